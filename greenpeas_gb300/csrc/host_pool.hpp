// host_pool.hpp -- a persistent pool of host threads.
//
// The host half of one compile (parse + lower + staging + fetch) takes a few
// hundred microseconds and hands work to the pool several times.  Creating
// threads for each hand-off costs tens of microseconds per thread, and so
// does waking threads parked on a condition variable (one futex wake after
// another).  So a worker that finishes keeps polling the call counter for a
// short while (spin_us, yielding its core between polls) before it parks: the
// hand-offs of one compile then reach running threads.  A call runs
// fn(0..n-1) on the caller and whichever workers join while indices remain;
// it returns once every index has run and no worker still holds the function.
// fn also gets the slot of the thread running it (0 the caller, 1.. the
// workers), so per-thread scratch memory can be indexed by it.
#pragma once

#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdint>
#include <exception>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace gpc {

class HostPool {
 public:
  explicit HostPool(unsigned workers, unsigned spin_us = 200) : spin_(std::chrono::microseconds(spin_us)) {
    for (unsigned i = 0; i < workers; ++i) threads_.emplace_back([this, i] { loop(i + 1); });
  }
  ~HostPool() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      stop_.store(true);
    }
    wake_.notify_all();
    for (auto &t : threads_) t.join();
  }
  HostPool(const HostPool &) = delete;
  HostPool &operator=(const HostPool &) = delete;

  unsigned workers() const { return (unsigned)threads_.size(); }

  // Runs fn(i, slot) for every i in [0, n); rethrows the first exception.
  // Calls from several threads take turns; fn must not call run() on the
  // same pool (the call would wait for its own turn).
  void run(uint32_t n, const std::function<void(uint32_t, uint32_t)> &fn) {
    if (n == 0) return;
    if (n == 1 || threads_.empty()) {
      for (uint32_t i = 0; i < n; ++i) fn(i, 0);
      return;
    }
    std::lock_guard<std::mutex> turn(call_mu_);
    fn_ = &fn;
    n_ = n;
    next_.store(0);
    err_ = nullptr;
    open_.store(true);
    gen_.fetch_add(1);
    if (parked_.load() > 0) {
      // a parked worker tests gen_ under mu_: taking it here orders this
      // call's gen_ before that test or the worker's wait before the notify
      { std::lock_guard<std::mutex> lk(mu_); }
      wake_.notify_all();
    }
    work(0);
    // every index is taken: workers that look from now on stay out; wait for
    // those inside (they finish their last index)
    open_.store(false);
    while (busy_.load() != 0) std::this_thread::yield();
    fn_ = nullptr;
    if (err_) std::rethrow_exception(err_);
  }

 private:
  void work(uint32_t slot) {
    for (uint32_t i; (i = next_.fetch_add(1)) < n_;) {
      try {
        (*fn_)(i, slot);
      } catch (...) {
        std::lock_guard<std::mutex> lk(err_mu_);
        if (!err_) err_ = std::current_exception();
      }
    }
  }
  // Joins the open call, if any.  busy_ is raised before open_ is read (both
  // sequentially consistent), so a caller that closed the call and then sees
  // busy_ == 0 has no worker left inside it.
  void join(uint32_t slot) {
    busy_.fetch_add(1);
    if (open_.load()) work(slot);
    busy_.fetch_sub(1);
  }
  void loop(uint32_t slot) {
    uint64_t seen = 0;
    while (true) {
      // poll for the next call for a while, then park
      const auto t0 = std::chrono::steady_clock::now();
      uint64_t g;
      while ((g = gen_.load()) == seen && !stop_.load()) {
        if (std::chrono::steady_clock::now() - t0 > spin_) break;
        std::this_thread::yield();
      }
      if (g == seen) {
        std::unique_lock<std::mutex> lk(mu_);
        parked_.fetch_add(1);
        wake_.wait(lk, [&] { return stop_.load() || gen_.load() != seen; });
        parked_.fetch_sub(1);
        g = gen_.load();
      }
      if (stop_.load()) return;
      seen = g;
      join(slot);
    }
  }

  std::vector<std::thread> threads_;
  const std::chrono::steady_clock::duration spin_;
  std::mutex call_mu_, mu_, err_mu_;
  std::condition_variable wake_;
  const std::function<void(uint32_t, uint32_t)> *fn_ = nullptr;
  uint32_t n_ = 0;
  std::atomic<uint32_t> next_{0};
  std::exception_ptr err_;
  std::atomic<uint64_t> gen_{0};
  std::atomic<int> busy_{0}, parked_{0};
  std::atomic<bool> open_{false}, stop_{false};
};

}  // namespace gpc
