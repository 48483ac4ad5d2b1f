// host_pool.hpp -- a persistent pool of parked host threads.
//
// The host half of one compile (parse + lower) takes a few hundred
// microseconds; creating threads for each call costs tens of microseconds
// per thread, waking parked ones a few.  A call runs fn(0..n-1) on the caller
// and whichever workers wake while indices remain; it returns once every
// index has run and no worker still holds the function.  fn also gets the
// slot of the thread running it (0 the caller, 1.. the workers), so per-thread
// scratch memory can be indexed by it.
#pragma once

#include <atomic>
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
  explicit HostPool(unsigned workers) {
    for (unsigned i = 0; i < workers; ++i) threads_.emplace_back([this, i] { loop(i + 1); });
  }
  ~HostPool() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      stop_ = true;
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
    {
      std::lock_guard<std::mutex> lk(mu_);
      fn_ = &fn;
      n_ = n;
      next_.store(0);
      err_ = nullptr;
      open_ = true;
      ++gen_;
    }
    wake_.notify_all();
    work(0);
    std::exception_ptr err;
    {
      std::unique_lock<std::mutex> lk(mu_);
      open_ = false;  // every index is taken: workers that wake from now on stay out
      done_.wait(lk, [&] { return busy_ == 0; });
      fn_ = nullptr;
      err = err_;
    }
    if (err) std::rethrow_exception(err);
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
  void loop(uint32_t slot) {
    uint64_t seen = 0;
    std::unique_lock<std::mutex> lk(mu_);
    while (true) {
      wake_.wait(lk, [&] { return stop_ || gen_ != seen; });
      if (stop_) return;
      seen = gen_;
      if (!open_) continue;
      ++busy_;
      lk.unlock();
      work(slot);
      lk.lock();
      if (--busy_ == 0) done_.notify_all();
    }
  }

  std::vector<std::thread> threads_;
  std::mutex call_mu_, mu_, err_mu_;
  std::condition_variable wake_, done_;
  const std::function<void(uint32_t, uint32_t)> *fn_ = nullptr;
  uint32_t n_ = 0;
  std::atomic<uint32_t> next_{0};
  std::exception_ptr err_;
  uint64_t gen_ = 0;
  unsigned busy_ = 0;
  bool open_ = false, stop_ = false;
};

}  // namespace gpc
