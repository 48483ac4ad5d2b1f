// Stress test of gpc::HostPool (host_pool.hpp): every index of every call runs
// exactly once, exceptions reach the caller, two callers take turns, and
// pools of several sizes and polling windows start and stop cleanly.  Built
// and run by tests/test_host_pool.py (optionally under ThreadSanitizer).
#include <cstdio>
#include <random>
#include <stdexcept>
#include "host_pool.hpp"
#include <atomic>
#include <cstdlib>
#include <thread>
#include <vector>
int main() {
  std::mt19937 rng(1);
  for (int round = 0; round < 20; ++round) {
    gpc::HostPool pool(1 + round % 7, round % 3 == 0 ? 0 : 50);
    std::vector<std::atomic<int>> hits(64);
    for (int it = 0; it < 300; ++it) {
      uint32_t n = rng() % 40;
      for (auto &h : hits) h = 0;
      bool thr = rng() % 10 == 0;
      try {
        pool.run(n, [&](uint32_t i, uint32_t) { hits[i]++; if (thr && i == n / 2) throw std::runtime_error("x"); });
        if (thr && n > 0) { printf("missing exception\n"); return 1; }
      } catch (const std::runtime_error &) {
        if (!thr) { printf("unexpected exception\n"); return 1; }
      }
      for (uint32_t i = 0; i < n; ++i) if (hits[i] != 1) { printf("index %u ran %d times\n", i, (int)hits[i]); return 1; }
      if (it % 50 == 0) std::this_thread::sleep_for(std::chrono::microseconds(rng() % 400));
    }
    // two callers taking turns
    std::thread a([&] { for (int k = 0; k < 200; ++k) { std::atomic<int> c{0}; pool.run(17, [&](uint32_t, uint32_t) { c++; }); if (c != 17) std::abort(); } });
    std::thread b([&] { for (int k = 0; k < 200; ++k) { std::atomic<int> c{0}; pool.run(9, [&](uint32_t, uint32_t) { c++; }); if (c != 9) std::abort(); } });
    a.join(); b.join();
  }
  printf("pool stress ok\n");
}
