// driver.cu -- the compile driver behind the C ABI (include/gpc.h).
//
// Counterpart of GreenPeas' Driver (QEC/ErrorAnalysis/Driver.hpp:37-219):
// it owns the device buffers (one arena that grows on demand instead of the
// reference's throw-on-overflow fitto, Driver.hpp:104-112), copies the tape
// host -> device with one asynchronous copy from pinned memory, runs the
// kernel pipeline on its own stream and copies back only the merged
// mechanisms (the reference copies the whole node x 32 class matrix,
// Driver.hpp:158-161).
#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <atomic>
#include <condition_variable>
#include <deque>
#include <exception>
#include <functional>
#include <mutex>
#include <unordered_map>
#include <thread>
#include <cstdio>
#include <cstring>
#include <limits>
#include <memory>
#include <string>
#include <vector>

#include "../../include/gpc.h"
#include "device.cuh"
#include "host_pool.hpp"
#include "lower.hpp"

using gpc::CircuitDev;
using gpc::Tape;

namespace {

thread_local std::string g_last_error;

gpc_status fail(gpc_status code, const std::string &msg) {
  g_last_error = msg;
  return code;
}

struct CudaError : std::runtime_error {
  explicit CudaError(const std::string &m) : std::runtime_error(m) {}
};

#define CK(x)                                                                                          \
  do {                                                                                                 \
    cudaError_t e_ = (x);                                                                              \
    if (e_ != cudaSuccess) throw CudaError(std::string(#x) + ": " + cudaGetErrorString(e_));          \
  } while (0)

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Runs fn(i) for i in [0, n) on up to `threads` host threads (the calling
// thread is one of them); rethrows the first exception after all joined.
uint32_t host_threads() { return std::max(1u, std::thread::hardware_concurrency()); }

// Device allocations of one driver: counted, and (a test of the failure
// path) the allocation numbered fail_at fails once as if the device were out
// of memory.
struct AllocCounter {
  uint64_t allocs = 0, frees = 0;
  int64_t fail_at = -1;  // -1: never
};

// Grow-only device allocation.
struct DevBuf {
  void *p = nullptr;
  size_t cap = 0;
  AllocCounter *ctr = nullptr;
  // A buffer that grows takes half again its old size when that is more (so
  // sizes that creep up, such as a batch's, do not reallocate every time);
  // off where an admission budget counts the exact bytes.
  bool slack = true;
  void ensure(size_t bytes) {
    if (bytes <= cap) return;
    const size_t old = cap;
    if (p) {
      CK(cudaFree(p));
      if (ctr) ++ctr->frees;
    }
    p = nullptr;
    cap = 0;
    if (ctr && ctr->fail_at >= 0 && ctr->allocs == (uint64_t)ctr->fail_at) {
      ctr->fail_at = -1;
      throw gpc::Error(GPC_ERR_OOM, "device allocation of " + std::to_string(bytes) + " bytes failed (injected)");
    }
    size_t want = slack ? std::max(bytes, old + old / 2) : bytes;
    cudaError_t e = cudaMalloc(&p, want);
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      e = cudaMalloc(&p, bytes);
      if (e != cudaSuccess) {
        (void)cudaGetLastError();
        throw gpc::Error(GPC_ERR_OOM, "device allocation of " + std::to_string(bytes) + " bytes failed");
      }
      want = bytes;
    }
    cap = want;
    if (ctr) ++ctr->allocs;
  }
  void release() {
    if (p) {
      cudaFree(p);
      if (ctr) ++ctr->frees;
    }
    p = nullptr;
    cap = 0;
  }
};

// Grow-only pinned host allocation.
struct HostBuf {
  void *p = nullptr;
  size_t cap = 0;
  void ensure(size_t bytes) {
    if (bytes <= cap) return;
    const size_t old = cap;  // (grows by half again, as DevBuf)
    if (p) CK(cudaFreeHost(p));
    p = nullptr;
    cap = 0;
    size_t want = std::max(bytes, old + old / 2);
    if (cudaHostAlloc(&p, want, cudaHostAllocDefault) != cudaSuccess) {
      (void)cudaGetLastError();
      throw gpc::Error(GPC_ERR_OOM, "pinned host allocation failed");
    }
    cap = want;
  }
  void release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
  }
};

// Byte offsets of one circuit's input arrays inside the arena.
struct CircLayout {
  size_t ops, ep_opoff, ep_k, ep_ptoff, ep_chunk, ch_off, ch_bytes, inj_lo, inj_hi, rec, rec_p, rec_moff, rec_src;
  size_t snap, band, nzm;
  uint32_t mbase, bbase, bbits;
};

// One walk launch: circuits with the same thread count, or (queue) every
// circuit of a batch in one persistent launch sized for the largest.
struct WalkClass {
  uint32_t qpad, item0, n_items, chunk_cap, max_epochs, max_chunks, words, qpt, queue;
};

// Byte offsets of every array inside the arena (staged inputs first, so they
// are one contiguous H2D copy; then the ops of tapes in page-locked memory,
// one copy each).
struct Layout {
  std::vector<CircLayout> c;
  size_t cdev, items, mbase, cbbase;
  size_t in_bytes;
  size_t ext_ops;  // bytes of page-locked tape ops
  size_t mdesc, mp, tl, tn, key, blk_r0, slot, bagg, bout, cout, big_list;
  size_t zero, err, totals, bcount, tsum, big_n, wq, zero_bytes;
  size_t sk0, sk1, pm0, pm1, hik;  // global path (single circuit)
  size_t src_off, src_rec, gq, grad_rec, ptab;  // noise-rate gradients (single circuit)
  size_t gzero, sort_scr, merge_status, merge_ctr, gzero_bytes;
  size_t out_prob, out_off;
  size_t seg_items, seg_aff, seg_state, seg_xcnt, seg_xlst;  // segmented walk (single circuit)
  size_t total;
  uint32_t M, nb, n_items;
  uint32_t sort_tiles, merge_tiles;
  size_t sort_words;
  std::vector<WalkClass> classes;
};

}  // namespace

namespace {
// Page-locked host memory, recycled by size class.  Freeing page-locked
// memory is slow and may wait for the device, so a freed buffer goes back to
// the free list of its class (two classes per power of two, from 64 KiB) and
// is handed out again.  At most kCapBytes are allocated; past that take()
// returns null and the caller uses the heap (staged copies).  Never destroyed
// (buffers may come back during process exit).
class PinnedPool {
 public:
  static size_t class_of(size_t bytes) {
    size_t c = (size_t)64 << 10;
    while (c < bytes) {
      const size_t mid = c + c / 2;  // between c and 2c
      if (mid >= bytes) return mid;
      c *= 2;
    }
    return c;
  }
  void *take(size_t bytes) {
    const size_t c = class_of(bytes);
    std::vector<void *> victims;
    bool room = false;
    {
      std::lock_guard<std::mutex> lk(mu_);
      auto &f = free_[c];
      if (!f.empty()) {
        void *p = f.back();
        f.pop_back();
        return p;
      }
      if (total_ + c > kCapBytes) {
        // make room from blocks of other sizes kept free (the largest first), so
        // that sizes of an earlier workload do not hold the pool from a later one
        std::vector<size_t> classes;
        for (auto &kv : free_)
          if (!kv.second.empty()) classes.push_back(kv.first);
        std::sort(classes.begin(), classes.end(), std::greater<size_t>());
        for (size_t k : classes) {
          auto &v = free_[k];
          while (!v.empty() && total_ + c > kCapBytes) {
            victims.push_back(v.back());
            v.pop_back();
            total_ -= k;
          }
          if (total_ + c <= kCapBytes) break;
        }
      }
      room = total_ + c <= kCapBytes;
      if (room) total_ += c;
    }
    for (void *q : victims) cudaFreeHost(q);
    if (!room) return nullptr;
    void *p = nullptr;
    if (cudaHostAlloc(&p, c, cudaHostAllocPortable) != cudaSuccess) {
      cudaGetLastError();
      std::lock_guard<std::mutex> lk(mu_);
      total_ -= c;
      return nullptr;
    }
    return p;
  }
  void give(void *p, size_t bytes) {
    if (!p) return;
    std::lock_guard<std::mutex> lk(mu_);
    free_[class_of(bytes)].push_back(p);
  }

 private:
  static constexpr size_t kCapBytes = (size_t)4 << 30;
  std::mutex mu_;
  std::unordered_map<size_t, std::vector<void *>> free_;
  size_t total_ = 0;
};
PinnedPool &pinned_pool() {
  static PinnedPool *p = new PinnedPool;
  return *p;
}

// Tape ops in page-locked memory (the device copy is made straight from them).
void *pinned_alloc(size_t bytes) { return pinned_pool().take(bytes); }
void pinned_free(void *p, size_t bytes) { pinned_pool().give(p, bytes); }
void pin_ops(Tape &T) { T.ops.set_allocator(pinned_alloc, pinned_free); }

// A DEM's host array: heap memory, or pinned memory that the device copies a
// single-circuit result into directly.  resize() keeps no contents (the array
// is written in full right after it is sized); pinned capacity grows with a
// quarter of slack, since cudaHostAlloc is slow.
template <typename T>
class DemArray {
 public:
  explicit DemArray(bool pinned = false) : pinned_(pinned) {}
  DemArray(const DemArray &) = delete;
  DemArray &operator=(const DemArray &) = delete;
  ~DemArray() { release(); }
  void resize(size_t m) {
    if (m > cap_) {
      release();
      const size_t want = pinned_ ? m + m / 4 : m;
      if (pinned_) {
        void *q = pinned_pool().take(want * sizeof(T));
        if (!q) throw gpc::Error(GPC_ERR_CUDA, "no page-locked memory for a DEM array");
        p_ = static_cast<T *>(q);
      } else {
        p_ = static_cast<T *>(::operator new(want * sizeof(T)));
      }
      cap_ = want;
    }
    n_ = m;
  }
  // Views n elements at p (memory owned elsewhere: a batch's result block);
  // the array's own buffer is released.
  void view(T *p, size_t n) {
    release();
    p_ = p;
    n_ = n;
    view_ = true;
  }
  void clear() {
    if (view_) release();
    n_ = 0;
  }
  T *data() { return p_; }
  const T *data() const { return p_; }
  size_t size() const { return n_; }
  size_t capacity() const { return cap_; }
  T &operator[](size_t i) { return p_[i]; }
  const T &operator[](size_t i) const { return p_[i]; }

 private:
  void release() {
    if (p_ && !view_) {
      if (pinned_)
        pinned_pool().give(p_, cap_ * sizeof(T));
      else
        ::operator delete(p_);
    }
    p_ = nullptr;
    n_ = cap_ = 0;
    view_ = false;
  }
  T *p_ = nullptr;
  size_t n_ = 0, cap_ = 0;
  bool pinned_;
  bool view_ = false;
};

// Page-locked memory that one batch's DEM arrays are copied back into.  The
// batch's DEMs view their probabilities and targets in it and share it; the
// last one freed gives it back to the page-locked pool.  When the pool has
// none to give (a caller holding many results), the DEMs own heap copies.
// Single circuits use pinned DEMs instead.
struct ResultBlock {
  void *p = nullptr;
  size_t cap = 0;
};
std::shared_ptr<ResultBlock> take_block(size_t bytes) {
  void *p = pinned_pool().take(bytes);
  if (!p) return nullptr;
  return std::shared_ptr<ResultBlock>(new ResultBlock{p, bytes}, [](ResultBlock *b) {
    pinned_pool().give(b->p, b->cap);
    delete b;
  });
}
}  // namespace

struct gpc_dem {  // arrays written in full right after they are sized
  explicit gpc_dem(bool pin = false) : probs(pin), offsets(pin), targets(pin), pinned(pin) {}
  DemArray<double> probs;
  DemArray<uint32_t> offsets;
  DemArray<uint32_t> targets;
  const bool pinned;
  std::shared_ptr<ResultBlock> block;  // the batch result block its probabilities and targets view
  uint32_t num_detectors = 0, num_observables = 0;
  uint64_t num_raw = 0;
  std::string text;
  bool text_ready = false;
};

namespace {
// DEMs freed by the caller keep their host arrays for the next fetch, up to a
// bound: a repeated compile then writes its result into memory that is
// already mapped instead of faulting in fresh pages (a [[144,12,12]] DEM is
// ~3 MB).  The cache is never destroyed (DEMs may be freed during process
// exit); what it holds at exit is returned with the process.
class DemCache {
 public:
  gpc_dem *take() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      if (!free_.empty()) {
        gpc_dem *d = free_.back();
        free_.pop_back();
        bytes_ -= size_of(d);
        return d;
      }
    }
    return new gpc_dem;
  }
  // A DEM with pinned arrays (a single-circuit fetch copies into it), or null
  // when kMaxPinned of them exist already (the caller holds them): pinned
  // memory stays bounded, and such a caller gets heap DEMs.
  gpc_dem *take_pinned() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      if (!free_pinned_.empty()) {
        gpc_dem *d = free_pinned_.back();
        free_pinned_.pop_back();
        return d;
      }
      if (live_pinned_ >= kMaxPinned) return nullptr;
      ++live_pinned_;
    }
    return new gpc_dem(true);
  }
  void give(gpc_dem *d) {
    d->probs.clear();  // sizes 0: a later resize past the capacity copies nothing (views dropped)
    d->offsets.clear();
    d->targets.clear();
    d->block.reset();
    std::string().swap(d->text);
    d->text_ready = false;
    d->num_detectors = d->num_observables = 0;
    d->num_raw = 0;
    if (d->pinned) {  // kept: at most kMaxPinned exist
      std::lock_guard<std::mutex> lk(mu_);
      free_pinned_.push_back(d);
      return;
    }
    const size_t b = size_of(d);
    {
      std::lock_guard<std::mutex> lk(mu_);
      if (free_.size() < kMaxDems && bytes_ + b <= kMaxBytes) {
        free_.push_back(d);
        bytes_ += b;
        return;
      }
    }
    delete d;
  }
  // A pinned DEM that failed to fill (its arrays could not grow): freed, not kept.
  void drop_pinned(gpc_dem *d) {
    delete d;
    std::lock_guard<std::mutex> lk(mu_);
    --live_pinned_;
  }

 private:
  static size_t size_of(const gpc_dem *d) {
    return d->probs.capacity() * 8 + (d->offsets.capacity() + d->targets.capacity()) * 4;
  }
  // (a batch's DEMs come back together: enough for one batch's offsets arrays)
  static constexpr size_t kMaxDems = 1024, kMaxBytes = (size_t)128 << 20, kMaxPinned = 4;
  std::mutex mu_;
  std::vector<gpc_dem *> free_, free_pinned_;
  size_t bytes_ = 0, live_pinned_ = 0;
};
DemCache &dem_cache() {
  static DemCache *c = new DemCache;
  return *c;
}
}  // namespace

namespace {
// Walk configurations chosen by gpc_autotune, kept for the process and keyed
// by the bitset widths of the batch they were tuned on: the set of its
// circuits' (walk slot count, detector words rounded up to a power of two)
// classes.  A coarse key on purpose: the chunks of a large batch, and other
// batches of the same workload, hold the same classes.  A batch prepared
// without explicit walk options on a driver that has not tuned itself takes
// the configuration cached for its key (the DEMs do not depend on it).
class TuneCache {
 public:
  bool get(uint64_t key, uint32_t cfg[3]) {
    std::lock_guard<std::mutex> lk(mu_);
    auto it = map_.find(key);
    if (it == map_.end()) return false;
    for (int k = 0; k < 3; ++k) cfg[k] = it->second[k];
    return true;
  }
  void put(uint64_t key, const uint32_t cfg[3]) {
    std::lock_guard<std::mutex> lk(mu_);
    map_[key] = {cfg[0], cfg[1], cfg[2]};
  }
  void clear() {
    std::lock_guard<std::mutex> lk(mu_);
    map_.clear();
  }

 private:
  std::mutex mu_;
  std::unordered_map<uint64_t, std::array<uint32_t, 3>> map_;
};
TuneCache &tune_cache() {
  static TuneCache *c = new TuneCache;
  return *c;
}
}  // namespace

struct gpc_driver {
  int device = 0;
  int level = 2;
  uint32_t sort_bits = 64;
  cudaStream_t stream = nullptr;
  static constexpr int kAux = 4;
  cudaStream_t aux[kAux] = {};
  cudaEvent_t fork_ev = nullptr, join_ev[kAux] = {};
  std::vector<Tape> tapes;
  std::vector<gpc::LowerScratch> lower_scratch;  // host memory of parse + lower, one per pool slot
  std::unique_ptr<gpc::HostPool> pool;            // host threads of this driver (made on first use)
  uint32_t pool_threads = 0;  // threads of the host pool, the caller included (0: every host thread)
  uint32_t pool_spin_us = 200;  // how long an idle pool thread polls for the next hand-off before parking
  gpc::HostPool &host_pool() {
    if (!pool) pool.reset(new gpc::HostPool((pool_threads ? pool_threads : host_threads()) - 1, pool_spin_us));
    return *pool;
  }
  // Circuit indices by decreasing size (the order batch work is handed out in).
  std::vector<uint32_t> big_first;
  template <typename F>
  void order_by_size(uint32_t n, F &&size) {
    big_first.resize(n);
    for (uint32_t i = 0; i < n; ++i) big_first[i] = i;
    std::stable_sort(big_first.begin(), big_first.end(), [&](uint32_t a, uint32_t b) { return size(a) > size(b); });
  }
  // Pieces of a large host copy: one per pool thread, at most 16.
  uint32_t copy_pieces() { return std::min<uint32_t>(16u, host_pool().workers() + 1); }
  // fn(i, slot) for i < n, on the host pool when `parallel`.
  void for_each(uint32_t n, bool parallel, const std::function<void(uint32_t, uint32_t)> &fn) {
    if (!parallel || n < 2) {
      for (uint32_t i = 0; i < n; ++i) fn(i, 0);
      return;
    }
    host_pool().run(n, fn);
  }
  bool have_tape = false;
  bool prepared = false;
  bool ran = false;
  Layout L{};
  AllocCounter alloc_ctr;
  DevBuf arena{nullptr, 0, &alloc_ctr}, tgbuf{nullptr, 0, &alloc_ctr};
  HostBuf pin_in, pin_out;
  uint32_t tg_cap = 0;
  cudaEvent_t ev[5] = {};
  cudaEvent_t tune_ev[2] = {};  // the autotuner's timing of whole runs
  // last run's global-path sort result
  uint32_t *perm_sorted = nullptr;
  uint64_t *sk_sorted = nullptr;
  uint64_t sort_mask = ~0ull;
  bool force_global = false;  // test option: skip the bucket path (single circuits)
  uint32_t walk_qpt = 0;      // qubits per walk thread (0: chosen per circuit)
  uint32_t walk_words = 0;    // detector words per walk CTA (0: two in batches, one for a single circuit)
  uint32_t bucket_mean = 0;   // target mechanisms per bucket (0: from the run's size; buckets are a power of two per circuit)
  uint32_t batch_words = 0, batch_qpt = 0;  // walk configuration of batches chosen by autotune (0: defaults)
  uint32_t batch_queue = 0;                  // 1: batches walk in one persistent launch (autotune's choice)
  int walk_queue = 0;                        // option walk_queue: 1 always, -1 never, 0 batch_queue
  bool key_split = true;                     // split key pass for one circuit when it pays (option key_split)
  int walk_segment = 0;                      // option walk_segment: 0 when it pays, -1 never, > 0 target cost
  unsigned long long spin_ns = 200ull * 1000 * 1000;  // option wait_limit_us: global-path look-back waits
  uint32_t hold_runs = 0;  // option test_hold_tile: global-path runs left whose first sort tile stays unpublished
  // Segmented walk of the current circuit (single circuits; plan_segments):
  // the cut epochs, launch A's items then launch B's, each word's AFF state
  // per segment, and the state buffer's size.
  bool seg_on = false;
  std::vector<uint32_t> seg_bounds;
  std::vector<gpc::SegItem> seg_items;
  uint32_t seg_na = 0, seg_nb = 0;
  std::vector<uint32_t> seg_aff;  // [w][S]
  uint32_t seg_states = 0, seg_xfer0 = 0, seg_ncol = 0, seg_qpt = 1, seg_ring = 1;
  bool seg_band_reset = false;    // a word without measurements: its band is zeroed before the walk
  // host phases of the last prepare / fetch (ms): lower, layout, staging,
  // wait for the pipeline + result sizes, D2H copies, DEM split
  double host_ms[6] = {};
  using HostClock = std::chrono::steady_clock;
  static double ms_since(HostClock::time_point t) {
    return std::chrono::duration<double, std::milli>(HostClock::now() - t).count();
  }

  static bool walk_qpt_fits(uint32_t qpad, uint32_t q) {
    const uint32_t mt = gpc::walk_max_threads(q);
    return mt && qpad % (32u * q) == 0 && qpad / q <= mt;
  }
  // Qubits per walk thread for a tape of qpad qubit slots (`pref` if it fits).
  static uint32_t walk_qpt_for(uint32_t qpad, uint32_t pref) {
    if (pref && walk_qpt_fits(qpad, pref)) return pref;
    return qpad <= 1024 ? 1u : qpad <= 2048 ? 2u : 4u;
  }
  // Serving: called by prepare() with the device bytes it must add to the
  // resident buffers and the bytes of all its buffers, before allocating them
  // (may release the buffers, block or throw).
  std::function<void(size_t, size_t)> admit;
  size_t resident_bytes() const { return arena.cap + tgbuf.cap; }
  // Frees the device buffers (a later prepare allocates them again).
  void release_device_memory() {
    if (stream) cudaStreamSynchronize(stream);
    drop_graph();
    arena.release();
    tgbuf.release();
    tg_cap = 0;
    prepared = false;
    ran = false;
    last_run_sig = 0;
  }
  // noise-rate gradients: record probabilities come from a device noise tensor
  bool param = false;
  const double *noise_dev = nullptr;
  uint32_t param_groups = 0;
  cudaEvent_t caller_ev = nullptr, done_ev = nullptr;
  cudaGraph_t graph = nullptr;  // captured kernel sequence of run() for one launch configuration
  cudaGraphExec_t graph_exec = nullptr;
  bool use_graph = true;
  uint64_t cfg_sig = 0, graph_sig = 0, last_run_sig = 0;
  uint32_t tcap = 32;      // target-list stride (grows when a symptom is longer)
  bool lists_off = false;  // symptoms too long for target lists: merge from snapshots
  uint64_t last_d2h = 0;   // bytes copied device -> host by the last fetch
  uint64_t last_h2d = 0;   // bytes copied host -> device by the last prepare (a chunked batch: all of its chunks)
  bool used_global = false;
  bool capturing = false;
  uint32_t ncirc() const { return (uint32_t)tapes.size(); }

  // Records timing event i on the stream (as a graph event node while capturing)
  // when stage timing is on.  Off by default: an event node between two
  // kernels of a captured graph costs ~4-5 us of the run (the [[144,12,12]]
  // pipeline: 105 -> 90 us without the three inner ones).
  bool stage_timing = false;
  bool timed_run = false;  // the last run recorded the stage events
  void rec(int i) {
    if (!stage_timing) return;
    if (capturing) CK(cudaEventRecordWithFlags(ev[i], stream, cudaEventRecordExternal));
    else CK(cudaEventRecord(ev[i], stream));
  }

  void drop_graph() {
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
    if (graph) cudaGraphDestroy(graph);
    graph_exec = nullptr;
    graph = nullptr;
    graph_sig = 0;
  }

  ~gpc_driver() {
    if (stream) cudaStreamSynchronize(stream);
    drop_graph();
    arena.release();
    tgbuf.release();
    pin_in.release();
    pin_out.release();
    for (auto &e : ev)
      if (e) cudaEventDestroy(e);
    for (auto &e : tune_ev)
      if (e) cudaEventDestroy(e);
    if (fork_ev) cudaEventDestroy(fork_ev);
    if (caller_ev) cudaEventDestroy(caller_ev);
    if (done_ev) cudaEventDestroy(done_ev);
    if (wait_ev) cudaEventDestroy(wait_ev);
    if (fetch_ev) cudaEventDestroy(fetch_ev);
    for (auto &e : join_ev)
      if (e) cudaEventDestroy(e);
    for (auto &a : aux)
      if (a) cudaStreamDestroy(a);
    if (stream) cudaStreamDestroy(stream);
  }

  // Waits for the driver's stream.  A server worker sleeps in the wait (an
  // event with blocking sync) so the lowering threads get its core while the
  // GPU runs its batch; otherwise the CUDA default (a spinning wait, lowest
  // latency) applies.
  bool blocking_wait = false;
  cudaEvent_t wait_ev = nullptr;
  void wait() {
    if (blocking_wait) {
      CK(cudaEventRecord(wait_ev, stream));
      CK(cudaEventSynchronize(wait_ev));
    } else {
      CK(cudaStreamSynchronize(stream));
    }
    ops_in_flight = false;
  }
  // A copy of page-locked tape ops to the device may still be reading them
  // (set by prepare, cleared by wait): the tapes are not rewritten or handed
  // back before the stream has caught up.
  bool ops_in_flight = false;

  void init_streams() {
    CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&wait_ev, cudaEventBlockingSync | cudaEventDisableTiming));
    for (auto &a : aux) CK(cudaStreamCreateWithFlags(&a, cudaStreamNonBlocking));
    for (auto &e : ev) CK(cudaEventCreate(&e));
    for (auto &e : tune_ev) CK(cudaEventCreate(&e));
    CK(cudaEventCreateWithFlags(&fork_ev, cudaEventDisableTiming));
    for (auto &e : join_ev) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }

  template <typename T>
  T *dptr(size_t off) const {
    return reinterpret_cast<T *>(static_cast<char *>(arena.p) + off);
  }

  void layout() {
    const uint32_t N = ncirc();
    size_t o = 0;
    auto take = [&](size_t bytes) {
      size_t r = o;
      o = align256(o + bytes);
      return r;
    };
    L.c.assign(N, CircLayout{});
    uint64_t M = 0, nb = 0, items = 0;
    // Bucket size, from each circuit's own mechanism count (so a circuit gets
    // the same buckets, and bit for bit the same DEM, alone and in a batch):
    // small circuits are latency-bound and want more buckets (more warps in
    // the grouping, fewer oversized buckets), large ones fewer (less
    // per-bucket work).  Measured on GB300: 16 mechanisms per bucket up to
    // 16k mechanisms, 48 up to 256k, then 96.
    auto bmean_of = [&](uint64_t m) -> uint64_t {
      return bucket_mean ? bucket_mean : m <= (16u << 10) ? 16 : m <= (256u << 10) ? 48 : 96;
    };
    for (uint32_t i = 0; i < N; ++i) {
      const Tape &T = tapes[i];
      CircLayout &c = L.c[i];
      c.ops = T.ops.external() ? 0 : take(T.ops.size() * 8);  // page-locked ops: placed below
      c.ep_opoff = take(T.ep_opoff.size() * 4);
      c.ep_k = take(T.ep_k.size() * 4);
      c.ep_ptoff = take(T.ep_ptoff.size() * 4);
      c.ep_chunk = take(T.ep_chunk.size() * 4);
      c.ch_off = take(T.ch_off.size() * 4);
      c.ch_bytes = take(T.ch_bytes.size() * 4);
      c.inj_lo = take(T.inj_lo.size() * 4);
      c.inj_hi = take(T.inj_hi.size() * 4);
      c.rec = take(T.rec.size() * 8);
      c.rec_p = take(T.rec_p.size() * 8);
      c.rec_moff = take(T.rec_moff.size() * 4);
      c.rec_src = take(param ? T.rec_src.size() * 4 : 0);  // record sources: read by the gradient kernels only
      // buckets: about bucket_mean mechanisms each, a power of two between 2^4 and 2^18
      uint32_t bb = 4;
      while (bb < 18 && (bmean_of(T.M) << bb) < T.M) ++bb;
      c.mbase = (uint32_t)M;
      c.bbase = (uint32_t)nb;
      c.bbits = bb;
      M += T.M;
      nb += 1ull << bb;
      items += T.w;
    }
    if (M >= 0xFFFFFFF0ull || nb >= 0x7FFFFFFFull) throw gpc::Error(GPC_ERR_CAPACITY, "batch too large");
    L.M = (uint32_t)M;
    L.nb = (uint32_t)nb;
    L.n_items = (uint32_t)items;
    L.cdev = take((size_t)N * sizeof(CircuitDev));
    L.items = take((size_t)items * sizeof(uint2));
    L.mbase = take((size_t)(N + 1) * 4);
    L.cbbase = take((size_t)N * 4);
    L.seg_items = take(seg_on ? seg_items.size() * sizeof(gpc::SegItem) : 0);
    L.seg_aff = take(seg_on ? seg_aff.size() * 4 : 0);
    if (param) {
      L.src_off = take(((size_t)tapes[0].n_ticks * gpc::SRC_CLASSES + 1) * 4);
      L.src_rec = take(tapes[0].rec.size() * 4);
    }
    L.in_bytes = o;  // the staged inputs (one copy from pinned memory)
    // ops in page-locked tape memory: copied to the device straight from it, one copy per tape
    L.ext_ops = 0;
    for (uint32_t i = 0; i < N; ++i)
      if (tapes[i].ops.external()) {
        L.c[i].ops = take(tapes[i].ops.size() * 8);
        L.ext_ops += tapes[i].ops.size() * 8;
      }
    for (uint32_t i = 0; i < N; ++i) {
      L.c[i].snap = take((size_t)tapes[i].w * tapes[i].npoints * 16);
      L.c[i].band = take((size_t)tapes[i].w * 8);
    }
    L.mdesc = take((size_t)M * 8);
    L.mp = take((size_t)M * 8);
    L.tl = take((size_t)M * tcap * 4);
    L.tn = take((size_t)M * 4);
    L.key = take((size_t)M * 16);
    L.blk_r0 = take((size_t)gpc::key_blocks((uint32_t)M) * 8);
    const size_t slots = (size_t)nb * gpc::SLOT_CAP;
    L.slot = take(slots * sizeof(gpc::Slot));
    L.bagg = take((size_t)nb * 8);
    L.bout = take((size_t)nb * 8);
    L.cout = take((size_t)N * 8);
    L.big_list = take((size_t)nb * 4);
    L.zero = o;
    L.err = take(4);
    L.totals = take(16);
    L.big_n = take(4);
    L.wq = take(4);
    L.bcount = take((size_t)nb * 4);
    L.tsum = take(((size_t)nb + gpc::SCAN_TILE - 1) / gpc::SCAN_TILE * 8);
    for (uint32_t i = 0; i < N; ++i)
      L.c[i].nzm = take((size_t)tapes[i].npoints * ((tapes[i].w + 63) / 64) * 8);
    const size_t seg_rows = seg_on ? (seg_bounds.size() - 1) * (size_t)2 * tapes[0].qpad : 0;
    L.seg_xcnt = take(seg_rows * 4);
    L.zero_bytes = o - L.zero;
    L.out_prob = take((size_t)M * 8);
    L.out_off = take((size_t)(M + 1) * 4);
    L.seg_state = take(seg_on ? (size_t)seg_states * 2 * tapes[0].qpad * 8 : 0);
    L.seg_xlst = take(seg_rows * gpc::kSegRowCap * 2);
    // global path (single circuit only)
    const uint32_t Mg = N == 1 ? (uint32_t)M : 0;
    L.sk0 = take((size_t)Mg * 8);
    L.sk1 = take((size_t)Mg * 8);
    L.pm0 = take((size_t)Mg * 4);
    L.pm1 = take((size_t)Mg * 4);
    L.hik = take((size_t)Mg * 8);
    L.sort_tiles = gpc::sort_tiles(Mg);
    L.merge_tiles = gpc::merge_tiles(Mg);
    L.sort_words = Mg ? gpc::sort_scratch_words(Mg, 64) : 0;
    L.gq = take(param ? (size_t)M * 8 : 0);
    L.grad_rec = take(param ? tapes[0].rec.size() * 8 : 0);
    L.ptab = take(param ? (size_t)tapes[0].n_ticks * gpc::SRC_CLASSES * 6 * 8 : 0);  // q and dq/dp tables
    L.gzero = o;
    L.sort_scr = take(L.sort_words * 4);
    L.merge_status = take((size_t)L.merge_tiles * 8);
    L.merge_ctr = take(4);
    L.gzero_bytes = o - L.gzero;
    L.total = o;
    // walk classes: circuits with the same qpad share a launch
    std::vector<uint32_t> order(N);
    for (uint32_t i = 0; i < N; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return tapes[a].qpad < tapes[b].qpad; });
    L.classes.clear();
    circ_words.assign(N, 1);
    walk_items.clear();
    if (N > 1 && build_queue_class()) return;
    uint32_t item = 0;
    for (uint32_t k = 0; k < N;) {
      uint32_t e = k;
      WalkClass wc{tapes[order[k]].qpad, item, 0, 0, 0, 0, 1, 1, 0};
      while (e < N && tapes[order[e]].qpad == wc.qpad) {
        const Tape &T = tapes[order[e]];
        wc.chunk_cap = std::max(wc.chunk_cap, T.chunk_cap);
        wc.max_epochs = std::max(wc.max_epochs, T.n_epochs);
        wc.max_chunks = std::max(wc.max_chunks, (uint32_t)T.ch_off.size());
        ++e;
      }
      // words per CTA: two in batches (half the CTAs; the walk is a chain of
      // latency-bound epochs) when the qubits-per-thread instance and shared
      // memory allow; one for a single circuit (latency)
      const uint32_t want = walk_words ? walk_words : (N > 1 ? (batch_words ? batch_words : 2u) : 1u);
      const uint32_t q = walk_qpt_for(wc.qpad, walk_qpt ? walk_qpt : (N > 1 ? batch_qpt : 0u));
      wc.qpt = q;
      if (want == 2 && (q == 1 || q == 2) &&
          gpc::walk_smem_bytes(wc.qpad, wc.chunk_cap, gpc::walk_table_bytes(wc.max_epochs, wc.max_chunks), 2) <=
              227 * 1024 - 1024)
        wc.words = 2;
      for (uint32_t x = k; x < e; ++x) {
        const uint32_t i = order[x];
        circ_words[i] = wc.words;
        for (uint32_t j = 0; j < tapes[i].w; j += wc.words) walk_items.push_back(make_uint2(i, j));
        wc.n_items += (tapes[i].w + wc.words - 1) / wc.words;
      }
      item += wc.n_items;
      L.classes.push_back(wc);
      k = e;
    }
  }

  // One persistent walk launch over every circuit of a batch (option
  // walk_queue, or the autotuner's choice): block size and shared memory of
  // the largest circuit, items ordered by estimated walk length, longest
  // first.  False (classes instead) when not chosen or when it does not fit.
  bool build_queue_class() {
    const uint32_t N = ncirc();
    if (walk_queue < 0 || (walk_queue == 0 && !batch_queue)) return false;
    WalkClass wc{0, 0, 0, 0, 0, 0, 1, 1, 1};
    for (uint32_t i = 0; i < N; ++i) {
      const Tape &T = tapes[i];
      wc.qpad = std::max(wc.qpad, T.qpad);
      wc.chunk_cap = std::max(wc.chunk_cap, T.chunk_cap);
      wc.max_epochs = std::max(wc.max_epochs, T.n_epochs);
      wc.max_chunks = std::max(wc.max_chunks, (uint32_t)T.ch_off.size());
    }
    const uint32_t want = walk_words ? walk_words : (batch_words ? batch_words : 2u);
    const uint32_t q = walk_qpt ? walk_qpt : (batch_qpt ? batch_qpt : 1u);
    wc.qpad = (wc.qpad + 32 * q - 1) / (32 * q) * (32 * q);  // q slots per thread, whole warps
    if (!gpc::walk_queue_supported(q, want) || wc.qpad / q > gpc::walk_max_threads(q)) return false;
    if (gpc::walk_smem_bytes(wc.qpad, wc.chunk_cap, gpc::walk_table_bytes(wc.max_epochs, wc.max_chunks), want) >
        227 * 1024 - 1024)
      return false;
    wc.qpt = q;
    wc.words = want;
    // estimated walk length of an item: its epochs (words holding observables
    // walk to the end; detector words stop a little after their last
    // injection) times the CTA's active warps plus a fixed cost per epoch
    std::vector<std::pair<uint64_t, uint2>> est;
    for (uint32_t i = 0; i < N; ++i) {
      const Tape &T = tapes[i];
      circ_words[i] = want;
      for (uint32_t j0 = 0; j0 < T.w; j0 += want) {
        uint32_t e0 = 0xFFFFFFFFu, e1 = 0;
        bool obs = false;
        for (uint32_t j = j0; j < std::min(T.w, j0 + want); ++j) {
          if ((uint64_t)(j + 1) * 64 > T.ndet) obs = true;
          if (T.inj_lo[j] == 0xFFFFFFFFu || T.inj_lo[j] >= T.n_epochs) continue;
          e0 = std::min(e0, T.inj_lo[j]);
          e1 = std::max(e1, T.inj_hi[j]);
        }
        const uint64_t ep = e0 == 0xFFFFFFFFu ? 0 : (obs ? T.n_epochs : std::min(T.n_epochs, e1 + 16)) - e0;
        est.push_back({ep * (T.qpad / 32 + 8), make_uint2(i, j0)});
      }
    }
    std::stable_sort(est.begin(), est.end(), [](const auto &a, const auto &b) { return a.first > b.first; });
    for (const auto &x : est) walk_items.push_back(x.second);
    wc.n_items = (uint32_t)walk_items.size();
    L.classes.push_back(wc);
    return true;
  }
  std::vector<uint2> walk_items;     // (circuit, first word) of each walk CTA, in launch order
  std::vector<uint32_t> circ_words;  // detector words per walk CTA of each circuit

  void stage_inputs() {
    const uint32_t N = ncirc();
    pin_in.ensure(L.in_bytes);
    char *h = static_cast<char *>(pin_in.p);
    auto put = [&](size_t off, const void *src, size_t bytes) {
      if (bytes) memcpy(h + off, src, bytes);
    };
    std::vector<CircuitDev> cd(N);
    std::vector<uint32_t> mb(N + 1), cb(N);
    // circuits fill disjoint regions of the staging buffer: a batch copies in parallel
    order_by_size(N, [&](uint32_t i) { return (uint64_t)tapes[i].ops.size() + tapes[i].rec.size(); });
    for_each(N, N >= 8, [&](uint32_t x, uint32_t) {
      const uint32_t i = big_first[x];
      const Tape &T = tapes[i];
      const CircLayout &l = L.c[i];
      struct Copy {
        size_t off;
        const void *src;
        size_t bytes;
      };
      const Copy cs[] = {{l.ops, T.ops.data(), T.ops.external() ? 0 : T.ops.size() * 8},
                         {l.ep_opoff, T.ep_opoff.data(), T.ep_opoff.size() * 4},
                         {l.ep_k, T.ep_k.data(), T.ep_k.size() * 4},
                         {l.ep_ptoff, T.ep_ptoff.data(), T.ep_ptoff.size() * 4},
                         {l.ep_chunk, T.ep_chunk.data(), T.ep_chunk.size() * 4},
                         {l.ch_off, T.ch_off.data(), T.ch_off.size() * 4},
                         {l.ch_bytes, T.ch_bytes.data(), T.ch_bytes.size() * 4},
                         {l.inj_lo, T.inj_lo.data(), T.inj_lo.size() * 4},
                         {l.inj_hi, T.inj_hi.data(), T.inj_hi.size() * 4},
                         {l.rec, T.rec.data(), T.rec.size() * 8},
                         {l.rec_p, T.rec_p.data(), T.rec_p.size() * 8},
                         {l.rec_moff, T.rec_moff.data(), T.rec_moff.size() * 4},
                         {l.rec_src, T.rec_src.data(), param ? T.rec_src.size() * 4 : 0}};
      size_t total = 0;
      for (const Copy &c : cs) total += c.bytes;
      // one large circuit: its arrays are copied as pieces of equal size on the host pool
      // (one thread's copy rate into pinned memory would dominate the staging)
      const uint32_t np = N == 1 && total >= (256u << 10) ? copy_pieces() : 1u;
      for_each(np, np > 1, [&](uint32_t q, uint32_t) {
        const size_t b0 = total * q / np, b1 = total * (q + 1) / np;
        size_t at = 0;
        for (const Copy &c : cs) {
          const size_t lo = std::max(b0, at), hi = std::min(b1, at + c.bytes);
          if (hi > lo) put(c.off + (lo - at), static_cast<const char *>(c.src) + (lo - at), hi - lo);
          at += c.bytes;
        }
      });
      CircuitDev &c = cd[i];
      c = CircuitDev{};
      c.ops = dptr<uint64_t>(l.ops);
      c.ep_opoff = dptr<uint32_t>(l.ep_opoff);
      c.ep_k = dptr<uint32_t>(l.ep_k);
      c.ep_ptoff = dptr<uint32_t>(l.ep_ptoff);
      c.ep_chunk = dptr<uint32_t>(l.ep_chunk);
      c.ch_off = dptr<uint32_t>(l.ch_off);
      c.ch_bytes = dptr<uint32_t>(l.ch_bytes);
      c.inj_lo = dptr<uint32_t>(l.inj_lo);
      c.inj_hi = dptr<uint32_t>(l.inj_hi);
      c.snap = dptr<ulonglong2>(l.snap);
      c.band = dptr<uint2>(l.band);
      c.nzm = dptr<unsigned long long>(l.nzm);
      c.mw = (T.w + 63) / 64;
      c.rec = dptr<uint64_t>(l.rec);
      c.rec_p = dptr<double>(l.rec_p);
      c.rec_moff = dptr<uint32_t>(l.rec_moff);
      c.mdesc = dptr<uint64_t>(L.mdesc) + l.mbase;
      c.mp = dptr<double>(L.mp) + l.mbase;
      c.tl = dptr<uint32_t>(L.tl) + (size_t)l.mbase * tcap;
      c.tn = dptr<uint32_t>(L.tn) + l.mbase;
      c.tcap = tcap;
      c.nq = T.nq;
      c.qpad = T.qpad;
      c.n_epochs = T.n_epochs;
      c.w = T.w;
      c.npoints = T.npoints;
      c.M = T.M;
      c.R = (uint32_t)T.rec.size();
      c.n_chunks = (uint32_t)T.ch_off.size();
      c.chunk_cap = T.chunk_cap;
      c.mbase = l.mbase;
      c.bbase = l.bbase;
      c.bbits = l.bbits;
      mb[i] = l.mbase;
      cb[i] = l.bbase;
    });
    mb[N] = L.M;
    put(L.cdev, cd.data(), cd.size() * sizeof(CircuitDev));
    put(L.mbase, mb.data(), mb.size() * 4);
    put(L.cbbase, cb.data(), cb.size() * 4);
    put(L.items, walk_items.data(), walk_items.size() * sizeof(uint2));
    if (seg_on) {
      put(L.seg_items, seg_items.data(), seg_items.size() * sizeof(gpc::SegItem));
      put(L.seg_aff, seg_aff.data(), seg_aff.size() * 4);
    }
    if (param) {
      // records of each (tick, class) source, in record order
      const Tape &T = tapes[0];
      const uint32_t ns = T.n_ticks * gpc::SRC_CLASSES;
      std::vector<uint32_t> off(ns + 1, 0), lst;
      for (uint32_t v : T.rec_src)
        if (v < ns) ++off[v + 1];
      for (uint32_t e = 0; e < ns; ++e) off[e + 1] += off[e];
      lst.resize(off[ns]);
      std::vector<uint32_t> cur(off.begin(), off.end() - 1);
      for (uint32_t r = 0; r < (uint32_t)T.rec_src.size(); ++r)
        if (T.rec_src[r] < ns) lst[cur[T.rec_src[r]]++] = r;
      put(L.src_off, off.data(), off.size() * 4);
      put(L.src_rec, lst.data(), lst.size() * 4);
    }
  }

  // Parses and lowers circuits (in parallel on host threads for batches).
  // The tapes and each thread's scratch memory are kept from one compile to
  // the next, so a repeated compile reuses mapped host memory.
  // n tapes, taken from and given back to the spares (tapes are not freed:
  // their op buffers are page-locked)
  std::vector<Tape> spare_tapes;
  void resize_tapes(uint32_t n) {
    while (tapes.size() > n) {
      spare_tapes.push_back(std::move(tapes.back()));
      tapes.pop_back();
    }
    while (tapes.size() < n) {
      if (spare_tapes.empty()) {
        tapes.emplace_back();
      } else {
        tapes.push_back(std::move(spare_tapes.back()));
        spare_tapes.pop_back();
      }
      pin_ops(tapes.back());
    }
  }

  void lower_all(const char *const *texts, const size_t *lens, uint32_t n) {
    if (ops_in_flight) wait();
    have_tape = false;  // the tapes are rewritten in place
    gpc::LowerOptions lo;
    lo.level = level;
    lo.sources = param;  // record sources feed the gradient kernels only
    if (n > 1) lo.chunk_min = gpc::kWalkChunkMin;
    // smaller segments than the default: one circuit's are scheduled side by side on the pool
    // (measured on GB300 + Grace: bb12 end to end 0.41 -> 0.36 ms; a batch's lowering, one
    // circuit per thread, 17.3 -> 16.8 ms)
    lo.segment_occ = 8192;
    // batches: each pool thread lowers its circuits against the previous one it lowered.  A single
    // circuit is lowered whole, on the pool: its parse and segments run side by side, while an
    // incremental lowering's text comparison and forward pass run on one thread (a bb12 branch:
    // 0.16 ms whole on the pool, about twice that incremental)
    lo.incremental = incremental && n > 1;
    gpc::HostPool &hp = host_pool();
    if (lower_scratch.size() < hp.workers() + 1) lower_scratch.resize(hp.workers() + 1);
    resize_tapes(n);
    order_by_size(n, [&](uint32_t i) { return (uint64_t)lens[i]; });
    if (n == 1)  // one circuit: a large text is parsed in pieces on the pool
      gpc::lower_text(texts[0], lens[0], lo, tapes[0], lower_scratch[0], &hp);
    else
      // largest texts first, so no large circuit starts last and holds up the batch
      hp.run(n, [&](uint32_t x, uint32_t slot) {
        const uint32_t i = big_first[x];
        gpc::lower_text(texts[i], lens[i], lo, tapes[i], lower_scratch[slot]);
      });
  }

  // Prepares circuits already lowered on the host (serving lowers requests as they arrive).
  // The driver's previous tapes come back in T (their memory can be reused).
  void prepare_tapes(std::vector<Tape> &T) {
    if (T.empty()) throw gpc::Error(GPC_ERR_INVALID, "empty batch");
    param = false;
    tcap = 32;
    lists_off = false;
    if (ops_in_flight) wait();
    tapes.swap(T);
    have_tape = true;
    prepare(nullptr, nullptr, 0);
  }

  void prepare(const char *const *texts, const size_t *lens, uint32_t n, bool param_mode = false) {
    CK(cudaSetDevice(device));
    if (texts) {
      if (param_mode && n != 1) throw gpc::Error(GPC_ERR_INVALID, "noise-rate gradients take one circuit");
      param = param_mode;
    }
    prepared = false;
    ran = false;
    if (texts) {
      if (n == 0) throw gpc::Error(GPC_ERR_INVALID, "empty batch");
      tcap = 32;
      lists_off = false;
      const auto t0 = HostClock::now();
      lower_all(texts, lens, n);
      host_ms[0] = ms_since(t0);
      have_tape = true;
    } else if (!have_tape) {
      throw gpc::Error(GPC_ERR_INVALID, "no circuit to compile");
    } else {
      host_ms[0] = 0;
    }
    const auto t1 = HostClock::now();
    if (!tuned && walk_words == 0 && walk_qpt == 0 && walk_queue == 0) {
      // a batch takes the walk configuration tuned for its widths, if any (else the defaults)
      uint32_t cfg[3] = {0, 0, 0};
      if (ncirc() > 1) tune_cache().get(width_key(), cfg);
      batch_words = cfg[0];
      batch_qpt = cfg[1];
      batch_queue = cfg[2];
    }
    plan_segments();
    layout();
    // The stream may still be reading the old arena: finish before regrowing.
    wait();
    uint32_t want_tg = std::max<uint32_t>(1024u, (uint32_t)std::min<uint64_t>(0xFFFFFFF0ull, (uint64_t)L.M * 16));
    if (admit) {
      const size_t tgb = (size_t)std::max(want_tg, tg_cap) * 4;
      const size_t grow = (L.total > arena.cap ? L.total - arena.cap : 0) + (tgb > tgbuf.cap ? tgb - tgbuf.cap : 0);
      if (grow) admit(grow, L.total + tgb);
    }
    arena.ensure(L.total);
    if (want_tg > tg_cap) {
      tgbuf.ensure((size_t)want_tg * 4);
      tg_cap = want_tg;
    }
    host_ms[1] = ms_since(t1);
    const auto t2 = HostClock::now();
    stage_inputs();
    host_ms[2] = ms_since(t2);
    CK(cudaMemcpyAsync(arena.p, pin_in.p, L.in_bytes, cudaMemcpyHostToDevice, stream));
    for (uint32_t i = 0; i < ncirc(); ++i)
      if (tapes[i].ops.external() && tapes[i].ops.size()) {
        CK(cudaMemcpyAsync(dptr<char>(L.c[i].ops), tapes[i].ops.data(), tapes[i].ops.size() * 8,
                           cudaMemcpyHostToDevice, stream));
        ops_in_flight = true;
      }
    last_h2d = L.in_bytes + L.ext_ops;
    // what a captured graph depends on: buffer addresses and launch sizes
    uint64_t h = 0xcbf29ce484222325ull;
    auto mix = [&](uint64_t v) { h = (h ^ v) * 0x100000001b3ull; };
    mix((uint64_t)(uintptr_t)arena.p);
    mix((uint64_t)(uintptr_t)tgbuf.p);
    mix(tg_cap);
    mix(L.total);
    mix(L.nb);
    mix(L.M);
    mix(tcap);
    mix((uint64_t)force_global);
    mix((uint64_t)lists_off);
    mix(L.in_bytes);
    mix(L.zero_bytes);
    for (const auto &c : L.classes) {
      mix(c.qpad);
      mix(c.n_items);
      mix(c.chunk_cap);
      mix(c.max_epochs);
      mix(c.max_chunks);
      mix(c.words);
      mix(c.qpt);
      mix(c.queue);
    }
    mix(split_word());
    mix((uint64_t)seg_on);
    if (seg_on) {
      mix(seg_na);
      mix(seg_nb);
      mix(seg_states);
      mix(seg_qpt);
      mix(seg_ring);
      for (uint32_t b : seg_bounds) mix(b);
    }
    cfg_sig = h;
    prepared = true;
  }

  // Runs the pipeline: from a CUDA graph of the kernel sequence when it can
  // (captured once a launch configuration runs twice in a row), else directly.
  void run() {
    if (!prepared) throw gpc::Error(GPC_ERR_INVALID, "no circuit prepared");
    CK(cudaSetDevice(device));
    used_global = false;
    const bool single_global = ncirc() == 1 && (force_global || lists_off);
    // (a graph with the stage events is another graph)
    const uint64_t sig = cfg_sig ^ (stage_timing ? 0x9e3779b97f4a7c15ull : 0ull);
    const bool graphable = use_graph && !single_global && ((graph_exec && graph_sig == sig) || last_run_sig == sig);
    last_run_sig = sig;
    if (graphable && graph_sig != sig) drop_graph();
    if (graphable && !graph_exec) {
      CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
      capturing = true;
      try {
        enqueue();
      } catch (...) {
        capturing = false;
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(stream, &g);
        if (g) cudaGraphDestroy(g);
        throw;
      }
      capturing = false;
      CK(cudaStreamEndCapture(stream, &graph));
      CK(cudaGraphInstantiate(&graph_exec, graph, 0));
      graph_sig = sig;
    }
    if (graphable) CK(cudaGraphLaunch(graph_exec, stream));
    else enqueue();
    ran = true;
    timed_run = stage_timing;
  }

  // The walks (one launch per class; several classes run on the auxiliary
  // streams), and meanwhile the key-block table on the main stream.
  void walk_one(const WalkClass &wc, cudaStream_t s) {
    gpc::WalkLaunch wl{};
    wl.circs = dptr<CircuitDev>(L.cdev);
    wl.items = dptr<uint2>(L.items) + wc.item0;
    wl.n_items = wc.n_items;
    wl.qpt = wc.qpt;
    wl.threads = wc.qpad / wl.qpt;
    wl.qpad = wc.qpad;
    wl.chunk_cap = wc.chunk_cap;
    wl.max_epochs = wc.max_epochs;
    wl.max_chunks = wc.max_chunks;
    wl.words = wc.words;
    wl.err = dptr<uint32_t>(L.err);
    wl.queue = wc.queue ? dptr<uint32_t>(L.wq) : nullptr;
    CK(gpc::launch_walk(wl, s));
  }

  void launch_walks(const gpc::KeyLaunch &kl) {
    const uint32_t nc = (uint32_t)L.classes.size();
    auto one = [&](const WalkClass &wc, cudaStream_t s) { walk_one(wc, s); };
    if (nc <= 1) {
      // the key-block table on an auxiliary stream beside the walk
      CK(cudaEventRecord(fork_ev, stream));
      CK(cudaStreamWaitEvent(aux[0], fork_ev, 0));
      CK(gpc::launch_key_prep(kl, aux[0]));
      if (nc == 1) one(L.classes[0], stream);
      CK(cudaEventRecord(join_ev[0], aux[0]));
      CK(cudaStreamWaitEvent(stream, join_ev[0], 0));
      return;
    }
    // fork: each class on an auxiliary stream, joined back into the main stream
    CK(cudaEventRecord(fork_ev, stream));
    const uint32_t used = std::min<uint32_t>(nc, kAux);
    for (uint32_t a = 0; a < used; ++a) CK(cudaStreamWaitEvent(aux[a], fork_ev, 0));
    for (uint32_t k = 0; k < nc; ++k) one(L.classes[k], aux[k % kAux]);
    CK(gpc::launch_key_prep(kl, stream));
    for (uint32_t a = 0; a < used; ++a) {
      CK(cudaEventRecord(join_ev[a], aux[a]));
      CK(cudaStreamWaitEvent(stream, join_ev[a], 0));
    }
  }

  // ---- segmented walk (one circuit) ----------------------------------------
  // Auto policy: segments of about kSegTarget cost units (an epoch costs its
  // slots + 2), taken when the longest word walk is at least kSegMinSpan
  // segments long.  Measured on GB300 (walk stage, L2 flushed between runs):
  // [[144,12,12]] r12 77 -> 41 us at 32 (16: 53, 48: 42), surface d = 7 61 ->
  // 34, d = 11 86 -> 41, [[72,12,6]] 42 -> 30, [[288,12,18]] 129 -> 77 (48:
  // 69); surface d = 3 walks 17 epochs and stays whole (segmenting it costs
  // 2-5 us; its longest walk costs 123 units, under kSegMinSpan segments).
  // A compose step costs about 1 us (instruction latency of one CTA
  // over a sparse transfer matrix), a segment epoch about 0.8 us.  Segment
  // walks copy the tape in chunks of at most kSegChunk bytes that never cross
  // a cut, so several segment CTAs share an SM and a segment's first copy is
  // short.
  static constexpr uint32_t kSegTarget = 32;
  static constexpr uint32_t kSegMinSpan = 4;
  static constexpr uint32_t kSegChunk = 24 * 1024;
  // A detector word's rows vanish some epochs after its last measurement
  // (the walk reaches the resets of the qubits they sit on); its segments
  // reach this many epochs past that measurement, the last one walking on.
  static constexpr uint32_t kSegTail = 12;

  // Chunks of whole epochs of at most the chunk capacity, cut at every bound.
  static void rechunk_at(Tape &T, const std::vector<uint32_t> &bounds, uint32_t cap_want) {
    const uint32_t nE = T.n_epochs;
    uint64_t big = 0;
    for (uint32_t e = 0; e < nE; ++e) big = std::max<uint64_t>(big, (uint64_t)T.ep_k[e] * T.qpad * 8);
    const uint64_t want = std::max<uint64_t>((big + 255) & ~(uint64_t)255, cap_want);
    T.chunk_cap = (uint32_t)std::min<uint64_t>(gpc::walk_chunk_cap(T.qpad), want);
    T.ep_chunk.assign(nE, 0);
    T.ch_off.clear();
    T.ch_bytes.clear();
    for (size_t s = 0; s + 1 < bounds.size(); ++s) {
      for (uint32_t e = bounds[s]; e < bounds[s + 1];) {
        const uint32_t c = (uint32_t)T.ch_off.size();
        uint64_t bytes = 0;
        uint32_t f = e;
        while (f < bounds[s + 1] && bytes + (uint64_t)T.ep_k[f] * T.qpad * 8 <= T.chunk_cap) {
          bytes += (uint64_t)T.ep_k[f] * T.qpad * 8;
          T.ep_chunk[f] = c;
          ++f;
        }
        T.ch_off.push_back(T.ep_opoff[e]);
        T.ch_bytes.push_back((uint32_t)bytes);
        e = f;
      }
    }
  }

  // Decides whether the single circuit's walk runs in segments and builds
  // the items of the two launches (device.cuh, SEG_*).
  void plan_segments() {
    seg_on = false;
    seg_band_reset = false;
    if (ncirc() != 1 || walk_segment < 0) return;
    Tape &T = tapes[0];
    const uint32_t nE = T.n_epochs;
    if (nE < 2 || T.w == 0) return;
    const uint32_t q = walk_qpt_for(T.qpad, walk_qpt);
    if (!gpc::walk_seg_supported(q) || !walk_qpt_fits(T.qpad, q)) return;
    std::vector<uint64_t> cum(nE + 1, 0);  // cost of epochs [0, e)
    for (uint32_t e = 0; e < nE; ++e) cum[e + 1] = cum[e] + gpc::walk_epoch_cost(T.ep_k[e]);
    auto holds_obs = [&](uint32_t j) { return (uint64_t)(j + 1) * 64 > T.ndet; };
    uint64_t longest = 0;
    for (uint32_t j = 0; j < T.w; ++j) {
      const uint32_t lo = T.inj_lo[j];
      if (lo == gpc::kNone || lo >= nE) continue;
      const uint32_t hi = holds_obs(j) ? nE : std::min(nE, T.inj_hi[j] + 1);
      longest = std::max<uint64_t>(longest, cum[hi] - cum[lo]);
    }
    const uint32_t target = walk_segment > 0 ? (uint32_t)walk_segment : kSegTarget;
    if (walk_segment == 0 && longest < (uint64_t)kSegMinSpan * target) return;
    gpc::walk_segment_bounds(T, target, seg_bounds);
    const uint32_t S = (uint32_t)seg_bounds.size() - 1;
    if (S < 2) return;
    const std::vector<uint32_t> &b = seg_bounds;
    auto seg_of = [&](uint32_t e) {
      return (uint32_t)(std::upper_bound(b.begin(), b.end(), e) - b.begin()) - 1;
    };
    seg_qpt = q;
    seg_ncol = (2 * T.qpad + 63) / 64;
    seg_aff.assign((size_t)T.w * S, gpc::kNone);
    std::vector<gpc::SegItem> A, B;
    std::vector<char> need_xfer(S, 0);
    uint32_t states = 0;
    for (uint32_t j = 0; j < T.w; ++j) {
      const uint32_t e0 = T.inj_lo[j];
      if (e0 == gpc::kNone || e0 >= nE) {
        seg_band_reset = true;  // no item writes this word's band
        continue;
      }
      const uint32_t elast = T.inj_hi[j];
      const uint32_t s0 = seg_of(e0);
      const uint32_t K = holds_obs(j) ? S - 1 : std::max(s0, seg_of(std::min(nE - 1, elast + kSegTail)));
      if (K == s0) {
        A.push_back(gpc::SegItem{gpc::SEG_FIRST, j, e0, nE, gpc::kNone, 0, 0, 0});
        continue;
      }
      const uint32_t ent = states++;
      A.push_back(gpc::SegItem{gpc::SEG_FIRST, j, e0, b[s0 + 1], ent, 0, 0, 0});
      for (uint32_t s = s0 + 1; s < K; ++s) {
        need_xfer[s] = 1;
        if (b[s] <= elast) {
          seg_aff[(size_t)j * S + s] = states;
          A.push_back(gpc::SegItem{gpc::SEG_AFF, j, b[s], b[s + 1], states++, 0, 0, 0});
        }
      }
      for (uint32_t s = s0 + 1; s <= K; ++s)
        B.push_back(gpc::SegItem{gpc::SEG_REST, j, b[s], s == K ? nE : b[s + 1], ent, s0 + 1, s, 0});
    }
    seg_xfer0 = states;
    for (uint32_t s = 0; s < S; ++s)
      if (need_xfer[s])
        for (uint32_t c = 0; c < seg_ncol; ++c)
          A.push_back(gpc::SegItem{gpc::SEG_XFER, c, b[s], b[s + 1], seg_xfer0 + s * seg_ncol + c, s, 0, 0});
    seg_states = seg_xfer0 + S * seg_ncol;
    rechunk_at(T, seg_bounds, kSegChunk);
    // compose ring: as many step buffers (2 to kSegRingMax: step k + 1 is copied while step k is
    // composed) as the REST CTA's shared memory holds
    uint32_t max_steps = 0;
    for (const auto &it : B) max_steps = std::max(max_steps, it.s_to - it.s_from);
    seg_ring = 0;
    for (uint32_t nb = std::min(gpc::kSegRingMax, std::max(2u, max_steps)); nb >= 2; --nb) {
      gpc::SegLaunch probe{};
      probe.qpad = T.qpad;
      probe.chunk_cap = T.chunk_cap;
      probe.max_epochs = nE;
      probe.max_chunks = (uint32_t)T.ch_off.size();
      probe.S = S;
      probe.ring_nb = nb;
      if (gpc::walk_seg_smem_bytes(probe)) {
        seg_ring = nb;
        break;
      }
    }
    if (seg_ring == 0) {  // no room for a compose step: the plain walk, with the tape's usual chunks
      rechunk_at(T, {0u, nE}, 0xFFFFFFFFu);
      return;
    }
    // longest items first (launch order is the order CTAs start in)
    auto span = [&](const gpc::SegItem &it) {
      return cum[it.e_end] - cum[it.e_begin] + (it.kind == gpc::SEG_REST ? 8ull * (it.s_to - it.s_from) : 0ull);
    };
    auto longer = [&](const gpc::SegItem &x, const gpc::SegItem &y) { return span(x) > span(y); };
    std::stable_sort(A.begin(), A.end(), longer);
    std::stable_sort(B.begin(), B.end(), longer);
    seg_na = (uint32_t)A.size();
    seg_nb = (uint32_t)B.size();
    seg_items = std::move(A);
    seg_items.insert(seg_items.end(), B.begin(), B.end());
    seg_on = true;
  }

  // Launch A (first parts, AFF and transfer walks) then launch B (the rest
  // of every segmented word) on the main stream; the key-block table beside
  // them on an auxiliary stream.
  void launch_walks_seg(const gpc::KeyLaunch &kl) {
    const Tape &T = tapes[0];
    CK(cudaEventRecord(fork_ev, stream));
    CK(cudaStreamWaitEvent(aux[0], fork_ev, 0));
    CK(gpc::launch_key_prep(kl, aux[0]));
    CK(cudaEventRecord(join_ev[0], aux[0]));
    if (seg_band_reset) CK(cudaMemsetAsync(dptr<char>(L.c[0].band), 0, (size_t)T.w * 8, stream));
    gpc::SegLaunch sl{};
    sl.circ = dptr<CircuitDev>(L.cdev);
    sl.items = dptr<gpc::SegItem>(L.seg_items);
    sl.n_items = seg_na;
    sl.qpt = seg_qpt;
    sl.qpad = T.qpad;
    sl.threads = T.qpad / seg_qpt;
    sl.chunk_cap = T.chunk_cap;
    sl.max_epochs = T.n_epochs;
    sl.max_chunks = (uint32_t)T.ch_off.size();
    sl.state = dptr<uint64_t>(L.seg_state);
    sl.xfer0 = seg_xfer0;
    sl.ncol = seg_ncol;
    sl.aff = dptr<uint32_t>(L.seg_aff);
    sl.S = (uint32_t)seg_bounds.size() - 1;
    sl.xcnt = dptr<uint32_t>(L.seg_xcnt);
    sl.xlst = dptr<uint16_t>(L.seg_xlst);
    sl.err = dptr<uint32_t>(L.err);
    sl.ring_nb = 0;
    CK(gpc::launch_walk_seg(sl, stream));
    sl.items += seg_na;
    sl.n_items = seg_nb;
    sl.ring_nb = seg_ring;
    CK(gpc::launch_walk_seg(sl, stream));
    CK(cudaStreamWaitEvent(stream, join_ev[0], 0));
  }

  // First word of a split key pass, or kNoSplit.  One circuit with target
  // lists whose observables sit in words after some detector-only words: the
  // observables never vanish, so their walk covers every epoch, while the
  // detector words stop early; their keys are computed beside that walk.
  uint32_t split_word() const {
    if (!key_split || seg_on || ncirc() != 1 || force_global || lists_off || tcap == 0 || L.classes.size() != 1)
      return gpc::kNoSplit;
    const Tape &T = tapes[0];
    if (T.nobs == 0 || T.n_epochs == 0) return gpc::kNoSplit;
    const uint32_t W = std::max(1u, L.classes[0].words);
    const uint32_t late = T.ndet / 64u / W * W;  // whole walk items before the first observable's word
    // worth a second launch only when the detector words' keys are a real
    // kernel and the observables' walk is long (measured: a loss for d = 5-9
    // surface circuits, a gain for [[144,12,12]] with 27 detector words)
    return late >= 8 && late < T.w && T.n_epochs >= 64 ? late : gpc::kNoSplit;
  }

  // The walks of a split key pass: the detector words on the main stream, the
  // late words (from `late`) and the key-block table on auxiliary streams; the
  // end of the late walk is timing event 1 and join_ev[1].
  void launch_walks_split(const gpc::KeyLaunch &kl, uint32_t late) {
    const WalkClass &wc = L.classes[0];
    WalkClass a = wc, b = wc;
    a.n_items = late / std::max(1u, wc.words);
    b.item0 = wc.item0 + a.n_items;
    b.n_items = wc.n_items - a.n_items;
    CK(cudaEventRecord(fork_ev, stream));
    CK(cudaStreamWaitEvent(aux[0], fork_ev, 0));
    CK(cudaStreamWaitEvent(aux[1], fork_ev, 0));
    CK(gpc::launch_key_prep(kl, aux[0]));
    CK(cudaEventRecord(join_ev[0], aux[0]));
    walk_one(b, aux[1]);
    if (stage_timing) {
      if (capturing) CK(cudaEventRecordWithFlags(ev[1], aux[1], cudaEventRecordExternal));
      else CK(cudaEventRecord(ev[1], aux[1]));
    }
    CK(cudaEventRecord(join_ev[1], aux[1]));
    walk_one(a, stream);
    CK(cudaStreamWaitEvent(stream, join_ev[0], 0));
  }

  gpc::KeyLaunch key_launch(bool write_all) {
    gpc::KeyLaunch kl{};
    kl.circs = dptr<CircuitDev>(L.cdev);
    kl.mbase = dptr<uint32_t>(L.mbase);
    kl.n_circ = ncirc();
    kl.M = L.M;
    kl.key = dptr<ulonglong2>(L.key);
    kl.bucket_count = dptr<uint32_t>(L.bcount);
    kl.blk_info = dptr<uint2>(L.blk_r0);
    kl.slot = dptr<gpc::Slot>(L.slot);
    kl.list_total = dptr<uint32_t>(L.totals) + 2;
    kl.err = dptr<uint32_t>(L.err);
    kl.write_all = write_all ? 1u : 0u;
    kl.late_word = gpc::kNoSplit;
    return kl;
  }

  void enqueue() {
    CK(cudaMemsetAsync(dptr<char>(L.zero), 0, L.zero_bytes, stream));
    for (uint32_t i = 0; i < ncirc(); ++i)
      if (tapes[i].n_epochs == 0) CK(cudaMemsetAsync(dptr<char>(L.c[i].band), 0, (size_t)tapes[i].w * 8, stream));
    gpc::KeyLaunch kl = key_launch(param || (ncirc() == 1 && (force_global || lists_off)));
    const uint32_t late = split_word();
    rec(0);
    if (seg_on) {
      launch_walks_seg(kl);
      rec(1);
      CK(gpc::launch_keys(kl, stream));
    } else if (late == gpc::kNoSplit) {
      launch_walks(kl);
      rec(1);
      CK(gpc::launch_keys(kl, stream));
    } else {
      launch_walks_split(kl, late);
      kl.late_word = late;
      CK(gpc::launch_keys(kl, stream));  // the detector words, beside the late walk
      CK(cudaStreamWaitEvent(stream, join_ev[1], 0));
      CK(gpc::launch_keys_late(kl, stream));
    }
    rec(2);
    if (ncirc() == 1 && (force_global || lists_off)) {
      run_global(false);
    } else {
      CK(gpc::launch_group(group_launch(), stream));
      rec(3);
      CK(gpc::launch_scan_emit(group_launch(), stream));
      rec(4);
    }
  }

  gpc::GroupLaunch group_launch() {
    gpc::GroupLaunch gl{};
    gl.tl = dptr<uint32_t>(L.tl);
    gl.tn = dptr<uint32_t>(L.tn);
    gl.tcap = tcap;
    gl.slot = dptr<gpc::Slot>(L.slot);
    gl.count = dptr<uint32_t>(L.bcount);
    gl.nb = L.nb;
    gl.bagg = dptr<uint2>(L.bagg);
    gl.bout = dptr<uint2>(L.bout);
    gl.tsum = dptr<uint2>(L.tsum);
    gl.big_n = dptr<uint32_t>(L.big_n);
    gl.big_list = dptr<uint32_t>(L.big_list);
    gl.out_prob = dptr<double>(L.out_prob);
    gl.out_off = dptr<uint32_t>(L.out_off);
    gl.out_tg = static_cast<uint32_t *>(tgbuf.p);
    gl.tg_cap = tg_cap;
    gl.totals = dptr<uint32_t>(L.totals);
    gl.cbbase = dptr<uint32_t>(L.cbbase);
    gl.n_circ = ncirc();
    gl.cout = dptr<uint2>(L.cout);
    gl.err = dptr<uint32_t>(L.err);
    return gl;
  }

  // Global path (single circuit): sort every mechanism (on sort_bits, or all
  // 128 bits) and merge from the snapshots.
  void run_global(bool full) {
    used_global = true;
    CK(cudaMemsetAsync(dptr<char>(L.gzero), 0, L.gzero_bytes, stream));
    CK(cudaMemsetAsync(dptr<char>(L.totals), 0, 8, stream));
    CK(gpc::launch_sort_init(dptr<ulonglong2>(L.key), dptr<uint64_t>(L.sk0), dptr<uint32_t>(L.pm0), L.M, stream));
    sort_and_merge(full);
  }

  void sort_and_merge(bool full) {
    const uint32_t M = L.M;
    uint32_t *sw = dptr<uint32_t>(L.sort_scr);
    const uint32_t passes = 8;
    const size_t one = (size_t)passes * gpc::RADIX + (size_t)passes * L.sort_tiles * gpc::RADIX + passes;
    const uint32_t hold = hold_runs ? 1u : 0u;
    if (hold_runs) --hold_runs;
    gpc::SortScratch s1{sw, sw + passes * gpc::RADIX, sw + passes * gpc::RADIX + (size_t)passes * L.sort_tiles * gpc::RADIX,
                        dptr<uint32_t>(L.err), spin_ns, hold};
    gpc::SortScratch s2{sw + one, sw + one + passes * gpc::RADIX,
                        sw + one + passes * gpc::RADIX + (size_t)passes * L.sort_tiles * gpc::RADIX, dptr<uint32_t>(L.err),
                        spin_ns, 0u};
    uint64_t *k0 = dptr<uint64_t>(L.sk0), *k1 = dptr<uint64_t>(L.sk1);
    uint32_t *p0 = dptr<uint32_t>(L.pm0), *p1 = dptr<uint32_t>(L.pm1);
    bool alt = false;
    CK(gpc::launch_sort(k0, k1, p0, p1, M, full ? 64 : sort_bits, s1, stream, &alt));
    uint64_t *ks = alt ? k1 : k0;
    uint32_t *ps = alt ? p1 : p0;
    if (full) {
      // second key: the high 64 bits, gathered in the current order, sorted stably
      uint64_t *hk = dptr<uint64_t>(L.hik);
      uint64_t *hk_alt = alt ? k0 : k1;
      uint32_t *ps_alt = alt ? p0 : p1;
      CK(gpc::launch_gather_hi(dptr<ulonglong2>(L.key), ps, hk, M, stream));
      bool alt2 = false;
      CK(gpc::launch_sort(hk, hk_alt, ps, ps_alt, M, 64, s2, stream, &alt2));
      ks = alt2 ? hk_alt : hk;
      ps = alt2 ? ps_alt : ps;
    }
    perm_sorted = ps;
    sk_sorted = ks;
    const uint32_t b = full ? 0 : sort_bits;
    sort_mask = b == 0 ? 0ull : (b >= 64 ? ~0ull : ((1ull << b) - 1));
    rec(3);
    launch_merge_now();
    rec(4);
  }

  void launch_merge_now() {
    gpc::MergeLaunch ml{};
    ml.c_dev = dptr<CircuitDev>(L.cdev);
    ml.w = tapes[0].w;
    ml.perm = perm_sorted;
    ml.sortkey = sk_sorted;
    ml.sort_mask = sort_mask;
    ml.key = dptr<ulonglong2>(L.key);
    ml.n = L.M;
    ml.out_prob = dptr<double>(L.out_prob);
    ml.out_off = dptr<uint32_t>(L.out_off);
    ml.out_tg = static_cast<uint32_t *>(tgbuf.p);
    ml.tg_cap = tg_cap;
    ml.status = dptr<unsigned long long>(L.merge_status);
    ml.tile_ctr = dptr<uint32_t>(L.merge_ctr);
    ml.totals = dptr<uint32_t>(L.totals);
    ml.err = dptr<uint32_t>(L.err);
    ml.spin_ns = spin_ns;
    CK(gpc::launch_merge(ml, stream));
  }

  void reset_merge_scratch() {
    CK(cudaMemsetAsync(dptr<char>(L.merge_status), 0, (size_t)L.merge_tiles * 8, stream));
    CK(cudaMemsetAsync(dptr<char>(L.merge_ctr), 0, 4, stream));
    CK(cudaMemsetAsync(dptr<char>(L.totals), 0, 8, stream));
  }

  enum class Finish { Ok, BatchFallback };

  // How often a run left the fast path (gpc_fallback_counts): [0] batches
  // compiled circuit by circuit, [1] runs through the global sort (a bucket
  // overflowed), [2] reruns with wider target lists (a long symptom), [3]
  // full 128-bit re-sorts, [4] target-buffer regrowths.
  std::atomic<uint64_t> fallbacks[5] = {};

  // Reads flags and totals; handles the rare fallbacks (bucket overflow,
  // long symptoms, short sort keys, target-buffer growth).
  Finish finish(uint32_t *groups, uint32_t *targets) {
    pin_out.ensure(64);
    uint32_t *h = static_cast<uint32_t *>(pin_out.p);
    bool did_full = false;
    for (int attempt = 0; attempt < 8; ++attempt) {
      CK(cudaMemcpyAsync(h, dptr<char>(L.err), 4, cudaMemcpyDeviceToHost, stream));
      CK(cudaMemcpyAsync(h + 1, dptr<char>(L.totals), 8, cudaMemcpyDeviceToHost, stream));
      wait();
      const uint32_t err = h[0];
      if (err & gpc::DEV_ERR_TIMEOUT) throw gpc::Error(GPC_ERR_TIMEOUT, "a bounded device wait timed out");
      if (err & gpc::DEV_ERR_COLLISION)
        throw gpc::Error(GPC_ERR_COLLISION, "two different symptoms share a 128-bit key");
      if ((err & (gpc::DEV_FLAG_LONG | gpc::DEV_FLAG_BIG_BUCKET)) && !used_global && ncirc() > 1) {
        ++fallbacks[0];
        return Finish::BatchFallback;  // compile the batch's circuits one by one
      }
      if ((err & gpc::DEV_FLAG_LONG) && !used_global) {
        ++fallbacks[2];
        // a symptom longer than the target-list stride: widen it (or merge from
        // the snapshots) and run again
        if (tcap < 256) {
          tcap *= 4;
        } else {
          tcap = 0;
          lists_off = true;
        }
        prepare(nullptr, nullptr, 0);
        if (param && noise_dev) launch_param_rec_now();
        run();
        continue;
      }
      if ((err & gpc::DEV_FLAG_BIG_BUCKET) && !used_global) {
        ++fallbacks[1];
        // a symptom repeated more often than a bucket holds: sort globally
        // (the bucket pass skipped the keys and descriptors this path reads)
        CK(cudaMemsetAsync(dptr<char>(L.err), 0, 4, stream));
        CK(gpc::launch_keys(key_launch(true), stream));
        CK(cudaMemsetAsync(dptr<char>(L.err), 0, 4, stream));
        run_global(false);
        continue;
      }
      if (used_global && (err & gpc::DEV_FLAG_MIXED) && !did_full) {
        ++fallbacks[3];
        // equal sort keys with different full keys: sort on all 128 bits
        CK(cudaMemsetAsync(dptr<char>(L.err), 0, 4, stream));
        run_global(true);
        did_full = true;
        continue;
      }
      if (err & gpc::DEV_FLAG_TG_OVF) {
        ++fallbacks[4];
        const uint32_t need = h[2];
        tgbuf.ensure((size_t)need * 4 + 1024);
        tg_cap = (uint32_t)std::min<size_t>(0xFFFFFFF0ull, tgbuf.cap / 4);
        drop_graph();  // the target buffer moved
        CK(cudaMemsetAsync(dptr<char>(L.err), 0, 4, stream));
        if (used_global) {
          reset_merge_scratch();
          launch_merge_now();
        } else {
          CK(gpc::launch_scan_emit(group_launch(), stream));  // the groups are already formed
        }
        continue;
      }
      if (h[1] > L.M || h[2] > tg_cap) throw gpc::Error(GPC_ERR_CUDA, "inconsistent merge totals");
      *groups = h[1];
      *targets = h[2];
      return Finish::Ok;
    }
    throw gpc::Error(GPC_ERR_CUDA, "merge did not converge");
  }

  // Device pointers to circuit i's merged mechanisms of the last run (no copy).
  void device_dem(uint32_t i, const double **probs, const uint32_t **offsets, const uint32_t **targets,
                  uint32_t *num_errors, uint32_t *targets_end) {
    if (!ran) throw gpc::Error(GPC_ERR_INVALID, "nothing has been run");
    if (i >= ncirc()) throw gpc::Error(GPC_ERR_INVALID, "circuit index out of range");
    CK(cudaSetDevice(device));
    uint32_t C = 0, NT = 0;
    if (finish(&C, &NT) != Finish::Ok)
      throw gpc::Error(GPC_ERR_UNSUPPORTED, "this batch was compiled circuit by circuit: no device arrays");
    uint2 first = make_uint2(0, 0), next = make_uint2(C, NT);
    pin_out.ensure(64);
    uint32_t *h = static_cast<uint32_t *>(pin_out.p);
    if (ncirc() > 1) {
      CK(cudaMemcpyAsync(h, dptr<char>(L.cout) + (size_t)i * 8, i + 1 < ncirc() ? 16 : 8, cudaMemcpyDeviceToHost,
                         stream));
      wait();
      first = make_uint2(h[0], h[1]);
      if (i + 1 < ncirc()) next = make_uint2(h[2], h[3]);
    }
    // the closing offset of the whole run (offsets are positions in the run's target array)
    h[8] = NT;
    CK(cudaMemcpyAsync(dptr<char>(L.out_off) + (size_t)C * 4, h + 8, 4, cudaMemcpyHostToDevice, stream));
    wait();
    *probs = dptr<double>(L.out_prob) + first.x;
    *offsets = dptr<uint32_t>(L.out_off) + first.x;
    *targets = static_cast<const uint32_t *>(tgbuf.p);
    *num_errors = next.x - first.x;
    *targets_end = next.y;
  }

  // ---- noise-rate gradients (one circuit) --------------------------------
  uint32_t n_src() const { return tapes.empty() ? 0 : tapes[0].n_ticks * gpc::SRC_CLASSES; }

  void launch_param_rec_now() {
    const Tape &T = tapes[0];
    gpc::ParamLaunch pl{};
    pl.rec = dptr<uint64_t>(L.c[0].rec);
    pl.rec_src = dptr<uint32_t>(L.c[0].rec_src);
    pl.rec_p = dptr<double>(L.c[0].rec_p);
    pl.R = (uint32_t)T.rec.size();
    pl.n_src = n_src();
    pl.qtab = dptr<double>(L.ptab);
    CK(gpc::launch_param_rec(pl, stream));
  }

  // The caller's stream waits for this driver's stream (and the reverse before work starts).
  void wait_caller(cudaStream_t caller) {
    if (!caller_ev) CK(cudaEventCreateWithFlags(&caller_ev, cudaEventDisableTiming));
    CK(cudaEventRecord(caller_ev, caller));
    CK(cudaStreamWaitEvent(stream, caller_ev, 0));
  }
  void signal_caller(cudaStream_t caller) {
    if (!done_ev) CK(cudaEventCreateWithFlags(&done_ev, cudaEventDisableTiming));
    CK(cudaEventRecord(done_ev, stream));
    CK(cudaStreamWaitEvent(caller, done_ev, 0));
  }

  uint32_t param_forward(const double *noise, cudaStream_t caller) {
    if (!param || !prepared) throw gpc::Error(GPC_ERR_INVALID, "no circuit prepared for noise-rate gradients");
    if (!noise) throw gpc::Error(GPC_ERR_INVALID, "noise tensor is null");
    CK(cudaSetDevice(device));
    wait_caller(caller);
    noise_dev = noise;
    // The rates come to the host (n_ticks x 4 doubles): each source's split
    // probability and slope per channel kind are evaluated with the same
    // host formulas as the text path, so a template run with a rate tensor
    // gives what compiling the instantiated text gives, bit for bit.  (The
    // DEPOLARIZE2 split 0.5 - 0.5 (1 - 16p/15)^(1/8) cancels: one ulp of the
    // root moves q by ~1e-12 relative at p ~ 1e-3, so the root must come from
    // the same pow.)
    const uint32_t ns = n_src();
    pin_out.ensure((size_t)ns * 8 * 7);
    double *h = static_cast<double *>(pin_out.p);
    CK(cudaMemcpyAsync(h, noise, (size_t)ns * 8, cudaMemcpyDeviceToHost, stream));
    wait();
    double *qt = h + ns, *st = h + 4 * (size_t)ns;
    for (uint32_t e = 0; e < ns; ++e) {
      const double p = h[e];
      if (!(p >= 0.0 && p <= 1.0)) throw gpc::Error(GPC_ERR_INVALID, "a noise rate is outside [0, 1]");
      qt[3 * e] = p;
      st[3 * e] = 1.0;
      const bool ok1 = p <= 0.75, ok2 = p <= 0.9375;
      if (!ok1 && (e % gpc::SRC_CLASSES) == gpc::SRC_DEP1)
        throw gpc::Error(GPC_ERR_INVALID, "a DEPOLARIZE1 rate is above 3/4");
      if (!ok2 && (e % gpc::SRC_CLASSES) == gpc::SRC_DEP2)
        throw gpc::Error(GPC_ERR_INVALID, "a DEPOLARIZE2 rate is above 15/16");
      const double s1 = ok1 ? std::sqrt(1.0 - 4.0 * p / 3.0) : 1.0;
      const double x2 = ok2 ? 1.0 - 16.0 * p / 15.0 : 1.0;
      qt[3 * e + 1] = ok1 ? gpc::split_dep1(p) : 0.0;
      st[3 * e + 1] = ok1 && s1 > 0 ? 1.0 / (3.0 * s1) : 0.0;
      qt[3 * e + 2] = ok2 ? gpc::split_dep2(p) : 0.0;
      st[3 * e + 2] = ok2 && x2 > 0 ? std::pow(x2, 0.125) / (15.0 * x2) : 0.0;
    }
    CK(cudaMemcpyAsync(dptr<char>(L.ptab), qt, (size_t)ns * 6 * 8, cudaMemcpyHostToDevice, stream));
    launch_param_rec_now();
    run();
    uint32_t C = 0, NT = 0;
    if (finish(&C, &NT) != Finish::Ok) throw gpc::Error(GPC_ERR_UNSUPPORTED, "batch fallback in a gradient run");
    param_groups = C;
    signal_caller(caller);
    return C;
  }

  void param_probs(double *out, cudaStream_t caller) {
    if (!param || !ran) throw gpc::Error(GPC_ERR_INVALID, "no forward run");
    if (param_groups) CK(cudaMemcpyAsync(out, dptr<char>(L.out_prob), (size_t)param_groups * 8, cudaMemcpyDeviceToDevice, stream));
    signal_caller(caller);
  }

  void param_backward(const double *grad_out, double *grad_noise, cudaStream_t caller) {
    if (!param || !ran) throw gpc::Error(GPC_ERR_INVALID, "no forward run");
    if (used_global)
      throw gpc::Error(GPC_ERR_UNSUPPORTED, "gradients need the bucket merge (this circuit took the global sort)");
    if (!grad_out || !grad_noise) throw gpc::Error(GPC_ERR_INVALID, "null gradient buffer");
    CK(cudaSetDevice(device));
    wait_caller(caller);
    const Tape &T = tapes[0];
    CK(cudaMemsetAsync(dptr<char>(L.gq), 0, (size_t)L.M * 8, stream));
    gpc::AdjointLaunch A{};
    A.slot = dptr<gpc::Slot>(L.slot);
    A.count = dptr<uint32_t>(L.bcount);
    A.bagg = dptr<uint2>(L.bagg);
    A.bout = dptr<uint2>(L.bout);
    A.nb = L.nb;
    A.blk_info = dptr<uint2>(L.blk_r0);
    A.rec_p = dptr<double>(L.c[0].rec_p);
    A.grad_out = grad_out;
    A.gq = dptr<double>(L.gq);
    A.rec = dptr<uint64_t>(L.c[0].rec);
    A.rec_src = dptr<uint32_t>(L.c[0].rec_src);
    A.rec_moff = dptr<uint32_t>(L.c[0].rec_moff);
    A.R = (uint32_t)T.rec.size();
    A.stab = dptr<double>(L.ptab) + (size_t)n_src() * 3;
    A.grad_rec = dptr<double>(L.grad_rec);
    A.src_off = dptr<uint32_t>(L.src_off);
    A.src_rec = dptr<uint32_t>(L.src_rec);
    A.n_src = n_src();
    A.grad_noise = grad_noise;
    CK(gpc::launch_adjoint(A, stream));
    signal_caller(caller);
    wait();
  }

  // Algorithmic bytes of each stage of the last run (walk, keys, bucket groups,
  // scan + emit): what the design must move, counted from the run's own sizes.
  void traffic(double out[4]) {
    wait();
    uint32_t tot[4] = {0, 0, 0, 0};
    uint32_t nonempty = 0;
    CK(cudaMemcpy(tot, dptr<char>(L.totals), 16, cudaMemcpyDeviceToHost));
    nonempty = tot[3];
    double walk = 0, pts = 0, R = 0;
    for (uint32_t i = 0; i < ncirc(); ++i) {
      const Tape &T = tapes[i];
      std::vector<uint2> band(T.w);
      CK(cudaMemcpy(band.data(), dptr<char>(L.c[i].band), (size_t)T.w * 8, cudaMemcpyDeviceToHost));
      // one walk CTA per group of circuit-words: it reads the tape of its
      // epochs once and writes each word's snapshots
      const uint32_t W = circ_words.size() > i ? circ_words[i] : 1u;
      for (uint32_t j0 = 0; j0 < T.w; j0 += W) {
        const uint32_t nw = std::min(W, T.w - j0);
        if (band[j0].y <= band[j0].x) continue;
        uint32_t e0 = 0xFFFFFFFFu;
        for (uint32_t j = j0; j < j0 + nw; ++j)
          if (T.inj_lo[j] != 0xFFFFFFFFu) e0 = std::min(e0, T.inj_lo[j]);
        if (e0 >= T.n_epochs) continue;
        uint32_t e1 = (uint32_t)(std::lower_bound(T.ep_ptoff.begin(), T.ep_ptoff.end(), band[j0].y) - T.ep_ptoff.begin());
        if (e1 > T.n_epochs) e1 = T.n_epochs;
        const uint64_t a = T.ep_opoff[e0], b = e1 < T.n_epochs ? T.ep_opoff[e1] : T.ops.size();
        const double p = (double)(band[j0].y - band[j0].x) * nw;
        walk += (double)(b - a) * 8 + 16.0 * p;
        pts += p;
      }
      R += (double)T.rec.size();
    }
    const double M = L.M, lists = tot[2], groups = tot[0], targets = tot[1], nb = L.nb;
    const double per_list = M > 0 ? lists / M : 0.0;
    out[0] = walk;
    // records, snapshot words read, count (+ key, descriptor, probability when kept), lists, bucket slots
    const bool all = param || (ncirc() == 1 && (force_global || lists_off));
    out[1] = R * 20 + 16.0 * pts + M * (all ? 36 : 4) + 4.0 * lists + (double)nonempty * 32;
    // slots read, lists compared for the non-head items, group records written, counts and aggregates
    out[2] = (double)nonempty * 32 + (double)(nonempty - std::min<double>(nonempty, groups)) * 8.0 * per_list +
             groups * 16 + nb * 12;
    // aggregates and prefixes, group records, head lists gathered and written, DEM probabilities and offsets
    out[3] = nb * 24 + groups * (16 + 4) + 8.0 * targets + groups * 12;
  }

  // A fetch whose copies are issued and whose DEMs are not built yet, with
  // what building them needs after the driver has moved on to other circuits.
  struct PendingFetch {
    bool active = false;
    std::vector<gpc_dem *> done;  // DEMs built already (single-circuit pinned path, fallback)
    std::shared_ptr<ResultBlock> blk;
    const char *h = nullptr;  // where the copies land (the block, else the staging buffer)
    uint32_t C = 0, NT = 0, N = 0;
    std::vector<uint32_t> ndet, nobs, order;
    std::vector<uint64_t> M;
  };
  cudaEvent_t fetch_ev = nullptr;  // the last begin_fetch's copies
  // Results copied into page-locked memory that the DEMs keep (pinned DEMs,
  // batch result blocks), as far as the page-locked pool reaches.
  bool pinned_results = true;
  bool incremental = false;  // lower each circuit against the previous one of its lowering slot

  // Waits for the pipeline and issues the copies of its result on the driver's
  // stream; end_fetch builds the DEMs.  A single circuit copied into a pinned
  // DEM, and a batch that falls back to circuit-by-circuit compiles, finish here.
  void begin_fetch(PendingFetch &pf) {
    if (!ran) throw gpc::Error(GPC_ERR_INVALID, "nothing has been run");
    CK(cudaSetDevice(device));
    pf = PendingFetch{};
    uint32_t C = 0, NT = 0;
    const auto t3 = HostClock::now();
    if (finish(&C, &NT) == Finish::BatchFallback) {
      batch_fallback(pf.done);
      return;
    }
    host_ms[3] = ms_since(t3);
    const auto t4 = HostClock::now();
    const uint32_t N = ncirc();
    if (N == 1 && pinned_results) {  // one circuit: straight into a pinned DEM's arrays when one is to be had
      gpc_dem *d = dem_cache().take_pinned();
      if (d) {
        try {
          d->probs.resize(C);
          d->offsets.resize((size_t)C + 1);
          d->targets.resize(NT);
        } catch (const gpc::Error &) {  // no pinned memory: the staged copy below
          dem_cache().drop_pinned(d);
          d = nullptr;
        }
      }
      if (d) {
        try {
          if (C) {
            CK(cudaMemcpyAsync(d->probs.data(), dptr<char>(L.out_prob), (size_t)C * 8, cudaMemcpyDeviceToHost,
                               stream));
            CK(cudaMemcpyAsync(d->offsets.data(), dptr<char>(L.out_off), (size_t)C * 4, cudaMemcpyDeviceToHost,
                               stream));
          }
          if (NT) CK(cudaMemcpyAsync(d->targets.data(), tgbuf.p, (size_t)NT * 4, cudaMemcpyDeviceToHost, stream));
          wait();
        } catch (...) {
          dem_cache().give(d);
          throw;
        }
        d->offsets[C] = NT;
        d->num_detectors = tapes[0].ndet;
        d->num_observables = tapes[0].nobs;
        d->num_raw = tapes[0].M;
        last_d2h = (uint64_t)C * 12 + (uint64_t)NT * 4 + 12;
        pf.done.assign(1, d);
        host_ms[4] = ms_since(t4);
        host_ms[5] = 0;
        return;
      }
    }
    const size_t bytes = (size_t)C * 8 + (size_t)C * 4 + (size_t)NT * 4 + (size_t)N * 8 + 64;
    // into a result block that the DEMs keep (they view their probabilities and targets in
    // it), else into the staging buffer, split into DEMs that own copies
    if (N > 1 && pinned_results) pf.blk = take_block(bytes);
    char *h;
    if (pf.blk) {
      h = static_cast<char *>(pf.blk->p);
    } else {
      pin_out.ensure(bytes);
      h = static_cast<char *>(pin_out.p);
    }
    char *hp = h, *ho = h + (size_t)C * 8, *ht = ho + (size_t)C * 4, *hc = ht + (size_t)NT * 4;
    if (C) {
      CK(cudaMemcpyAsync(hp, dptr<char>(L.out_prob), (size_t)C * 8, cudaMemcpyDeviceToHost, stream));
      CK(cudaMemcpyAsync(ho, dptr<char>(L.out_off), (size_t)C * 4, cudaMemcpyDeviceToHost, stream));
    }
    if (NT) CK(cudaMemcpyAsync(ht, tgbuf.p, (size_t)NT * 4, cudaMemcpyDeviceToHost, stream));
    if (N > 1) CK(cudaMemcpyAsync(hc, dptr<char>(L.cout), (size_t)N * 8, cudaMemcpyDeviceToHost, stream));
    if (!fetch_ev)  // (a blocking wait sleeps, as wait() does: serving workers leave the cores to lowering)
      CK(cudaEventCreateWithFlags(&fetch_ev, cudaEventDisableTiming | (blocking_wait ? cudaEventBlockingSync : 0u)));
    CK(cudaEventRecord(fetch_ev, stream));
    last_d2h = (uint64_t)C * 12 + (uint64_t)NT * 4 + 12 + (N > 1 ? (uint64_t)N * 8 : 0);
    pf.active = true;
    pf.h = h;
    pf.C = C;
    pf.NT = NT;
    pf.N = N;
    pf.ndet.resize(N);
    pf.nobs.resize(N);
    pf.M.resize(N);
    for (uint32_t i = 0; i < N; ++i) {
      pf.ndet[i] = tapes[i].ndet;
      pf.nobs[i] = tapes[i].nobs;
      pf.M[i] = tapes[i].M;
    }
    pf.order = big_first;
    if (pf.order.size() != N) {
      pf.order.resize(N);
      for (uint32_t i = 0; i < N; ++i) pf.order[i] = i;
    }
    host_ms[4] = ms_since(t4);
  }

  // Waits for begin_fetch's copies and builds the DEMs: views into the result
  // block, or copies out of the staging buffer.
  void end_fetch(PendingFetch &pf, std::vector<gpc_dem *> &outs) {
    if (!pf.active) {
      outs.swap(pf.done);
      return;
    }
    const auto t4 = HostClock::now();
    CK(cudaEventSynchronize(fetch_ev));
    host_ms[4] += ms_since(t4);
    const auto t5 = HostClock::now();
    const uint32_t C = pf.C, NT = pf.NT, N = pf.N;
    const char *h = pf.h;
    const double *P = reinterpret_cast<const double *>(h);
    const uint32_t *O = reinterpret_cast<const uint32_t *>(h + (size_t)C * 8);
    const uint32_t *TG = reinterpret_cast<const uint32_t *>(h + (size_t)C * 12);
    const uint2 *CO = reinterpret_cast<const uint2 *>(h + (size_t)C * 12 + (size_t)NT * 4);
    const std::shared_ptr<ResultBlock> blk = std::move(pf.blk);
    pf.active = false;
    outs.assign(N, nullptr);
    try {
      for_each(N, N >= 8, [&](uint32_t x, uint32_t) {
        const uint32_t i = pf.order[x];
        const uint32_t c0 = N > 1 ? CO[i].x : 0, c1 = (N > 1 && i + 1 < N) ? CO[i + 1].x : C;
        const uint32_t t0 = N > 1 ? CO[i].y : 0, t1 = (N > 1 && i + 1 < N) ? CO[i + 1].y : NT;
        if (c1 < c0 || c1 > C || t1 < t0 || t1 > NT) throw gpc::Error(GPC_ERR_CUDA, "inconsistent batch ranges");
        std::unique_ptr<gpc_dem> dem(dem_cache().take());
        dem->num_detectors = pf.ndet[i];
        dem->num_observables = pf.nobs[i];
        dem->num_raw = pf.M[i];
        const uint32_t ne = c1 - c0, nt = t1 - t0;
        if (blk) {  // views into the block; the offsets rebased to the DEM's first target
          dem->block = blk;
          dem->probs.view(const_cast<double *>(P) + c0, ne);
          dem->targets.view(const_cast<uint32_t *>(TG) + t0, nt);
          dem->offsets.resize((size_t)ne + 1);
          uint32_t *dof = dem->offsets.data();
          for (uint32_t k = 0; k < ne; ++k) dof[k] = O[c0 + k] - t0;
          dof[ne] = nt;
          outs[i] = dem.release();
          return;
        }
        dem->probs.resize(ne);
        dem->offsets.resize((size_t)ne + 1);
        dem->targets.resize(nt);
        double *dp = dem->probs.data();
        uint32_t *dof = dem->offsets.data(), *dt = dem->targets.data();
        // one large result is copied in pieces on the host pool (a single
        // thread's copy rate would dominate the fetch)
        const uint32_t np = N == 1 && (size_t)ne * 12 + (size_t)nt * 4 >= (256u << 10) ? copy_pieces() : 1u;
        for_each(np, np > 1, [&](uint32_t q, uint32_t) {
          const uint32_t e0 = (uint32_t)((uint64_t)ne * q / np), e1 = (uint32_t)((uint64_t)ne * (q + 1) / np);
          const uint32_t g0 = (uint32_t)((uint64_t)nt * q / np), g1 = (uint32_t)((uint64_t)nt * (q + 1) / np);
          if (e1 > e0) memcpy(dp + e0, P + c0 + e0, (size_t)(e1 - e0) * 8);
          for (uint32_t k = e0; k < e1; ++k) dof[k] = O[c0 + k] - t0;
          if (g1 > g0) memcpy(dt + g0, TG + t0 + g0, (size_t)(g1 - g0) * 4);
        });
        dof[ne] = nt;
        outs[i] = dem.release();
      });
    } catch (...) {
      for (auto &d : outs)
        if (d) dem_cache().give(d);
      outs.assign(N, nullptr);
      throw;
    }
    host_ms[5] = ms_since(t5);
  }

  // Copies the merged arrays of the last run to the host and splits them per circuit.
  void fetch_all(std::vector<gpc_dem *> &outs) {
    PendingFetch pf;
    begin_fetch(pf);
    end_fetch(pf, outs);
  }

  // A batch whose merge needs a fallback (a symptom repeated more than a
  // bucket holds, or a symptom longer than the target lists): compile its
  // circuits one at a time on the single-circuit path.
  void batch_fallback(std::vector<gpc_dem *> &outs) {
    std::vector<Tape> T = std::move(tapes);
    const uint32_t N = (uint32_t)T.size();
    outs.assign(N, nullptr);
    try {
      for (uint32_t i = 0; i < N; ++i) {
        for (Tape &x : tapes) spare_tapes.push_back(std::move(x));  // kept (page-locked ops)
        tapes.clear();
        tapes.push_back(std::move(T[i]));
        tcap = 32;
        lists_off = false;
        prepare(nullptr, nullptr, 0);
        run();
        std::vector<gpc_dem *> one;
        fetch_all(one);
        outs[i] = one[0];
      }
    } catch (...) {
      for (auto &d : outs)
        if (d) dem_cache().give(d);
      outs.assign(N, nullptr);
      throw;
    }
  }

  gpc_dem *fetch() {
    std::vector<gpc_dem *> outs;
    fetch_all(outs);
    for (size_t i = 1; i < outs.size(); ++i)
      if (outs[i]) dem_cache().give(outs[i]);
    return outs.empty() ? nullptr : outs[0];
  }

  // Times the batched pipeline of these circuits in each walk configuration
  // (words per CTA x qubits per thread, one launch per thread-count class or
  // one persistent launch) and keeps the fastest for batches.
  // The tuning key of the prepared circuits (see TuneCache).
  uint64_t width_key() const {
    std::vector<uint64_t> cls;
    for (const Tape &T : tapes) {
      uint64_t w = 1;
      while (w < T.w) w <<= 1;
      cls.push_back(((uint64_t)T.qpad << 32) | w);
    }
    std::sort(cls.begin(), cls.end());
    cls.erase(std::unique(cls.begin(), cls.end()), cls.end());
    uint64_t h = 0xcbf29ce484222325ull;
    for (uint64_t v : cls) h = (h ^ v) * 0x100000001b3ull;
    return h;
  }
  bool tuned = false;  // this driver chose its batches' walk configuration itself

  void autotune(const char *const *texts, const size_t *lens, uint32_t n, uint32_t reps, gpc_tuning &out) {
    static const uint32_t cand[][3] = {{2, 1, 0}, {1, 1, 0}, {2, 2, 0}, {1, 2, 0}, {1, 4, 0},
                                       {2, 1, 1}, {1, 1, 1}, {2, 2, 1}, {1, 2, 1}};
    out = gpc_tuning{};
    tuned = true;
    prepare(texts, lens, n);  // lowered once: each configuration lays out the same tapes again
    float best = std::numeric_limits<float>::infinity();
    uint32_t bw = batch_words, bq = batch_qpt, bz = batch_queue;
    try {
      for (const auto &c : cand) {
        batch_words = c[0];
        batch_qpt = c[1];
        batch_queue = c[2];
        prepare(nullptr, nullptr, 0);
        // a persistent configuration that does not fit these circuits runs as classes: skip it
        const bool queued = L.classes.size() == 1 && L.classes[0].queue;
        if (c[2] && !queued) continue;
        run();  // first launches of this configuration
        float t = std::numeric_limits<float>::infinity();
        for (uint32_t r = 0; r < std::max(1u, reps); ++r) {
          CK(cudaEventRecord(tune_ev[0], stream));  // around the run (outside its graph)
          run();
          CK(cudaEventRecord(tune_ev[1], stream));
          CK(cudaEventSynchronize(tune_ev[1]));
          float ms = 0;
          CK(cudaEventElapsedTime(&ms, tune_ev[0], tune_ev[1]));
          t = std::min(t, ms);
        }
        if (out.num_tried < 12)
          out.tried[out.num_tried++] = gpc_tuning_entry{(int32_t)c[0], (int32_t)c[1], (int32_t)c[2], t};
        if (t < best) {
          best = t;
          bw = c[0];
          bq = c[1];
          bz = c[2];
        }
      }
    } catch (...) {
      batch_words = 0;
      batch_qpt = 0;
      batch_queue = 0;
      throw;
    }
    batch_words = bw;
    batch_qpt = bq;
    batch_queue = bz;
    const uint32_t cfg[3] = {bw, bq, bz};
    tune_cache().put(width_key(), cfg);  // for other drivers' batches of these widths
    prepare(nullptr, nullptr, 0);
    out.walk_words = (int32_t)bw;
    out.walk_qpt = (int32_t)bq;
    out.walk_queue = (int32_t)bz;
    out.ms = best;
  }

  // A second pipeline (own stream and buffers, same settings) for compile_batch.
  std::unique_ptr<gpc_driver> partner;
  gpc_driver &twin() {
    if (!partner) {
      std::unique_ptr<gpc_driver> d(new gpc_driver());
      d->device = device;
      d->level = level;
      d->sort_bits = sort_bits;
      d->force_global = force_global;
      d->walk_qpt = walk_qpt;
      d->bucket_mean = bucket_mean;
      d->walk_words = walk_words;
      d->key_split = key_split;
      d->batch_words = batch_words;
      d->batch_qpt = batch_qpt;
      d->batch_queue = batch_queue;
      d->walk_queue = walk_queue;
      d->walk_segment = walk_segment;
      d->pinned_results = pinned_results;
      d->incremental = incremental;
      d->spin_ns = spin_ns;
      d->init_streams();
      partner = std::move(d);
    }
    return *partner;
  }

  // Compiles n circuits to n DEMs (in order).  A large batch is cut into up to
  // four chunks that alternate between this pipeline and its twin: chunk c is
  // lowered on the host while chunk c-1 runs on the device, and chunk c-1's
  // results are split on the host while chunk c runs.  A circuit's DEM does not
  // depend on the circuits beside it, so the result equals one pipeline's.
  void compile_batch(const char *const *texts, const size_t *lens, uint32_t n, std::vector<gpc_dem *> &outs) {
    size_t bytes = 0;
    for (uint32_t i = 0; i < n; ++i) bytes += lens[i];
    const uint32_t K = n >= 32 && bytes >= (8u << 20) ? 4u : 1u;
    if (K == 1) {
      prepare(texts, lens, n);
      run();
      fetch_all(outs);
      return;
    }
    std::vector<uint32_t> cut{0};  // chunk c: circuits [cut[c], cut[c + 1]), about bytes / K of text each
    size_t acc = 0;
    for (uint32_t i = 0; i < n && cut.size() < K; ++i) {
      acc += lens[i];
      if (acc * K >= bytes * cut.size() && i + 1 < n) cut.push_back(i + 1);
    }
    cut.push_back(n);
    const uint32_t nc = (uint32_t)cut.size() - 1;
    gpc_driver *D[2] = {this, &twin()};
    outs.assign(n, nullptr);
    uint64_t h2d = 0, d2h = 0;
    double ms[6] = {};  // host phases summed over the chunks of both pipelines
    auto add_ms = [&](const gpc_driver *d, int k0, int k1) {
      for (int k = k0; k < k1; ++k) ms[k] += d->host_ms[k];
    };
    // Chunk c - 1's copies back are issued once chunk c is running, and its
    // DEMs built after chunk c + 1 is prepared on the same pipeline (whose
    // stream has drained them meanwhile): the host lowers while they copy.
    std::vector<PendingFetch> pend(nc);
    auto begin = [&](uint32_t c) {
      D[c & 1]->begin_fetch(pend[c]);
      add_ms(D[c & 1], 3, 5);
      d2h += D[c & 1]->last_d2h;
    };
    auto end = [&](uint32_t c) {
      std::vector<gpc_dem *> v;
      const double issued = D[c & 1]->host_ms[4];
      D[c & 1]->end_fetch(pend[c], v);
      ms[4] += D[c & 1]->host_ms[4] - issued;  // the wait for the copies
      add_ms(D[c & 1], 5, 6);
      for (uint32_t i = 0; i < (uint32_t)v.size(); ++i) outs[cut[c] + i] = v[i];
    };
    try {
      for (uint32_t c = 0; c < nc; ++c) {
        if (c == 1) {  // the second pipeline walks as the first one settled (tuned or cached)
          D[1]->batch_words = D[0]->batch_words;
          D[1]->batch_qpt = D[0]->batch_qpt;
          D[1]->batch_queue = D[0]->batch_queue;
          D[1]->tuned = true;
        }
        D[c & 1]->prepare(texts + cut[c], lens + cut[c], cut[c + 1] - cut[c]);
        add_ms(D[c & 1], 0, 3);
        h2d += D[c & 1]->last_h2d;
        if (c >= 2) end(c - 2);
        D[c & 1]->run();
        if (c >= 1) begin(c - 1);
      }
      begin(nc - 1);
      if (nc >= 2) end(nc - 2);
      end(nc - 1);
      last_h2d = h2d;
      last_d2h = d2h;
      for (int k = 0; k < 6; ++k) host_ms[k] = ms[k];
    } catch (...) {
      for (auto &d : outs)
        if (d) dem_cache().give(d);
      for (auto &pf : pend)
        for (auto &d : pf.done)
          if (d) dem_cache().give(d);
      outs.assign(n, nullptr);
      throw;
    }
  }
};

namespace {

template <typename F>
gpc_status guarded(F &&f) {
  try {
    f();
    g_last_error.clear();
    return GPC_OK;
  } catch (const gpc::Error &e) {
    return fail(e.code, e.what());
  } catch (const CudaError &e) {
    return fail(GPC_ERR_CUDA, e.what());
  } catch (const std::bad_alloc &) {
    return fail(GPC_ERR_OOM, "host allocation failed");
  } catch (const std::exception &e) {
    return fail(GPC_ERR_INVALID, e.what());
  }
}

}  // namespace

// ---- serving: continuous batching of compile requests ----------------------
//
// Requests wait in one FIFO queue.  Each of `slots` workers owns a resident
// driver (its own stream and device buffers, kept between requests) and loops:
// take every queued request up to max_batch, lower them on the host, admit
// the device bytes its buffers must grow by against the HBM budget (waiting
// until enough is free; a request that alone exceeds the budget fails), run
// the batched pipeline, deliver each DEM.  Workers run concurrently, so one
// batch's kernels overlap another's host lowering and kernels; requests that
// arrive while the GPU is busy join the next batch of the first free worker.
// When a worker waits for budget, others give their buffers back as they
// finish a batch.
struct gpc_server {
  struct Req {
    std::string text;
    std::chrono::steady_clock::time_point t0, t1;
    bool done = false;
    gpc_status status = GPC_OK;
    std::string msg;
    gpc_dem *dem = nullptr;
    std::unique_ptr<Tape> tape;  // lowered, waiting for a worker
  };
  std::deque<uint64_t> lower_queue;  // submitted, not yet lowered
  std::condition_variable cv_lower;
  std::vector<std::thread> lowerers;
  std::vector<Tape> spare;  // tapes of compiled batches, lowered into again (their memory kept)
  static constexpr size_t kSpareTapes = 32;
  int device = 0, level = 2;
  uint32_t max_batch = 16;
  bool incremental = false;  // each lowering thread lowers a request against its previous one
  size_t budget = 0, used = 0, peak = 0;
  uint32_t budget_waiters = 0;
  uint64_t next_ticket = 1, completed = 0, batches = 0;
  bool stop = false;
  std::mutex mu;
  std::condition_variable cv_work, cv_done, cv_budget;
  std::deque<uint64_t> queue;
  std::unordered_map<uint64_t, std::unique_ptr<Req>> reqs;
  std::vector<std::unique_ptr<gpc_driver>> drivers;
  std::vector<size_t> held;  // budget bytes held by each worker's buffers
  size_t max_ahead() const { return (size_t)2 * drivers.size() * max_batch; }  // lowered, waiting for a worker
  std::vector<std::thread> workers;

  // Admits `grow` more bytes for worker w (whose buffers will total `total`).
  // A worker that must wait first gives its own buffers back, so waiting
  // workers hold nothing and the running ones can always finish and free.
  void acquire(uint32_t w, size_t grow, size_t total) {
    std::unique_lock<std::mutex> lk(mu);
    if (total > budget) throw gpc::Error(GPC_ERR_CAPACITY, "the request needs more device memory than the serving budget");
    if (used + grow <= budget) {
      used += grow;
      held[w] += grow;
      peak = std::max(peak, used);
      return;
    }
    used -= held[w];
    held[w] = 0;
    lk.unlock();
    drivers[w]->release_device_memory();
    lk.lock();
    cv_budget.notify_all();
    ++budget_waiters;
    cv_budget.wait(lk, [&] { return stop || used + total <= budget; });
    --budget_waiters;
    if (stop) throw gpc::Error(GPC_ERR_INVALID, "server stopped");
    used += total;
    held[w] = total;
    peak = std::max(peak, used);
  }

  void give_back(uint32_t w) {
    drivers[w]->release_device_memory();
    std::lock_guard<std::mutex> lk(mu);
    used -= held[w];
    held[w] = 0;
    cv_budget.notify_all();
  }

  void deliver(uint64_t t, gpc_status st, const std::string &msg, gpc_dem *dem) {
    std::lock_guard<std::mutex> lk(mu);
    Req &r = *reqs.at(t);
    r.status = st;
    r.msg = msg;
    r.dem = dem;
    r.t1 = std::chrono::steady_clock::now();
    r.done = true;
    ++completed;
  }

  // Lowering threads: parse and lower each request as it arrives (in
  // parallel across requests), then hand it to the GPU workers.
  void lowerer() {
    gpc::LowerScratch scratch;
    gpc::LowerOptions lo;
    lo.level = level;
    lo.chunk_min = gpc::kWalkChunkMin;  // requests are compiled in batches
    lo.sources = false;
    lo.segment_occ = 8192;  // as the driver lowers
    lo.incremental = incremental;
    while (true) {
      uint64_t t;
      const char *text;
      size_t len;
      {
        // back-pressure: at most two rounds of full batches lowered ahead of the workers (bounded
        // host memory; their tapes stay within the page-locked pool)
        std::unique_lock<std::mutex> lk(mu);
        cv_lower.wait(lk, [&] { return stop || (!lower_queue.empty() && queue.size() < max_ahead()); });
        if (stop) return;
        t = lower_queue.front();
        lower_queue.pop_front();
        text = reqs.at(t)->text.data();
        len = reqs.at(t)->text.size();
      }
      try {
        auto tape = std::make_unique<Tape>();
        {
          std::lock_guard<std::mutex> lk(mu);
          if (!spare.empty()) {
            *tape = std::move(spare.back());
            spare.pop_back();
          }
        }
        pin_ops(*tape);
        gpc::lower_text(text, len, lo, *tape, scratch);
        {
          std::lock_guard<std::mutex> lk(mu);
          reqs.at(t)->tape = std::move(tape);
          queue.push_back(t);
        }
        cv_work.notify_one();
      } catch (const gpc::Error &e) {
        deliver(t, e.code, e.what(), nullptr);
        cv_done.notify_all();
      } catch (const std::bad_alloc &) {
        deliver(t, GPC_ERR_OOM, "host allocation failed", nullptr);
        cv_done.notify_all();
      } catch (const std::exception &e) {
        deliver(t, GPC_ERR_INVALID, e.what(), nullptr);
        cv_done.notify_all();
      }
    }
  }

  // Compiles tickets ts on worker w's driver (one batched pipeline over their
  // lowered tapes, or from their texts when `from_text`).
  void compile(uint32_t w, const std::vector<uint64_t> &ts, bool from_text) {
    gpc_driver &d = *drivers[w];
    if (from_text) {
      std::vector<const char *> texts;
      std::vector<size_t> lens;
      {
        std::lock_guard<std::mutex> lk(mu);
        for (uint64_t t : ts) {
          texts.push_back(reqs.at(t)->text.data());
          lens.push_back(reqs.at(t)->text.size());
        }
      }
      d.prepare(texts.data(), lens.data(), (uint32_t)ts.size());
    } else {
      std::vector<Tape> tapes;
      {
        std::lock_guard<std::mutex> lk(mu);
        for (uint64_t t : ts) {
          tapes.push_back(std::move(*reqs.at(t)->tape));
          reqs.at(t)->tape.reset();
        }
      }
      d.prepare_tapes(tapes);
      {
        std::lock_guard<std::mutex> lk(mu);
        for (auto &x : tapes)
          if (spare.size() < kSpareTapes) spare.push_back(std::move(x));
      }
    }
    d.run();
    std::vector<gpc_dem *> outs;
    d.fetch_all(outs);
    for (size_t i = 0; i < ts.size(); ++i) deliver(ts[i], GPC_OK, "", outs[i]);
  }

  void worker(uint32_t w) {
    cudaSetDevice(device);
    while (true) {
      std::vector<uint64_t> ts;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv_work.wait(lk, [&] { return stop || !queue.empty(); });
        if (stop) return;
        while (!queue.empty() && ts.size() < max_batch) {
          ts.push_back(queue.front());
          queue.pop_front();
        }
      }
      cv_lower.notify_all();  // room below the back-pressure bound
      auto run_one_by_one = [&](const std::vector<uint64_t> &list) {
        for (uint64_t t : list) {
          try {
            compile(w, {t}, true);
          } catch (const gpc::Error &e) {
            deliver(t, e.code, e.what(), nullptr);
          } catch (const std::exception &e) {
            deliver(t, GPC_ERR_CUDA, e.what(), nullptr);
          }
        }
      };
      try {
        compile(w, ts, false);
      } catch (const gpc::Error &e) {
        // one request's failure must not fail the others: compile them singly
        if (ts.size() > 1) run_one_by_one(ts);
        else deliver(ts[0], e.code, e.what(), nullptr);
      } catch (const std::exception &e) {
        if (ts.size() > 1) run_one_by_one(ts);
        else deliver(ts[0], GPC_ERR_CUDA, e.what(), nullptr);
      }
      bool waiting;
      {
        std::lock_guard<std::mutex> lk(mu);
        ++batches;
        waiting = budget_waiters > 0;
      }
      cv_done.notify_all();
      if (waiting) give_back(w);
    }
  }

  ~gpc_server() {
    {
      std::lock_guard<std::mutex> lk(mu);
      stop = true;
    }
    cv_work.notify_all();
    cv_budget.notify_all();
    cv_lower.notify_all();
    for (auto &t : workers)
      if (t.joinable()) t.join();
    for (auto &t : lowerers)
      if (t.joinable()) t.join();
    for (auto &kv : reqs)
      if (kv.second->dem) delete kv.second->dem;
  }
};

extern "C" {

const char *gpc_last_error(void) { return g_last_error.c_str(); }

gpc_status gpc_get_driver(const char *stim_text, size_t len, int32_t correlation_level, const gpc_options *options,
                          gpc_driver **out) {
  if (!out) return fail(GPC_ERR_INVALID, "out is null");
  *out = nullptr;
  if (!stim_text) return fail(GPC_ERR_INVALID, "circuit text is null");
  if (correlation_level < 0 || correlation_level > 2) return fail(GPC_ERR_INVALID, "correlation level must be 0, 1 or 2");
  std::unique_ptr<gpc_driver> d(new (std::nothrow) gpc_driver());
  if (!d) return fail(GPC_ERR_OOM, "host allocation failed");
  d->level = correlation_level;
  if (options) {
    d->device = options->device;
    if (options->sort_bits < 0 || options->sort_bits > 64) return fail(GPC_ERR_INVALID, "sort_bits must be in 0..64");
    if (options->sort_bits) d->sort_bits = (uint32_t)options->sort_bits;
    d->force_global = options->global_sort != 0;
    if (options->walk_qpt < 0 || (options->walk_qpt && !gpc::walk_max_threads((uint32_t)options->walk_qpt)))
      return fail(GPC_ERR_INVALID, "walk_qpt must be 0, 1, 2, 3, 4, 6, 8, 12 or 16");
    d->walk_qpt = (uint32_t)options->walk_qpt;
    if (options->bucket_mean < 0 || (options->bucket_mean && (options->bucket_mean < 8 || options->bucket_mean > 128)))
      return fail(GPC_ERR_INVALID, "bucket_mean must be 0 or 8..128");
    d->bucket_mean = (uint32_t)options->bucket_mean;
    if (options->walk_words < 0 || options->walk_words > 2) return fail(GPC_ERR_INVALID, "walk_words must be 0, 1 or 2");
    d->walk_words = (uint32_t)options->walk_words;
    if (options->key_split != 0 && options->key_split != -1) return fail(GPC_ERR_INVALID, "key_split must be 0 or -1");
    d->key_split = options->key_split == 0;
    if (options->walk_queue < -1 || options->walk_queue > 1) return fail(GPC_ERR_INVALID, "walk_queue must be -1, 0 or 1");
    d->walk_queue = options->walk_queue;
    if (options->walk_segment < -1) return fail(GPC_ERR_INVALID, "walk_segment must be -1, 0 or positive");
    d->walk_segment = options->walk_segment;
    if (options->wait_limit_us < 0 || options->test_hold_tile < 0)
      return fail(GPC_ERR_INVALID, "wait_limit_us and test_hold_tile must be >= 0");
    if (options->wait_limit_us) d->spin_ns = (unsigned long long)options->wait_limit_us * 1000ull;
    d->hold_runs = (uint32_t)options->test_hold_tile;
    if (options->test_fail_alloc < 0) return fail(GPC_ERR_INVALID, "test_fail_alloc must be >= 0");
    if (options->test_fail_alloc) d->alloc_ctr.fail_at = options->test_fail_alloc - 1;
    if (options->heap_results != 0 && options->heap_results != 1) return fail(GPC_ERR_INVALID, "heap_results must be 0 or 1");
    d->pinned_results = options->heap_results == 0;
    if (options->incremental != 0 && options->incremental != 1) return fail(GPC_ERR_INVALID, "incremental must be 0 or 1");
    d->incremental = options->incremental == 1;
  }
  gpc_status st = guarded([&] {
    int n = 0;
    CK(cudaGetDeviceCount(&n));
    if (d->device < 0 || d->device >= n) throw gpc::Error(GPC_ERR_CUDA, "no such CUDA device");
    CK(cudaSetDevice(d->device));
    d->init_streams();
    CK(gpc::walk_set_smem_limit());  // per device: the driver's device is current here
    d->prepare(&stim_text, &len, 1);
  });
  if (st != GPC_OK) return st;
  *out = d.release();
  return GPC_OK;
}

gpc_status gpc_prepare(gpc_driver *driver, const char *stim_text, size_t len) {
  if (!driver) return fail(GPC_ERR_INVALID, "driver is null");
  return guarded([&] {
    if (stim_text) driver->prepare(&stim_text, &len, 1);
    else driver->prepare(nullptr, nullptr, 0);
  });
}

gpc_status gpc_prepare_batch(gpc_driver *driver, const char *const *texts, const size_t *lens, int32_t n) {
  if (!driver || !texts || !lens || n <= 0) return fail(GPC_ERR_INVALID, "bad batch arguments");
  for (int32_t i = 0; i < n; ++i)
    if (!texts[i]) return fail(GPC_ERR_INVALID, "null circuit text in batch");
  return guarded([&] { driver->prepare(texts, lens, (uint32_t)n); });
}

gpc_status gpc_fetch_batch(gpc_driver *driver, gpc_dem **outs, int32_t n) {
  if (!driver || !outs || n <= 0) return fail(GPC_ERR_INVALID, "bad batch arguments");
  for (int32_t i = 0; i < n; ++i) outs[i] = nullptr;
  return guarded([&] {
    if ((uint32_t)n != driver->ncirc()) throw gpc::Error(GPC_ERR_INVALID, "batch size differs from the prepared batch");
    std::vector<gpc_dem *> v;
    driver->fetch_all(v);
    for (int32_t i = 0; i < n; ++i) outs[i] = v[i];
  });
}

gpc_status gpc_device_dem(gpc_driver *driver, int32_t circuit, const double **probs, const uint32_t **offsets,
                          const uint32_t **targets, uint32_t *num_errors, uint32_t *targets_end) {
  if (!driver || !probs || !offsets || !targets || !num_errors || !targets_end || circuit < 0)
    return fail(GPC_ERR_INVALID, "bad arguments");
  return guarded([&] { driver->device_dem((uint32_t)circuit, probs, offsets, targets, num_errors, targets_end); });
}

gpc_status gpc_param_prepare(gpc_driver *driver, const char *stim_text, size_t len, uint32_t *num_ticks) {
  if (!driver || !stim_text) return fail(GPC_ERR_INVALID, "bad arguments");
  return guarded([&] {
    driver->prepare(&stim_text, &len, 1, true);
    if (num_ticks) *num_ticks = driver->tapes[0].n_ticks;
  });
}

gpc_status gpc_param_forward(gpc_driver *driver, const double *noise, void *stream, uint32_t *num_errors) {
  if (!driver) return fail(GPC_ERR_INVALID, "driver is null");
  return guarded([&] {
    const uint32_t c = driver->param_forward(noise, static_cast<cudaStream_t>(stream));
    if (num_errors) *num_errors = c;
  });
}

gpc_status gpc_param_probs(gpc_driver *driver, double *probs, void *stream) {
  if (!driver || !probs) return fail(GPC_ERR_INVALID, "bad arguments");
  return guarded([&] { driver->param_probs(probs, static_cast<cudaStream_t>(stream)); });
}

gpc_status gpc_param_backward(gpc_driver *driver, const double *grad_probs, double *grad_noise, void *stream) {
  if (!driver) return fail(GPC_ERR_INVALID, "driver is null");
  return guarded([&] { driver->param_backward(grad_probs, grad_noise, static_cast<cudaStream_t>(stream)); });
}

gpc_status gpc_run_device(gpc_driver *driver) {
  if (!driver) return fail(GPC_ERR_INVALID, "driver is null");
  return guarded([&] { driver->run(); });
}

gpc_status gpc_fetch(gpc_driver *driver, gpc_dem **out) {
  if (!driver || !out) return fail(GPC_ERR_INVALID, "null argument");
  *out = nullptr;
  return guarded([&] { *out = driver->fetch(); });
}

gpc_status gpc_compile(gpc_driver *driver, const char *stim_text, size_t len, gpc_dem **out) {
  if (!driver || !out) return fail(GPC_ERR_INVALID, "null argument");
  *out = nullptr;
  return guarded([&] {
    if (stim_text) driver->prepare(&stim_text, &len, 1);
    else driver->prepare(nullptr, nullptr, 0);  // re-upload the parsed circuit, as the reference re-copies it
    driver->run();
    *out = driver->fetch();
  });
}

gpc_status gpc_compile_batch(gpc_driver *driver, const char *const *texts, const size_t *lens, int32_t n,
                             gpc_dem **outs) {
  if (!driver || !texts || !lens || !outs || n <= 0) return fail(GPC_ERR_INVALID, "bad batch arguments");
  for (int32_t i = 0; i < n; ++i) outs[i] = nullptr;
  for (int32_t i = 0; i < n; ++i)
    if (!texts[i]) return fail(GPC_ERR_INVALID, "null circuit text in batch");
  return guarded([&] {
    std::vector<gpc_dem *> v;
    driver->compile_batch(texts, lens, (uint32_t)n, v);
    for (int32_t i = 0; i < n; ++i) outs[i] = v[i];
  });
}

gpc_status gpc_autotune(gpc_driver *driver, const char *const *texts, const size_t *lens, int32_t n, int32_t reps,
                        gpc_tuning *out) {
  if (!driver || !texts || !lens || !out || n < 2) return fail(GPC_ERR_INVALID, "autotune takes a batch of two or more circuits");
  for (int32_t i = 0; i < n; ++i)
    if (!texts[i]) return fail(GPC_ERR_INVALID, "null circuit text in batch");
  return guarded([&] {
    driver->autotune(texts, lens, (uint32_t)n, (uint32_t)std::max(1, reps), *out);
    if (driver->partner) {  // the second pipeline of compile_batch follows the choice
      driver->partner->batch_words = driver->batch_words;
      driver->partner->batch_qpt = driver->batch_qpt;
      driver->partner->batch_queue = driver->batch_queue;
    }
  });
}

gpc_status gpc_dem_arrays(const gpc_dem *dem, const uint32_t **offsets, const uint32_t **targets, const double **probs,
                          uint32_t *num_errors) {
  if (!dem) return fail(GPC_ERR_INVALID, "dem is null");
  if (offsets) *offsets = dem->offsets.data();
  if (targets) *targets = dem->targets.data();
  if (probs) *probs = dem->probs.data();
  if (num_errors) *num_errors = (uint32_t)dem->probs.size();
  return GPC_OK;
}

gpc_status gpc_dem_info(const gpc_dem *dem, uint32_t *num_detectors, uint32_t *num_observables,
                        uint64_t *num_raw_mechanisms) {
  if (!dem) return fail(GPC_ERR_INVALID, "dem is null");
  if (num_detectors) *num_detectors = dem->num_detectors;
  if (num_observables) *num_observables = dem->num_observables;
  if (num_raw_mechanisms) *num_raw_mechanisms = dem->num_raw;
  return GPC_OK;
}

gpc_status gpc_dem_text(const gpc_dem *dem_c, const char **text, size_t *len) {
  if (!dem_c || !text) return fail(GPC_ERR_INVALID, "null argument");
  gpc_dem *dem = const_cast<gpc_dem *>(dem_c);
  return guarded([&] {
    if (!dem->text_ready) {
      std::string s;
      s.reserve(dem->probs.size() * 48);
      char buf[64];
      for (size_t i = 0; i < dem->probs.size(); ++i) {
        int n = snprintf(buf, sizeof buf, "error(%.17g)", dem->probs[i]);
        s.append(buf, (size_t)n);
        for (uint32_t k = dem->offsets[i]; k < dem->offsets[i + 1]; ++k) {
          uint32_t t = dem->targets[k];
          n = t < dem->num_detectors ? snprintf(buf, sizeof buf, " D%u", t)
                                     : snprintf(buf, sizeof buf, " L%u", t - dem->num_detectors);
          s.append(buf, (size_t)n);
        }
        s.push_back('\n');
      }
      dem->text = std::move(s);
      dem->text_ready = true;
    }
    *text = dem->text.c_str();
    if (len) *len = dem->text.size();
  });
}

void gpc_dem_free(gpc_dem *dem) {
  if (dem) dem_cache().give(dem);
}

gpc_status gpc_server_create(const gpc_server_options *options, gpc_server **out) {
  if (!out) return fail(GPC_ERR_INVALID, "out is null");
  *out = nullptr;
  gpc_server_options o{};
  o.slots = 4;
  o.max_batch = 16;
  o.hbm_budget = 120ull << 30;
  o.correlation_level = 2;
  if (options) o = *options;
  if (o.slots == 0 || o.slots > 64 || o.max_batch == 0 || o.hbm_budget == 0)
    return fail(GPC_ERR_INVALID, "bad server options");
  if (o.correlation_level < 0 || o.correlation_level > 2) return fail(GPC_ERR_INVALID, "bad correlation level");
  std::unique_ptr<gpc_server> sv(new (std::nothrow) gpc_server());
  if (!sv) return fail(GPC_ERR_OOM, "host allocation failed");
  sv->device = o.device;
  sv->level = o.correlation_level;
  sv->max_batch = o.max_batch;
  sv->budget = o.hbm_budget;
  if (o.incremental > 1) return fail(GPC_ERR_INVALID, "incremental must be 0 or 1");
  sv->incremental = o.incremental == 1;
  gpc_status st = guarded([&] {
    int n = 0;
    CK(cudaGetDeviceCount(&n));
    if (sv->device < 0 || sv->device >= n) throw gpc::Error(GPC_ERR_CUDA, "no such CUDA device");
    CK(cudaSetDevice(sv->device));
    CK(gpc::walk_set_smem_limit());
    sv->held.assign(o.slots, 0);
    gpc_server *raw = sv.get();
    // host threads: about one core per GPU worker, the rest lowering requests.
    // Workers sleep while their batch runs, so one lowering thread more than
    // the cores left fits (on 16 Grace cores, 4 slots: 13 lowering threads
    // measured ~5.9k DEM/s, 12 ~5.5k, 14 ~5.7k; far more threads than cores
    // measured 27% less); a worker's own pool for staging and splitting its
    // batches gets its share of the cores
    const uint32_t hw = host_threads();
    for (uint32_t w = 0; w < o.slots; ++w) {
      std::unique_ptr<gpc_driver> d(new gpc_driver());
      d->device = sv->device;
      d->level = sv->level;
      d->pool_threads = std::max(1u, hw / o.slots);
      d->pool_spin_us = 0;  // the lowering threads need the cores between a worker's hand-offs
      d->blocking_wait = true;  // and while the GPU runs the worker's batch
      d->init_streams();
      d->admit = [raw, w](size_t grow, size_t total) { raw->acquire(w, grow, total); };
      d->arena.slack = d->tgbuf.slack = false;  // the budget counts exact bytes
      sv->drivers.push_back(std::move(d));
    }
    for (uint32_t w = 0; w < o.slots; ++w) sv->workers.emplace_back([raw, w] { raw->worker(w); });
    const uint32_t nl = o.lower_threads ? o.lower_threads : std::max(1u, hw > o.slots ? hw - o.slots + 1 : 1u);
    for (uint32_t i = 0; i < nl; ++i) sv->lowerers.emplace_back([raw] { raw->lowerer(); });
  });
  if (st != GPC_OK) return st;
  *out = sv.release();
  return GPC_OK;
}

gpc_status gpc_server_submit(gpc_server *server, const char *stim_text, size_t len, uint64_t *ticket) {
  if (!server || !stim_text || !ticket) return fail(GPC_ERR_INVALID, "null argument");
  return guarded([&] {
    auto r = std::make_unique<gpc_server::Req>();
    r->text.assign(stim_text, len);
    r->t0 = std::chrono::steady_clock::now();
    {
      std::lock_guard<std::mutex> lk(server->mu);
      const uint64_t t = server->next_ticket++;
      server->reqs.emplace(t, std::move(r));
      server->lower_queue.push_back(t);
      *ticket = t;
    }
    server->cv_lower.notify_one();
  });
}

gpc_status gpc_server_wait(gpc_server *server, uint64_t ticket, double timeout_s, gpc_dem **out, double *latency_s) {
  if (!server || !out) return fail(GPC_ERR_INVALID, "null argument");
  *out = nullptr;
  std::unique_ptr<gpc_server::Req> r;
  {
    std::unique_lock<std::mutex> lk(server->mu);
    auto it = server->reqs.find(ticket);
    if (it == server->reqs.end()) return fail(GPC_ERR_INVALID, "unknown ticket");
    gpc_server::Req *p = it->second.get();
    const auto until = std::chrono::steady_clock::now() + std::chrono::duration<double>(std::max(0.0, timeout_s));
    if (!server->cv_done.wait_until(lk, until, [&] { return p->done; }))
      return fail(GPC_ERR_TIMEOUT, "request not finished");
    r = std::move(it->second);
    server->reqs.erase(it);
  }
  if (latency_s) *latency_s = std::chrono::duration<double>(r->t1 - r->t0).count();
  if (r->status != GPC_OK) return fail(r->status, r->msg);
  *out = r->dem;
  return GPC_OK;
}

gpc_status gpc_fallback_counts(gpc_driver *driver, uint64_t *counts5) {
  if (!driver || !counts5) return fail(GPC_ERR_INVALID, "null argument");
  for (int i = 0; i < 5; ++i) {
    counts5[i] = driver->fallbacks[i].load();
    if (driver->partner) counts5[i] += driver->partner->fallbacks[i].load();
  }
  return GPC_OK;
}

gpc_status gpc_server_fallback_counts(gpc_server *server, uint64_t *counts5) {
  if (!server || !counts5) return fail(GPC_ERR_INVALID, "null argument");
  for (int i = 0; i < 5; ++i) counts5[i] = 0;
  std::lock_guard<std::mutex> lk(server->mu);
  for (const auto &d : server->drivers) {
    if (!d) continue;
    uint64_t c[5];
    gpc_fallback_counts(d.get(), c);
    for (int i = 0; i < 5; ++i) counts5[i] += c[i];
  }
  return GPC_OK;
}

gpc_status gpc_server_stats(gpc_server *server, uint64_t *completed, uint64_t *batches, uint64_t *budget_used,
                            uint64_t *budget_peak) {
  if (!server) return fail(GPC_ERR_INVALID, "server is null");
  std::lock_guard<std::mutex> lk(server->mu);
  if (completed) *completed = server->completed;
  if (batches) *batches = server->batches;
  if (budget_used) *budget_used = server->used;
  if (budget_peak) *budget_peak = server->peak;
  return GPC_OK;
}

void gpc_server_destroy(gpc_server *server) { delete server; }

void gpc_driver_destroy(gpc_driver *driver) { delete driver; }

void *gpc_driver_stream(gpc_driver *driver) { return driver ? (void *)driver->stream : nullptr; }

gpc_status gpc_walk_config(gpc_driver *driver, int32_t *words, int32_t *qpt, int32_t *queue) {
  if (!driver || !words || !qpt || !queue) return fail(GPC_ERR_INVALID, "null argument");
  *words = (int32_t)driver->batch_words;
  *qpt = (int32_t)driver->batch_qpt;
  *queue = (int32_t)driver->batch_queue;
  return GPC_OK;
}

void gpc_tune_cache_clear(void) { tune_cache().clear(); }

gpc_status gpc_walk_form(gpc_driver *driver, int32_t *launches, int32_t *persistent) {
  if (!driver || !launches || !persistent) return fail(GPC_ERR_INVALID, "null argument");
  if (!driver->prepared) return fail(GPC_ERR_INVALID, "no circuit prepared");
  *launches = (int32_t)driver->L.classes.size();
  *persistent = driver->L.classes.size() == 1 && driver->L.classes[0].queue ? 1 : 0;
  return GPC_OK;
}

gpc_status gpc_alloc_counts(gpc_driver *driver, uint64_t *device_allocs, uint64_t *device_frees) {
  if (!driver || !device_allocs || !device_frees) return fail(GPC_ERR_INVALID, "null argument");
  *device_allocs = driver->alloc_ctr.allocs;
  *device_frees = driver->alloc_ctr.frees;
  return GPC_OK;
}

gpc_status gpc_walk_segments(gpc_driver *driver, uint32_t *segments, uint32_t *items_first, uint32_t *items_rest) {
  if (!driver || !segments || !items_first || !items_rest) return fail(GPC_ERR_INVALID, "null argument");
  if (!driver->prepared) return fail(GPC_ERR_INVALID, "no circuit prepared");
  *segments = driver->seg_on ? (uint32_t)driver->seg_bounds.size() - 1 : 0u;
  *items_first = driver->seg_on ? driver->seg_na : 0u;
  *items_rest = driver->seg_on ? driver->seg_nb : 0u;
  return GPC_OK;
}

gpc_status gpc_last_host_timings(gpc_driver *driver, double *ms6) {
  if (!driver || !ms6) return fail(GPC_ERR_INVALID, "null argument");
  for (int k = 0; k < 6; ++k) ms6[k] = driver->host_ms[k];
  return GPC_OK;
}

gpc_status gpc_set_stage_timing(gpc_driver *driver, int32_t on) {
  if (!driver) return fail(GPC_ERR_INVALID, "null argument");
  driver->stage_timing = on != 0;
  return GPC_OK;
}

gpc_status gpc_last_timings(gpc_driver *driver, float *ms5) {
  if (!driver || !ms5) return fail(GPC_ERR_INVALID, "null argument");
  if (!driver->ran) return fail(GPC_ERR_INVALID, "nothing has been run");
  if (!driver->timed_run) return fail(GPC_ERR_INVALID, "the last run had stage timing off (gpc_set_stage_timing)");
  return guarded([&] {
    CK(cudaEventSynchronize(driver->ev[4]));
    for (int i = 0; i < 4; ++i) CK(cudaEventElapsedTime(&ms5[i], driver->ev[i], driver->ev[i + 1]));
    CK(cudaEventElapsedTime(&ms5[4], driver->ev[0], driver->ev[4]));
  });
}

gpc_status gpc_last_traffic(gpc_driver *driver, double *bytes4) {
  if (!driver || !bytes4) return fail(GPC_ERR_INVALID, "null argument");
  if (!driver->ran) return fail(GPC_ERR_INVALID, "nothing has been run");
  return guarded([&] { driver->traffic(bytes4); });
}

gpc_status gpc_last_io_bytes(gpc_driver *driver, uint64_t *h2d, uint64_t *d2h) {
  if (!driver) return fail(GPC_ERR_INVALID, "driver is null");
  if (h2d) *h2d = driver->last_h2d;
  if (d2h) *d2h = driver->last_d2h;
  return GPC_OK;
}

gpc_status gpc_last_sizes(gpc_driver *driver, uint64_t *raw, uint64_t *points, uint32_t *epochs, uint32_t *words,
                          uint32_t *qubits) {
  if (!driver) return fail(GPC_ERR_INVALID, "driver is null");
  uint64_t r = 0, p = 0;
  uint32_t e = 0, w = 0, q = 0;
  for (const auto &T : driver->tapes) {  // sums over a batch; epochs/words/qubits: the largest circuit
    r += T.M;
    p += T.npoints;
    e = std::max(e, T.n_epochs);
    w = std::max(w, T.w);
    q = std::max(q, T.nq);
  }
  if (raw) *raw = r;
  if (points) *points = p;
  if (epochs) *epochs = e;
  if (words) *words = w;
  if (qubits) *qubits = q;
  return GPC_OK;
}

}  // extern "C"
