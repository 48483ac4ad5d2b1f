// walk.cu -- the backward Pauli-frame walk (propagate + emit), sm_103a.
//
// Replaces the reference's sensitivity generation (K1 scatterInitialSensitivities
// + K2 backwardsLayerTraversalKernel, Policies/Compute/CUDA.hpp:27-52,388-414,
// CUDAHandlers.hpp:38-62), which materialises a node x word matrix for 8 nodes
// per qubit per tick and needs a grid-wide sync per tick.
//
// Here one CTA walks one 64-bit word j of the detector bitset for one circuit.
// Thread t owns qubits t, t+T, ... and keeps their rows X_q, Z_q (the
// detectors among bits 64j..64j+63 flipped by an X / Z error on q at the
// current time) in registers.  Words are independent, so CTAs never talk.
// Per epoch:
//   1. every thread publishes its rows to shared memory (double buffered);
//   2. __syncthreads_or() -- the only barrier of the epoch -- also tells the
//      CTA whether any row is non-zero; once every row is zero and no
//      measurement of word j remains, the rest of the walk would only see
//      zeros, so the CTA stops and records the point range it covered;
//   3. the epoch's ops are read from shared memory: the tape is cut (on the
//      host) into chunks of whole epochs, and one thread copies chunk c+1
//      with a single cp.async.bulk (TMA) into the second of two buffers
//      while the CTA executes chunk c; a chunk's copy completes on its
//      buffer's mbarrier, which every thread waits on once per chunk (waits
//      are bounded by %globaltimer and report DEV_ERR_TIMEOUT);
//   4. ops: one-qubit Cliffords, two-qubit Cliffords (partner rows from the
//      published buffer), resets, measurements (XOR in the measurement's bits
//      that fall in word j; the bits ride in the tape itself), snapshots of
//      (X, Z) at noise points; a non-zero snapshot also sets word j's bit in
//      the point's mask (an atomic OR), so later stages visit only the
//      non-zero words of a point.
// The epoch and chunk tables are staged in shared memory at start, so no
// global load sits on the per-epoch critical path.
//
// Two launch forms share that body (walk_item): one CTA per item for the
// circuits of one thread-count class (walk_kernel), or one persistent launch
// over a whole batch (walk_queue_kernel) whose resident CTAs, sized for the
// largest circuit, take (circuit, word group) items from a queue counter,
// longest first, until it runs dry.
#include <algorithm>
#include <cstdint>

#include "device.cuh"
#include "lower.hpp"

namespace gpc {
namespace {

constexpr unsigned long long kWaitLimitNs = 200ull * 1000 * 1000;  // 200 ms

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Waits for phase `parity` of `bar`; false after kWaitLimitNs.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = globaltimer();
  while (!mbar_try_wait(bar, parity)) {
    if (globaltimer() - t0 > kWaitLimitNs) return false;
  }
  return true;
}

// *p |= v as a reduction that returns nothing: the thread does not wait for
// the atomic's round trip through L2 (measured 8 us of an 82 us walk).
__device__ __forceinline__ void red_or(unsigned long long *p, unsigned long long v) {
  asm volatile("red.global.or.b64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// 1D bulk copy global -> shared, completing `bytes` of transaction count on `bar`.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ uint64_t lds64(uint32_t a) {
  uint64_t v;
  asm volatile("ld.shared.u64 %0, [%1];" : "=l"(v) : "r"(a));
  return v;
}

__device__ __forceinline__ ulonglong2 lds128(uint32_t a) {
  ulonglong2 v;
  asm volatile("ld.shared.v2.u64 {%0, %1}, [%2];" : "=l"(v.x), "=l"(v.y) : "r"(a));
  return v;
}

__device__ __forceinline__ uint64_t sel2(uint32_t m, uint64_t x, uint64_t z) {
  return (x & (0ull - (uint64_t)(m & 1u))) ^ (z & (0ull - (uint64_t)((m >> 1) & 1u)));
}

__device__ __forceinline__ uint64_t sel4(uint32_t m, uint64_t a, uint64_t b, uint64_t c, uint64_t d) {
  return sel2(m & 3u, a, b) ^ sel2((m >> 2) & 3u, c, d);
}

// Largest block of each qubits-per-thread instance (registers: 4 QPT u64 of state per thread).
template <int QPT>
struct WalkBound {
  static constexpr int value = QPT <= 2 || QPT == 4 ? 1024 : QPT == 3 ? 512 : QPT <= 8 ? 256 : 128;
};

__device__ __forceinline__ void mbar_inval(uint64_t *bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

enum : uint32_t { ITEM_DONE = 0, ITEM_EMPTY = 1, ITEM_ABORTED = 2 };

// What walk_item runs: the plain walk of words j0 .. j0+W-1, or one item of
// the segmented walk (device.cuh: SEG_*; one word per CTA).
enum : int { MODE_PLAIN = 0, MODE_FIRST = 1, MODE_AFF = 2, MODE_XFER = 3, MODE_REST = 4 };

// One segment item as walk_item sees it.
struct SegCtx {
  uint32_t e_begin, e_end;  // epochs walked
  uint64_t *out;            // FIRST / AFF / XFER: exit rows ([2 qpad]; null: none)
  const uint64_t *in;       // REST: entry rows of segment s_from
  const uint64_t *state;    // all states (transfer columns, AFF exits)
  const uint32_t *aff_row;  // REST: [S] AFF state of this word in each segment (kNoState: none)
  uint32_t *xcnt;           // [S][2 qpad] entries of each transfer row (XFER adds, REST reads)
  uint16_t *xlst;           // entries (the rows at the segment's start, as word offsets in a published
                            // buffer: 2 slot for X, 2 slot + 1 for Z): [S][2 qpad][kSegRingCap] entries
                            // 0..7, then [S][2 qpad][kSegRowCap - kSegRingCap] entries 8..15
  uint32_t xfer0, ncol, s_from, s_to;
  uint32_t col, seg;        // XFER: the unit column walked, its segment
  uint32_t ring_nb;         // REST: step buffers of the compose ring
  uint32_t S;               // segments of the plan (sizes the staged AFF table)
};
constexpr uint32_t kNoState = 0xFFFFFFFFu;

// Bytes of one compose step in shared memory: entry counts (u32), entries
// 0..7 (kSegRingCap u16) and the segment's AFF rows (u64) of every row.
__host__ __device__ constexpr size_t seg_step_bytes(uint32_t qpad) {
  return (size_t)2 * qpad * (4 + 2 * kSegRingCap + 8);
}

// XFER exit: the set bits of row r's word of column col, as entries of the
// row's sparse list (order is free: the compose XORs them).  An entry is the
// row's word offset in a published buffer, so the compose adds it to the
// buffer's address as it is.
__device__ __forceinline__ void seg_list_add(const SegCtx &sc, uint32_t n2, uint32_t r, uint64_t w) {
  const size_t row = (size_t)sc.seg * n2 + r;
  const uint32_t qpad = n2 / 2u;
  uint16_t *const hi = sc.xlst + (size_t)sc.S * n2 * kSegRingCap;
  for (; w; w &= w - 1) {
    const uint32_t j = sc.col * 64u + (uint32_t)(__ffsll((long long)w) - 1);
    const uint16_t wj = (uint16_t)(j < qpad ? 2u * j : 2u * (j - qpad) + 1u);
    const uint32_t pos = atomicAdd(sc.xcnt + row, 1u);
    if (pos < kSegRingCap)
      sc.xlst[row * kSegRingCap + pos] = wj;
    else if (pos < kSegRowCap)
      hi[row * (kSegRowCap - kSegRingCap) + pos - kSegRingCap] = wj;
  }
}

// One transfer row of one compose step, held in registers: its entry count,
// its first eight entries (u16 pairs) and its AFF row.
struct SegRow {
  uint32_t n;
  uint32_t e[4];
  uint64_t c;
};

// REST: composes the entry rows of segment s_to from those of s_from, one
// segment at a time: rows <- A_s rows ^ c_s.  Row r of A_s is the sparse list
// of the rows at the segment's start that feed it (XFER built it; a row
// with more than kSegRowCap entries is read from the dense transfer columns
// instead: bit r' mod 64 of word r of column r' / 64).  The current rows sit
// in the published buffer, so a thread reads the rows its entries name from
// shared memory.  Each step's lists and AFF rows are copied into a ring of
// ring_nb shared-memory buffers by cp.async.bulk, issued ring_nb - 1 steps
// ahead by lane 0 of the last warp on one mbarrier per buffer (mbar[2 + b]);
// thread 0 issues the walk's first tape copies (issue_walk_copies).  A thread keeps the
// next step's row lists in registers (loaded while the current step runs: they
// do not depend on its result), so a step's chain is: publish the rows, one
// barrier, the entries' loads from the published rows, XOR.  Waits are
// bounded and a timeout aborts the item.  CTA-wide (barriers); one word per
// CTA.  Returns false after a wait gave up (in-flight ring copies have been
// waited for).
template <int QPT, typename F>
__device__ __forceinline__ bool seg_compose(uint64_t (&X)[QPT][1], uint64_t (&Z)[QPT][1], const SegCtx &sc,
                                            ulonglong2 *pub, const uint32_t qpad, uint64_t *mbar,
                                            unsigned char *ring, const uint32_t *s_aff, uint32_t *err,
                                            F &&issue_walk_copies) {
  const uint32_t T = blockDim.x, tid = threadIdx.x;
  const uint32_t n2 = 2 * qpad;
  const uint32_t steps = sc.s_to - sc.s_from, NB = sc.ring_nb;
  const size_t step_bytes = seg_step_bytes(qpad);
  const uint32_t cnt_b = n2 * 4u, lst_b = n2 * 2u * kSegRingCap, c_b = n2 * 8u;
  const uint16_t *const xhi = sc.xlst + (size_t)sc.S * n2 * kSegRingCap;  // entries 8..15
  // the ring's copies are issued by lane 0 of the last warp (whose slots are
  // the packing's padding when there is any), so the first warp is not held up
  const uint32_t issuer = T - 32u;
  uint32_t issued = 0, waited = 0;  // steps issued (issuer) / seen complete (this thread)
  auto issue = [&]() {  // issuer: the next step into its ring buffer
    const uint32_t k = issued++;
    const uint32_t s = sc.s_from + k;
    unsigned char *dst = ring + (size_t)(k % NB) * step_bytes;
    uint64_t *bar = &mbar[2 + k % NB];
    const uint32_t ai = s_aff[s];
    mbar_expect_tx(bar, cnt_b + lst_b + (ai == kNoState ? 0u : c_b));
    bulk_g2s(dst, sc.xcnt + (size_t)s * n2, cnt_b, bar);
    bulk_g2s(dst + cnt_b, sc.xlst + (size_t)s * n2 * kSegRingCap, lst_b, bar);
    if (ai != kNoState) bulk_g2s(dst + cnt_b + lst_b, sc.state + (size_t)ai * n2, c_b, bar);
  };
  if (tid == issuer) {
    while (issued < min(NB, steps)) issue();
  }
  if (tid == 0) issue_walk_copies();  // the walk's first tape chunks (thread 0 owns them), needed after the compose
  bool bad = false;
  auto wait_step = [&](uint32_t k) {
    if (!mbar_wait_bounded(&mbar[2 + k % NB], (k / NB) & 1u)) bad = true;
    else waited = k + 1;
  };
  const unsigned char *const ring_c = ring;
  auto load_row = [&](uint32_t k, uint32_t r, SegRow &m) {
    const unsigned char *buf = ring_c + (size_t)(k % NB) * step_bytes;
    m.n = reinterpret_cast<const uint32_t *>(buf)[r];
    const uint4 e = reinterpret_cast<const uint4 *>(buf + cnt_b)[r];  // entries 0..7
    m.e[0] = e.x;
    m.e[1] = e.y;
    m.e[2] = e.z;
    m.e[3] = e.w;
    m.c = s_aff[sc.s_from + k] != kNoState ? reinterpret_cast<const uint64_t *>(buf + cnt_b + lst_b)[r] : 0ull;
  };
  // the published rows as words: word 2 j of a buffer is X of slot j, word 2 j + 1 its Z
  const uint32_t pub_s0 = smem_u32(pub);
  auto word_addr = [&](uint32_t pbuf, uint32_t j) -> uint32_t {
    return pbuf + (j < qpad ? j * 16u : (j - qpad) * 16u + 8u);
  };
  // row r of step k: its AFF row XOR the published rows its entries name.
  // The loads of a row issue together, without branches: entries past the
  // row's count read a shared word that is always zero (four loads always,
  // four more for a row of five to eight entries: rows of one role share a
  // warp).  A step takes as long as its slowest row's chain, since a barrier
  // follows.
  __shared__ uint64_t s_zero;
  if (tid == 0) s_zero = 0;  // read after the first step's barrier
  const uint32_t zaddr = smem_u32(&s_zero);
  auto apply = [&](uint32_t k, uint32_t r, const SegRow &m, uint64_t self, uint32_t pbuf) -> uint64_t {
    uint64_t v = m.c;
    if (m.n <= kSegRowCap) {
#pragma unroll
      for (uint32_t i = 0; i < 4; ++i) {
        const uint32_t wj = (m.e[i >> 1] >> ((i & 1u) * 16u)) & 0xFFFFu;
        v ^= lds64(i < m.n ? pbuf + wj * 8u : zaddr);
      }
      if (m.n > 4) {
#pragma unroll
        for (uint32_t i = 4; i < kSegRingCap; ++i) {
          const uint32_t wj = (m.e[i >> 1] >> ((i & 1u) * 16u)) & 0xFFFFu;
          v ^= lds64(i < m.n ? pbuf + wj * 8u : zaddr);
        }
      }
      if (m.n > kSegRingCap) {  // entries 8..15 (rare): from global memory
        const uint4 t = __ldg(reinterpret_cast<const uint4 *>(
            xhi + ((size_t)(sc.s_from + k) * n2 + r) * (kSegRowCap - kSegRingCap)));
        const uint32_t e2[4] = {t.x, t.y, t.z, t.w};
#pragma unroll
        for (uint32_t i = 0; i < kSegRowCap - kSegRingCap; ++i) {
          const uint32_t wj = (e2[i >> 1] >> ((i & 1u) * 16u)) & 0xFFFFu;
          v ^= lds64(i + kSegRingCap < m.n ? pbuf + wj * 8u : zaddr);
        }
      }
    } else {  // a long row: its words from the dense transfer columns
      const uint64_t *tm = sc.state + (size_t)(sc.xfer0 + (sc.s_from + k) * sc.ncol) * n2;
      for (uint32_t c = 0; c < sc.ncol; ++c)
        for (uint64_t w = __ldg(tm + (size_t)c * n2 + r); w; w &= w - 1) {
          const uint32_t j = c * 64u + (uint32_t)(__ffsll((long long)w) - 1);
          v ^= j == r ? self : j < n2 ? lds64(word_addr(pbuf, j)) : 0ull;
        }
    }
    return v;
  };
  SegRow mx[QPT], mz[QPT];
  if (steps) {
    wait_step(0);
#pragma unroll
    for (int u = 0; u < QPT; ++u) {
      load_row(0, tid + (uint32_t)u * T, mx[u]);
      load_row(0, qpad + tid + (uint32_t)u * T, mz[u]);
    }
  }
  for (uint32_t k = 0; k < steps; ++k) {
    ulonglong2 *pb = pub + (size_t)(k & 1u) * qpad;
#pragma unroll
    for (int u = 0; u < QPT; ++u) pb[tid + u * T] = make_ulonglong2(X[u][0], Z[u][0]);
    if (__syncthreads_or(bad ? 1 : 0)) {
      bad = true;
      break;
    }
    // every thread is done with step k - 1's buffer
    if (tid == issuer && k >= 1 && issued < steps) issue();
    const uint32_t pbuf = pub_s0 + (k & 1u) * qpad * 16u;
#pragma unroll
    for (int u = 0; u < QPT; ++u) {
      const uint32_t slot = tid + (uint32_t)u * T;
      const uint64_t nx = apply(k, slot, mx[u], X[u][0], pbuf);
      const uint64_t nz = apply(k, qpad + slot, mz[u], Z[u][0], pbuf);
      X[u][0] = nx;
      Z[u][0] = nz;
    }
    if (k + 1 < steps) {
      wait_step(k + 1);
#pragma unroll
      for (int u = 0; u < QPT; ++u) {
        load_row(k + 1, tid + (uint32_t)u * T, mx[u]);
        load_row(k + 1, qpad + tid + (uint32_t)u * T, mz[u]);
      }
    }
  }
  if (bad && tid == issuer) {
    atomicOr(err, DEV_ERR_TIMEOUT);
    // copies still in flight target this CTA's shared memory
    for (uint32_t k = waited; k < issued; ++k)
      if (!mbar_wait_bounded(&mbar[2 + k % NB], (k / NB) & 1u)) break;
  }
  __syncthreads();  // the walk publishes into buffer 0 next, which may have been read last
  return !bad;
}

// One walk item: the words j0 .. j0+W-1 of circuit C (rows W x 64 bits per
// qubit; a batch halves its CTAs with W = 2 while each epoch's latency chain
// stays about the same), walked by the whole CTA.  `pub_slots` lays out the
// shared memory (the circuit's slot count, or the largest of a persistent
// launch).  QUEUE: the CTA may have more threads than the circuit has qubit
// slots (a persistent launch sized for its largest circuit); thread slots at
// or past C.qpad hold nothing, publish nothing and skip the ops (qpad is a
// multiple of 32, so whole warps idle).  Returns ITEM_EMPTY when the words
// inject nothing (the mbarriers were not initialised), ITEM_ABORTED after a
// bounded wait gave up, else ITEM_DONE.  CTA-uniform.
//
// Segment items (MODE != MODE_PLAIN, W = 1, `sc` given) walk [e_begin, e_end)
// only: FIRST from zero rows with snapshots (and the word's band), AFF from
// zero rows without snapshots, XFER from unit rows without measurement bits
// or snapshots (stopping once the rows vanish), REST from composed entry rows
// with snapshots (a REST that stops early lowers the band's end).
template <int QPT, int W, bool QUEUE, int MODE = MODE_PLAIN>
__device__ __forceinline__ uint32_t walk_item(const CircuitDev &C, const uint32_t j0, unsigned char *smem,
                                              const uint32_t pub_slots, const uint32_t chunk_cap,
                                              const uint32_t table_bytes, uint32_t *__restrict__ err,
                                              uint32_t &s_abort, const SegCtx *sc = nullptr) {
  constexpr bool SEG = MODE != MODE_PLAIN;
  constexpr bool SNAPS = MODE == MODE_PLAIN || MODE == MODE_FIRST || MODE == MODE_REST;
  static_assert(!SEG || (W == 1 && !QUEUE), "segment items walk one word per CTA");
  const uint32_t nw = SEG ? 1u : min((uint32_t)W, C.w - j0);  // words of this CTA (the circuit's last group may be short)
  const uint32_t T = blockDim.x;
  const uint32_t tid = threadIdx.x;
  const uint32_t qpad = C.qpad;
  const uint32_t nE = C.n_epochs;
  bool act[QPT];  // thread slot tid + u * T holds a qubit slot of the circuit
#pragma unroll
  for (int u = 0; u < QPT; ++u) act[u] = !QUEUE || tid + (uint32_t)u * T < qpad;

  // the CTA walks from the earliest first injection of its words to the
  // latest last injection (and on until every row is zero)
  uint32_t e0 = 0xFFFFFFFFu, elast = 0, e_end = nE;
  if constexpr (SEG) {
    e0 = sc->e_begin;
    e_end = sc->e_end;
    if constexpr (MODE != MODE_XFER) elast = C.inj_hi[j0];
  } else {
#pragma unroll
    for (int wi = 0; wi < W; ++wi) {
      if ((uint32_t)wi >= nw) break;
      const uint32_t lo = C.inj_lo[j0 + wi];
      if (lo == 0xFFFFFFFFu || lo >= nE) continue;
      e0 = min(e0, lo);
      elast = max(elast, C.inj_hi[j0 + wi]);
    }
    if (e0 == 0xFFFFFFFFu) {
      if (tid < nw) C.band[j0 + tid] = make_uint2(0u, 0u);
      return ITEM_EMPTY;
    }
  }

  // shared memory: [published rows x2][mbarriers][tables][chunk buffer x2]
  ulonglong2 *pub = reinterpret_cast<ulonglong2 *>(smem);
  size_t off = (size_t)2 * pub_slots * W * sizeof(ulonglong2);
  uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + off);
  off += 128;
  uint2 *etab = reinterpret_cast<uint2 *>(smem + off);  // epoch e0+i: (op offset, slots | chunk << 8)
  const uint32_t c0 = C.ep_chunk[e0];
  const uint32_t c_end = SEG ? C.ep_chunk[e_end - 1] + 1 : C.n_chunks;  // chunks past the last one walked
  const uint32_t ne = e_end - e0, nc = c_end - c0;
  const bool staged = ((size_t)ne + nc) * sizeof(uint2) <= table_bytes;
  uint2 *ctab = etab + ne;  // chunk c0+i: (op offset, bytes)
  off += table_bytes;
  unsigned char *buf = smem + off;  // two buffers of chunk_cap bytes
  // REST: [S aff states (u32, 16-byte rounded)][ring_nb compose step buffers]
  uint32_t *s_aff = nullptr;
  unsigned char *ring = nullptr;
  if constexpr (MODE == MODE_REST) {
    off += (size_t)2 * chunk_cap;
    s_aff = reinterpret_cast<uint32_t *>(smem + off);
    off += ((size_t)sc->S * 4 + 15) & ~(size_t)15;
    ring = smem + ((off + 127) & ~(size_t)127);
    for (uint32_t i = tid; i < sc->s_to; i += T) s_aff[i] = sc->aff_row[i];
  }

  if (staged) {
    for (uint32_t i = tid; i < ne; i += T)
      etab[i] = make_uint2(C.ep_opoff[e0 + i], C.ep_k[e0 + i] | (C.ep_chunk[e0 + i] << 8));
    for (uint32_t i = tid; i < nc; i += T) ctab[i] = make_uint2(C.ch_off[c0 + i], C.ch_bytes[c0 + i]);
  }
  if (tid == 0) {
    s_abort = 0;
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    if constexpr (MODE == MODE_REST)
      for (uint32_t b = 0; b < sc->ring_nb; ++b) mbar_init(&mbar[2 + b], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  auto epoch = [&](uint32_t e) -> uint2 {
    return staged ? etab[e - e0]
                  : make_uint2(__ldg(C.ep_opoff + e), __ldg(C.ep_k + e) | (__ldg(C.ep_chunk + e) << 8));
  };
  auto chunk = [&](uint32_t c) -> uint2 {
    return staged ? ctab[c - c0] : make_uint2(__ldg(C.ch_off + c), __ldg(C.ch_bytes + c));
  };
  // Producer (thread 0): chunk c goes to buffer (c - c0) & 1.
  uint32_t issued = 0;  // chunks c0 .. c0+issued-1 have been issued
  auto issue = [&]() {
    const uint32_t c = c0 + issued;
    const uint2 ck = chunk(c);
    uint64_t *bar = &mbar[issued & 1u];
    mbar_expect_tx(bar, ck.y);
    bulk_g2s(buf + (size_t)(issued & 1u) * chunk_cap, C.ops + ck.x, ck.y, bar);
    ++issued;
  };
  auto issue_first_chunks = [&]() {
    issue();
    if (nc > 1) issue();
  };
  // (REST: after the compose ring's first copies, which are needed first)
  if (MODE != MODE_REST && tid == 0) issue_first_chunks();

  uint64_t X[QPT][W], Z[QPT][W], acc[QPT][W], last_inj[QPT][W];
  bool compose_bad = false;
#pragma unroll
  for (int u = 0; u < QPT; ++u)
#pragma unroll
    for (int wi = 0; wi < W; ++wi) X[u][wi] = Z[u][wi] = acc[u][wi] = last_inj[u][wi] = 0;
  if constexpr (MODE == MODE_XFER) {
    // unit rows of column col: row r (X of slot r, or Z of slot r - qpad) holds bit r - 64 col
#pragma unroll
    for (int u = 0; u < QPT; ++u) {
      const uint32_t xr = tid + (uint32_t)u * T, zr = qpad + xr;
      if constexpr (W == 1) {
        X[u][0] = (xr >> 6) == sc->col ? 1ull << (xr & 63u) : 0ull;
        Z[u][0] = (zr >> 6) == sc->col ? 1ull << (zr & 63u) : 0ull;
      }
    }
  } else if constexpr (MODE == MODE_REST) {
    if constexpr (W == 1) {
#pragma unroll
      for (int u = 0; u < QPT; ++u) {
        const uint32_t slot = tid + (uint32_t)u * T;
        X[u][0] = __ldg(sc->in + slot);
        Z[u][0] = __ldg(sc->in + qpad + slot);
      }
      compose_bad = !seg_compose<QPT>(X, Z, *sc, reinterpret_cast<ulonglong2 *>(smem), qpad, mbar, ring, s_aff,
                                      err, issue_first_chunks);
    }
  }

  const uint32_t np = C.npoints;
  ulonglong2 *snap0 = C.snap + (size_t)j0 * np;  // word j0 + wi at + wi * np
  const uint32_t jlo = j0 * 64u;
  // non-zero masks: W divides 64 and groups start at multiples of W, so the
  // CTA's words share one 64-bit mask word
  unsigned long long *nzm0 = C.nzm + (j0 >> 6);
  const uint32_t mw = C.mw;
  const uint32_t jsh = j0 & 63u;
  bool timed_out = compose_bad, aborted = false;  // (the walk's first barrier aborts after a failed compose)
  uint32_t e = e0;
  uint32_t seq = 0;
  uint32_t cur = 0xFFFFFFFFu;  // chunk whose data this thread has waited for
  uint32_t waited = 0;         // chunks (from c0) whose copy this thread saw complete
  const unsigned char *cbase = nullptr;
  uint32_t cbase_off = 0;
  uint2 ek_next = epoch(e0);
  // stores the W words' snapshots of one point and sets their mask bits
  auto snapshot = [&](uint32_t arg, const uint64_t *xs, const uint64_t *zs) {
    if constexpr (W == 1) {
      snap0[arg] = make_ulonglong2(xs[0], zs[0]);
      if (xs[0] | zs[0]) red_or(nzm0 + arg * mw, 1ull << jsh);
    } else {
      unsigned long long bits = 0;
#pragma unroll
      for (int wi = 0; wi < W; ++wi) {
        if ((uint32_t)wi < nw) {
          snap0[(size_t)wi * np + arg] = make_ulonglong2(xs[wi], zs[wi]);
          if (xs[wi] | zs[wi]) bits |= 1ull << (jsh + wi);
        }
      }
      if (bits) red_or(nzm0 + arg * mw, bits);
    }
  };
  for (;; ++e, ++seq) {
    // (1) publish rows (the state after epoch e-1): slot s holds its W words at [s * W, s * W + W)
    ulonglong2 *pb = pub + (size_t)(seq & 1u) * qpad * W;
    bool nz = false;
#pragma unroll
    for (int u = 0; u < QPT; ++u)
#pragma unroll
      for (int wi = 0; wi < W; ++wi) {
        if (!act[u]) continue;
        asm volatile("st.shared.v2.u64 [%0], {%1, %2};" ::"r"(smem_u32(pb + (tid + u * T) * W + wi)),
                     "l"(X[u][wi]), "l"(Z[u][wi])
                     : "memory");
        nz |= (X[u][wi] | Z[u][wi]) != 0;
      }
    if (timed_out) s_abort = 1;
    // (2) the epoch barrier
    const int any = __syncthreads_or(nz ? 1 : 0);
    if (s_abort) {
      if (tid == 0) atomicOr(err, DEV_ERR_TIMEOUT);
      aborted = true;
      break;
    }
    // (XFER has no measurement bits: its rows stay zero once they vanish)
    if ((!any && (MODE == MODE_XFER || e > elast)) || e >= e_end) break;
    const uint2 ek = ek_next;
    if (e + 1 < e_end) ek_next = epoch(e + 1);  // used next epoch: its latency hides behind this one
    const uint32_t K = ek.y & 0xFFu;
    const uint32_t ch = ek.y >> 8;
    if (ch != cur) {
      // (3) first epoch of a chunk: every thread has finished the previous
      //     chunk (barrier above), so its buffer can take the chunk after this one
      if (tid == 0 && ch + 1 < c_end && c0 + issued == ch + 1) issue();
      const uint32_t i = ch - c0;
      if (!mbar_wait_bounded(&mbar[i & 1u], (i >> 1) & 1u)) {
        timed_out = true;
        continue;
      }
      waited = i + 1;
      cur = ch;
      cbase = buf + (size_t)(i & 1u) * chunk_cap;
      cbase_off = chunk(ch).x;
    }
    // (4) execute the epoch's ops in order (shared-memory addresses are kept
    //     as 32-bit shared-window offsets so every load is an ld.shared)
    const uint32_t ops_s = smem_u32(cbase) + (ek.x - cbase_off) * 8u + tid * 8u;
    const uint32_t pub_s = smem_u32(pb);
    for (uint32_t k = 0; k < K; ++k) {
#pragma unroll
      for (int u = 0; u < QPT; ++u) {
        if (!act[u]) continue;
        const uint64_t op = lds64(ops_s + (k * qpad + (uint32_t)u * T) * 8u);
        const uint32_t opc = (uint32_t)op & 0xFFu;
        if (opc == OP_NOP) continue;
        const uint32_t arg = (uint32_t)(op >> 32);
        const uint32_t pa = pub_s + arg * W * 16u;  // the partner slot's published words
        if (opc == OP_XPX) {
#pragma unroll
          for (int wi = 0; wi < W; ++wi) X[u][wi] ^= lds64(pa + wi * 16u);
        } else if (opc == OP_ZPZ) {
#pragma unroll
          for (int wi = 0; wi < W; ++wi) Z[u][wi] ^= lds64(pa + wi * 16u + 8u);
        } else if (opc == OP_SNAP) {
          if constexpr (SNAPS) snapshot(arg, X[u], Z[u]);
        } else if (opc == OP_XPZ) {
#pragma unroll
          for (int wi = 0; wi < W; ++wi) X[u][wi] ^= lds64(pa + wi * 16u + 8u);
        } else {
          const uint32_t sub = ((uint32_t)op >> 8) & 0xFFu;
          if (opc == OP_C2) {
#pragma unroll
            for (int wi = 0; wi < W; ++wi) {
              const ulonglong2 p = lds128(pa + wi * 16u);
              const uint64_t x = X[u][wi], z = Z[u][wi];
              X[u][wi] = sel4(sub & 15u, x, z, p.x, p.y);
              Z[u][wi] = sel4(sub >> 4, x, z, p.x, p.y);
            }
          } else if (opc == OP_C1) {
#pragma unroll
            for (int wi = 0; wi < W; ++wi) {
              const uint64_t x = X[u][wi], z = Z[u][wi];
              X[u][wi] = sel2(sub & 3u, x, z);
              Z[u][wi] = sel2(sub >> 2, x, z);
            }
          } else if (opc == OP_R) {
#pragma unroll
            for (int wi = 0; wi < W; ++wi) X[u][wi] = Z[u][wi] = 0;
          } else if (opc == OP_INJ) {
            if constexpr (MODE == MODE_XFER) continue;  // the linear part only
            // measurement bits (one or two) that fall in this CTA's words
            const uint32_t b2 = ((uint32_t)op >> 8) & 0xFFFFFFu;
            const uint32_t d1 = arg - jlo, d2 = b2 - jlo;
#pragma unroll
            for (int wi = 0; wi < W; ++wi) {
              if (d1 - wi * 64u < 64u) acc[u][wi] |= 1ull << (d1 & 63u);
              if (b2 != 0xFFFFFFu && d2 - wi * 64u < 64u) acc[u][wi] |= 1ull << (d2 & 63u);
            }
          } else if (opc == OP_M) {
            const uint32_t d1 = arg - jlo;
            const uint32_t basis = sub & 3u;
#pragma unroll
            for (int wi = 0; wi < W; ++wi) {
              uint64_t inj = acc[u][wi];
              if (d1 - wi * 64u < 64u) inj |= 1ull << (d1 & 63u);
              if constexpr (MODE == MODE_XFER) inj = 0;
              acc[u][wi] = 0;
              if (sub & 4u) X[u][wi] = Z[u][wi] = 0;
              if (basis != 1u) X[u][wi] ^= inj;
              if (basis != 0u) Z[u][wi] ^= inj;
              last_inj[u][wi] = inj;
            }
          } else if (opc == OP_SNAPD) {
            if constexpr (!SNAPS) continue;
            if constexpr (W == 1) {
              snap0[arg] = make_ulonglong2(last_inj[u][0], 0ull);
              if (last_inj[u][0]) red_or(nzm0 + arg * mw, 1ull << jsh);
            } else {
              uint64_t zero[W];
#pragma unroll
              for (int wi = 0; wi < W; ++wi) zero[wi] = 0;
              snapshot(arg, last_inj[u], zero);
            }
          }
        }
      }
    }
  }
  if constexpr (MODE == MODE_PLAIN) {
    if (tid < nw) C.band[j0 + tid] = make_uint2(C.ep_ptoff[e0], C.ep_ptoff[e < nE ? e : nE]);
  } else if constexpr (MODE == MODE_FIRST) {
    // later segments (if any) cover up to the end unless they stop early
    if (tid == 0) C.band[j0] = make_uint2(C.ep_ptoff[e0], C.ep_ptoff[e < e_end ? e : nE]);
  } else if constexpr (MODE == MODE_REST) {
    if (tid == 0 && e < e_end) atomicMin(&C.band[j0].y, C.ep_ptoff[e]);
  }
  if constexpr (MODE == MODE_XFER) {
#pragma unroll
    for (int u = 0; u < QPT; ++u) {
      const uint32_t slot = tid + (uint32_t)u * T;
      seg_list_add(*sc, 2 * qpad, slot, X[u][0]);
      seg_list_add(*sc, 2 * qpad, qpad + slot, Z[u][0]);
    }
  }
  if constexpr (MODE == MODE_FIRST || MODE == MODE_AFF || MODE == MODE_XFER) {
    if (sc->out) {
#pragma unroll
      for (int u = 0; u < QPT; ++u) {
        const uint32_t slot = tid + (uint32_t)u * T;
        sc->out[slot] = X[u][0];
        sc->out[qpad + slot] = Z[u][0];
      }
    }
  }
  if (tid == 0) {
    // Copies still in flight target this CTA's shared memory: wait for them
    // (bounded) before the CTA exits or takes another item.
    for (uint32_t i = waited; i < issued; ++i) {
      if (!mbar_wait_bounded(&mbar[i & 1u], (i >> 1) & 1u)) {
        atomicOr(err, DEV_ERR_TIMEOUT);
        s_abort = 1;
        break;
      }
    }
  }
  return aborted ? ITEM_ABORTED : ITEM_DONE;
}

// One CTA per item (circuit, first word), all circuits of the launch with
// the same slot count.
template <int QPT, int W>
__global__ void __launch_bounds__(WalkBound<QPT>::value) walk_kernel(const CircuitDev *__restrict__ circs,
                                                    const uint2 *__restrict__ items, uint32_t chunk_cap, uint32_t table_bytes,
                                                    uint32_t *__restrict__ err) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint32_t s_abort;
  const uint2 item = items[blockIdx.x];
  const CircuitDev C = circs[item.x];
  walk_item<QPT, W, false>(C, item.y, smem, C.qpad, chunk_cap, table_bytes, err, s_abort);
}

// Persistent walk: one launch over the items of circuits of every size, at
// most as many CTAs as fit on the GPU at once.  Each CTA takes the next item
// from the queue counter (items are ordered longest first, so the longest
// walks start first and the short ones fill in behind them) until the queue
// is empty.  A CTA stops taking items after a wait gave up.
template <int QPT, int W>
__global__ void __launch_bounds__(WalkBound<QPT>::value) walk_queue_kernel(const CircuitDev *__restrict__ circs,
                                                          const uint2 *__restrict__ items, uint32_t n_items,
                                                          uint32_t *__restrict__ next, uint32_t pub_slots,
                                                          uint32_t chunk_cap, uint32_t table_bytes,
                                                          uint32_t *__restrict__ err) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint32_t s_item, s_abort;
  uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + (size_t)2 * pub_slots * W * sizeof(ulonglong2));
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(next, 1u);
    __syncthreads();
    const uint32_t it = s_item;
    if (it >= n_items) return;
    const uint2 item = items[it];
    const CircuitDev C = circs[item.x];
    const uint32_t st = walk_item<QPT, W, true>(C, item.y, smem, pub_slots, chunk_cap, table_bytes, err, s_abort);
    // every thread is done with the item's shared memory and mbarriers (and
    // thread 0 has seen every copy of the item complete)
    __syncthreads();
    if (st == ITEM_ABORTED || s_abort) return;
    if (st == ITEM_DONE && threadIdx.x == 0) {
      mbar_inval(&mbar[0]);
      mbar_inval(&mbar[1]);
    }
  }
}

// Segmented walk of one circuit: one CTA per segment item (SEG_*).
template <int QPT>
__global__ void __launch_bounds__(WalkBound<QPT>::value) walk_seg_kernel(const SegLaunch L, uint32_t table_bytes) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint32_t s_abort;
  const SegItem it = L.items[blockIdx.x];
  if (it.kind == SEG_REST && L.ring_nb < 2) {  // no compose ring in this launch
    if (threadIdx.x == 0) atomicOr(L.err, DEV_ERR_TIMEOUT);
    return;
  }
  const CircuitDev C = *L.circ;
  const size_t n2 = (size_t)2 * C.qpad;
  SegCtx sc;
  sc.e_begin = it.e_begin;
  sc.e_end = it.e_end;
  sc.out = it.kind != SEG_REST && it.state != kNoState ? L.state + (size_t)it.state * n2 : nullptr;
  sc.in = it.kind == SEG_REST ? L.state + (size_t)it.state * n2 : nullptr;
  sc.state = L.state;
  sc.aff_row = L.aff + (size_t)(it.kind == SEG_XFER ? 0u : it.idx) * L.S;
  sc.xfer0 = L.xfer0;
  sc.ncol = L.ncol;
  sc.s_from = it.s_from;
  sc.s_to = it.s_to;
  sc.col = it.idx;
  sc.seg = it.s_from;
  sc.xcnt = L.xcnt;
  sc.xlst = L.xlst;
  sc.ring_nb = L.ring_nb;
  sc.S = L.S;
  switch (it.kind) {
    case SEG_FIRST:
      walk_item<QPT, 1, false, MODE_FIRST>(C, it.idx, smem, C.qpad, L.chunk_cap, table_bytes, L.err, s_abort, &sc);
      break;
    case SEG_AFF:
      walk_item<QPT, 1, false, MODE_AFF>(C, it.idx, smem, C.qpad, L.chunk_cap, table_bytes, L.err, s_abort, &sc);
      break;
    case SEG_XFER:
      walk_item<QPT, 1, false, MODE_XFER>(C, 0, smem, C.qpad, L.chunk_cap, table_bytes, L.err, s_abort, &sc);
      break;
    default:
      walk_item<QPT, 1, false, MODE_REST>(C, it.idx, smem, C.qpad, L.chunk_cap, table_bytes, L.err, s_abort, &sc);
      break;
  }
}

}  // namespace

uint32_t walk_table_bytes(uint32_t max_epochs, uint32_t max_chunks) {
  const uint64_t b = ((uint64_t)max_epochs + max_chunks) * sizeof(uint2);
  return b <= kWalkTableBudget ? (uint32_t)((b + 127) & ~(uint64_t)127) : 0u;
}

size_t walk_smem_bytes(uint32_t qpad, uint32_t chunk_cap, uint32_t table_bytes, uint32_t words) {
  return (size_t)2 * qpad * words * sizeof(ulonglong2) + 128 + table_bytes + (size_t)2 * chunk_cap;
}

// Raises the dynamic shared-memory limit of the walk kernels once (not a
// stream operation, so it is done here rather than inside a graph capture).
template <int QPT, int W>
cudaError_t walk_set_limit_one(int optin) {
  cudaFuncAttributes a{};
  cudaError_t e = cudaFuncGetAttributes(&a, walk_kernel<QPT, W>);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(walk_kernel<QPT, W>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              optin - (int)a.sharedSizeBytes);
}

template <int QPT, int W>
cudaError_t walk_queue_set_limit_one(int optin) {
  cudaFuncAttributes a{};
  cudaError_t e = cudaFuncGetAttributes(&a, walk_queue_kernel<QPT, W>);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(walk_queue_kernel<QPT, W>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              optin - (int)a.sharedSizeBytes);
}

template <int QPT>
cudaError_t walk_seg_set_limit_one(int optin) {
  cudaFuncAttributes a{};
  cudaError_t e = cudaFuncGetAttributes(&a, walk_seg_kernel<QPT>);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(walk_seg_kernel<QPT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              optin - (int)a.sharedSizeBytes);
}

cudaError_t walk_set_smem_limit() {
  int dev = 0, optin = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e == cudaSuccess) e = walk_set_limit_one<1, 1>(optin);
  if (e == cudaSuccess) e = walk_set_limit_one<2, 1>(optin);
  if (e == cudaSuccess) e = walk_set_limit_one<3, 1>(optin);
  if (e == cudaSuccess) e = walk_set_limit_one<4, 1>(optin);
  if (e == cudaSuccess) e = walk_set_limit_one<6, 1>(optin);
  if (e == cudaSuccess) e = walk_set_limit_one<8, 1>(optin);
  if (e == cudaSuccess) e = walk_set_limit_one<12, 1>(optin);
  if (e == cudaSuccess) e = walk_set_limit_one<16, 1>(optin);
  if (e == cudaSuccess) e = walk_set_limit_one<1, 2>(optin);
  if (e == cudaSuccess) e = walk_set_limit_one<2, 2>(optin);
  if (e == cudaSuccess) e = walk_queue_set_limit_one<1, 1>(optin);
  if (e == cudaSuccess) e = walk_queue_set_limit_one<2, 1>(optin);
  if (e == cudaSuccess) e = walk_queue_set_limit_one<1, 2>(optin);
  if (e == cudaSuccess) e = walk_queue_set_limit_one<2, 2>(optin);
  if (e == cudaSuccess) e = walk_seg_set_limit_one<1>(optin);
  if (e == cudaSuccess) e = walk_seg_set_limit_one<2>(optin);
  return e;
}

uint32_t walk_max_threads(uint32_t qpt) {
  switch (qpt) {
    case 1: return WalkBound<1>::value;
    case 2: return WalkBound<2>::value;
    case 3: return WalkBound<3>::value;
    case 4: return WalkBound<4>::value;
    case 6: return WalkBound<6>::value;
    case 8: return WalkBound<8>::value;
    case 12: return WalkBound<12>::value;
    case 16: return WalkBound<16>::value;
    default: return 0;
  }
}

bool walk_queue_supported(uint32_t qpt, uint32_t words) {
  return (qpt == 1 || qpt == 2) && (words == 1 || words == 2);
}

namespace {
// As many CTAs as can be resident at once (occupancy of this block size and
// shared memory), at most one per item.
template <int QPT, int W>
cudaError_t launch_walk_queue_one(const WalkLaunch &L, uint32_t tb, size_t smem, cudaStream_t s) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, walk_queue_kernel<QPT, W>, (int)L.threads, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  const uint32_t grid = (uint32_t)std::min<uint64_t>((uint64_t)sms * (uint64_t)per_sm, L.n_items);
  walk_queue_kernel<QPT, W><<<grid, L.threads, smem, s>>>(L.circs, L.items, L.n_items, L.queue, L.qpad, L.chunk_cap,
                                                         tb, L.err);
  return cudaGetLastError();
}
}  // namespace

cudaError_t launch_walk(const WalkLaunch &L, cudaStream_t s) {
  if (L.n_items == 0) return cudaSuccess;
  const uint32_t tb = walk_table_bytes(L.max_epochs, L.max_chunks);
  const size_t smem = walk_smem_bytes(L.qpad, L.chunk_cap, tb, L.words);
  if (smem > 227 * 1024 - 1024) return cudaErrorInvalidValue;
  if (L.words != 1 && !(L.words == 2 && (L.qpt == 1 || L.qpt == 2))) return cudaErrorInvalidValue;
  if (L.threads * L.qpt != L.qpad || L.threads > walk_max_threads(L.qpt)) return cudaErrorInvalidValue;
  if (L.queue) {
    // every circuit of the launch has at most L.qpad slots (checked by the caller)
    if (!walk_queue_supported(L.qpt, L.words)) return cudaErrorInvalidValue;
    if (L.words == 2) return L.qpt == 1 ? launch_walk_queue_one<1, 2>(L, tb, smem, s) : launch_walk_queue_one<2, 2>(L, tb, smem, s);
    return L.qpt == 1 ? launch_walk_queue_one<1, 1>(L, tb, smem, s) : launch_walk_queue_one<2, 1>(L, tb, smem, s);
  }
#define GPC_WALK(Q) walk_kernel<Q, 1><<<L.n_items, L.threads, smem, s>>>(L.circs, L.items, L.chunk_cap, tb, L.err)
#define GPC_WALK2(Q) walk_kernel<Q, 2><<<L.n_items, L.threads, smem, s>>>(L.circs, L.items, L.chunk_cap, tb, L.err)
  if (L.words == 2) {
    if (L.qpt == 1) GPC_WALK2(1);
    else GPC_WALK2(2);
    return cudaGetLastError();
  }
  switch (L.qpt) {
    case 1:
      GPC_WALK(1);
      break;
    case 2:
      GPC_WALK(2);
      break;
    case 3:
      GPC_WALK(3);
      break;
    case 4:
      GPC_WALK(4);
      break;
    case 6:
      GPC_WALK(6);
      break;
    case 8:
      GPC_WALK(8);
      break;
    case 12:
      GPC_WALK(12);
      break;
    case 16:
      GPC_WALK(16);
      break;
    default:
      return cudaErrorInvalidValue;
  }
#undef GPC_WALK
#undef GPC_WALK2
  return cudaGetLastError();
}

bool walk_seg_supported(uint32_t qpt) { return qpt == 1 || qpt == 2; }

size_t walk_seg_smem_bytes(const SegLaunch &L) {
  const uint32_t tb = walk_table_bytes(L.max_epochs, L.max_chunks);
  size_t b = walk_smem_bytes(L.qpad, L.chunk_cap, tb, 1);
  if (L.ring_nb) b = ((b + ((size_t)L.S * 4 + 15) / 16 * 16 + 127) & ~(size_t)127) + L.ring_nb * seg_step_bytes(L.qpad);
  return b <= 227 * 1024 - 1024 ? b : 0;
}

cudaError_t launch_walk_seg(const SegLaunch &L, cudaStream_t s) {
  if (L.n_items == 0) return cudaSuccess;
  const uint32_t tb = walk_table_bytes(L.max_epochs, L.max_chunks);
  const size_t smem = walk_seg_smem_bytes(L);
  // a compose ring needs two buffers at least: step k + 1's copy is issued
  // only once every thread is done with step k - 1's buffer
  if (smem == 0 || L.ring_nb > kSegRingMax || L.ring_nb == 1) return cudaErrorInvalidValue;
  if (!walk_seg_supported(L.qpt) || L.threads * L.qpt != L.qpad || L.threads > walk_max_threads(L.qpt))
    return cudaErrorInvalidValue;
  if (L.qpt == 1) walk_seg_kernel<1><<<L.n_items, L.threads, smem, s>>>(L, tb);
  else walk_seg_kernel<2><<<L.n_items, L.threads, smem, s>>>(L, tb);
  return cudaGetLastError();
}

}  // namespace gpc
