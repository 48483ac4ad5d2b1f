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
template <int QPT, int W, bool QUEUE>
__device__ __forceinline__ uint32_t walk_item(const CircuitDev &C, const uint32_t j0, unsigned char *smem,
                                              const uint32_t pub_slots, const uint32_t chunk_cap,
                                              const uint32_t table_bytes, uint32_t *__restrict__ err,
                                              uint32_t &s_abort) {
  const uint32_t nw = min((uint32_t)W, C.w - j0);  // words of this CTA (the circuit's last group may be short)
  const uint32_t T = blockDim.x;
  const uint32_t tid = threadIdx.x;
  const uint32_t qpad = C.qpad;
  const uint32_t nE = C.n_epochs;
  bool act[QPT];  // thread slot tid + u * T holds a qubit slot of the circuit
#pragma unroll
  for (int u = 0; u < QPT; ++u) act[u] = !QUEUE || tid + (uint32_t)u * T < qpad;

  // the CTA walks from the earliest first injection of its words to the
  // latest last injection (and on until every row is zero)
  uint32_t e0 = 0xFFFFFFFFu, elast = 0;
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

  // shared memory: [published rows x2][mbarriers][tables][chunk buffer x2]
  ulonglong2 *pub = reinterpret_cast<ulonglong2 *>(smem);
  size_t off = (size_t)2 * pub_slots * W * sizeof(ulonglong2);
  uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + off);
  off += 128;
  uint2 *etab = reinterpret_cast<uint2 *>(smem + off);  // epoch e0+i: (op offset, slots | chunk << 8)
  const uint32_t c0 = C.ep_chunk[e0];
  const uint32_t ne = nE - e0, nc = C.n_chunks - c0;
  const bool staged = ((size_t)ne + nc) * sizeof(uint2) <= table_bytes;
  uint2 *ctab = etab + ne;  // chunk c0+i: (op offset, bytes)
  off += table_bytes;
  unsigned char *buf = smem + off;  // two buffers of chunk_cap bytes

  if (staged) {
    for (uint32_t i = tid; i < ne; i += T)
      etab[i] = make_uint2(C.ep_opoff[e0 + i], C.ep_k[e0 + i] | (C.ep_chunk[e0 + i] << 8));
    for (uint32_t i = tid; i < nc; i += T) ctab[i] = make_uint2(C.ch_off[c0 + i], C.ch_bytes[c0 + i]);
  }
  if (tid == 0) {
    s_abort = 0;
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
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
  if (tid == 0) {
    issue();
    if (nc > 1) issue();
  }

  uint64_t X[QPT][W], Z[QPT][W], acc[QPT][W], last_inj[QPT][W];
#pragma unroll
  for (int u = 0; u < QPT; ++u)
#pragma unroll
    for (int wi = 0; wi < W; ++wi) X[u][wi] = Z[u][wi] = acc[u][wi] = last_inj[u][wi] = 0;

  const uint32_t np = C.npoints;
  ulonglong2 *snap0 = C.snap + (size_t)j0 * np;  // word j0 + wi at + wi * np
  const uint32_t jlo = j0 * 64u;
  // non-zero masks: W divides 64 and groups start at multiples of W, so the
  // CTA's words share one 64-bit mask word
  unsigned long long *nzm0 = C.nzm + (j0 >> 6);
  const uint32_t mw = C.mw;
  const uint32_t jsh = j0 & 63u;
  bool timed_out = false, aborted = false;
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
    if ((!any && e > elast) || e >= nE) break;
    const uint2 ek = ek_next;
    if (e + 1 < nE) ek_next = epoch(e + 1);  // used next epoch: its latency hides behind this one
    const uint32_t K = ek.y & 0xFFu;
    const uint32_t ch = ek.y >> 8;
    if (ch != cur) {
      // (3) first epoch of a chunk: every thread has finished the previous
      //     chunk (barrier above), so its buffer can take the chunk after this one
      if (tid == 0 && ch + 1 < C.n_chunks && c0 + issued == ch + 1) issue();
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
          snapshot(arg, X[u], Z[u]);
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
              acc[u][wi] = 0;
              if (sub & 4u) X[u][wi] = Z[u][wi] = 0;
              if (basis != 1u) X[u][wi] ^= inj;
              if (basis != 0u) Z[u][wi] ^= inj;
              last_inj[u][wi] = inj;
            }
          } else if (opc == OP_SNAPD) {
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
  if (tid < nw) C.band[j0 + tid] = make_uint2(C.ep_ptoff[e0], C.ep_ptoff[e < nE ? e : nE]);
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

}  // namespace gpc
