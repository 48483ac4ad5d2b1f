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
//   3. the epoch's ops are read from a shared-memory ring that one thread
//      fills ahead of time with cp.async.bulk (TMA) copies completing on an
//      mbarrier; waits are bounded by %globaltimer and report DEV_ERR_TIMEOUT;
//   4. ops: one-qubit Cliffords, two-qubit Cliffords (partner rows from the
//      published buffer), resets, measurements (XOR in the measurement's bits
//      that fall in word j; the bits ride in the tape itself), snapshots of
//      (X, Z) at noise points.
// The epoch table (slot count and tape offset per epoch) is staged in shared
// memory at start, so no global load sits on the per-epoch critical path.
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

// 1D bulk copy global -> shared, completing `bytes` of transaction count on `bar`.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ uint64_t sel2(uint32_t m, uint64_t x, uint64_t z) {
  return (x & (0ull - (uint64_t)(m & 1u))) ^ (z & (0ull - (uint64_t)((m >> 1) & 1u)));
}

__device__ __forceinline__ uint64_t sel4(uint32_t m, uint64_t a, uint64_t b, uint64_t c, uint64_t d) {
  return sel2(m & 3u, a, b) ^ sel2((m >> 2) & 3u, c, d);
}

constexpr uint32_t kEpochTabMax = 6144;  // epochs whose table is staged in shared memory

template <int QPT>
__global__ void __launch_bounds__(1024) walk_kernel(const CircuitDev *__restrict__ circs,
                                                    const uint2 *__restrict__ items, uint32_t ring_slots,
                                                    uint32_t slot_bytes, uint32_t tab_epochs,
                                                    uint32_t *__restrict__ err) {
  extern __shared__ __align__(128) unsigned char smem[];
  const uint2 item = items[blockIdx.x];
  const CircuitDev C = circs[item.x];
  const uint32_t j = item.y;
  const uint32_t T = blockDim.x;
  const uint32_t tid = threadIdx.x;
  const uint32_t qpad = C.qpad;
  const uint32_t nE = C.n_epochs;

  const uint32_t e0 = C.inj_lo[j];
  if (e0 == 0xFFFFFFFFu || e0 >= nE) {
    if (tid == 0) C.band[j] = make_uint2(0u, 0u);
    return;
  }
  const uint32_t elast = C.inj_hi[j];

  ulonglong2 *pub = reinterpret_cast<ulonglong2 *>(smem);  // [2][qpad]
  size_t off = (size_t)2 * qpad * sizeof(ulonglong2);
  uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + off);  // ring_slots <= 16
  off += 128;
  uint2 *etab = reinterpret_cast<uint2 *>(smem + off);  // (opoff, k) of epochs e0.. (if staged)
  off += ((size_t)tab_epochs * sizeof(uint2) + 127) / 128 * 128;
  unsigned char *ring = smem + off;
  __shared__ uint32_t s_abort;

  const bool staged = nE - e0 <= tab_epochs;
  if (staged) {
    for (uint32_t i = tid; i < nE - e0; i += T) etab[i] = make_uint2(C.ep_opoff[e0 + i], C.ep_k[e0 + i]);
  }
  if (tid == 0) {
    s_abort = 0;
    for (uint32_t s = 0; s < ring_slots; ++s) mbar_init(&mbar[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  auto epoch = [&](uint32_t e) -> uint2 {
    return staged ? etab[e - e0] : make_uint2(__ldg(C.ep_opoff + e), __ldg(C.ep_k + e));
  };

  // Producer state (thread 0 only): next epoch to load, sequences issued.
  uint32_t next_load = e0;
  uint32_t issued = 0;
  auto issue = [&](uint32_t seq) {
    const uint32_t slot = seq % ring_slots;
    const uint2 ek = epoch(next_load);
    const uint32_t bytes = ek.y * qpad * (uint32_t)sizeof(uint64_t);
    mbar_expect_tx(&mbar[slot], bytes);
    bulk_g2s(ring + (size_t)slot * slot_bytes, C.ops + ek.x, bytes, &mbar[slot]);
    ++next_load;
    ++issued;
  };
  if (tid == 0) {
    for (uint32_t s = 0; s < ring_slots && next_load < nE; ++s) issue(s);
  }

  uint64_t X[QPT], Z[QPT], acc[QPT], last_inj[QPT];
#pragma unroll
  for (int u = 0; u < QPT; ++u) X[u] = Z[u] = acc[u] = last_inj[u] = 0;

  ulonglong2 *snap_j = C.snap + (size_t)j * C.npoints;
  const uint32_t jlo = j * 64u;
  bool timed_out = false;
  uint32_t e = e0;
  uint32_t seq = 0;
  uint32_t consumed = 0;  // sequences whose copy this thread has seen complete
  for (;; ++e, ++seq) {
    // (1) publish rows (the state after epoch e-1)
    ulonglong2 *pb = pub + (size_t)(seq & 1u) * qpad;
    bool nz = false;
#pragma unroll
    for (int u = 0; u < QPT; ++u) {
      pb[tid + u * T] = make_ulonglong2(X[u], Z[u]);
      nz |= (X[u] | Z[u]) != 0;
    }
    if (timed_out) s_abort = 1;
    // (2) the epoch barrier
    const int any = __syncthreads_or(nz ? 1 : 0);
    if (s_abort) {
      if (tid == 0) atomicOr(err, DEV_ERR_TIMEOUT);
      break;
    }
    if ((!any && e > elast) || e >= nE) break;
    // (3) refill the slot freed by epoch e-1 (every thread finished reading it
    //     before the barrier above), then wait for epoch e
    if (tid == 0 && seq > 0 && next_load < nE) issue(issued);
    const uint32_t slot = seq % ring_slots;
    const uint32_t K = epoch(e).y;
    if (!mbar_wait_bounded(&mbar[slot], (seq / ring_slots) & 1u)) {
      timed_out = true;
      continue;
    }
    ++consumed;
    const uint64_t *ops = reinterpret_cast<const uint64_t *>(ring + (size_t)slot * slot_bytes);
    // (4) execute
    for (uint32_t k = 0; k < K; ++k) {
#pragma unroll
      for (int u = 0; u < QPT; ++u) {
        const uint64_t op = ops[(size_t)k * qpad + tid + u * T];
        const uint32_t opc = (uint32_t)op & 0xFFu;
        if (opc == OP_NOP) continue;
        const uint32_t sub = ((uint32_t)op >> 8) & 0xFFu;
        const uint32_t arg = (uint32_t)(op >> 32);
        switch (opc) {
          case OP_C1: {
            const uint64_t x = X[u], z = Z[u];
            X[u] = sel2(sub & 3u, x, z);
            Z[u] = sel2(sub >> 2, x, z);
            break;
          }
          case OP_C2: {
            const ulonglong2 p = pb[arg];
            const uint64_t x = X[u], z = Z[u];
            X[u] = sel4(sub & 15u, x, z, p.x, p.y);
            Z[u] = sel4(sub >> 4, x, z, p.x, p.y);
            break;
          }
          case OP_R:
            X[u] = Z[u] = 0;
            break;
          case OP_INJ: {
            const uint32_t b2 = ((uint32_t)op >> 8) & 0xFFFFFFu;
            if (arg - jlo < 64u) acc[u] |= 1ull << (arg - jlo);
            if (b2 != 0xFFFFFFu && b2 - jlo < 64u) acc[u] |= 1ull << (b2 - jlo);
            break;
          }
          case OP_M: {
            uint64_t inj = acc[u];
            if (arg - jlo < 64u) inj |= 1ull << (arg - jlo);
            acc[u] = 0;
            if (sub & 4u) X[u] = Z[u] = 0;
            const uint32_t basis = sub & 3u;
            if (basis != 1u) X[u] ^= inj;
            if (basis != 0u) Z[u] ^= inj;
            last_inj[u] = inj;
            break;
          }
          case OP_SNAP:
            snap_j[arg] = make_ulonglong2(X[u], Z[u]);
            break;
          case OP_SNAPD:
            snap_j[arg] = make_ulonglong2(last_inj[u], 0ull);
            break;
          default:
            break;
        }
      }
    }
  }
  if (tid == 0) {
    C.band[j] = make_uint2(C.ep_ptoff[e0], C.ep_ptoff[e < nE ? e : nE]);
    // Copies still in flight target this CTA's shared memory: wait for them
    // (bounded) before the CTA exits.
    for (uint32_t s = consumed; s < issued; ++s) {
      if (!mbar_wait_bounded(&mbar[s % ring_slots], (s / ring_slots) & 1u)) {
        atomicOr(err, DEV_ERR_TIMEOUT);
        break;
      }
    }
  }
}

}  // namespace

size_t walk_smem_bytes(uint32_t qpad, uint32_t ring_slots, uint32_t slot_bytes, uint32_t max_epochs) {
  const uint32_t tab = max_epochs <= kEpochTabMax ? max_epochs : 0;
  return (size_t)2 * qpad * sizeof(ulonglong2) + 128 + ((size_t)tab * sizeof(uint2) + 127) / 128 * 128 +
         (size_t)ring_slots * slot_bytes;
}

cudaError_t launch_walk(const WalkLaunch &L, cudaStream_t s) {
  if (L.n_items == 0) return cudaSuccess;
  if (L.ring_slots < 1 || L.ring_slots > 16) return cudaErrorInvalidValue;
  const uint32_t tab = L.max_epochs <= kEpochTabMax ? L.max_epochs : 0;
  const size_t smem = walk_smem_bytes(L.qpad, L.ring_slots, L.slot_bytes, L.max_epochs);
  cudaError_t e;
#define GPC_WALK(Q)                                                                                      \
  e = cudaFuncSetAttribute(walk_kernel<Q>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);     \
  if (e != cudaSuccess) return e;                                                                        \
  walk_kernel<Q><<<L.n_items, L.threads, smem, s>>>(L.circs, L.items, L.ring_slots, L.slot_bytes, tab, L.err)
  switch (L.qpt) {
    case 1:
      GPC_WALK(1);
      break;
    case 2:
      GPC_WALK(2);
      break;
    case 4:
      GPC_WALK(4);
      break;
    default:
      return cudaErrorInvalidValue;
  }
#undef GPC_WALK
  return cudaGetLastError();
}

}  // namespace gpc
