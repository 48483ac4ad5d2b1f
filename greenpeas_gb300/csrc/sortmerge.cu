// sortmerge.cu -- symptom keys, onesweep radix sort, segmented merge (sm_103a).
//
// Replaces the reference's K3-K7 (Policies/Compute/CUDA.hpp:184-189,276-343,
// 422-497; CUDAHandlers.hpp:67-139): set-bit extraction truncated at 32 bits
// + a 64-bit FNV hash with no collision check, CUB radix sort, a gather of
// probabilities, CUB reduce-by-key and a gather of the full class matrix.
//
//  * key_kernel: one thread per mechanism computes its symptom words from
//    the walk's snapshots (word j of mechanism m is the XOR of the selected
//    rows of its one or two points, zero outside word j's band) and folds them
//    into a 128-bit key  K = XOR_j H(j, word_j), H(j, 0) = 0, so the empty
//    symptom has key 0 and the key is independent of padding.
//  * onesweep radix sort (one histogram kernel + one kernel per 8-bit digit):
//    every tile ranks its items per digit with warp match/popc, publishes its
//    digit counts and resolves its global offsets by decoupled look-back on
//    the preceding tiles' status words.  Stable, so equal keys keep
//    ascending mechanism order.
//  * merge_kernel: one thread per sorted item.  A group is a run of equal
//    128-bit keys; every item checks its full symptom against its
//    predecessor (collision check).  Group heads fold the probabilities of
//    their run left to right with p <- p(1-q) + q(1-p) (CUDAHandlers.hpp:
//    635-640) in FP64, extract the targets of the symptom, and get their
//    output slot from a block scan plus decoupled look-back.  The empty
//    symptom (key 0) is dropped (Driver.hpp:185).
#include <cstdint>

#include "device.cuh"

namespace gpc {
namespace {

constexpr unsigned long long kSpinLimitNs = 200ull * 1000 * 1000;  // 200 ms

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// murmur3 64-bit finaliser (a published bijective mixer).
__device__ __forceinline__ uint64_t fmix64(uint64_t k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdull;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ull;
  k ^= k >> 33;
  return k;
}

// Two independent mixes of (word index, non-zero word value).
__device__ __forceinline__ ulonglong2 word_hash(uint32_t j, uint64_t v) {
  const uint64_t jj = (uint64_t)j + 1;
  return make_ulonglong2(fmix64(v * 0x9E3779B97F4A7C15ull + jj * 0xC2B2AE3D27D4EB4Full),
                         fmix64(v * 0xD6E8FEB86659FD93ull + jj * 0xA0761D6478BD642Full + 0x8EBC6AF09C88C6E3ull));
}

__device__ __forceinline__ uint64_t pauli_sel(ulonglong2 s, uint32_t P) {
  return (s.x & (0ull - (uint64_t)(P & 1u))) ^ (s.y & (0ull - (uint64_t)((P >> 1) & 1u)));
}

// Word j of mechanism descriptor d (band-aware).
__device__ __forceinline__ uint64_t symptom_word(const CircuitDev &C, uint64_t d, uint32_t j, uint2 b) {
  const uint32_t pa = (uint32_t)(d & 0x3FFFFFFFu), Pa = (uint32_t)((d >> 30) & 3u);
  const uint32_t pb = (uint32_t)((d >> 32) & 0x3FFFFFFFu), Pb = (uint32_t)(d >> 62);
  const ulonglong2 *sj = C.snap + (size_t)j * C.npoints;
  uint64_t v = 0;
  if (Pa && pa - b.x < b.y - b.x) v ^= pauli_sel(sj[pa], Pa);
  if (Pb && pb - b.x < b.y - b.x) v ^= pauli_sel(sj[pb], Pb);
  return v;
}

__global__ void key_kernel(const CircuitDev *__restrict__ cdev, uint32_t M, uint32_t w, ulonglong2 *__restrict__ key,
                           uint64_t *__restrict__ sortkey, uint32_t *__restrict__ perm) {
  extern __shared__ uint2 sband[];
  const CircuitDev C = *cdev;
  for (uint32_t j = threadIdx.x; j < w; j += blockDim.x) sband[j] = C.band[j];
  __syncthreads();
  for (uint32_t m = blockIdx.x * blockDim.x + threadIdx.x; m < M; m += gridDim.x * blockDim.x) {
    const uint64_t d = __ldg(C.desc + m);
    uint64_t hx = 0, hy = 0;
    for (uint32_t j = 0; j < w; ++j) {
      const uint64_t v = symptom_word(C, d, j, sband[j]);
      if (v) {
        const ulonglong2 h = word_hash(j, v);
        hx ^= h.x;
        hy ^= h.y;
      }
    }
    key[m] = make_ulonglong2(hx, hy);
    sortkey[m] = hx;
    perm[m] = m;
  }
}

// ---- onesweep radix sort ----------------------------------------------------

__global__ void sort_hist_kernel(const uint64_t *__restrict__ keys, uint32_t n, uint32_t passes,
                                 uint32_t *__restrict__ hist) {
  __shared__ uint32_t h[8][RADIX];
  for (uint32_t i = threadIdx.x; i < 8 * RADIX; i += blockDim.x) (&h[0][0])[i] = 0;
  __syncthreads();
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint64_t k = keys[i];
    for (uint32_t p = 0; p < passes; ++p) atomicAdd(&h[p][(k >> (p * RADIX_BITS)) & (RADIX - 1)], 1u);
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < passes * RADIX; i += blockDim.x) {
    const uint32_t v = (&h[0][0])[i];
    if (v) atomicAdd(hist + i, v);
  }
}

// Exclusive scan of each pass's histogram (one block of RADIX threads per pass).
__global__ void sort_scan_kernel(uint32_t *__restrict__ hist) {
  __shared__ uint32_t s[RADIX];
  uint32_t *h = hist + blockIdx.x * RADIX;
  const uint32_t t = threadIdx.x;
  s[t] = h[t];
  __syncthreads();
  for (uint32_t off = 1; off < RADIX; off <<= 1) {
    const uint32_t v = t >= off ? s[t - off] : 0;
    __syncthreads();
    s[t] += v;
    __syncthreads();
  }
  h[t] = s[t] - h[t];
}

constexpr uint32_t ST_AGG = 1u << 30;     // tile aggregate published
constexpr uint32_t ST_PREFIX = 2u << 30;  // inclusive prefix published
constexpr uint32_t ST_MASK = (1u << 30) - 1;

__global__ void __launch_bounds__(SORT_THREADS) sort_pass_kernel(
    const uint64_t *__restrict__ kin, const uint32_t *__restrict__ vin, uint64_t *__restrict__ kout,
    uint32_t *__restrict__ vout, uint32_t n, uint32_t shift, const uint32_t *__restrict__ gofs,
    uint32_t *__restrict__ status, uint32_t *__restrict__ tile_ctr, uint32_t *__restrict__ err) {
  constexpr int WARPS = SORT_THREADS / 32;
  __shared__ uint32_t wcount[WARPS][RADIX];
  __shared__ uint32_t dbase[RADIX];
  __shared__ uint32_t s_tile;
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  for (uint32_t i = threadIdx.x; i < WARPS * RADIX; i += SORT_THREADS) (&wcount[0][0])[i] = 0;
  if (threadIdx.x == 0) s_tile = atomicAdd(tile_ctr, 1u);
  __syncthreads();
  const uint32_t tile = s_tile;
  const uint32_t base = tile * SORT_TILE + warp * (32 * SORT_IPT) + lane;

  uint64_t key[SORT_IPT];
  uint32_t val[SORT_IPT];
  uint32_t dig[SORT_IPT];
  uint32_t rank[SORT_IPT];
#pragma unroll
  for (int k = 0; k < SORT_IPT; ++k) {
    const uint32_t idx = base + k * 32;
    if (idx < n) {
      key[k] = kin[idx];
      val[k] = vin[idx];
      dig[k] = (uint32_t)(key[k] >> shift) & (RADIX - 1);
    } else {
      key[k] = 0;
      val[k] = 0;
      dig[k] = RADIX;  // not counted
    }
  }
  const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
  for (int k = 0; k < SORT_IPT; ++k) {
    const uint32_t peers = __match_any_sync(0xFFFFFFFFu, dig[k]);
    const uint32_t leader = __ffs(peers) - 1u;
    uint32_t b = 0;
    if (dig[k] < RADIX) b = wcount[warp][dig[k]];
    rank[k] = b + __popc(peers & lt);
    __syncwarp();
    if (lane == leader && dig[k] < RADIX) wcount[warp][dig[k]] = b + __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  // per digit: exclusive scan over warps, tile count, look-back
  {
    const uint32_t d = threadIdx.x;  // SORT_THREADS == RADIX
    uint32_t sum = 0;
#pragma unroll
    for (int w = 0; w < WARPS; ++w) {
      const uint32_t c = wcount[w][d];
      wcount[w][d] = sum;
      sum += c;
    }
    volatile uint32_t *st = status;
    if (tile == 0) {
      st[d] = ST_PREFIX | sum;
      dbase[d] = gofs[d];
    } else {
      st[(size_t)tile * RADIX + d] = ST_AGG | sum;
      uint32_t excl = 0;
      int32_t t = (int32_t)tile - 1;
      unsigned long long t0 = 0;
      while (t >= 0) {
        const uint32_t s = st[(size_t)t * RADIX + d];
        if ((s & ~ST_MASK) == 0) {
          if (t0 == 0) t0 = globaltimer();
          else if (globaltimer() - t0 > kSpinLimitNs) {
            atomicOr(err, DEV_ERR_TIMEOUT);
            break;
          }
          continue;
        }
        t0 = 0;
        excl += s & ST_MASK;
        if (s & ST_PREFIX) break;
        --t;
      }
      __threadfence();
      st[(size_t)tile * RADIX + d] = ST_PREFIX | (excl + sum);
      dbase[d] = gofs[d] + excl;
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < SORT_IPT; ++k) {
    if (dig[k] < RADIX) {
      const uint32_t pos = dbase[dig[k]] + wcount[warp][dig[k]] + rank[k];
      if (pos < n) {  // always true unless a look-back wait timed out
        kout[pos] = key[k];
        vout[pos] = val[k];
      }
    }
  }
}

__global__ void gather_hi_kernel(const ulonglong2 *__restrict__ key, const uint32_t *__restrict__ perm,
                                 uint64_t *__restrict__ out, uint32_t n) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    out[i] = key[perm[i]].y;
}

// ---- merge ------------------------------------------------------------------

constexpr unsigned long long MS_AGG = 1ull << 62;
constexpr unsigned long long MS_PREFIX = 2ull << 62;

__device__ __forceinline__ unsigned long long ms_pack(uint32_t cnt, uint32_t tg) {
  return ((unsigned long long)(cnt & 0x3FFFFFFFu) << 32) | tg;
}

__global__ void __launch_bounds__(MERGE_THREADS) merge_kernel(MergeLaunch L) {
  const CircuitDev C = *L.c_dev;
  extern __shared__ uint2 sband[];  // [w]
  __shared__ uint32_t s_tile;
  __shared__ uint32_t wsum_c[MERGE_THREADS / 32], wsum_t[MERGE_THREADS / 32];
  __shared__ uint32_t s_pre_c, s_pre_t;
  const uint32_t w = L.w;
  for (uint32_t j = threadIdx.x; j < w; j += blockDim.x) sband[j] = C.band[j];
  if (threadIdx.x == 0) s_tile = atomicAdd(L.tile_ctr, 1u);
  __syncthreads();
  const uint32_t tile = s_tile;
  const uint32_t i = tile * MERGE_THREADS + threadIdx.x;
  const uint32_t n = L.n;
  const uint32_t ntiles = (n + MERGE_THREADS - 1) / MERGE_THREADS;

  bool head = false;
  uint32_t ntg = 0, m = 0;
  ulonglong2 k = make_ulonglong2(0, 0);
  if (i < n) {
    m = L.perm[i];
    k = L.key[m];
    const uint64_t d = __ldg(C.desc + m);
    bool newgroup = true;
    if (i > 0) {
      const uint32_t mp = L.perm[i - 1];
      const ulonglong2 kp = L.key[mp];
      if (kp.x == k.x && kp.y == k.y) {
        newgroup = false;
        const uint64_t dp = __ldg(C.desc + mp);
        for (uint32_t j = 0; j < w; ++j) {
          if (symptom_word(C, d, j, sband[j]) != symptom_word(C, dp, j, sband[j])) {
            atomicOr(L.err, DEV_ERR_COLLISION);
            break;
          }
        }
      } else if (((L.sortkey[i] ^ L.sortkey[i - 1]) & L.sort_mask) == 0 && L.sort_mask) {
        atomicOr(L.err, DEV_FLAG_MIXED);
      }
    }
    const bool empty = (k.x | k.y) == 0;
    if (newgroup && empty) {
      for (uint32_t j = 0; j < w; ++j)
        if (symptom_word(C, d, j, sband[j])) {
          atomicOr(L.err, DEV_ERR_COLLISION);
          break;
        }
    }
    head = newgroup && !empty;
    if (head)
      for (uint32_t j = 0; j < w; ++j) ntg += __popcll(symptom_word(C, d, j, sband[j]));
  }
  // block-wide exclusive scan of (head, ntg)
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint32_t c_in = head ? 1u : 0u, t_in = ntg;
  uint32_t c_inc = c_in, t_inc = t_in;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const uint32_t a = __shfl_up_sync(0xFFFFFFFFu, c_inc, off), b = __shfl_up_sync(0xFFFFFFFFu, t_inc, off);
    if (lane >= (uint32_t)off) {
      c_inc += a;
      t_inc += b;
    }
  }
  if (lane == 31) {
    wsum_c[warp] = c_inc;
    wsum_t[warp] = t_inc;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t ac = 0, at = 0;
    for (int x = 0; x < MERGE_THREADS / 32; ++x) {
      const uint32_t c = wsum_c[x], t = wsum_t[x];
      wsum_c[x] = ac;
      wsum_t[x] = at;
      ac += c;
      at += t;
    }
    // decoupled look-back over preceding tiles
    volatile unsigned long long *st = L.status;
    uint32_t pc = 0, pt = 0;
    if (tile == 0) {
      st[0] = MS_PREFIX | ms_pack(ac, at);
    } else {
      st[tile] = MS_AGG | ms_pack(ac, at);
      int32_t t = (int32_t)tile - 1;
      unsigned long long t0 = 0;
      while (t >= 0) {
        const unsigned long long s = st[t];
        if ((s >> 62) == 0) {
          if (t0 == 0) t0 = globaltimer();
          else if (globaltimer() - t0 > kSpinLimitNs) {
            atomicOr(L.err, DEV_ERR_TIMEOUT);
            break;
          }
          continue;
        }
        t0 = 0;
        pc += (uint32_t)((s >> 32) & 0x3FFFFFFFu);
        pt += (uint32_t)s;
        if (s & MS_PREFIX) break;
        --t;
      }
      __threadfence();
      st[tile] = MS_PREFIX | ms_pack(pc + ac, pt + at);
    }
    s_pre_c = pc;
    s_pre_t = pt;
    if (tile == ntiles - 1) {
      L.totals[0] = pc + ac;
      L.totals[1] = pt + at;
      if (pt + at > L.tg_cap) atomicOr(L.err, DEV_FLAG_TG_OVF);
    }
  }
  __syncthreads();
  if (!head) return;
  const uint32_t slot = s_pre_c + wsum_c[warp] + c_inc - c_in;
  if (slot >= n) return;  // only after a timed-out look-back
  const uint32_t toff = s_pre_t + wsum_t[warp] + t_inc - t_in;
  // fold the run's probabilities left to right
  double p = __ldg(C.prob + m);
  for (uint32_t i2 = i + 1; i2 < n; ++i2) {
    const uint32_t m2 = L.perm[i2];
    const ulonglong2 k2 = L.key[m2];
    if (k2.x != k.x || k2.y != k.y) break;
    const double q = __ldg(C.prob + m2);
    p = p * (1.0 - q) + q * (1.0 - p);
  }
  L.out_prob[slot] = p;
  L.out_off[slot] = toff;
  if (toff + ntg <= L.tg_cap) {
    const uint64_t d = __ldg(C.desc + m);
    uint32_t o = toff;
    for (uint32_t j = 0; j < w; ++j) {
      uint64_t v = symptom_word(C, d, j, sband[j]);
      while (v) {
        L.out_tg[o++] = j * 64u + (uint32_t)(__ffsll((long long)v) - 1);
        v &= v - 1;
      }
    }
  }
}

}  // namespace

cudaError_t launch_keys(const CircuitDev *c_dev, uint32_t M, uint32_t w, ulonglong2 *key, uint64_t *sortkey,
                        uint32_t *perm, cudaStream_t s) {
  if (M == 0) return cudaSuccess;
  const uint32_t threads = 256;
  uint32_t blocks = (M + threads - 1) / threads;
  if (blocks > 152u * 16u) blocks = 152u * 16u;
  key_kernel<<<blocks, threads, (size_t)w * sizeof(uint2), s>>>(c_dev, M, w, key, sortkey, perm);
  return cudaGetLastError();
}

size_t sort_scratch_words(uint32_t n, uint32_t bits) {
  const uint32_t passes = (bits + RADIX_BITS - 1) / RADIX_BITS;
  // hist + status + tile counters, for a 128-bit fallback as well (2 sorts)
  return 2 * ((size_t)passes * RADIX + (size_t)passes * sort_tiles(n) * RADIX + passes);
}

cudaError_t launch_sort(uint64_t *keys, uint64_t *keys_alt, uint32_t *vals, uint32_t *vals_alt, uint32_t n,
                        uint32_t bits, const SortScratch &scr, cudaStream_t s, bool *result_in_alt) {
  *result_in_alt = false;
  if (n == 0) return cudaSuccess;
  const uint32_t passes = (bits + RADIX_BITS - 1) / RADIX_BITS;
  if (passes == 0 || passes > 8) return cudaErrorInvalidValue;
  const uint32_t tiles = sort_tiles(n);
  uint32_t hb = (n + 1023) / 1024;
  if (hb > 152u * 4u) hb = 152u * 4u;
  sort_hist_kernel<<<hb, 1024, 0, s>>>(keys, n, passes, scr.hist);
  sort_scan_kernel<<<passes, RADIX, 0, s>>>(scr.hist);
  uint64_t *ki = keys, *ko = keys_alt;
  uint32_t *vi = vals, *vo = vals_alt;
  for (uint32_t p = 0; p < passes; ++p) {
    sort_pass_kernel<<<tiles, SORT_THREADS, 0, s>>>(ki, vi, ko, vo, n, p * RADIX_BITS, scr.hist + p * RADIX,
                                                    scr.status + (size_t)p * tiles * RADIX, scr.tile_ctr + p,
                                                    scr.err);
    uint64_t *tk = ki;
    ki = ko;
    ko = tk;
    uint32_t *tv = vi;
    vi = vo;
    vo = tv;
  }
  *result_in_alt = (passes & 1u) != 0;
  return cudaGetLastError();
}

cudaError_t launch_gather_hi(const ulonglong2 *key, const uint32_t *perm, uint64_t *out, uint32_t n, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  uint32_t blocks = (n + 255) / 256;
  if (blocks > 152u * 16u) blocks = 152u * 16u;
  gather_hi_kernel<<<blocks, 256, 0, s>>>(key, perm, out, n);
  return cudaGetLastError();
}

cudaError_t launch_merge(const MergeLaunch &L, cudaStream_t s) {
  if (L.n == 0) return cudaSuccess;
  const uint32_t tiles = merge_tiles(L.n);
  merge_kernel<<<tiles, MERGE_THREADS, (size_t)L.w * sizeof(uint2), s>>>(L);
  return cudaGetLastError();
}

}  // namespace gpc
