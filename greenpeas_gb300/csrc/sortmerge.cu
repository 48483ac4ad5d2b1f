// sortmerge.cu -- symptom keys, radix bucketing / onesweep sort, merge (sm_103a).
//
// Replaces the reference's K3-K7 (Policies/Compute/CUDA.hpp:184-189,276-343,
// 422-497; CUDAHandlers.hpp:67-139): set-bit extraction truncated at 32 bits
// + a 64-bit FNV hash with no collision check, CUB radix sort, a gather of
// probabilities, CUB reduce-by-key and a gather of the full class matrix.
//
//  * key_kernel: one thread per noise record.  It expands the record into
//    its mechanisms (the Pauli components of the channel), computes each
//    mechanism's symptom words from the walk's snapshots -- word j is the
//    XOR of the selected rows of its one or two points, zero outside word
//    j's band -- and folds them into a 128-bit key K = XOR_j H(j, word_j)
//    with H(j, 0) = 0, so the empty symptom has key 0.  Non-empty keys are
//    counted per bucket (the top bits of K: one MSD radix digit).
//  * bucket scan + scatter: the radix partition pass.
//  * bucket_merge_kernel: one CTA per bucket sorts its items in shared memory
//    by (K, mechanism), so a group (run of equal K) keeps ascending mechanism
//    order; every item checks its full symptom against its predecessor
//    (collision check); group heads fold their run's probabilities left to
//    right with p <- p(1-q) + q(1-p) (CUDAHandlers.hpp:635-640) in FP64,
//    extract their targets and get an output slot from a block scan plus a
//    warp-wide decoupled look-back over the preceding buckets.  The empty
//    symptom is dropped (Driver.hpp:185).
//  * global path, used when a bucket exceeds one CTA (a symptom repeated
//    more than BUCKET_CAP times): LSD onesweep radix sort of all keys (one
//    kernel per 8-bit digit, tile ranks by warp match/popc, decoupled
//    look-back for digit offsets) and a merge kernel over the sorted run.
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

__device__ __forceinline__ uint64_t mk_desc(uint32_t pa, uint32_t Pa, uint32_t pb, uint32_t Pb) {
  return (uint64_t)(pa & 0x3FFFFFFFu) | ((uint64_t)(Pa & 3u) << 30) | ((uint64_t)(pb & 0x3FFFFFFFu) << 32) |
         ((uint64_t)(Pb & 3u) << 62);
}

// Components of each record type as (Pauli a | Pauli b << 2); Pauli: 1 X, 2 Z, 3 Y.
// Two-qubit lists follow stim's order IX IY IZ XI XX XY XZ YI YX YY YZ ZI ZX ZY ZZ,
// restricted to the correlation level's set (Mixer.hpp:13-20).
#define PP(a, b) ((a) | ((b) << 2))
__constant__ uint8_t kComp[6][15] = {
    {0},
    {PP(1, 0), PP(2, 0)},
    {PP(1, 0), PP(3, 0), PP(2, 0)},
    {PP(0, 1), PP(0, 2), PP(1, 0), PP(1, 1), PP(2, 0), PP(2, 2)},
    {PP(0, 1), PP(0, 3), PP(0, 2), PP(1, 0), PP(1, 1), PP(1, 2), PP(3, 0), PP(2, 0), PP(2, 1), PP(2, 2)},
    {PP(0, 1), PP(0, 3), PP(0, 2), PP(1, 0), PP(1, 1), PP(1, 3), PP(1, 2), PP(3, 0), PP(3, 1), PP(3, 3), PP(3, 2),
     PP(2, 0), PP(2, 1), PP(2, 3), PP(2, 2)},
};
__constant__ uint8_t kNComp[6] = {1, 2, 3, 6, 10, 15};
#undef PP

__global__ void __launch_bounds__(256) key_kernel(KeyLaunch L) {
  __shared__ uint32_t smb[kMaxCircuitsStaged + 1];
  __shared__ uint2 sband[1024];
  __shared__ uint32_t s_c0, s_c1;
  const bool staged = L.n_circ <= kMaxCircuitsStaged;
  for (uint32_t i = threadIdx.x; staged && i <= L.n_circ; i += blockDim.x) smb[i] = L.mbase[i];
  __syncthreads();
  const uint32_t *mb = staged ? smb : L.mbase;
  const uint32_t m0 = blockIdx.x * blockDim.x;
  const uint32_t mg = m0 + threadIdx.x;
  // the circuits of this block's first and last mechanisms; one circuit: stage its bands
  if (threadIdx.x == 0) {
    s_c0 = find_circuit(mb, L.n_circ, m0);
    s_c1 = find_circuit(mb, L.n_circ, min(L.M - 1, m0 + blockDim.x - 1));
  }
  __syncthreads();
  const uint32_t c0 = s_c0;
  const bool oneband = s_c0 == s_c1 && L.circs[c0].w <= 1024;
  if (oneband)
    for (uint32_t j = threadIdx.x; j < L.circs[c0].w; j += blockDim.x) sband[j] = L.circs[c0].band[j];
  __syncthreads();
  if (mg >= L.M) return;
  const uint32_t c = oneband ? c0 : find_circuit(mb, L.n_circ, mg);
  const CircuitDev &C = L.circs[c];
  const uint32_t m = mg - mb[c];
  const uint32_t w = C.w;
  const uint32_t tcap = C.tcap;
  const uint32_t R = C.R;
  // the record holding mechanism m: the last r with rec_moff[r] <= m
  uint32_t lo = 0, hi = R;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (__ldg(C.rec_moff + mid) <= m) lo = mid;
    else hi = mid;
  }
  const uint32_t r = lo;
  const uint64_t d = __ldg(C.rec + r);
  const uint32_t ci = m - __ldg(C.rec_moff + r);
  const uint32_t type = (uint32_t)((d >> 56) & 15u);
  const uint32_t comp = type == 0 ? (uint32_t)((d >> 60) & 3u) | ((uint32_t)(d >> 62) << 2) : kComp[type][ci];
  uint32_t pa = (uint32_t)(d & 0x0FFFFFFFu), pb = (uint32_t)((d >> 28) & 0x0FFFFFFFu);
  uint32_t Pa = comp & 3u, Pb = comp >> 2;
  if (Pa == 0) {  // a component on point b only is stored with b as its first point
    pa = pb;
    Pa = Pb;
    Pb = 0;
  }
  if (Pb == 0) pb = 0;
  C.mdesc[m] = mk_desc(pa, Pa, pb, Pb);
  C.mp[m] = __ldg(C.rec_p + r);
  uint64_t hx = 0, hy = 0;
  uint32_t cnt = 0;
  bool nonzero = false;
  uint32_t *out = C.tl + (size_t)m * tcap;
  const ulonglong2 *snap = C.snap;
  const uint32_t np = C.npoints;
  for (uint32_t j = 0; j < w; ++j) {
    const uint2 b = oneband ? sband[j] : C.band[j];
    const ulonglong2 *sj = snap + (size_t)j * np;
    uint64_t v = 0;
    if (pa - b.x < b.y - b.x) v = pauli_sel(sj[pa], Pa);
    if (Pb && pb - b.x < b.y - b.x) v ^= pauli_sel(sj[pb], Pb);
    if (!v) continue;
    nonzero = true;
    const ulonglong2 h = word_hash(j, v);
    hx ^= h.x;
    hy ^= h.y;
    if (tcap) {
      uint64_t x = v;
      while (x) {
        if (cnt < tcap) out[cnt] = j * 64u + (uint32_t)(__ffsll((long long)x) - 1);
        ++cnt;
        x &= x - 1;
      }
    }
  }
  L.key[mg] = make_ulonglong2(hx, hy);
  if (tcap) {
    C.tn[m] = cnt;
    if (cnt > tcap) atomicOr(L.err, DEV_FLAG_LONG);
    if (cnt) atomicAdd(L.list_total, cnt);
  }
  if ((hx | hy) == 0) {
    if (cnt || (!tcap && nonzero)) atomicOr(L.err, DEV_ERR_COLLISION);  // a non-empty symptom hashed to 0
  } else {
    atomicAdd(L.bucket_count + C.bbase + (uint32_t)(hx >> (64u - C.bbits)), 1u);
  }
}

// Exclusive scan of nb bucket counts (one block); offset[nb] = total.
__global__ void __launch_bounds__(1024) bucket_scan_kernel(const uint32_t *__restrict__ count,
                                                           uint32_t *__restrict__ offset, uint32_t nb) {
  __shared__ uint32_t part[1024];
  const uint32_t t = threadIdx.x;
  const uint32_t per = (nb + 1023) / 1024;
  const uint32_t lo = min(nb, t * per), hi = min(nb, lo + per);
  uint32_t sum = 0;
  for (uint32_t i = lo; i < hi; ++i) sum += count[i];
  part[t] = sum;
  __syncthreads();
  for (uint32_t off = 1; off < 1024; off <<= 1) {
    const uint32_t v = t >= off ? part[t - off] : 0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  uint32_t run = part[t] - sum;
  for (uint32_t i = lo; i < hi; ++i) {
    const uint32_t c = count[i];
    offset[i] = run;
    run += c;
  }
  if (t == 1023) offset[nb] = part[1023];
}

__global__ void bucket_scatter_kernel(const ulonglong2 *__restrict__ key, uint32_t M, uint32_t shift,
                                      const uint32_t *__restrict__ offset, uint32_t *__restrict__ cursor,
                                      ulonglong2 *__restrict__ bkey, uint32_t *__restrict__ bm) {
  for (uint32_t m = blockIdx.x * blockDim.x + threadIdx.x; m < M; m += gridDim.x * blockDim.x) {
    const ulonglong2 k = key[m];
    if ((k.x | k.y) == 0) continue;
    const uint32_t b = (uint32_t)(k.x >> shift);
    const uint32_t pos = offset[b] + atomicAdd(cursor + b, 1u);
    bkey[pos] = k;
    bm[pos] = m;
  }
}

__global__ void bucket_scatter_p_kernel(const CircuitDev *__restrict__ circs, const uint32_t *__restrict__ mbase,
                                        uint32_t n_circ, const ulonglong2 *__restrict__ key,
                                        const double *__restrict__ mp, uint32_t M,
                                        const uint32_t *__restrict__ offset, uint32_t *__restrict__ cursor,
                                        ulonglong2 *__restrict__ bkey, uint32_t *__restrict__ bm,
                                        double *__restrict__ bp) {
  __shared__ uint32_t smb[kMaxCircuitsStaged + 1];
  const bool staged = n_circ <= kMaxCircuitsStaged;
  for (uint32_t i = threadIdx.x; staged && i <= n_circ; i += blockDim.x) smb[i] = mbase[i];
  __syncthreads();
  const uint32_t *mb = staged ? smb : mbase;
  for (uint32_t m = blockIdx.x * blockDim.x + threadIdx.x; m < M; m += gridDim.x * blockDim.x) {
    const ulonglong2 k = key[m];
    if ((k.x | k.y) == 0) continue;
    const uint32_t c = n_circ == 1 ? 0u : find_circuit(mb, n_circ, m);
    const uint32_t b = circs[c].bbase + (uint32_t)(k.x >> (64u - circs[c].bbits));
    const uint32_t pos = offset[b] + atomicAdd(cursor + b, 1u);
    bkey[pos] = k;
    bm[pos] = m;
    bp[pos] = mp[m];
  }
}

__global__ void sort_init_kernel(const ulonglong2 *__restrict__ key, uint64_t *__restrict__ sortkey,
                                 uint32_t *__restrict__ perm, uint32_t M) {
  for (uint32_t m = blockIdx.x * blockDim.x + threadIdx.x; m < M; m += gridDim.x * blockDim.x) {
    sortkey[m] = key[m].x;
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
    const uint64_t d = __ldg(C.mdesc + m);
    bool newgroup = true;
    if (i > 0) {
      const uint32_t mp = L.perm[i - 1];
      const ulonglong2 kp = L.key[mp];
      if (kp.x == k.x && kp.y == k.y) {
        newgroup = false;
        const uint64_t dp = __ldg(C.mdesc + mp);
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
  double p = __ldg(C.mp + m);
  for (uint32_t i2 = i + 1; i2 < n; ++i2) {
    const uint32_t m2 = L.perm[i2];
    const ulonglong2 k2 = L.key[m2];
    if (k2.x != k.x || k2.y != k.y) break;
    const double q = __ldg(C.mp + m2);
    p = p * (1.0 - q) + q * (1.0 - p);
  }
  L.out_prob[slot] = p;
  L.out_off[slot] = toff;
  if (toff + ntg <= L.tg_cap) {
    const uint64_t d = __ldg(C.mdesc + m);
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

// ---- bucket sort + merge ---------------------------------------------------

// (key, m) order: key.x, then key.y, then mechanism id.
__device__ __forceinline__ bool item_less(ulonglong2 a, uint32_t ma, ulonglong2 b, uint32_t mb) {
  if (a.x != b.x) return a.x < b.x;
  if (a.y != b.y) return a.y < b.y;
  return ma < mb;
}

// Warp 0 resolves the exclusive prefix of tile `tile` over tiles [0, tile)
// by decoupled look-back: 32 predecessors per step.  `agg` is this tile's
// (count, targets) aggregate.  Returns the prefix in lane 0.
__device__ __forceinline__ void warp_lookback(unsigned long long *status, uint32_t tile, uint32_t agg_c,
                                              uint32_t agg_t, uint32_t *err, uint32_t *pre_c, uint32_t *pre_t) {
  const uint32_t lane = threadIdx.x & 31u;
  volatile unsigned long long *st = status;
  if (tile == 0) {
    if (lane == 0) st[0] = MS_PREFIX | ms_pack(agg_c, agg_t);
    *pre_c = 0;
    *pre_t = 0;
    return;
  }
  if (lane == 0) st[tile] = MS_AGG | ms_pack(agg_c, agg_t);
  uint32_t ec = 0, et = 0;
  int32_t base = (int32_t)tile - 1;
  unsigned long long t0 = 0;
  while (base >= 0) {
    const int32_t idx = base - (int32_t)lane;
    const unsigned long long s = idx >= 0 ? st[idx] : (MS_PREFIX | 0ull);
    const uint32_t flag = (uint32_t)(s >> 62);
    const uint32_t ready = __ballot_sync(0xFFFFFFFFu, flag != 0);
    const uint32_t pref = __ballot_sync(0xFFFFFFFFu, flag == 2u);
    // lanes up to (and including) the nearest prefix must all be ready
    const uint32_t need = pref ? ((pref & (0u - pref)) << 1) - 1u : 0xFFFFFFFFu;
    if ((ready & need) != need) {
      if (t0 == 0) t0 = globaltimer();
      else if (globaltimer() - t0 > kSpinLimitNs) {
        if (lane == 0) atomicOr(err, DEV_ERR_TIMEOUT);
        break;
      }
      continue;
    }
    t0 = 0;
    uint32_t c = (need >> lane) & 1u ? (uint32_t)((s >> 32) & 0x3FFFFFFFu) : 0u;
    uint32_t t = (need >> lane) & 1u ? (uint32_t)s : 0u;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      c += __shfl_xor_sync(0xFFFFFFFFu, c, o);
      t += __shfl_xor_sync(0xFFFFFFFFu, t, o);
    }
    ec += c;
    et += t;
    if (pref) break;
    base -= 32;
  }
  if (lane == 0) {
    __threadfence();
    st[tile] = MS_PREFIX | ms_pack(ec + agg_c, et + agg_t);
  }
  *pre_c = ec;
  *pre_t = et;
}

// Loads a target list as 16-byte vectors (rows are 16-byte aligned).
__device__ __forceinline__ bool lists_equal(const uint32_t *a, const uint32_t *b, uint32_t n) {
  const uint4 *va = reinterpret_cast<const uint4 *>(a), *vb = reinterpret_cast<const uint4 *>(b);
  for (uint32_t k = 0; k * 4 < n; ++k) {
    const uint4 x = __ldg(va + k), y = __ldg(vb + k);
    const uint32_t rem = n - k * 4;
    if (x.x != y.x || (rem > 1 && x.y != y.y) || (rem > 2 && x.z != y.z) || (rem > 3 && x.w != y.w)) return false;
  }
  return true;
}

__global__ void __launch_bounds__(BUCKET_THREADS) bucket_merge_kernel(BucketMergeLaunch L) {
  constexpr int NT = BUCKET_THREADS;
  constexpr int NW = NT / 32;
  __shared__ ulonglong2 sk[BUCKET_CAP];
  __shared__ uint32_t sm[BUCKET_CAP];
  __shared__ uint16_t ord[BUCKET_CAP];
  __shared__ uint32_t sntg[BUCKET_CAP];  // targets of a group starting at a sorted position, else ~0u
  __shared__ uint2 sexc[BUCKET_CAP];     // exclusive (groups, targets) before each sorted position
  __shared__ uint32_t wc[NW], wt[NW];
  __shared__ uint32_t s_b, s_pre_c, s_pre_t;
  extern __shared__ uint2 sband[];
  const CircuitDev C = *L.c_dev;
  const uint32_t w = L.w;
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  for (uint32_t j = threadIdx.x; j < w; j += NT) sband[j] = C.band[j];
  if (threadIdx.x == 0) s_b = atomicAdd(L.ticket, 1u);
  __syncthreads();
  const uint32_t b = s_b;
  uint32_t n = L.count[b];
  const uint32_t base = L.offset[b];
  if (n > (uint32_t)BUCKET_CAP) {
    if (threadIdx.x == 0) atomicOr(L.err, DEV_FLAG_BIG_BUCKET);
    n = 0;
  }
  for (uint32_t i = threadIdx.x; i < n; i += NT) {
    sk[i] = L.bkey[base + i];
    sm[i] = L.bm[base + i];
  }
  __syncthreads();
  // rank sort by (key, m): every key is distinct once m is included
  for (uint32_t i = threadIdx.x; i < n; i += NT) {
    const ulonglong2 ki = sk[i];
    const uint32_t mi = sm[i];
    uint32_t r = 0;
    for (uint32_t k = 0; k < n; ++k) r += item_less(sk[k], sm[k], ki, mi) ? 1u : 0u;
    ord[r] = (uint16_t)i;
  }
  __syncthreads();
  // group heads, collision checks (full target lists), target counts
  const uint32_t tcap = C.tcap;
  for (uint32_t s = threadIdx.x; s < n; s += NT) {
    const uint32_t i = ord[s];
    const uint32_t m = sm[i];
    const uint32_t nt = __ldg(C.tn + m);
    bool head = true;
    if (s > 0) {
      const uint32_t ip = ord[s - 1];
      if (sk[ip].x == sk[i].x && sk[ip].y == sk[i].y) {
        head = false;
        const uint32_t mq = sm[ip];
        if (__ldg(C.tn + mq) != nt ||
            !lists_equal(C.tl + (size_t)m * tcap, C.tl + (size_t)mq * tcap, nt))
          atomicOr(L.err, DEV_ERR_COLLISION);
      }
    }
    sntg[s] = head ? nt : ~0u;
  }
  __syncthreads();
  // block-wide exclusive scan of (heads, targets) over sorted positions, NT at a time
  uint32_t carry_c = 0, carry_t = 0;
  for (uint32_t r0 = 0; r0 < n; r0 += NT) {
    const uint32_t s = r0 + threadIdx.x;
    const uint32_t v = s < n ? sntg[s] : ~0u;
    const uint32_t c_in = v != ~0u ? 1u : 0u, t_in = v != ~0u ? v : 0u;
    uint32_t ic = c_in, it = t_in;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t a = __shfl_up_sync(0xFFFFFFFFu, ic, o), bb = __shfl_up_sync(0xFFFFFFFFu, it, o);
      if (lane >= (uint32_t)o) {
        ic += a;
        it += bb;
      }
    }
    if (lane == 31) {
      wc[warp] = ic;
      wt[warp] = it;
    }
    __syncthreads();
    uint32_t pc = carry_c, pt = carry_t;
    for (uint32_t x = 0; x < warp; ++x) {
      pc += wc[x];
      pt += wt[x];
    }
    if (s < n) sexc[s] = make_uint2(pc + ic - c_in, pt + it - t_in);
    for (uint32_t x = 0; x < (uint32_t)NW; ++x) {
      carry_c += wc[x];
      carry_t += wt[x];
    }
    __syncthreads();
  }
  if (threadIdx.x < 32) {
    uint32_t pc = 0, pt = 0;
    warp_lookback(L.status, b, carry_c, carry_t, L.err, &pc, &pt);
    if (threadIdx.x == 0) {
      s_pre_c = pc;
      s_pre_t = pt;
      if (b == L.nb - 1) {
        L.totals[0] = pc + carry_c;
        L.totals[1] = pt + carry_t;
        if (pt + carry_t > L.tg_cap) atomicOr(L.err, DEV_FLAG_TG_OVF);
      }
    }
  }
  __syncthreads();
  for (uint32_t s = threadIdx.x; s < n; s += NT) {
    const uint32_t ntg = sntg[s];
    if (ntg == ~0u) continue;
    const uint32_t slot = s_pre_c + sexc[s].x, toff = s_pre_t + sexc[s].y;
    if (slot >= L.max_groups) continue;  // only after a timed-out look-back
    const uint32_t i = ord[s];
    const uint32_t m = sm[i];
    double p = __ldg(C.mp + m);
    for (uint32_t s2 = s + 1; s2 < n; ++s2) {
      const uint32_t i2 = ord[s2];
      if (sk[i2].x != sk[i].x || sk[i2].y != sk[i].y) break;
      const double q = __ldg(C.mp + sm[i2]);
      p = p * (1.0 - q) + q * (1.0 - p);
    }
    L.out_prob[slot] = p;
    L.out_off[slot] = toff;
    if (toff + ntg <= L.tg_cap) {
      const uint4 *src = reinterpret_cast<const uint4 *>(C.tl + (size_t)m * tcap);
      for (uint32_t k = 0; k * 4 < ntg; ++k) {
        const uint4 x = __ldg(src + k);
        const uint32_t o = toff + k * 4, rem = ntg - k * 4;
        L.out_tg[o] = x.x;
        if (rem > 1) L.out_tg[o + 1] = x.y;
        if (rem > 2) L.out_tg[o + 2] = x.z;
        if (rem > 3) L.out_tg[o + 3] = x.w;
      }
    }
  }
}

// ---- three-kernel merge -----------------------------------------------------

__global__ void __launch_bounds__(BUCKET_THREADS) group_kernel(GroupLaunch L) {
  constexpr int NT = BUCKET_THREADS;
  constexpr int NW = NT / 32;
  __shared__ ulonglong2 sk[BUCKET_CAP];
  __shared__ uint32_t sm[BUCKET_CAP];
  __shared__ double sp[BUCKET_CAP];
  __shared__ uint16_t ord[BUCKET_CAP];
  __shared__ uint32_t sntg[BUCKET_CAP];  // targets of a group head at a sorted position, else ~0u
  __shared__ uint32_t wc[NW], wt[NW];
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const uint32_t b = blockIdx.x;
  uint32_t n = L.count[b];
  const uint32_t base = L.offset[b];
  if (n > (uint32_t)BUCKET_CAP) {
    if (threadIdx.x == 0) atomicOr(L.err, DEV_FLAG_BIG_BUCKET);
    n = 0;
  }
  for (uint32_t i = threadIdx.x; i < n; i += NT) {
    sk[i] = L.bkey[base + i];
    sm[i] = L.bm[base + i];
    sp[i] = L.bp[base + i];
  }
  __syncthreads();
  // rank sort by (key, m), four comparisons per step
  for (uint32_t i = threadIdx.x; i < n; i += NT) {
    const ulonglong2 ki = sk[i];
    const uint32_t mi = sm[i];
    uint32_t r = 0;
    uint32_t k = 0;
    for (; k + 4 <= n; k += 4) {
      r += item_less(sk[k], sm[k], ki, mi) ? 1u : 0u;
      r += item_less(sk[k + 1], sm[k + 1], ki, mi) ? 1u : 0u;
      r += item_less(sk[k + 2], sm[k + 2], ki, mi) ? 1u : 0u;
      r += item_less(sk[k + 3], sm[k + 3], ki, mi) ? 1u : 0u;
    }
    for (; k < n; ++k) r += item_less(sk[k], sm[k], ki, mi) ? 1u : 0u;
    ord[r] = (uint16_t)i;
  }
  __syncthreads();
  // group heads, collision checks (full target lists), target counts
  const uint32_t tcap = L.tcap;
  for (uint32_t s = threadIdx.x; s < n; s += NT) {
    const uint32_t i = ord[s];
    const uint32_t m = sm[i];
    const uint32_t nt = __ldg(L.tn + m);
    bool head = true;
    if (s > 0) {
      const uint32_t ip = ord[s - 1];
      if (sk[ip].x == sk[i].x && sk[ip].y == sk[i].y) {
        head = false;
        const uint32_t mq = sm[ip];
        if (__ldg(L.tn + mq) != nt || !lists_equal(L.tl + (size_t)m * tcap, L.tl + (size_t)mq * tcap, nt))
          atomicOr(L.err, DEV_ERR_COLLISION);
      }
    }
    sntg[s] = head ? nt : ~0u;
  }
  __syncthreads();
  // compact the heads (block scan over sorted positions, NT at a time) and
  // write one record per group; fold the run's probabilities left to right
  uint32_t carry_c = 0, carry_t = 0;
  for (uint32_t r0 = 0; r0 < n; r0 += NT) {
    const uint32_t s = r0 + threadIdx.x;
    const uint32_t v = s < n ? sntg[s] : ~0u;
    const uint32_t c_in = v != ~0u ? 1u : 0u, t_in = v != ~0u ? v : 0u;
    uint32_t ic = c_in, it = t_in;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t a = __shfl_up_sync(0xFFFFFFFFu, ic, o), bb = __shfl_up_sync(0xFFFFFFFFu, it, o);
      if (lane >= (uint32_t)o) {
        ic += a;
        it += bb;
      }
    }
    if (lane == 31) {
      wc[warp] = ic;
      wt[warp] = it;
    }
    __syncthreads();
    uint32_t pc = carry_c, pt = carry_t;
    for (uint32_t x = 0; x < warp; ++x) {
      pc += wc[x];
      pt += wt[x];
    }
    if (c_in) {
      const uint32_t g = pc + ic - 1;
      const uint32_t i = ord[s];
      double p = sp[i];
      for (uint32_t s2 = s + 1; s2 < n; ++s2) {
        const uint32_t i2 = ord[s2];
        if (sk[i2].x != sk[i].x || sk[i2].y != sk[i].y) break;
        const double q = sp[i2];
        p = p * (1.0 - q) + q * (1.0 - p);
      }
      L.gm[base + g] = sm[i];
      L.gp[base + g] = p;
      L.gt[base + g] = pt + it - t_in;
    }
    for (uint32_t x = 0; x < (uint32_t)NW; ++x) {
      carry_c += wc[x];
      carry_t += wt[x];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) L.bagg[b] = make_uint2(carry_c, carry_t);
}

// Exclusive scan of the nb bucket aggregates (one block of 1024 threads).
__global__ void __launch_bounds__(1024) group_scan_kernel(GroupLaunch L) {
  __shared__ uint32_t pc[1024], pt[1024];
  const uint32_t t = threadIdx.x, nb = L.nb;
  const uint32_t per = (nb + 1023) / 1024;
  const uint32_t lo = min(nb, t * per), hi = min(nb, lo + per);
  uint32_t c = 0, g = 0;
  for (uint32_t i = lo; i < hi; ++i) {
    const uint2 a = L.bagg[i];
    c += a.x;
    g += a.y;
  }
  pc[t] = c;
  pt[t] = g;
  __syncthreads();
  for (uint32_t off = 1; off < 1024; off <<= 1) {
    const uint32_t a = t >= off ? pc[t - off] : 0, b = t >= off ? pt[t - off] : 0;
    __syncthreads();
    pc[t] += a;
    pt[t] += b;
    __syncthreads();
  }
  uint32_t rc = pc[t] - c, rt = pt[t] - g;
  for (uint32_t i = lo; i < hi; ++i) {
    const uint2 a = L.bagg[i];
    L.bout[i] = make_uint2(rc, rt);
    rc += a.x;
    rt += a.y;
  }
  if (t == 1023) {
    L.totals[0] = pc[1023];
    L.totals[1] = pt[1023];
    if (pt[1023] > L.tg_cap) atomicOr(L.err, DEV_FLAG_TG_OVF);
  }
  __syncthreads();  // bout written by the whole block
  for (uint32_t c = t; c < L.n_circ; c += 1024) L.cout[c] = L.bout[L.cbbase[c]];
}

__global__ void __launch_bounds__(BUCKET_THREADS) emit_kernel(GroupLaunch L) {
  const uint32_t b = blockIdx.x;
  const uint2 agg = L.bagg[b], out = L.bout[b];
  const uint32_t base = L.offset[b];
  const uint32_t tcap = L.tcap;
  for (uint32_t g = threadIdx.x; g < agg.x; g += BUCKET_THREADS) {
    const uint32_t slot = out.x + g;
    const uint32_t toff = out.y + L.gt[base + g];
    const uint32_t m = L.gm[base + g];
    L.out_prob[slot] = L.gp[base + g];
    L.out_off[slot] = toff;
    const uint32_t ntg = __ldg(L.tn + m);
    if (toff + ntg <= L.tg_cap) {
      const uint4 *src = reinterpret_cast<const uint4 *>(L.tl + (size_t)m * tcap);
      for (uint32_t k = 0; k * 4 < ntg; ++k) {
        const uint4 x = __ldg(src + k);
        const uint32_t o = toff + k * 4, rem = ntg - k * 4;
        L.out_tg[o] = x.x;
        if (rem > 1) L.out_tg[o + 1] = x.y;
        if (rem > 2) L.out_tg[o + 2] = x.z;
        if (rem > 3) L.out_tg[o + 3] = x.w;
      }
    }
  }
}

}  // namespace

cudaError_t launch_keys(const KeyLaunch &L, cudaStream_t s) {
  if (L.M == 0) return cudaSuccess;
  const uint32_t threads = 256;
  const uint32_t blocks = (L.M + threads - 1) / threads;
  key_kernel<<<blocks, threads, 0, s>>>(L);
  return cudaGetLastError();
}

cudaError_t launch_bucket_scan(const uint32_t *count, uint32_t *offset, uint32_t nb, cudaStream_t s) {
  bucket_scan_kernel<<<1, 1024, 0, s>>>(count, offset, nb);
  return cudaGetLastError();
}

cudaError_t launch_bucket_scatter(const ulonglong2 *key, uint32_t M, uint32_t bucket_bits, const uint32_t *offset,
                                  uint32_t *cursor, ulonglong2 *bkey, uint32_t *bm, cudaStream_t s) {
  if (M == 0) return cudaSuccess;
  uint32_t blocks = (M + 255) / 256;
  if (blocks > 152u * 16u) blocks = 152u * 16u;
  bucket_scatter_kernel<<<blocks, 256, 0, s>>>(key, M, 64u - bucket_bits, offset, cursor, bkey, bm);
  return cudaGetLastError();
}

cudaError_t launch_bucket_scatter_p(const CircuitDev *circs, const uint32_t *mbase, uint32_t n_circ,
                                    const ulonglong2 *key, const double *mp, uint32_t M, const uint32_t *offset,
                                    uint32_t *cursor, ulonglong2 *bkey, uint32_t *bm, double *bp, cudaStream_t s) {
  if (M == 0) return cudaSuccess;
  uint32_t blocks = (M + 255) / 256;
  if (blocks > 152u * 16u) blocks = 152u * 16u;
  bucket_scatter_p_kernel<<<blocks, 256, 0, s>>>(circs, mbase, n_circ, key, mp, M, offset, cursor, bkey, bm, bp);
  return cudaGetLastError();
}

cudaError_t launch_group_merge(const GroupLaunch &L, cudaStream_t s) {
  if (L.nb == 0) return cudaSuccess;
  group_kernel<<<L.nb, BUCKET_THREADS, 0, s>>>(L);
  group_scan_kernel<<<1, 1024, 0, s>>>(L);
  emit_kernel<<<L.nb, BUCKET_THREADS, 0, s>>>(L);
  return cudaGetLastError();
}

cudaError_t launch_bucket_merge(const BucketMergeLaunch &L, cudaStream_t s) {
  if (L.nb == 0) return cudaSuccess;
  bucket_merge_kernel<<<L.nb, BUCKET_THREADS, (size_t)L.w * sizeof(uint2), s>>>(L);
  return cudaGetLastError();
}

cudaError_t launch_sort_init(const ulonglong2 *key, uint64_t *sortkey, uint32_t *perm, uint32_t M, cudaStream_t s) {
  if (M == 0) return cudaSuccess;
  uint32_t blocks = (M + 255) / 256;
  if (blocks > 152u * 16u) blocks = 152u * 16u;
  sort_init_kernel<<<blocks, 256, 0, s>>>(key, sortkey, perm, M);
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
