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
//    right with p <- p(1-q) + q(1-p) (CUDAHandlers.hpp:124-139) in FP64,
//    extract their targets and get an output slot from a block scan plus a
//    warp-wide decoupled look-back over the preceding buckets.  The empty
//    symptom is dropped (Driver.hpp:185).
//  * global path, used when a bucket exceeds one CTA (a symptom repeated
//    more than BUCKET_CAP times): LSD onesweep radix sort of all keys (one
//    kernel per 8-bit digit, tile ranks by warp match/popc, decoupled
//    look-back for digit offsets) and a merge kernel over the sorted run.
#include <cstdint>

#include "device.cuh"
#include "lower.hpp"

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
#undef PP

// Thread per key block: the record holding the block's first mechanism, the
// block's circuit, and whether the block spans more than one circuit.
__global__ void key_prep_kernel(KeyLaunch L) {
  const uint32_t blk = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t m0 = blk * KEY_THREADS;
  if (m0 >= L.M) return;
  const uint32_t c = find_circuit(L.mbase, L.n_circ, m0);
  const uint32_t c1 = find_circuit(L.mbase, L.n_circ, min(L.M - 1, m0 + KEY_THREADS - 1));
  const CircuitDev &C = L.circs[c];
  const uint32_t m = m0 - L.mbase[c];
  uint32_t lo = 0, hi = C.R;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (__ldg(C.rec_moff + mid) <= m) lo = mid;
    else hi = mid;
  }
  L.blk_info[blk] = make_uint2(lo, c | (c1 != c ? 0x80000000u : 0u));
}

// One thread per mechanism (global numbering over the batch).  Writes the
// mechanism's descriptor, probability, 128-bit key, target list, and its item
// into a slot of its bucket.  The symptom's words are the words set in the
// non-zero masks of the mechanism's points (ascending); a block inside one
// circuit finds its mechanisms' records in shared memory.
__global__ void __launch_bounds__(KEY_THREADS, 5) key_kernel(KeyLaunch L) {
  __shared__ uint32_t srm[KEY_THREADS + 1];  // rec_moff of the block's records
  __shared__ uint8_t sown[KEY_THREADS];      // record (from r0) of each of the block's mechanisms
  __shared__ uint32_t stg[8][KEY_THREADS];   // each thread's first eight targets ([slot][thread]: no bank conflicts)
  const uint32_t tid = threadIdx.x, lane = tid & 31u;
  const uint32_t m0 = blockIdx.x * KEY_THREADS;
  const uint32_t mg = m0 + tid;
  const uint2 info = L.blk_info[blockIdx.x];
  const uint32_t r0 = info.x, c0 = info.y & 0x7FFFFFFFu;
  const bool one = (info.y >> 31) == 0;
  // every record holds at least one mechanism, so the block's records are r0 .. r0 + KEY_THREADS - 1
  const uint32_t nr = one ? min(KEY_THREADS, L.circs[c0].R - r0) : 0;
  if (one) {
    for (uint32_t k = tid; k <= nr; k += KEY_THREADS) srm[k] = __ldg(L.circs[c0].rec_moff + r0 + k);
    __syncthreads();
    // each record marks its mechanisms inside the block (at most 15), so a
    // mechanism finds its record with one shared load instead of a search
    const uint32_t mb0 = m0 - __ldg(L.mbase + c0);  // the block's first mechanism within its circuit
    for (uint32_t k = tid; k < nr; k += KEY_THREADS) {
      const uint32_t a = max(srm[k], mb0), b = min(srm[k + 1], mb0 + KEY_THREADS);
      for (uint32_t j = a; j < b; ++j) sown[j - mb0] = (uint8_t)k;
    }
  }
  __syncthreads();
  if (mg >= L.M) return;

  const uint32_t c = one ? c0 : find_circuit(L.mbase, L.n_circ, mg);
  const CircuitDev &C = L.circs[c];
  const uint32_t m = mg - __ldg(L.mbase + c);
  uint32_t r;
  if (one) {
    r = r0 + sown[tid];
  } else {
    uint32_t lo = 0, hi = C.R;
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (__ldg(C.rec_moff + mid) <= m) lo = mid;
      else hi = mid;
    }
    r = lo;
  }
  const uint64_t d = __ldg(C.rec + r);
  const uint32_t ci = m - (one ? srm[r - r0] : __ldg(C.rec_moff + r));
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
  const double prob = __ldg(C.rec_p + r);
  const bool split = L.late_word != kNoSplit;
  if (L.write_all || split) {  // descriptors and probabilities: global merge path, gradients, second pass
    C.mdesc[m] = mk_desc(pa, Pa, pb, Pb);
    C.mp[m] = prob;
  }

  const uint32_t tcap = C.tcap;
  uint64_t hx = 0, hy = 0;
  uint32_t cnt = 0;
  bool nonzero = false;
  uint32_t *out = C.tl + (size_t)m * tcap;
  // the first eight targets are staged in shared memory and leave as two
  // 16-byte stores (a row per thread: one scattered store per target would
  // cost an L2 transaction each); later ones are stored as they come
  auto put = [&](uint32_t c, uint32_t v) {
    if (c < 8) stg[c][tid] = v;
    else if (c < tcap) out[c] = v;
  };
  const ulonglong2 *snap = C.snap;
  const uint32_t np = C.npoints, mw = C.mw;
  const unsigned long long *ma = C.nzm + (size_t)pa * mw, *mb = C.nzm + (size_t)pb * mw;
  const uint32_t jend = split ? L.late_word : mw * 64u;  // words of this pass: j < jend
  for (uint32_t i = 0; i < mw && i * 64u < jend; ++i) {
    // a point's snapshot of word j exists only where its own bit is set
    const uint64_t ba = __ldg(ma + i), bb = Pb ? __ldg(mb + i) : 0ull;
    uint64_t bits = ba | bb;
    if (jend - i * 64u < 64u) bits &= (1ull << (jend - i * 64u)) - 1ull;
    while (bits) {
      const uint32_t bit = (uint32_t)(__ffsll((long long)bits) - 1);
      const uint32_t j = i * 64u + bit;
      bits &= bits - 1;
      const ulonglong2 *sj = snap + (size_t)j * np;
      uint64_t v = 0;
      if ((ba >> bit) & 1ull) v = pauli_sel(sj[pa], Pa);
      if ((bb >> bit) & 1ull) v ^= pauli_sel(sj[pb], Pb);
      if (!v) continue;
      nonzero = true;
      const ulonglong2 h = word_hash(j, v);
      hx ^= h.x;
      hy ^= h.y;
      if (tcap) {
        uint64_t x = v;
        while (x) {
          put(cnt, j * 64u + (uint32_t)(__ffsll((long long)x) - 1));
          ++cnt;
          x &= x - 1;
        }
      }
    }
  }
  const ulonglong2 key = make_ulonglong2(hx, hy);
  if (L.write_all || split) L.key[mg] = key;  // a split pass leaves the partial key
  if (tcap) {
    // rows are 16-byte aligned (tcap is a multiple of 4, at least 32)
    // (both halves even for four targets or fewer: a whole 32-byte sector per row; entries past
    // the count are never read)
    if (cnt) {
      reinterpret_cast<uint4 *>(out)[0] = make_uint4(stg[0][tid], stg[1][tid], stg[2][tid], stg[3][tid]);
      reinterpret_cast<uint4 *>(out)[1] = make_uint4(stg[4][tid], stg[5][tid], stg[6][tid], stg[7][tid]);
    }
    C.tn[m] = cnt;
    if (cnt > tcap) atomicOr(L.err, DEV_FLAG_LONG);
    const uint32_t am = __activemask();
    const uint32_t tot = __reduce_add_sync(am, cnt);
    if (lane == (uint32_t)(__ffs(am) - 1) && tot) red_add(L.list_total, tot);
  }
  if (split) return;  // filed in its bucket by the second pass
  if ((hx | hy) == 0) {
    if (cnt || (!tcap && nonzero)) atomicOr(L.err, DEV_ERR_COLLISION);  // a non-empty symptom hashed to 0
  } else {
    const uint32_t b = C.bbase + (uint32_t)(hx >> (64u - C.bbits));
    const uint32_t slot = atomicAdd(L.bucket_count + b, 1u);
    if (slot < SLOT_CAP) {
      const size_t pos = (size_t)b * SLOT_CAP + slot;
      L.slot[pos] = Slot{key, SlotTail{mg, cnt, prob}};
    } else {
      atomicOr(L.err, DEV_FLAG_BIG_BUCKET);
    }
  }
}

// Second pass of a split key pass (one circuit, target lists on): adds the
// words from late_word on to each mechanism's partial key, appends their
// targets after the first pass's (they are the larger indices, so the list
// stays ascending), and files the mechanism in its bucket.
__global__ void __launch_bounds__(KEY_THREADS) key_late_kernel(KeyLaunch L) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t m = blockIdx.x * KEY_THREADS + threadIdx.x;
  if (m >= L.M) return;
  const CircuitDev &C = L.circs[0];
  const uint64_t d = C.mdesc[m];
  const uint32_t pa = (uint32_t)(d & 0x3FFFFFFFu), Pa = (uint32_t)((d >> 30) & 3u);
  const uint32_t pb = (uint32_t)((d >> 32) & 0x3FFFFFFFu), Pb = (uint32_t)(d >> 62);
  const double prob = C.mp[m];
  ulonglong2 key = L.key[m];
  const uint32_t tcap = C.tcap;
  uint32_t *out = C.tl + (size_t)m * tcap;
  const uint32_t cnt1 = C.tn[m];
  uint32_t cnt = cnt1;
  const ulonglong2 *snap = C.snap;
  const uint32_t np = C.npoints, mw = C.mw, jbeg = L.late_word;
  const unsigned long long *ma = C.nzm + (size_t)pa * mw, *mb = C.nzm + (size_t)pb * mw;
  for (uint32_t i = jbeg / 64u; i < mw; ++i) {
    const uint64_t ba = __ldg(ma + i), bb = Pb ? __ldg(mb + i) : 0ull;
    uint64_t bits = ba | bb;
    if (jbeg > i * 64u) bits &= ~((1ull << (jbeg - i * 64u)) - 1ull);
    while (bits) {
      const uint32_t bit = (uint32_t)(__ffsll((long long)bits) - 1);
      const uint32_t j = i * 64u + bit;
      bits &= bits - 1;
      const ulonglong2 *sj = snap + (size_t)j * np;
      uint64_t v = 0;
      if ((ba >> bit) & 1ull) v = pauli_sel(sj[pa], Pa);
      if ((bb >> bit) & 1ull) v ^= pauli_sel(sj[pb], Pb);
      if (!v) continue;
      const ulonglong2 h = word_hash(j, v);
      key.x ^= h.x;
      key.y ^= h.y;
      for (uint64_t x = v; x; x &= x - 1) {
        if (cnt < tcap) out[cnt] = j * 64u + (uint32_t)(__ffsll((long long)x) - 1);
        ++cnt;
      }
    }
  }
  if (L.write_all) L.key[m] = key;
  if (cnt != cnt1) C.tn[m] = cnt;
  if (cnt > tcap) atomicOr(L.err, DEV_FLAG_LONG);
  const uint32_t am = __activemask();
  const uint32_t tot = __reduce_add_sync(am, cnt - cnt1);
  if (lane == (uint32_t)(__ffs(am) - 1) && tot) red_add(L.list_total, tot);
  if ((key.x | key.y) == 0) {
    if (cnt) atomicOr(L.err, DEV_ERR_COLLISION);  // a non-empty symptom hashed to 0
  } else {
    const uint32_t b = C.bbase + (uint32_t)(key.x >> (64u - C.bbits));
    const uint32_t slot = atomicAdd(L.bucket_count + b, 1u);
    if (slot < SLOT_CAP) {
      const size_t pos = (size_t)b * SLOT_CAP + slot;
      L.slot[pos] = Slot{key, SlotTail{m, cnt, prob}};
    } else {
      atomicOr(L.err, DEV_FLAG_BIG_BUCKET);
    }
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
    uint32_t *__restrict__ status, uint32_t *__restrict__ tile_ctr, uint32_t *__restrict__ err,
    unsigned long long spin_ns, uint32_t hold_tile0) {
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
      if (!hold_tile0) st[d] = ST_PREFIX | sum;  // (held: a test of the waits below)
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
          else if (globaltimer() - t0 > spin_ns) {
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
    out[i] = perm[i] < n ? key[perm[i]].y : 0ull;  // (an index past n: a sort pass timed out)
}

// ---- merge ------------------------------------------------------------------

constexpr unsigned long long MS_AGG = 1ull << 62;
constexpr unsigned long long MS_PREFIX = 2ull << 62;

__device__ __forceinline__ unsigned long long ms_pack(uint32_t cnt, uint32_t tg) {
  return ((unsigned long long)(cnt & 0x3FFFFFFFu) << 32) | tg;
}

// Mask word i of the words where mechanism d's symptom can be non-zero: the
// union of its points' non-zero masks (a word whose mask bit is clear has a
// zero snapshot at that point, so it adds nothing to the symptom).
__device__ __forceinline__ uint64_t symptom_mask(const CircuitDev &C, uint64_t d, uint32_t i) {
  const uint32_t pa = (uint32_t)(d & 0x3FFFFFFFu), Pa = (uint32_t)((d >> 30) & 3u);
  const uint32_t pb = (uint32_t)((d >> 32) & 0x3FFFFFFFu), Pb = (uint32_t)(d >> 62);
  uint64_t b = 0;
  if (Pa) b |= __ldg(C.nzm + (size_t)pa * C.mw + i);
  if (Pb) b |= __ldg(C.nzm + (size_t)pb * C.mw + i);
  return b;
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
  // After a sort pass timed out (DEV_ERR_TIMEOUT, the compile fails) the
  // permutation may hold stale entries: an index past n is never followed.
  m = i < n ? L.perm[i] : 0u;
  if (i < n && m >= n) {
    atomicOr(L.err, DEV_ERR_TIMEOUT);
    m = 0;
  } else if (i < n) {
    k = L.key[m];
    const uint64_t d = __ldg(C.mdesc + m);
    bool newgroup = true;
    const uint32_t mp = i > 0 ? L.perm[i - 1] : 0u;
    if (i > 0 && mp < n) {
      const ulonglong2 kp = L.key[mp];
      if (kp.x == k.x && kp.y == k.y) {
        newgroup = false;
        const uint64_t dp = __ldg(C.mdesc + mp);
        // the full symptoms, compared on the words either can be non-zero in
        bool diff = false;
        for (uint32_t mi = 0; mi < C.mw && !diff; ++mi)
          for (uint64_t bits = symptom_mask(C, d, mi) | symptom_mask(C, dp, mi); bits && !diff; bits &= bits - 1) {
            const uint32_t j = mi * 64u + (uint32_t)(__ffsll((long long)bits) - 1);
            diff = j < w && symptom_word(C, d, j, sband[j]) != symptom_word(C, dp, j, sband[j]);
          }
        if (diff) atomicOr(L.err, DEV_ERR_COLLISION);
      } else if (((L.sortkey[i] ^ L.sortkey[i - 1]) & L.sort_mask) == 0 && L.sort_mask) {
        atomicOr(L.err, DEV_FLAG_MIXED);
      }
    }
    const bool empty = (k.x | k.y) == 0;
    if (newgroup) {
      // a non-empty symptom hashed to zero is a collision; a head counts its targets
      bool nonzero = false;
      for (uint32_t mi = 0; mi < C.mw; ++mi)
        for (uint64_t bits = symptom_mask(C, d, mi); bits; bits &= bits - 1) {
          const uint32_t j = mi * 64u + (uint32_t)(__ffsll((long long)bits) - 1);
          const uint32_t c = j < w ? __popcll(symptom_word(C, d, j, sband[j])) : 0u;
          nonzero |= c != 0;
          ntg += c;
        }
      if (empty && nonzero) atomicOr(L.err, DEV_ERR_COLLISION);
    }
    head = newgroup && !empty;
    if (!head) ntg = 0;
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
          else if (globaltimer() - t0 > L.spin_ns) {
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
    if (m2 >= n) break;  // stale entry after a timed-out sort pass
    const ulonglong2 k2 = L.key[m2];
    if (k2.x != k.x || k2.y != k.y) break;
    const double q = __ldg(C.mp + m2);
    p = p * (1.0 - q) + q * (1.0 - p);
  }
  L.out_prob[slot] = p;
  L.out_off[slot] = toff;
  if ((uint64_t)toff + ntg <= L.tg_cap) {
    const uint64_t d = __ldg(C.mdesc + m);
    uint32_t o = toff;
    for (uint32_t mi = 0; mi < C.mw; ++mi)  // the masked words, ascending: the targets stay ascending
      for (uint64_t bits = symptom_mask(C, d, mi); bits; bits &= bits - 1) {
        const uint32_t j = mi * 64u + (uint32_t)(__ffsll((long long)bits) - 1);
        uint64_t v = j < w ? symptom_word(C, d, j, sband[j]) : 0ull;
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
  // A caller's list longer than the stride was reported (and cut to the
  // stride) by the key pass; every read of a count here is cut the same way,
  // so no list is read past its row.
  const uint32_t tcap = C.tcap;
  for (uint32_t s = threadIdx.x; s < n; s += NT) {
    const uint32_t i = ord[s];
    const uint32_t m = sm[i];
    const uint32_t nt = min(__ldg(C.tn + m), tcap);
    bool head = true;
    if (s > 0) {
      const uint32_t ip = ord[s - 1];
      if (sk[ip].x == sk[i].x && sk[ip].y == sk[i].y) {
        head = false;
        const uint32_t mq = sm[ip];
        if (min(__ldg(C.tn + mq), tcap) != nt ||
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
        if ((uint64_t)pt + carry_t > L.tg_cap) atomicOr(L.err, DEV_FLAG_TG_OVF);
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
    if ((uint64_t)toff + ntg <= L.tg_cap) {
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

// ---- merge of the compile pipeline ---------------------------------------

constexpr uint32_t GW_WARPS = 8;  // buckets per group/emit block (one warp each)

__device__ __forceinline__ bool key_eq(ulonglong2 a, ulonglong2 b) { return a.x == b.x && a.y == b.y; }

// a(1-b) + b(1-a), written as a + b(1-2a): two fused multiply-adds.
__device__ __forceinline__ double xor_merge(double a, double b) { return fma(b, fma(-2.0, a, 1.0), a); }

// One warp per bucket of at most WARP_CAP items; larger buckets are listed
// for group_big_kernel.  Items are ordered by sub-bin (top 6 bits of the
// key's second half), then by (key, m) inside the sub-bin: equal keys end up
// adjacent in ascending mechanism order, at O(n) work per bucket.
__global__ void __launch_bounds__(GW_WARPS * 32) group_warp_kernel(GroupLaunch L) {
  constexpr uint32_t NBIN = 64;
  __shared__ ulonglong2 s_k[GW_WARPS][WARP_CAP];
  __shared__ uint32_t s_m[GW_WARPS][WARP_CAP];
  __shared__ double s_p[GW_WARPS][WARP_CAP];
  __shared__ uint32_t s_t[GW_WARPS][WARP_CAP];
  __shared__ uint8_t s_o[GW_WARPS][WARP_CAP];   // sorted position -> item
  __shared__ uint8_t s_q[GW_WARPS][WARP_CAP];   // item -> place inside its sub-bin (arrival order)
  __shared__ uint8_t s_x[GW_WARPS][WARP_CAP];   // items grouped by sub-bin
  __shared__ uint32_t s_h[GW_WARPS][NBIN];      // sub-bin counts, then offsets
  const uint32_t lane = threadIdx.x & 31u, wi = threadIdx.x >> 5;
  const uint32_t b = blockIdx.x * GW_WARPS + wi;
  if (b >= L.nb) return;
  const uint32_t n = L.count[b];
  if (n == 0) {
    if (lane == 0) L.bagg[b] = make_uint2(0, 0);
    return;
  }
  if (n > WARP_CAP) {
    if (lane == 0) {
      if (n > SLOT_CAP) {
        atomicOr(L.err, DEV_FLAG_BIG_BUCKET);  // slots overflowed; the run is redone another way
        L.bagg[b] = make_uint2(0, 0);
      } else {
        L.big_list[atomicAdd(L.big_n, 1u)] = b;
      }
    }
    return;
  }
  ulonglong2 *K = s_k[wi];
  uint32_t *Mm = s_m[wi], *T = s_t[wi], *H = s_h[wi];
  double *P = s_p[wi];
  uint8_t *O = s_o[wi], *Q = s_q[wi], *X = s_x[wi];
  const size_t base = (size_t)b * SLOT_CAP;
  H[lane] = 0;
  H[lane + 32] = 0;
  __syncwarp();
  for (uint32_t i = lane; i < n; i += 32) {
    const Slot sl = L.slot[base + i];
    const ulonglong2 k = sl.key;
    const SlotTail t = sl.tail;
    K[i] = k;
    Mm[i] = t.m;
    T[i] = t.t;
    P[i] = t.p;
    Q[i] = (uint8_t)atomicAdd(H + (uint32_t)(k.y >> 58), 1u);
  }
  __syncwarp();
  {  // sub-bin offsets: lane owns bins 2*lane and 2*lane + 1
    const uint32_t c0 = H[2 * lane], c1 = H[2 * lane + 1];
    uint32_t inc = c0 + c1;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t a = __shfl_up_sync(0xFFFFFFFFu, inc, o);
      if (lane >= (uint32_t)o) inc += a;
    }
    const uint32_t ex = inc - c0 - c1;
    __syncwarp();
    H[2 * lane] = ex;
    H[2 * lane + 1] = ex + c0;
  }
  __syncwarp();
  for (uint32_t i = lane; i < n; i += 32) X[H[(uint32_t)(K[i].y >> 58)] + Q[i]] = (uint8_t)i;
  __syncwarp();
  for (uint32_t i = lane; i < n; i += 32) {
    const ulonglong2 ki = K[i];
    const uint32_t mi = Mm[i];
    const uint32_t bin = (uint32_t)(ki.y >> 58);
    const uint32_t lo = H[bin], hi = bin + 1 < NBIN ? H[bin + 1] : n;
    uint32_t r = lo;
    for (uint32_t j = lo; j < hi; ++j) {
      const uint32_t x = X[j];
      r += item_less(K[x], Mm[x], ki, mi) ? 1u : 0u;
    }
    O[r] = (uint8_t)i;
  }
  __syncwarp();
  // the saved permutation for the adjoint: mechanism at each sorted position
  // (every key of this bucket is in shared memory already)
  Slot *const bslot = L.slot + base;
  for (uint32_t s = lane; s < n; s += 32) slot_perm(bslot, s)[0] = Mm[O[s]];
  // Groups, 32 sorted positions at a time.  Each group's probability is a
  // segmented inclusive scan of the XOR-merge over its run: log2(longest run
  // in the chunk) shuffle steps with every lane busy (FP64 throughput is
  // scarce on this part), plus the value carried in from the previous chunk.
  // The scan is a tree, so its rounding differs from a left-to-right fold by
  // a few ulps; it is deterministic.
  const uint32_t tcap = L.tcap;
  uint32_t gcount = 0, tcount = 0;
  uint32_t carry_head = 0;  // item of the run open at the end of the previous chunk
  double carry = 0.0;
  for (uint32_t s0 = 0; s0 < n; s0 += 32) {
    const uint32_t s = s0 + lane;
    const bool in = s < n;
    bool head = false;
    uint32_t i = 0, nt = 0;
    if (in) {
      i = O[s];
      nt = T[i];
      head = s == 0 || !key_eq(K[O[s - 1]], K[i]);
    }
    const uint32_t hb = __ballot_sync(0xFFFFFFFFu, head);
    {
      // collision check: every item of a run against the run's head (full target lists)
      const uint32_t le0 = hb & (0xFFFFFFFFu >> (31u - lane));
      const uint32_t ih = le0 ? (uint32_t)O[s0 + 31 - __clz(le0)] : carry_head;
      // (a list longer than the stride holds only its first tcap targets; the
      // key pass flagged it and the run is redone with wider lists)
      if (in && !head && nt <= tcap &&
          (T[ih] != nt || !lists_equal(L.tl + (size_t)Mm[i] * tcap, L.tl + (size_t)Mm[ih] * tcap, nt)))
        atomicOr(L.err, DEV_ERR_COLLISION);
      carry_head = __shfl_sync(0xFFFFFFFFu, ih, 31);
    }
    const uint32_t tv = head ? nt : 0u;
    uint32_t inc = tv;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t a = __shfl_up_sync(0xFFFFFFFFu, inc, o);
      if (lane >= (uint32_t)o) inc += a;
    }
    // the run of each position: it starts at lane `seg` of this chunk, or
    // (seg < 0) continues the run open at the end of the previous chunk
    const uint32_t le = hb & (0xFFFFFFFFu >> (31u - lane));
    const int seg = le ? 31 - __clz(le) : -1;
    const uint32_t seg0 = seg < 0 ? 0u : (uint32_t)seg;
    double x = in ? P[i] : 0.0;
    const uint32_t maxlen = __reduce_max_sync(0xFFFFFFFFu, in ? lane - seg0 + 1 : 0u);
    for (uint32_t d = 1; d < maxlen; d <<= 1) {
      const double y = __shfl_up_sync(0xFFFFFFFFu, x, d);
      if (lane >= d && lane - d >= seg0) x = xor_merge(y, x);
    }
    if (seg < 0) x = xor_merge(carry, x);
    const uint32_t gh = gcount + __popc(hb & ((1u << lane) - 1u));  // group of a head at this lane
    // every slot of this bucket was read into shared memory above
    if (head) {
      bslot[gh].tail.m = Mm[i];
      bslot[gh].tail.t = tcount + inc - tv;
      slot_perm(bslot, gh)[1] = s;
    }
    if (in && (s + 1 >= n || !key_eq(K[O[s + 1]], K[i]))) {  // the run's last item holds its value
      const uint32_t g = seg < 0 ? gcount - 1u : gcount + __popc(hb & ((1u << seg0) - 1u));
      bslot[g].tail.p = x;
    }
    carry = __shfl_sync(0xFFFFFFFFu, x, 31);
    gcount += __popc(hb);
    tcount += __shfl_sync(0xFFFFFFFFu, inc, 31);
  }
  if (lane == 0) {
    L.bagg[b] = make_uint2(gcount, tcount);
    red_add(&L.tsum[b / SCAN_TILE].x, gcount);
    red_add(&L.tsum[b / SCAN_TILE].y, tcount);
    red_add(L.totals + 3, n);
  }
}

// One CTA per listed bucket (WARP_CAP < items <= SLOT_CAP), persistent over
// the list; one thread per slot.  Same order and arithmetic as
// group_warp_kernel: sub-bin counting sort, rank inside a sub-bin, then each
// warp takes 32 sorted positions (heads, target offsets, segmented scan of
// the XOR-merge) and one thread chains the runs across the warps' chunks.
constexpr uint32_t GB_THREADS = SLOT_CAP;
__global__ void __launch_bounds__(GB_THREADS) group_big_kernel(GroupLaunch L) {
  constexpr uint32_t NBIN = 64, NWARP = GB_THREADS / 32;
  __shared__ ulonglong2 sk[SLOT_CAP];
  __shared__ uint32_t sm[SLOT_CAP], st[SLOT_CAP];
  __shared__ double sp[SLOT_CAP];
  __shared__ uint16_t ord[SLOT_CAP], sx[SLOT_CAP];
  __shared__ uint8_t sq[SLOT_CAP];
  __shared__ uint32_t sh[NBIN];
  __shared__ uint32_t c_groups[NWARP], c_targets[NWARP], c_head[NWARP], c_gbase[NWARP], c_tbase[NWARP];
  __shared__ double c_tail[NWARP], c_carry[NWARP];
  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  const uint32_t nbig = *L.big_n;
  const uint32_t tcap = L.tcap;
  for (uint32_t kb = blockIdx.x; kb < nbig; kb += gridDim.x) {
    const uint32_t b = L.big_list[kb];
    const uint32_t n = L.count[b];  // WARP_CAP < n <= SLOT_CAP
    const size_t base = (size_t)b * SLOT_CAP;
    if (tid < NBIN) sh[tid] = 0;
    __syncthreads();
    if (tid < n) {
      const Slot sl = L.slot[base + tid];
      const ulonglong2 k = sl.key;
      const SlotTail t = sl.tail;
      sk[tid] = k;
      sm[tid] = t.m;
      st[tid] = t.t;
      sp[tid] = t.p;
      sq[tid] = (uint8_t)atomicAdd(sh + (uint32_t)(k.y >> 58), 1u);
    }
    __syncthreads();
    if (warp == 0) {
      const uint32_t c0 = sh[2 * lane], c1 = sh[2 * lane + 1];
      uint32_t inc = c0 + c1;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t a = __shfl_up_sync(0xFFFFFFFFu, inc, o);
        if (lane >= (uint32_t)o) inc += a;
      }
      const uint32_t ex = inc - c0 - c1;
      __syncwarp();
      sh[2 * lane] = ex;
      sh[2 * lane + 1] = ex + c0;
    }
    __syncthreads();
    if (tid < n) sx[sh[(uint32_t)(sk[tid].y >> 58)] + sq[tid]] = (uint16_t)tid;
    __syncthreads();
    if (tid < n) {
      const ulonglong2 ki = sk[tid];
      const uint32_t mi = sm[tid];
      const uint32_t bin = (uint32_t)(ki.y >> 58);
      const uint32_t lo = sh[bin], hi = bin + 1 < NBIN ? sh[bin + 1] : n;
      uint32_t r = lo;
      for (uint32_t j = lo; j < hi; ++j) {
        const uint32_t x = sx[j];
        r += item_less(sk[x], sm[x], ki, mi) ? 1u : 0u;
      }
      ord[r] = (uint16_t)tid;
    }
    __syncthreads();
    // position s = tid: heads, collisions, per-chunk scans
    const uint32_t s = tid;
    const bool in = s < n;
    bool head = false;
    uint32_t i = 0, nt = 0;
    if (in) {
      i = ord[s];
      nt = st[i];
      head = true;
      if (s > 0) {
        const uint32_t ip = ord[s - 1];
        if (key_eq(sk[ip], sk[i])) {
          head = false;
          // (lists longer than the stride: flagged by the key pass, redone wider)
          if (nt <= tcap && (st[ip] != nt || !lists_equal(L.tl + (size_t)sm[i] * tcap, L.tl + (size_t)sm[ip] * tcap, nt)))
            atomicOr(L.err, DEV_ERR_COLLISION);
        }
      }
    }
    const uint32_t hb = __ballot_sync(0xFFFFFFFFu, head);
    const uint32_t tv = head ? nt : 0u;
    uint32_t inc = tv;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t a = __shfl_up_sync(0xFFFFFFFFu, inc, o);
      if (lane >= (uint32_t)o) inc += a;
    }
    const uint32_t le = hb & (0xFFFFFFFFu >> (31u - lane));
    const int seg = le ? 31 - __clz(le) : -1;
    const uint32_t seg0 = seg < 0 ? 0u : (uint32_t)seg;
    double x = in ? sp[i] : 0.0;
    const uint32_t maxlen = __reduce_max_sync(0xFFFFFFFFu, in ? lane - seg0 + 1 : 0u);
    for (uint32_t d = 1; d < maxlen; d <<= 1) {
      const double y = __shfl_up_sync(0xFFFFFFFFu, x, d);
      if (lane >= d && lane - d >= seg0) x = xor_merge(y, x);
    }
    if (lane == 31) {
      c_groups[warp] = __popc(hb);
      c_targets[warp] = inc;
      c_head[warp] = hb != 0u;
      c_tail[warp] = x;
    }
    __syncthreads();
    if (tid == 0) {  // chain the chunks: group/target bases and the run carried into each chunk
      uint32_t g = 0, t = 0;
      double run = 0.0;
      for (uint32_t c = 0; c < NWARP; ++c) {
        c_gbase[c] = g;
        c_tbase[c] = t;
        c_carry[c] = run;
        g += c_groups[c];
        t += c_targets[c];
        run = c_head[c] ? c_tail[c] : xor_merge(run, c_tail[c]);
      }
      L.bagg[b] = make_uint2(g, t);
      red_add(&L.tsum[b / SCAN_TILE].x, g);
      red_add(&L.tsum[b / SCAN_TILE].y, t);
      red_add(L.totals + 3, n);
    }
    __syncthreads();
    if (seg < 0) x = xor_merge(c_carry[warp], x);
    const uint32_t gb = c_gbase[warp];
    Slot *const bslot = L.slot + base;
    if (in) slot_perm(bslot, s)[0] = sm[i];
    if (head) {
      const uint32_t g = gb + __popc(hb & ((1u << lane) - 1u));
      bslot[g].tail.m = sm[i];
      bslot[g].tail.t = c_tbase[warp] + inc - tv;
      slot_perm(bslot, g)[1] = s;
    }
    if (in && (s + 1 >= n || !key_eq(sk[ord[s + 1]], sk[i]))) {
      const uint32_t g = seg < 0 ? gb - 1u : gb + __popc(hb & ((1u << seg0) - 1u));
      bslot[g].tail.p = x;
    }
    __syncthreads();
  }
}

// Block sum of a pair over 1024 threads (result in every thread).
__device__ __forceinline__ uint2 block_sum1024(uint2 v, uint2 *scratch) {
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  v.x = __reduce_add_sync(0xFFFFFFFFu, v.x);
  v.y = __reduce_add_sync(0xFFFFFFFFu, v.y);
  if (lane == 0) scratch[warp] = v;
  __syncthreads();
  uint2 a = lane < 32 ? scratch[lane] : make_uint2(0, 0);
  a.x = __reduce_add_sync(0xFFFFFFFFu, a.x);
  a.y = __reduce_add_sync(0xFFFFFFFFu, a.y);
  __syncthreads();
  return a;
}

// Exclusive scan of the bucket aggregates: block t covers buckets
// [t * SCAN_TILE, (t + 1) * SCAN_TILE) and starts from the sum of the tile
// sums before it.  The aggregates go through shared memory both ways, so the
// block's global loads and stores are coalesced while each thread scans
// SCAN_TILE / SCAN_THREADS consecutive ones.  The last block writes the totals.
__global__ void __launch_bounds__(SCAN_THREADS) group_scan_kernel(GroupLaunch L) {
  constexpr uint32_t PER = SCAN_TILE / SCAN_THREADS, NW = SCAN_THREADS / 32;
  __shared__ uint2 stage[SCAN_TILE];
  __shared__ uint2 red[NW], wsum[NW];
  const uint32_t t = threadIdx.x, lane = t & 31u, warp = t >> 5;
  const uint32_t tile = blockIdx.x;
  const size_t b0 = (size_t)tile * SCAN_TILE;
#pragma unroll
  for (uint32_t k = 0; k < PER; ++k) {
    const size_t i = b0 + (size_t)k * SCAN_THREADS + t;
    stage[k * SCAN_THREADS + t] = i < L.nb ? L.bagg[i] : make_uint2(0, 0);
  }
  uint2 pre = make_uint2(0, 0);
  for (uint32_t k = t; k < tile; k += SCAN_THREADS) {
    const uint2 a = L.tsum[k];
    pre.x += a.x;
    pre.y += a.y;
  }
  pre.x = __reduce_add_sync(0xFFFFFFFFu, pre.x);
  pre.y = __reduce_add_sync(0xFFFFFFFFu, pre.y);
  if (lane == 0) red[warp] = pre;
  __syncthreads();  // (also: the staged aggregates are visible)
  pre = make_uint2(0, 0);
#pragma unroll
  for (uint32_t w = 0; w < NW; ++w) {
    pre.x += red[w].x;
    pre.y += red[w].y;
  }
  uint2 v[PER];
  uint2 loc = make_uint2(0, 0);
#pragma unroll
  for (uint32_t k = 0; k < PER; ++k) {
    v[k] = stage[t * PER + k];
    loc.x += v[k].x;
    loc.y += v[k].y;
  }
  // exclusive scan of loc over the block
  uint2 inc = loc;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t ax = __shfl_up_sync(0xFFFFFFFFu, inc.x, o), ay = __shfl_up_sync(0xFFFFFFFFu, inc.y, o);
    if (lane >= (uint32_t)o) {
      inc.x += ax;
      inc.y += ay;
    }
  }
  if (lane == 31) wsum[warp] = inc;
  __syncthreads();
  uint2 run = make_uint2(pre.x + inc.x - loc.x, pre.y + inc.y - loc.y);
  for (uint32_t w = 0; w < warp; ++w) {
    run.x += wsum[w].x;
    run.y += wsum[w].y;
  }
#pragma unroll
  for (uint32_t k = 0; k < PER; ++k) {
    stage[t * PER + k] = run;  // (each thread rewrites only the entries it read)
    run.x += v[k].x;
    run.y += v[k].y;
  }
  __syncthreads();
#pragma unroll
  for (uint32_t k = 0; k < PER; ++k) {
    const size_t i = b0 + (size_t)k * SCAN_THREADS + t;
    if (i < L.nb) L.bout[i] = stage[k * SCAN_THREADS + t];
  }
  if (tile == gridDim.x - 1 && t == SCAN_THREADS - 1) {
    L.totals[0] = run.x;
    L.totals[1] = run.y;
    if (run.y > L.tg_cap) atomicOr(L.err, DEV_FLAG_TG_OVF);
  }
}

// One warp per bucket: the bucket's groups to the DEM arrays.  Block 0 also
// writes each circuit's first output slot and target.
__global__ void __launch_bounds__(GW_WARPS * 32) emit_kernel(GroupLaunch L) {
  if (blockIdx.x == 0)
    for (uint32_t c = threadIdx.x; c < L.n_circ; c += GW_WARPS * 32) L.cout[c] = L.bout[L.cbbase[c]];
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t b = blockIdx.x * GW_WARPS + (threadIdx.x >> 5);
  if (b >= L.nb) return;
  const size_t base = (size_t)b * SLOT_CAP;
  // the first records load beside the bucket's aggregate and offset (a slot
  // past the groups holds whatever it held: only the ones below agg.x are used)
  SlotTail t = L.slot[base + lane].tail, tn1 = L.slot[base + lane + 1].tail;
  const uint2 agg = L.bagg[b], out = L.bout[b];
  const uint32_t tcap = L.tcap;
  for (uint32_t g = lane; g < agg.x; g += 32) {
    if (g != lane) {
      t = L.slot[base + g].tail;
      if (g + 1 < agg.x) tn1 = L.slot[base + g + 1].tail;  // (slot g + 1 <= SLOT_CAP - 1)
    }
    const uint32_t slot = out.x + g;
    const uint32_t toff = out.y + t.t;
    const uint32_t m = t.m;
    L.out_prob[slot] = t.p;
    L.out_off[slot] = toff;
    // the group's targets run to the next group's (the bucket's total after
    // the last); a list longer than the stride was flagged by the key pass
    // and the run is redone with wider lists, so only the stride's targets
    // are copied here
    const uint32_t ntg = min((g + 1 < agg.x ? tn1.t : agg.y) - t.t, tcap);
    if ((uint64_t)toff + ntg <= L.tg_cap) {
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

// ---- noise-rate gradients ---------------------------------------------------

// Channel kind of a record type: 0 X/Y/Z error or measurement flip, 1 DEPOLARIZE1, 2 DEPOLARIZE2.
__device__ __forceinline__ uint32_t channel_kind(uint32_t type) {
  return (type == REC_DEP1_L0 || type == REC_DEP1_L12) ? 1u : type >= REC_DEP2_L0 ? 2u : 0u;
}

__global__ void param_rec_kernel(ParamLaunch L) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= L.R) return;
  const uint32_t src = L.rec_src[r];
  if (src >= L.n_src) return;
  L.rec_p[r] = L.qtab[(size_t)src * 3 + channel_kind((uint32_t)((L.rec[r] >> 56) & 15u))];
}

// Record of mechanism m (one circuit): a search of rec_moff between the
// record of m's key block's first mechanism and KEY_THREADS + 15 records
// after it (each record holds 1 to 15 mechanisms, so m's record lies there).
__device__ __forceinline__ uint32_t record_of(const AdjointLaunch &A, uint32_t m) {
  uint32_t lo = A.blk_info[m / KEY_THREADS].x;
  uint32_t hi = min(A.R, lo + KEY_THREADS + 15u);
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (__ldg(A.rec_moff + mid) <= m) lo = mid;
    else hi = mid;
  }
  return lo;
}

__global__ void __launch_bounds__(GW_WARPS * 32) adjoint_group_kernel(AdjointLaunch A) {
  __shared__ double s_q[GW_WARPS][SLOT_CAP];  // probability of the mechanism at each sorted position
  const uint32_t lane = threadIdx.x & 31u, wi = threadIdx.x >> 5;
  const uint32_t b = blockIdx.x * GW_WARPS + wi;
  if (b >= A.nb) return;
  const uint32_t n = A.count[b];
  if (n == 0 || n > SLOT_CAP) return;
  const uint32_t groups = A.bagg[b].x, out0 = A.bout[b].x;
  const Slot *const bslot = A.slot + (size_t)b * SLOT_CAP;
  double *q = s_q[wi];
  // the forward's mechanism probabilities, recomputed from the records (every
  // component of a record carries the record's probability)
  for (uint32_t s = lane; s < n; s += 32) q[s] = __ldg(A.rec_p + record_of(A, slot_perm(bslot, s)[0]));
  __syncwarp();
  for (uint32_t g = lane; g < groups; g += 32) {
    const uint32_t s0 = slot_perm(bslot, g)[1], s1 = g + 1 < groups ? slot_perm(bslot, g + 1)[1] : n;
    const double dl = A.grad_out[out0 + g];
    double pre = 1.0;
    for (uint32_t s = s0; s < s1; ++s) {
      A.gq[slot_perm(bslot, s)[0]] = pre;
      pre *= 1.0 - 2.0 * q[s];
    }
    double suf = 1.0;
    for (uint32_t s = s1; s-- > s0;) {
      const uint32_t m = slot_perm(bslot, s)[0];
      A.gq[m] = dl * A.gq[m] * suf;
      suf *= 1.0 - 2.0 * q[s];
    }
  }
}

__global__ void adjoint_record_kernel(AdjointLaunch A) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= A.R) return;
  const uint32_t src = A.rec_src[r];
  if (src >= A.n_src) {
    A.grad_rec[r] = 0.0;
    return;
  }
  double sum = 0.0;
  for (uint32_t m = A.rec_moff[r]; m < A.rec_moff[r + 1]; ++m) sum += A.gq[m];
  A.grad_rec[r] = sum * A.stab[(size_t)src * 3 + channel_kind((uint32_t)((A.rec[r] >> 56) & 15u))];
}

__global__ void adjoint_source_kernel(AdjointLaunch A) {
  const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= A.n_src) return;
  double sum = 0.0;
  for (uint32_t k = A.src_off[e]; k < A.src_off[e + 1]; ++k) sum += A.grad_rec[A.src_rec[k]];
  A.grad_noise[e] = sum;
}

}  // namespace

cudaError_t launch_param_rec(const ParamLaunch &L, cudaStream_t s) {
  if (L.R == 0) return cudaSuccess;
  param_rec_kernel<<<(L.R + 255) / 256, 256, 0, s>>>(L);
  return cudaGetLastError();
}

cudaError_t launch_adjoint(const AdjointLaunch &A, cudaStream_t s) {
  if (A.nb) adjoint_group_kernel<<<(A.nb + GW_WARPS - 1) / GW_WARPS, GW_WARPS * 32, 0, s>>>(A);
  if (A.R) adjoint_record_kernel<<<(A.R + 255) / 256, 256, 0, s>>>(A);
  if (A.n_src) adjoint_source_kernel<<<(A.n_src + 255) / 256, 256, 0, s>>>(A);
  return cudaGetLastError();
}

cudaError_t launch_key_prep(const KeyLaunch &L, cudaStream_t s) {
  if (L.M == 0) return cudaSuccess;
  const uint32_t nblk = key_blocks(L.M);
  key_prep_kernel<<<(nblk + 127) / 128, 128, 0, s>>>(L);
  return cudaGetLastError();
}

cudaError_t launch_keys(const KeyLaunch &L, cudaStream_t s) {
  if (L.M == 0) return cudaSuccess;
  key_kernel<<<key_blocks(L.M), KEY_THREADS, 0, s>>>(L);
  return cudaGetLastError();
}

cudaError_t launch_keys_late(const KeyLaunch &L, cudaStream_t s) {
  if (L.M == 0) return cudaSuccess;
  if (L.late_word == kNoSplit || L.n_circ != 1) return cudaErrorInvalidValue;
  key_late_kernel<<<key_blocks(L.M), KEY_THREADS, 0, s>>>(L);
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

cudaError_t launch_group(const GroupLaunch &L, cudaStream_t s) {
  if (L.nb == 0) return cudaSuccess;
  group_warp_kernel<<<(L.nb + GW_WARPS - 1) / GW_WARPS, GW_WARPS * 32, 0, s>>>(L);
  group_big_kernel<<<2 * 152, GB_THREADS, 0, s>>>(L);
  return cudaGetLastError();
}

cudaError_t launch_scan_emit(const GroupLaunch &L, cudaStream_t s) {
  if (L.nb == 0) return cudaSuccess;
  group_scan_kernel<<<(L.nb + SCAN_TILE - 1) / SCAN_TILE, SCAN_THREADS, 0, s>>>(L);
  emit_kernel<<<(L.nb + GW_WARPS - 1) / GW_WARPS, GW_WARPS * 32, 0, s>>>(L);
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
                                                    scr.err, scr.spin_ns, p == 0 ? scr.hold_first : 0u);
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
