// static_merge.cu -- merge raw error mechanisms into a DEM without allocating memory.
//
// Some callers cannot call cudaMalloc: code that runs while another runtime
// owns the device memory pool (a decoder or control loop that reserved its
// memory up front and must not grow it or synchronise the device in an
// allocation), or code whose memory budget is fixed at start-up.  For them,
// gpc_merge_mechanisms_static() runs the merge stage of the compile -- key
// hashing, radix bucketing, in-CTA sort and the FP64 XOR-merge -- on
// buffers the caller passes, with every piece of scratch memory taken from
// one file-scope static device array instead of an allocation.
//
// The scratch array is kStaticScratchBytes (about 2.3 MiB) and stays
// resident on every GPU that loads this library until the process exits.
// It bounds one call to kStaticMaxMechanisms (65,536) mechanisms.  All calls
// on a device share it: calls that overlap on the GPU (different streams,
// or different host threads) race and corrupt each other's results, so
// callers must serialise them.  Each call clears the counters it needs.
//
// Host code cannot use the array's name as a device address; the first call
// on each device looks the address up with cudaGetSymbolAddress (so make
// that first call outside any stream capture) and caches it per device.
#include <cstdint>
#include <mutex>

#include "../../include/gpc.h"
#include "device.cuh"

namespace gpc {
namespace {

constexpr uint32_t kStaticMaxMechanisms = 1u << 16;
constexpr uint32_t kStaticBucketBits = 10;
constexpr uint32_t kStaticBuckets = 1u << kStaticBucketBits;
constexpr uint32_t kMaxDevices = 64;

// Byte layout of the scratch array.
constexpr size_t A256(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t kOffKey = 0;                                                    // ulonglong2[max]
constexpr size_t kOffBKey = A256(kOffKey + 16ull * kStaticMaxMechanisms);        // ulonglong2[max]
constexpr size_t kOffBM = A256(kOffBKey + 16ull * kStaticMaxMechanisms);         // uint32[max]
constexpr size_t kOffOffset = A256(kOffBM + 4ull * kStaticMaxMechanisms);        // uint32[nb + 1]
constexpr size_t kOffCDev = A256(kOffOffset + 4ull * (kStaticBuckets + 1));      // CircuitDev
constexpr size_t kOffZero = A256(kOffCDev + sizeof(CircuitDev));                 // start of per-call zeroed part
constexpr size_t kOffCount = kOffZero;                                           // uint32[nb]
constexpr size_t kOffCursor = A256(kOffCount + 4ull * kStaticBuckets);           // uint32[nb]
constexpr size_t kOffStatus = A256(kOffCursor + 4ull * kStaticBuckets);          // u64[nb]
constexpr size_t kOffTicket = A256(kOffStatus + 8ull * kStaticBuckets);          // uint32
constexpr size_t kOffErr = kOffTicket + 4;                                       // uint32
constexpr size_t kOffTotals = kOffTicket + 16;                                   // uint32[4]
constexpr size_t kStaticScratchBytes = A256(kOffTotals + 16);
constexpr size_t kZeroBytes = kStaticScratchBytes - kOffZero;

static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

std::mutex g_setup_mu;
void *g_scratch_addr[kMaxDevices] = {};

__device__ __forceinline__ uint64_t fmix64s(uint64_t k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdull;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ull;
  k ^= k >> 33;
  return k;
}

// Same word hash as the compile pipeline: two independent mixes of (j, word).
__device__ __forceinline__ ulonglong2 word_hash_s(uint32_t j, uint64_t v) {
  const uint64_t jj = (uint64_t)j + 1;
  return make_ulonglong2(fmix64s(v * 0x9E3779B97F4A7C15ull + jj * 0xC2B2AE3D27D4EB4Full),
                         fmix64s(v * 0xD6E8FEB86659FD93ull + jj * 0xA0761D6478BD642Full + 0x8EBC6AF09C88C6E3ull));
}

enum : uint32_t { STATIC_ERR_BAD_LIST = 64u };

// Describes the caller's mechanism arrays to the bucket-merge kernel.
__global__ void static_setup_kernel(CircuitDev *cdev, const uint32_t *tn, const uint32_t *tl, const double *p,
                                    uint32_t n, uint32_t stride) {
  CircuitDev c{};
  c.tl = const_cast<uint32_t *>(tl);
  c.tn = const_cast<uint32_t *>(tn);
  c.mp = const_cast<double *>(p);
  c.M = n;
  c.tcap = stride;
  c.w = 0;
  *cdev = c;
}

// One thread per mechanism: 128-bit key of its target list, bucket histogram.
__global__ void static_key_kernel(const uint32_t *__restrict__ tn, const uint32_t *__restrict__ tl, uint32_t n,
                                  uint32_t stride, ulonglong2 *__restrict__ key, uint32_t *__restrict__ count,
                                  uint32_t *__restrict__ err) {
  const uint32_t shift = 64u - kStaticBucketBits;
  for (uint32_t m = blockIdx.x * blockDim.x + threadIdx.x; m < n; m += gridDim.x * blockDim.x) {
    uint32_t nt = tn[m];
    if (nt > stride) {
      atomicOr(err, STATIC_ERR_BAD_LIST);
      nt = stride;
    }
    const uint32_t *t = tl + (size_t)m * stride;
    uint64_t hx = 0, hy = 0, v = 0;
    uint32_t cur = 0xFFFFFFFFu, prev = 0;
    for (uint32_t k = 0; k < nt; ++k) {
      const uint32_t b = t[k];
      if (k > 0 && b <= prev) atomicOr(err, STATIC_ERR_BAD_LIST);  // targets must ascend
      prev = b;
      const uint32_t j = b >> 6;
      if (j != cur) {
        if (v) {
          const ulonglong2 h = word_hash_s(cur, v);
          hx ^= h.x;
          hy ^= h.y;
        }
        cur = j;
        v = 0;
      }
      v |= 1ull << (b & 63u);
    }
    if (v) {
      const ulonglong2 h = word_hash_s(cur, v);
      hx ^= h.x;
      hy ^= h.y;
    }
    key[m] = make_ulonglong2(hx, hy);
    if ((hx | hy) == 0) {
      if (nt) atomicOr(err, DEV_ERR_COLLISION);
    } else {
      atomicAdd(count + (hx >> shift), 1u);
    }
  }
}

// Copies the totals and flags to the caller and closes the offsets array.
__global__ void static_finish_kernel(const uint32_t *totals, const uint32_t *err, uint32_t n, uint32_t *out_off,
                                     uint32_t *result) {
  const uint32_t groups = totals[0], targets = totals[1];
  result[0] = groups;
  result[1] = targets;
  result[2] = *err;
  result[3] = 0;
  if (groups <= n) out_off[groups] = targets;
}

}  // namespace
}  // namespace gpc

extern "C" gpc_status gpc_merge_mechanisms_static(const uint32_t *num_targets, const uint32_t *targets,
                                                  uint32_t stride, const double *probs, uint32_t n,
                                                  double *out_probs, uint32_t *out_offsets, uint32_t *out_targets,
                                                  uint32_t out_target_cap, uint32_t *result, void *stream) {
  using namespace gpc;
  if (n > kStaticMaxMechanisms) return GPC_ERR_CAPACITY;  // more mechanisms than the static scratch holds
  if (!num_targets || !targets || !probs || !out_probs || !out_offsets || !out_targets || !result || stride == 0)
    return GPC_ERR_INVALID;
  // target lists are read as 16-byte vectors
  if (stride % 4 != 0 || (reinterpret_cast<uintptr_t>(targets) & 15u) != 0) return GPC_ERR_INVALID;
  // list lengths are cut to the stride, so n * stride bounds every target
  // count and offset the kernels form in 32 bits
  if ((uint64_t)n * stride > 0xFFFFFFFFull) return GPC_ERR_CAPACITY;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || (uint32_t)dev >= kMaxDevices) return GPC_ERR_CUDA;
  char *base;
  {
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_addr[dev]) {
      void *p = nullptr;
      if (cudaGetSymbolAddress(&p, g_static_scratch) != cudaSuccess || !p) {
        (void)cudaGetLastError();
        return GPC_ERR_CUDA;
      }
      g_scratch_addr[dev] = p;
    }
    base = static_cast<char *>(g_scratch_addr[dev]);
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  ulonglong2 *key = reinterpret_cast<ulonglong2 *>(base + kOffKey);
  ulonglong2 *bkey = reinterpret_cast<ulonglong2 *>(base + kOffBKey);
  uint32_t *bm = reinterpret_cast<uint32_t *>(base + kOffBM);
  uint32_t *offset = reinterpret_cast<uint32_t *>(base + kOffOffset);
  CircuitDev *cdev = reinterpret_cast<CircuitDev *>(base + kOffCDev);
  uint32_t *count = reinterpret_cast<uint32_t *>(base + kOffCount);
  uint32_t *cursor = reinterpret_cast<uint32_t *>(base + kOffCursor);
  unsigned long long *status = reinterpret_cast<unsigned long long *>(base + kOffStatus);
  uint32_t *ticket = reinterpret_cast<uint32_t *>(base + kOffTicket);
  uint32_t *err = reinterpret_cast<uint32_t *>(base + kOffErr);
  uint32_t *totals = reinterpret_cast<uint32_t *>(base + kOffTotals);

  if (cudaMemsetAsync(base + kOffZero, 0, kZeroBytes, s) != cudaSuccess) return GPC_ERR_CUDA;
  static_setup_kernel<<<1, 1, 0, s>>>(cdev, num_targets, targets, probs, n, stride);
  if (n) {
    uint32_t blocks = (n + 255) / 256;
    static_key_kernel<<<blocks, 256, 0, s>>>(num_targets, targets, n, stride, key, count, err);
  }
  if (launch_bucket_scan(count, offset, kStaticBuckets, s) != cudaSuccess) return GPC_ERR_CUDA;
  if (launch_bucket_scatter(key, n, kStaticBucketBits, offset, cursor, bkey, bm, s) != cudaSuccess)
    return GPC_ERR_CUDA;
  BucketMergeLaunch bl{};
  bl.c_dev = cdev;
  bl.w = 0;
  bl.bkey = bkey;
  bl.bm = bm;
  bl.count = count;
  bl.offset = offset;
  bl.nb = kStaticBuckets;
  bl.max_groups = n;
  bl.out_prob = out_probs;
  bl.out_off = out_offsets;
  bl.out_tg = out_targets;
  bl.tg_cap = out_target_cap;
  bl.status = status;
  bl.ticket = ticket;
  bl.totals = totals;
  bl.err = err;
  if (launch_bucket_merge(bl, s) != cudaSuccess) return GPC_ERR_CUDA;
  static_finish_kernel<<<1, 1, 0, s>>>(totals, err, n, out_offsets, result);
  return cudaGetLastError() == cudaSuccess ? GPC_OK : GPC_ERR_CUDA;
}
