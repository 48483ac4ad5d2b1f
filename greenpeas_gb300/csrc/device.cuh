// device.cuh -- structures shared by the host driver and the sm_103a kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace gpc {

// Device error bits (one word per pipeline run).
enum : uint32_t {
  DEV_ERR_TIMEOUT = 1u,    // a bounded wait (mbarrier or look-back) gave up
  DEV_ERR_COLLISION = 2u,  // equal 128-bit keys, different symptoms
  DEV_FLAG_MIXED = 4u,     // equal sort keys, different 128-bit keys: re-sort on 128 bits
  DEV_FLAG_TG_OVF = 8u,    // target buffer too small: grow and re-run the merge
  DEV_FLAG_BIG_BUCKET = 16u,  // a bucket exceeds the in-CTA capacity: use the global sort
  DEV_FLAG_LONG = 32u,        // a symptom has more targets than the target-list stride: widen it
  DEV_ERR_NOISE = 128u,       // a noise-tensor entry is outside its channel's range
};

// One circuit as the kernels see it.  All arrays are device pointers.
struct CircuitDev {
  const uint64_t *ops;        // tape, epoch-major, [slot][qubit] inside an epoch
  const uint32_t *ep_opoff;   // [n_epochs]
  const uint32_t *ep_k;       // [n_epochs]
  const uint32_t *ep_ptoff;   // [n_epochs + 1]
  const uint32_t *ep_chunk;   // [n_epochs] copy chunk of each epoch
  const uint32_t *ch_off;     // [n_chunks] first op of each chunk
  const uint32_t *ch_bytes;   // [n_chunks]
  const uint32_t *inj_lo;     // [w] first epoch injecting into word j (0xFFFFFFFF: none)
  const uint32_t *inj_hi;     // [w] last epoch injecting into word j
  ulonglong2 *snap;           // [w][npoints] (X row, Z row) at each point
  uint2 *band;                // [w] point range written by the walk of word j
  unsigned long long *nzm;    // [npoints][mw] (zeroed) bit j: word j's rows at the point are non-zero
  const uint64_t *rec;        // [R] noise records
  const double *rec_p;        // [R]
  const uint32_t *rec_moff;   // [R + 1]
  uint64_t *mdesc;            // [M] mechanism descriptors (written by the key kernel)
  double *mp;                 // [M] mechanism probabilities (written by the key kernel)
  uint32_t *tl;               // [M][tcap] targets of each mechanism, ascending (written by the key kernel)
  uint32_t *tn;               // [M] number of targets of each mechanism
  uint32_t nq, qpad, n_epochs, w;
  uint32_t npoints, M, R;
  uint32_t tcap;              // stride of tl (0: no target lists, merge from snapshots)
  uint32_t n_chunks, chunk_cap;
  uint32_t mbase;             // first mechanism of this circuit in the batch-wide arrays
  uint32_t bbase, bbits;      // first bucket of this circuit, log2 of its bucket count
  uint32_t mw;                // 64-bit mask words per point: ceil(w / 64)
};

// *p += v as a reduction that returns nothing (the thread does not wait for
// the L2 round trip of an atomic whose old value it would not use).
__device__ __forceinline__ void red_add(uint32_t *p, uint32_t v) {
  asm volatile("red.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

constexpr uint32_t kMaxCircuitsStaged = 2048;  // batch tables staged in shared memory up to this size

// Index of the circuit holding item x: the last c with base[c] <= x (base has n+1 entries).
__device__ __forceinline__ uint32_t find_circuit(const uint32_t *base, uint32_t n, uint32_t x) {
  uint32_t lo = 0, hi = n;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (base[mid] <= x) lo = mid;
    else hi = mid;
  }
  return lo;
}

constexpr int SORT_THREADS = 256;
constexpr int SORT_IPT = 8;
constexpr int SORT_TILE = SORT_THREADS * SORT_IPT;
constexpr int RADIX_BITS = 8;
constexpr int RADIX = 1 << RADIX_BITS;
constexpr int MERGE_THREADS = 256;
constexpr int BUCKET_THREADS = 128;
constexpr int BUCKET_CAP = 1024;  // items one CTA sorts in shared memory (allocation-free merge)
constexpr uint32_t SLOT_CAP = 256;  // slots of one bucket in the compile pipeline
constexpr uint32_t WARP_CAP = 128;  // bucket items one warp merges; larger buckets take a CTA
constexpr uint32_t SCAN_TILE = 1024;    // bucket aggregates one scan block covers
constexpr uint32_t SCAN_THREADS = 256;  // threads of a scan block (4 aggregates each)

inline uint32_t sort_tiles(uint32_t n) { return (n + SORT_TILE - 1) / SORT_TILE; }
inline uint32_t merge_tiles(uint32_t n) { return (n + MERGE_THREADS - 1) / MERGE_THREADS; }

// ---- launch wrappers (defined in the .cu files) ----------------------------
struct WalkLaunch {
  const CircuitDev *circs;  // device array
  const uint2 *items;       // device array of (circuit, first word of the CTA)
  uint32_t n_items;
  uint32_t threads, qpt, qpad;
  uint32_t chunk_cap;       // bytes of each of the two chunk buffers
  uint32_t max_epochs, max_chunks;  // largest tables of the launch (staged in shared memory if they fit)
  uint32_t words;           // detector words per CTA (1, or 2 with 1 or 2 qubits per thread)
  uint32_t *err;
  // Persistent launch (null: one CTA per item): a zeroed counter from which
  // resident CTAs take items until none are left.  Circuits of any slot count
  // up to qpad share the launch; the items should come longest first.
  uint32_t *queue;
};
cudaError_t launch_walk(const WalkLaunch &L, cudaStream_t s);
cudaError_t walk_set_smem_limit();  // call once per device before launching walks

// ---- segmented walk (one circuit) -------------------------------------------
// The epochs are cut into time segments s = [b_s, b_{s+1}) at clean cuts
// (walk_segment_bounds, lower.hpp).  A word whose walk spans segments s0..K
// (K: the last segment for words holding observables, else the one holding
// the word's last measurement) runs as
//   launch A: SEG_FIRST  -- [e0, b_{s0+1}) from zero rows, with snapshots; exit rows -> a state;
//             SEG_AFF    -- each segment s in (s0, K) holding measurements of the word,
//                           from zero rows, no snapshots; exit rows -> a state (c_s);
//             SEG_XFER   -- per segment s and 64-row column c, the walk of unit rows
//                           without measurement bits: column c of the transfer matrix A_s;
//   launch B: SEG_REST   -- segment s in (s0, K]: entry rows composed from the
//                           first part's exit through A and c of segments
//                           (s0, s), then the segment walked with snapshots
//                           (the last one on to the end, or until the rows vanish).
// A word that spans one segment is a single SEG_FIRST item walking to the end.
// States are [2 qpad] u64 rows: X of slots 0..qpad-1, then Z of the same slots.
enum : uint32_t { SEG_FIRST = 0, SEG_AFF = 1, SEG_XFER = 2, SEG_REST = 3 };
// Entries of a transfer row kept as a sparse list (rows with more are read
// from the dense transfer columns): measured on code circuits, rows hold 1-3
// entries on average and up to 12 where a cut falls inside a round.
constexpr uint32_t kSegRowCap = 16;
// Entries of a row that the compose ring copies into shared memory (entries
// kSegRingCap .. kSegRowCap - 1, rare, are read from global memory).
constexpr uint32_t kSegRingCap = 8;
// Most compose steps a REST item keeps in flight (shared-memory ring).
constexpr uint32_t kSegRingMax = 4;
struct SegItem {
  uint32_t kind;
  uint32_t idx;             // word (SEG_XFER: transfer column)
  uint32_t e_begin, e_end;  // epochs walked
  uint32_t state;           // FIRST/AFF/XFER: state written at exit (0xFFFFFFFF: none); REST: entry state
  uint32_t s_from, s_to;    // REST: compose through segments [s_from, s_to) before walking; XFER: s_from
                            // is the segment
  uint32_t pad;
};
static_assert(sizeof(SegItem) == 32, "segment item is 32 bytes");
struct SegLaunch {
  const CircuitDev *circ;   // the circuit
  const SegItem *items;
  uint32_t n_items;
  uint32_t threads, qpt, qpad;
  uint32_t chunk_cap, max_epochs, max_chunks;
  uint64_t *state;          // [states][2 qpad]
  uint32_t xfer0;           // state of segment s's transfer column c: xfer0 + s * ncol + c
  uint32_t ncol;            // 64-row columns of a transfer matrix: ceil(2 qpad / 64)
  const uint32_t *aff;      // [w][S] state of word j's SEG_AFF walk of segment s (0xFFFFFFFF: no measurements)
  uint32_t S;
  uint32_t *xcnt;           // [S][2 qpad] (zeroed) entries of each transfer row
  uint16_t *xlst;           // entries 0..7 [S][2 qpad][kSegRingCap], then entries 8..15 [S][2 qpad][8]
  uint32_t ring_nb;         // compose step buffers of a REST CTA (launch B; 0 in launch A)
  uint32_t *err;
};
// Dynamic shared memory of a segment launch (0: it does not fit a CTA).
size_t walk_seg_smem_bytes(const SegLaunch &L);
cudaError_t launch_walk_seg(const SegLaunch &L, cudaStream_t s);
bool walk_seg_supported(uint32_t qpt);
// Staged epoch/chunk table bytes for a launch (0: the tables are read from global memory).
uint32_t walk_table_bytes(uint32_t max_epochs, uint32_t max_chunks);
size_t walk_smem_bytes(uint32_t qpad, uint32_t chunk_cap, uint32_t table_bytes, uint32_t words);
uint32_t walk_max_threads(uint32_t qpt);  // 0: no walk instance for this many qubits per thread
bool walk_queue_supported(uint32_t qpt, uint32_t words);  // a persistent walk instance exists

// Key kernel: one thread per noise record; expands the record into its
// mechanisms (mdesc, mp), computes each mechanism's 128-bit key, and counts
// non-empty keys per bucket (top `bucket_bits` bits of key.x).
// One bucket slot (32 bytes, one sector): the mechanism's 128-bit key, then
// (mechanism, target count, probability).  The group stage overwrites the
// second half of a bucket's first slots with one record per group:
// (head mechanism, targets before the group inside the bucket, probability).
struct SlotTail {
  uint32_t m, t;
  double p;
};
static_assert(sizeof(SlotTail) == 16, "slot tail is 16 bytes");
// A slot: key and tail side by side, so a mechanism's item is one 32-byte
// sector written once and read once.  After grouping, the key half of slot s
// holds the saved permutation as two 32-bit words: [0] the mechanism at
// sorted position s, [1] (for s < groups) the first sorted position of group s.
struct Slot {
  ulonglong2 key;
  SlotTail tail;
};
static_assert(sizeof(Slot) == 32, "a slot is one 32-byte sector");
__host__ __device__ __forceinline__ uint32_t *slot_perm(Slot *bucket, uint32_t s) {
  return reinterpret_cast<uint32_t *>(&bucket[s].key);
}
__host__ __device__ __forceinline__ const uint32_t *slot_perm(const Slot *bucket, uint32_t s) {
  return reinterpret_cast<const uint32_t *>(&bucket[s].key);
}

struct KeyLaunch {
  const CircuitDev *circs;  // [n_circ]
  const uint32_t *mbase;    // [n_circ + 1] first mechanism of each circuit (+ total)
  uint32_t n_circ, M;       // circuits, mechanisms of the whole batch
  uint2 *blk_info;          // [key blocks] (record of the block's first mechanism, its circuit | spans << 31)
  ulonglong2 *key;          // [M]
  uint32_t *bucket_count;   // [buckets of the batch] (zeroed)
  Slot *slot;               // [buckets * SLOT_CAP] bucket slots
  uint32_t *list_total;     // += targets written to the lists (for traffic accounting)
  uint32_t *err;
  uint32_t write_all;       // also write key[], and descriptors/probabilities (global path, gradients)
  // One circuit whose key pass is split (kNoSplit: one pass over every word):
  // key_kernel covers the words below late_word and leaves each mechanism's
  // descriptor, probability, targets and partial key; key_late_kernel adds
  // the words from late_word on (the observables', whose walk is the longest)
  // and files the mechanism in its bucket.
  uint32_t late_word;
};
constexpr uint32_t kNoSplit = 0xFFFFFFFFu;
constexpr uint32_t KEY_THREADS = 256;
inline uint32_t key_blocks(uint32_t M) { return (M + KEY_THREADS - 1) / KEY_THREADS; }
// Finds each key block's first record (one thread per block).
cudaError_t launch_key_prep(const KeyLaunch &L, cudaStream_t s);
cudaError_t launch_keys(const KeyLaunch &L, cudaStream_t s);
cudaError_t launch_keys_late(const KeyLaunch &L, cudaStream_t s);  // second pass of a split key pass

// Exclusive scan of the bucket counts into bucket offsets (+ total at [nb]).
cudaError_t launch_bucket_scan(const uint32_t *count, uint32_t *offset, uint32_t nb, cudaStream_t s);

// Moves every non-empty mechanism to its bucket: items (key, m).
cudaError_t launch_bucket_scatter(const ulonglong2 *key, uint32_t M, uint32_t bucket_bits, const uint32_t *offset,
                                  uint32_t *cursor, ulonglong2 *bkey, uint32_t *bm, cudaStream_t s);

struct BucketMergeLaunch {
  const CircuitDev *c_dev;
  uint32_t w;
  const ulonglong2 *bkey;   // bucketed keys
  const uint32_t *bm;       // bucketed mechanism ids
  const uint32_t *count;    // [nb]
  const uint32_t *offset;   // [nb]
  uint32_t nb;
  uint32_t max_groups;      // capacity of out_prob / out_off (the mechanism count)
  double *out_prob;
  uint32_t *out_off;
  uint32_t *out_tg;
  uint32_t tg_cap;
  unsigned long long *status;  // [nb]
  uint32_t *ticket;
  uint32_t *totals;  // [0] groups, [1] targets
  uint32_t *err;
};
cudaError_t launch_bucket_merge(const BucketMergeLaunch &L, cudaStream_t s);

// Merge of the compile pipeline (no inter-CTA waits).  The key kernel has put
// every non-empty mechanism into a slot of its bucket (SLOT_CAP slots per
// bucket; more raises DEV_FLAG_BIG_BUCKET).
//  group: one warp per bucket of <= WARP_CAP items (one CTA per larger bucket)
//         orders its items (by 64 sub-bins on the top bits of the key's second
//         half, then by (key, m) inside a sub-bin), checks collisions, folds each group's
//         probability and overwrites the bucket's first slots with one record
//         per group (head mechanism, probability, targets before it in the
//         bucket); bucket aggregates (groups, targets) and their per-tile sums;
//  scan:  exclusive scan of the bucket aggregates, one block per SCAN_TILE
//         buckets (tile sums give each block its prefix);
//  emit:  one warp per bucket writes its groups' probabilities, offsets and
//         target lists to the DEM arrays.
struct GroupLaunch {
  const uint32_t *tl;       // [M][tcap] batch-wide target lists
  const uint32_t *tn;       // [M]
  uint32_t tcap;
  Slot *slot;               // [nb * SLOT_CAP] items; afterwards the saved permutation in the
                            // key halves (slot_perm) and one group record per group in the tails
  const uint32_t *count;    // [nb]
  uint32_t nb;
  uint2 *bagg;              // [nb] (groups, targets) of each bucket
  uint2 *bout;              // [nb] exclusive prefix of bagg
  uint2 *tsum;              // [ceil(nb / SCAN_TILE)] (zeroed) per-tile sums of bagg
  uint32_t *big_n;          // (zeroed) buckets with more than WARP_CAP items
  uint32_t *big_list;       // [nb]
  double *out_prob;
  uint32_t *out_off;
  uint32_t *out_tg;
  uint32_t tg_cap;
  uint32_t *totals;         // [0] groups, [1] targets, [3] += bucketed items
  const uint32_t *cbbase;   // [n_circ] first bucket of each circuit
  uint32_t n_circ;
  uint2 *cout;              // [n_circ] (first slot, first target) of each circuit's output
  uint32_t *err;
};
cudaError_t launch_group(const GroupLaunch &L, cudaStream_t s);

// ---- noise-rate gradients (single circuit) ----------------------------------
// Record probabilities from a [n_ticks][4] FP64 noise tensor: record r takes
// its source's rate through its channel's split, looked up in qtab[src][kind]
// (kind 0: X/Y/Z error or measurement flip, 1: DEPOLARIZE1, 2: DEPOLARIZE2),
// which the host fills with the same split formulas as the text path.
// Records without a source keep their probability.
struct ParamLaunch {
  const uint64_t *rec;
  const uint32_t *rec_src;
  double *rec_p;
  uint32_t R, n_src;
  const double *qtab;  // [n_src][3]
};
cudaError_t launch_param_rec(const ParamLaunch &L, cudaStream_t s);

// Adjoint of the merge and of the channel splits:
//  group:  one warp per bucket, a lane per group: dL/dq_m = dL/dp_g *
//          prod_{j in g, j != m} (1 - 2 q_j) from prefix and suffix products
//          along the group's run in the saved permutation;
//  record: dL/dp_r = (sum of its mechanisms' dL/dq) * dq/dp, the split's
//          slope at the source's rate (stab[src][kind], filled by the host);
//  source: dL/dnoise[e] = sum over the records of source e, in record order.
struct AdjointLaunch {
  const Slot *slot;        // saved permutation (see GroupLaunch)
  const uint32_t *count;
  const uint2 *bagg, *bout;
  uint32_t nb;
  const uint2 *blk_info;   // [key blocks] record of each key block's first mechanism (the forward's key pass)
  const double *rec_p;     // [R] each record's component probability of the forward (from the noise tensor)
  const double *grad_out;  // [groups] dL/dp of each merged mechanism
  double *gq;              // [M] (zeroed) dL/dq of each mechanism
  const uint64_t *rec;
  const uint32_t *rec_src, *rec_moff;
  uint32_t R;
  const double *stab;      // [n_src][3] dq/dp of each source and channel kind
  double *grad_rec;        // [R]
  const uint32_t *src_off, *src_rec;  // records of each source (CSR, record order)
  uint32_t n_src;
  double *grad_noise;      // [n_src]
};
cudaError_t launch_adjoint(const AdjointLaunch &L, cudaStream_t s);
cudaError_t launch_scan_emit(const GroupLaunch &L, cudaStream_t s);

// ---- global path (used when a bucket is too large for one CTA) -------------
// Onesweep radix sort of (u64 key, u32 value) pairs on the low `bits` bits.
struct SortScratch {
  uint32_t *hist;      // [passes][RADIX]
  uint32_t *status;    // [passes][tiles][RADIX]
  uint32_t *tile_ctr;  // [passes]
  uint32_t *err;
  unsigned long long spin_ns;  // a look-back wait gives up (DEV_ERR_TIMEOUT) after this long
  // Test of the bounded look-back: tile 0 of the first pass keeps its digit
  // counts to itself, so the waits of the tiles after it run out.
  uint32_t hold_first;
};
size_t sort_scratch_words(uint32_t n, uint32_t bits);
cudaError_t launch_sort(uint64_t *keys, uint64_t *keys_alt, uint32_t *vals, uint32_t *vals_alt, uint32_t n,
                        uint32_t bits, const SortScratch &scr, cudaStream_t s, bool *result_in_alt);

// sortkey[m] = key[m].x, perm[m] = m (inputs of the global sort).
cudaError_t launch_sort_init(const ulonglong2 *key, uint64_t *sortkey, uint32_t *perm, uint32_t M, cudaStream_t s);

// Gathers key128[perm[i]].y into out[i] (second pass of a 128-bit sort).
cudaError_t launch_gather_hi(const ulonglong2 *key, const uint32_t *perm, uint64_t *out, uint32_t n, cudaStream_t s);

struct MergeLaunch {
  const CircuitDev *c_dev;  // single circuit
  uint32_t w;
  const uint32_t *perm;     // sorted mechanism ids
  const uint64_t *sortkey;  // sorted keys (for the mixed-run check)
  uint64_t sort_mask;       // key bits the sort compared (0: skip the mixed-run check)
  const ulonglong2 *key;    // 128-bit key per mechanism
  uint32_t n;
  double *out_prob;
  uint32_t *out_off;
  uint32_t *out_tg;
  uint32_t tg_cap;
  unsigned long long *status;  // [tiles]
  uint32_t *tile_ctr;
  uint32_t *totals;  // [0] groups, [1] targets
  uint32_t *err;
  unsigned long long spin_ns;  // a look-back wait gives up (DEV_ERR_TIMEOUT) after this long
};
cudaError_t launch_merge(const MergeLaunch &L, cudaStream_t s);

}  // namespace gpc
