// lower.hpp -- stim circuit text -> device tick tape.
//
// The host half of the compile.  It replaces the reference's circuit
// lowering (Circuit::parseFromStimCircuit + Mixer + STEPG,
// QEC/ErrorAnalysis/Circuit.hpp:426-478, Mixer.hpp:97-533), which builds a
// layered node graph, with a tape for a backward Pauli-frame walk:
//
//  * qubit q is owned by one thread of a walk CTA (one CTA per 64-bit word
//    of the detector bitset);
//  * ops are grouped into epochs; a two-qubit Clifford opens a new epoch for
//    both its qubits and reads the partner's rows, published at the epoch
//    barrier; every other op is thread-local;
//  * the tape is stored epoch by epoch as [slot k][qubit q] u64 ops so a warp
//    reads one slot with one coalesced load;
//  * a noise op becomes a SNAP op that stores the qubit's two rows (X, Z)
//    at a "point"; each error component (mechanism) is a descriptor naming
//    up to two (point, Pauli) terms, its symptom is the XOR of the selected
//    rows.  A measurement flip stores its measurement's bits at a point.
#pragma once

#include <cstdint>
#include <cstdlib>
#include <new>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace gpc {

class HostPool;

// Allocator whose resize() leaves new elements of trivial types uninitialised,
// for host arrays that are written in full after they are sized.
template <typename T>
struct UninitAlloc : std::allocator<T> {
  template <typename U>
  struct rebind {
    using other = UninitAlloc<U>;
  };
  UninitAlloc() = default;
  template <typename U>
  UninitAlloc(const UninitAlloc<U> &) noexcept {}
  template <typename U>
  void construct(U *) noexcept {}
  template <typename U, typename... A>
  void construct(U *p, A &&...a) {
    ::new ((void *)p) U(std::forward<A>(a)...);
  }
};
template <typename T>
using HostArray = std::vector<T, UninitAlloc<T>>;

// Errors thrown by the lowering carry a gpc_status code.
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

// ---- tape op encoding (u64) ----------------------------------------------
// bits 0-7 opcode, bits 8-15 sub, bits 16-31 aux, bits 32-63 operand.
enum : uint32_t {
  OP_NOP = 0,
  OP_C1 = 1,     // sub: newX mask (bits 0-1 over X,Z) | newZ mask << 2
  OP_C2 = 2,     // sub: newX mask (4 bits over selfX,selfZ,partX,partZ) | newZ mask << 4; operand: partner qubit
  OP_R = 3,      // clear both rows
  OP_M = 4,      // sub: basis (0 Z, 1 X, 2 Y) | 4 (clear first: MR); operand: one bit of the measurement
                 // (0xFFFFFFFF: none); the bits of preceding OP_INJ ops are added; rows ^= bits in word j
  OP_INJ = 5,    // two more bits of the next OP_M: operand, and bits 8-31 (0xFFFFFF: none)
  OP_SNAP = 6,   // operand: point; point <- (X, Z)
  OP_SNAPD = 7,  // operand: point; point <- (bits of the last measurement, 0)
  // two-qubit Cliffords whose update is one XOR (operand: partner qubit)
  OP_XPX = 8,    // X ^= partner X   (CX control)
  OP_ZPZ = 9,    // Z ^= partner Z   (CX target)
  OP_XPZ = 10,   // X ^= partner Z   (CZ, either qubit)
};

inline uint64_t make_op(uint32_t opc, uint32_t sub, uint32_t operand) {
  return (uint64_t)opc | ((uint64_t)(sub & 0xFF) << 8) | ((uint64_t)operand << 32);
}
inline uint64_t make_inj(uint32_t bit1, uint32_t bit2) {
  return (uint64_t)OP_INJ | ((uint64_t)(bit2 & 0xFFFFFFu) << 8) | ((uint64_t)bit1 << 32);
}

// Mechanism descriptor (device, one per mechanism): point a (30 bits) |
// Pauli a (2 bits) | point b | Pauli b.  Pauli: 0 none, 1 X, 2 Z, 3 Y (X|Z).
inline uint64_t make_desc(uint32_t pa, uint32_t Pa, uint32_t pb, uint32_t Pb) {
  return (uint64_t)(pa & 0x3FFFFFFFu) | ((uint64_t)(Pa & 3) << 30) | ((uint64_t)(pb & 0x3FFFFFFFu) << 32) |
         ((uint64_t)(Pb & 3) << 62);
}

// Noise record (host -> device, one per noise instance): point a (28 bits) |
// point b (28 bits) << 28 | type (4 bits) << 56 | Pauli a << 60 | Pauli b << 62.
// The device expands a record into its mechanisms (components).
enum : uint32_t {
  REC_PAULI = 0,     // one mechanism: Pauli a on point a, Pauli b on point b (b optional)
  REC_DEP1_L0 = 1,   // X, Z on point a
  REC_DEP1_L12 = 2,  // X, Y, Z on point a
  REC_DEP2_L0 = 3,   // IX IZ XI XX ZI ZZ on (a, b)
  REC_DEP2_L1 = 4,   // + IY XZ YI ZX
  REC_DEP2_L2 = 5,   // all 15
};
constexpr uint32_t kRecComps[6] = {1, 2, 3, 6, 10, 15};
constexpr uint32_t kMaxPoint28 = (1u << 28) - 1;

inline uint64_t make_rec(uint32_t pa, uint32_t pb, uint32_t type, uint32_t Pa, uint32_t Pb) {
  return (uint64_t)(pa & kMaxPoint28) | ((uint64_t)(pb & kMaxPoint28) << 28) | ((uint64_t)(type & 15u) << 56) |
         ((uint64_t)(Pa & 3u) << 60) | ((uint64_t)(Pb & 3u) << 62);
}

constexpr uint32_t kNone = 0xFFFFFFFFu;

// Parsed instruction: gate id, args, a span of targets in a shared pool.
struct Instr {
  uint16_t gate;
  uint8_t nargs;
  uint8_t kinds;  // its targets: bit 0 some record target, 1 all records, 2 some Pauli target, 3 all Pauli
  uint32_t maxq;  // the largest qubit index (low 24 bits) among its targets
  double args[3];
  uint32_t t0, tn;
};
constexpr uint8_t kAnyRec = 1, kAllRec = 2, kAnyPau = 4, kAllPau = 8;

// A top-level statement that opens its line: the text offset of the line,
// its line number, and the instructions and targets parsed before it.
struct ParseMark {
  size_t off, line, ins, tpos;
};

struct Parsed {
  std::vector<Instr> ins;
  HostArray<uint32_t> pool;  // targets of every instruction (a REPEAT body's once)
  bool want_marks = false;   // record `marks` (the incremental lowering reads them)
  std::vector<ParseMark> marks;
  size_t end_line = 1;       // line number at the end of the text
};

// Parses stim circuit text, flattening REPEAT blocks.  Throws gpc::Error.
Parsed parse_stim(const char *text, size_t len);
// The same into `out`, whose buffers are reused.
void parse_stim_into(const char *text, size_t len, Parsed &out);

// A lowered circuit: everything the device pipeline needs.
// A tape's op array.  Its memory comes from the allocator its owner set
// (page-locked memory for the tapes a driver owns: the device copy of the ops
// is made straight from it) or, without one or when that allocator has none
// to give, from the heap.  resize() keeps no contents: the lowering writes
// every op after sizing the array.
class OpArray {
 public:
  using AllocFn = void *(*)(size_t bytes);
  using FreeFn = void (*)(void *, size_t bytes);  // bytes: as allocated
  OpArray() = default;
  OpArray(OpArray &&o) noexcept { take(o); }
  OpArray &operator=(OpArray &&o) noexcept {
    if (this != &o) {
      release();
      take(o);
    }
    return *this;
  }
  OpArray(const OpArray &) = delete;
  OpArray &operator=(const OpArray &) = delete;
  ~OpArray() { release(); }
  // Takes effect from the next allocation (a held buffer is released now).
  void set_allocator(AllocFn a, FreeFn f) {
    if (a == alloc_ && f == free_) return;
    release();
    alloc_ = a;
    free_ = f;
  }
  void resize(size_t n) {
    if (n > cap_) {
      release();
      const size_t want = n + n / 4;  // slack: page-locked allocations are slow
      void *q = alloc_ ? alloc_(want * sizeof(uint64_t)) : nullptr;
      ext_ = q != nullptr;
      if (!q) q = std::malloc(want * sizeof(uint64_t));
      if (!q) throw std::bad_alloc();
      p_ = static_cast<uint64_t *>(q);
      cap_ = want;
    }
    n_ = n;
  }
  void clear() { n_ = 0; }
  uint64_t *data() { return p_; }
  const uint64_t *data() const { return p_; }
  size_t size() const { return n_; }
  uint64_t &operator[](size_t i) { return p_[i]; }
  const uint64_t &operator[](size_t i) const { return p_[i]; }
  // The buffer came from the owner's allocator.
  bool external() const { return ext_; }

 private:
  void release() {
    if (p_) {
      if (ext_)
        free_(p_, cap_ * sizeof(uint64_t));
      else
        std::free(p_);
    }
    p_ = nullptr;
    n_ = cap_ = 0;
    ext_ = false;
  }
  void take(OpArray &o) {
    p_ = o.p_;
    n_ = o.n_;
    cap_ = o.cap_;
    ext_ = o.ext_;
    alloc_ = o.alloc_;
    free_ = o.free_;
    o.p_ = nullptr;
    o.n_ = o.cap_ = 0;
    o.ext_ = false;
  }
  uint64_t *p_ = nullptr;
  size_t n_ = 0, cap_ = 0;
  bool ext_ = false;
  AllocFn alloc_ = nullptr;
  FreeFn free_ = nullptr;
};

struct Tape {
  uint32_t nq = 0, qpad = 0, nmeas = 0, ndet = 0, nobs = 0, nbits = 0, w = 0;
  uint32_t n_epochs = 0, kmax = 0;
  OpArray ops;                      // sum_e K_e * qpad (every op written by the lowering)
  std::vector<uint32_t> ep_opoff;   // [n_epochs]     first op of epoch e
  std::vector<uint32_t> ep_k;       // [n_epochs]     slots in epoch e
  std::vector<uint32_t> ep_ptoff;   // [n_epochs + 1] first point of epoch e
  std::vector<uint32_t> ep_chunk;   // [n_epochs]     copy chunk holding epoch e
  std::vector<uint32_t> ch_off;     // [n_chunks]     first op of each chunk (= ep_opoff of its first epoch)
  std::vector<uint32_t> ch_bytes;   // [n_chunks]     bytes of each chunk (a whole number of epochs)
  uint32_t chunk_cap = 0;           // bytes of one shared-memory chunk buffer
  std::vector<uint32_t> inj_lo;     // [w] first epoch (walk order) injecting into word j, kNone if none
  std::vector<uint32_t> inj_hi;     // [w] last such epoch
  uint32_t npoints = 0;
  HostArray<uint64_t> rec;          // [R] noise records
  HostArray<double> rec_p;          // [R] probability of each of the record's mechanisms
  std::vector<uint32_t> rec_moff;   // [R + 1] first mechanism of each record
  uint32_t M = 0;                   // mechanisms (components)
  // Source of each record for the noise-rate gradient: tick * 4 + class, or
  // kNone.  The tick of an instruction is the number of TICKs before it;
  // classes: 0 DEPOLARIZE2, 1 DEPOLARIZE1, 2 measurement flip (X/Y/Z_ERROR
  // not directly after a reset of its qubit, or the flip argument of a
  // measurement), 3 reset flip (X/Y/Z_ERROR whose qubit's last operation was
  // a reset).  PAULI_CHANNEL_1 and E have no source.
  HostArray<uint32_t> rec_src;      // [R]
  uint32_t n_ticks = 1;             // TICK instructions + 1

  // Empties the tape, keeping the capacity of its arrays.
  void reset();
};

enum : uint32_t { SRC_DEP2 = 0, SRC_DEP1 = 1, SRC_MEAS_FLIP = 2, SRC_RESET_FLIP = 3, SRC_CLASSES = 4 };

// Smallest tape chunk for circuits compiled in a batch: chunks hold whole
// epochs, and small chunks (sized from the tape's largest epoch) let several
// walk CTAs share an SM.  A single circuit takes the largest chunk its walk's
// shared memory holds (fewer chunk switches on its latency-bound walk).
constexpr uint32_t kWalkChunkMin = 16 * 1024;

struct LowerOptions {
  int level = 2;     // correlation level 0/1/2
  uint32_t kcap = 8; // max slots per epoch
  uint32_t chunk_min = 0xFFFFFFFFu;  // smallest tape chunk (bytes; capped by the walk's shared memory)
  bool sources = true;  // fill Tape::rec_src (read by the noise-rate gradient only)
  // Target occurrences per time segment of the backward pass (at most 8
  // segments, of equal size).  Segments are scheduled on the host pool when
  // one is given; each cut adds at most about one epoch to the walk.  The
  // DEM does not depend on it.
  uint32_t segment_occ = 16384;
  // Keep this circuit's parse and time segments in the scratch, and lower the
  // next circuit of the same scratch against them: only the statements that
  // differ are parsed again, and a time segment whose instructions are
  // unchanged is scheduled again only if its measurements' detector bits or
  // its noise sources changed other than by one common shift (see
  // lower_text).  The tape equals a full lowering with the same segment cuts.
  bool incremental = false;
  // Cut the backward pass at these instruction indices (descending, from the
  // instruction count to 0) instead of by segment_occ.
  const std::vector<size_t> *cuts = nullptr;
};

// Shared-memory plan of the walk kernel (bytes): double-buffered tape chunks,
// the published rows, and the epoch/chunk tables when they fit.
constexpr uint32_t kWalkSmemBudget = 224 * 1024;  // of 227 KiB per CTA, leaving room for static shared memory
constexpr uint32_t kWalkTableBudget = 32 * 1024;  // most epoch/chunk table bytes a walk CTA stages
constexpr uint32_t kWalkChunkMax = 96 * 1024;
inline uint32_t walk_chunk_cap(uint32_t qpad) {
  const uint32_t pub = 2 * qpad * 16 + 128;
  if (pub + kWalkTableBudget >= kWalkSmemBudget) return 0;
  uint32_t c = (kWalkSmemBudget - pub - kWalkTableBudget) / 2;
  c = c < kWalkChunkMax ? c : kWalkChunkMax;
  return c & ~255u;
}

Tape lower(const Parsed &p, const LowerOptions &opt);

// Reusable host memory of parse + lower.  A caller that lowers circuit after
// circuit keeps one (per thread) and lowers into a kept Tape, so later
// circuits write memory that is already mapped instead of fresh pages.
struct LowerScratch {
  LowerScratch();
  ~LowerScratch();
  LowerScratch(LowerScratch &&) noexcept;
  LowerScratch &operator=(LowerScratch &&) noexcept;
  Parsed parsed;
  std::vector<Parsed> pieces;  // a text parsed in pieces on several threads
  struct Buffers;
  std::unique_ptr<Buffers> b;
  // The last lowering: its time segments (the backward pass's cuts,
  // descending instruction indices), how many were taken over from the
  // lowering before it, and how many text bytes were parsed.
  struct Stats {
    bool incremental = false;  // lowered against the scratch's previous circuit
    uint32_t segments = 0, reused = 0;
    size_t parsed_bytes = 0;
  } stats;
  const std::vector<size_t> &last_cuts() const;
  // Forget the previous circuit (the next incremental lowering is a full one).
  void forget();
};
// lower() into T (reset first), with S's buffers; a large tape is assembled
// in pieces on `pool`'s threads when a pool is given.
void lower_into(const Parsed &p, const LowerOptions &opt, Tape &T, LowerScratch &S, HostPool *pool = nullptr);
// parse_stim + lower_into, parsing into S.parsed (a large text in pieces on
// `pool`'s threads when a pool is given).
void lower_text(const char *text, size_t len, const LowerOptions &opt, Tape &T, LowerScratch &S,
                HostPool *pool = nullptr);
// parse_stim_into, cutting a large text without REPEAT blocks at line ends
// into pieces parsed on `pool`'s threads; the same result as one parse.
void parse_stim_pieces(const char *text, size_t len, Parsed &out, std::vector<Parsed> &pieces, HostPool &pool);

// ---- time segments of one circuit's walk ---------------------------------
// The walk of a word is affine over GF(2) in the rows it starts from: across
// epochs [a, b) the rows at b are A_ab * (rows at a) ^ c_ab, where A_ab (the
// Cliffords and resets, the same for every word) is a (2 qpad x 2 qpad) bit
// matrix and c_ab comes from the measurements in [a, b).  So a long walk can
// be cut at epoch boundaries into segments walked side by side, once each
// segment's entry rows are known (A and c of the segments before it, composed
// in walk order).  A cut must not split a measurement: its OP_INJ ops carry
// bits into the OP_M, and its OP_SNAPD reads the OP_M's bits, through
// per-slot registers.  Such a pair straddles an epoch boundary only when the
// later op was pushed into slot 0 of the next epoch, so an epoch whose slot 0
// holds no OP_INJ, OP_M or OP_SNAPD is a clean cut.
//
// Epoch cost in the walk's units: its slots plus two (a barrier and the
// publish of the rows cost about two slots' work).
inline uint32_t walk_epoch_cost(uint32_t slots) { return slots + 2u; }
// True if a segment may start at epoch e (0 < e < n_epochs).
bool walk_clean_cut(const Tape &T, uint32_t e);
// Cuts [0, n_epochs) into segments of about `target` cost units at clean
// cuts: bounds = {0 = b_0 < b_1 < ... < b_S = n_epochs}.  The last segment is
// merged into the one before when it would cost less than target / 2.
void walk_segment_bounds(const Tape &T, uint32_t target, std::vector<uint32_t> &bounds);

// Independent-component probability of DEPOLARIZE1(p) and DEPOLARIZE2(p)
// (Mixer.hpp:164,184): 0.5 - 0.5 sqrt(1 - 4p/3), 0.5 - 0.5 (1 - 16p/15)^(1/8).
double split_dep1(double p);
double split_dep2(double p);

}  // namespace gpc
