// lower.cpp -- stim text parser and the tick-tape lowering (see lower.hpp).
#include "lower.hpp"

#include "host_pool.hpp"

#include <algorithm>
#include <atomic>
#include <cctype>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <string_view>
#include <unordered_map>

#include "../../include/gpc.h"

namespace gpc {
namespace {

enum Kind : uint8_t { G_NOP, G_TICK, G_DET, G_OBS, G_PAULI, G_C1, G_C2, G_M, G_MR, G_R, G_N1, G_N2, G_CORR, G_MPAD };
enum { N1_X, N1_Y, N1_Z, N1_DEP1, N1_PC1 };

// Pauli masks: bit0 = X, bit1 = Z.  Two-qubit masks: bit0 Xa, bit1 Za, bit2 Xb, bit3 Zb.
struct Gate {
  const char *name;
  Kind kind;
  uint8_t a, b;       // C1: image masks of X and Z;  M/MR/R: basis;  N1: channel
  uint8_t img[4];     // C2: images of Xa, Za, Xb, Zb
  uint8_t nargs_min, nargs_max;
};

constexpr uint8_t XA = 1, ZA = 2, XB = 4, ZB = 8;

const Gate kGates[] = {
    {"TICK", G_TICK, 0, 0, {}, 0, 0},
    {"DETECTOR", G_DET, 0, 0, {}, 0, 255},
    {"OBSERVABLE_INCLUDE", G_OBS, 0, 0, {}, 1, 1},
    {"QUBIT_COORDS", G_NOP, 0, 0, {}, 0, 255},
    {"SHIFT_COORDS", G_NOP, 0, 0, {}, 0, 255},
    {"MPAD", G_MPAD, 0, 0, {}, 0, 1},
    {"I", G_PAULI, 0, 0, {}, 0, 0},
    {"X", G_PAULI, 0, 0, {}, 0, 0},
    {"Y", G_PAULI, 0, 0, {}, 0, 0},
    {"Z", G_PAULI, 0, 0, {}, 0, 0},
    {"H", G_C1, 2, 1, {}, 0, 0},
    {"H_XZ", G_C1, 2, 1, {}, 0, 0},
    {"H_XY", G_C1, 3, 2, {}, 0, 0},
    {"H_YZ", G_C1, 1, 3, {}, 0, 0},
    {"S", G_C1, 3, 2, {}, 0, 0},
    {"SQRT_Z", G_C1, 3, 2, {}, 0, 0},
    {"S_DAG", G_C1, 3, 2, {}, 0, 0},
    {"SQRT_Z_DAG", G_C1, 3, 2, {}, 0, 0},
    {"SQRT_X", G_C1, 1, 3, {}, 0, 0},
    {"SQRT_X_DAG", G_C1, 1, 3, {}, 0, 0},
    {"SQRT_Y", G_C1, 2, 1, {}, 0, 0},
    {"SQRT_Y_DAG", G_C1, 2, 1, {}, 0, 0},
    {"C_XYZ", G_C1, 3, 1, {}, 0, 0},
    {"C_ZYX", G_C1, 2, 3, {}, 0, 0},
    {"CX", G_C2, 0, 0, {XA | XB, ZA, XB, ZA | ZB}, 0, 0},
    {"CNOT", G_C2, 0, 0, {XA | XB, ZA, XB, ZA | ZB}, 0, 0},
    {"ZCX", G_C2, 0, 0, {XA | XB, ZA, XB, ZA | ZB}, 0, 0},
    {"CZ", G_C2, 0, 0, {XA | ZB, ZA, ZA | XB, ZB}, 0, 0},
    {"ZCZ", G_C2, 0, 0, {XA | ZB, ZA, ZA | XB, ZB}, 0, 0},
    {"CY", G_C2, 0, 0, {XA | XB | ZB, ZA, ZA | XB, ZA | ZB}, 0, 0},
    {"ZCY", G_C2, 0, 0, {XA | XB | ZB, ZA, ZA | XB, ZA | ZB}, 0, 0},
    {"XCZ", G_C2, 0, 0, {XA, ZA | ZB, XA | XB, ZB}, 0, 0},
    {"XCX", G_C2, 0, 0, {XA, ZA | XB, XB, XA | ZB}, 0, 0},
    {"SWAP", G_C2, 0, 0, {XB, ZB, XA, ZA}, 0, 0},
    {"M", G_M, 0, 0, {}, 0, 1},
    {"MZ", G_M, 0, 0, {}, 0, 1},
    {"MX", G_M, 1, 0, {}, 0, 1},
    {"MY", G_M, 2, 0, {}, 0, 1},
    {"MR", G_MR, 0, 0, {}, 0, 1},
    {"MRZ", G_MR, 0, 0, {}, 0, 1},
    {"MRX", G_MR, 1, 0, {}, 0, 1},
    {"MRY", G_MR, 2, 0, {}, 0, 1},
    {"R", G_R, 0, 0, {}, 0, 0},
    {"RZ", G_R, 0, 0, {}, 0, 0},
    {"RX", G_R, 1, 0, {}, 0, 0},
    {"RY", G_R, 2, 0, {}, 0, 0},
    {"X_ERROR", G_N1, N1_X, 0, {}, 1, 1},
    {"Y_ERROR", G_N1, N1_Y, 0, {}, 1, 1},
    {"Z_ERROR", G_N1, N1_Z, 0, {}, 1, 1},
    {"DEPOLARIZE1", G_N1, N1_DEP1, 0, {}, 1, 1},
    {"PAULI_CHANNEL_1", G_N1, N1_PC1, 0, {}, 3, 3},
    {"DEPOLARIZE2", G_N2, 0, 0, {}, 1, 1},
    {"E", G_CORR, 0, 0, {}, 1, 1},
    {"CORRELATED_ERROR", G_CORR, 0, 0, {}, 1, 1},
};
constexpr int kNumGates = sizeof(kGates) / sizeof(kGates[0]);

const std::unordered_map<std::string_view, int> &gateIndex() {
  static const std::unordered_map<std::string_view, int> m = [] {
    std::unordered_map<std::string_view, int> r;
    for (int i = 0; i < kNumGates; ++i) r.emplace(kGates[i].name, i);
    return r;
  }();
  return m;
}

// Target encoding in the pool: qubit q -> q; rec[-k] -> kRec | k;
// Pauli target P q -> kPau | P << 24 | q (P: 1 X, 2 Z, 3 Y).
constexpr uint32_t kRec = 0x80000000u;
constexpr uint32_t kPau = 0x40000000u;
constexpr uint32_t kMaxQubit = 1u << 24;

// ASCII character classes (the locale-aware <cctype> calls cost a call per byte).
inline bool is_digit(char c) { return (unsigned)(c - '0') < 10u; }
inline bool is_name_char(char c) {
  return is_digit(c) || (unsigned)((c | 0x20) - 'a') < 26u || c == '_';
}
inline char to_upper(char c) { return (unsigned)(c - 'a') < 26u ? (char)(c - 32) : c; }

struct TextParser {
  const char *s, *e;
  size_t line = 1;
  Parsed *out;
  const char *s0 = nullptr;  // start of the text (offsets of the marks)
  const char *ls = nullptr;  // start of the current line
  // targets are written through this cursor into out->pool, sized up front:
  // targets are separated by whitespace, so a text of n bytes holds at most
  // n / 2 + 1 of them (a REPEAT body's are stored once)
  uint32_t *tw = nullptr;
  // the gate of the previous instruction line (consecutive lines repeat names, e.g. DETECTOR)
  char last_name[40] = {0};
  size_t last_len = 0;
  int last_gate = -1;

  [[noreturn]] void fail(int code, const std::string &m) { throw Error(code, "line " + std::to_string(line) + ": " + m); }
  void sp() {
    while (s < e && (*s == ' ' || *s == '\t' || *s == '\r')) ++s;
  }
  uint32_t uint() {
    if (s >= e || *s < '0' || *s > '9') fail(GPC_ERR_PARSE, "expected an integer");
    uint64_t v = 0;
    while (s < e && *s >= '0' && *s <= '9') {
      v = v * 10 + (uint64_t)(*s++ - '0');
      if (v > 0xFFFFFFFull) fail(GPC_ERR_PARSE, "integer out of range");
    }
    return (uint32_t)v;
  }

  // Parses statements into `dst` until '}' or the end of the text.
  void block(std::vector<Instr> &dst, bool inner, int depth) {
    if (depth > 64) fail(GPC_ERR_PARSE, "REPEAT nesting too deep");
    char name[40];
    while (true) {
      sp();
      if (s >= e) {
        if (inner) fail(GPC_ERR_PARSE, "unterminated REPEAT block");
        return;
      }
      char c = *s;
      if (c == '\n') {
        ++s;
        ++line;
        ls = s;
        continue;
      }
      if (c == '#') {
        while (s < e && *s != '\n') ++s;
        continue;
      }
      if (c == '}') {
        if (!inner) fail(GPC_ERR_PARSE, "unmatched '}'");
        ++s;
        return;
      }
      if (depth == 0 && out->want_marks) {
        // a top-level statement that opens its line: a place where the text
        // may be re-parsed from (the incremental lowering)
        const char *q = ls;
        while (q < s && (*q == ' ' || *q == '\t' || *q == '\r')) ++q;
        if (q == s)
          out->marks.push_back({(size_t)(ls - s0), line, dst.size(), (size_t)(tw - out->pool.data())});
      }
      size_t n = 0;
      while (s < e && is_name_char(*s)) {
        if (n + 1 >= sizeof(name)) fail(GPC_ERR_PARSE, "instruction name too long");
        name[n++] = to_upper(*s++);
      }
      name[n] = 0;
      if (n == 0) fail(GPC_ERR_PARSE, std::string("unexpected character '") + c + "'");
      if (s < e && *s == '[') {  // tag: ignored
        while (s < e && *s != ']' && *s != '\n') ++s;
        if (s >= e || *s != ']') fail(GPC_ERR_PARSE, "unterminated tag");
        ++s;
      }
      std::string_view nv(name, n);
      if (nv == "REPEAT") {
        sp();
        uint32_t reps = uint();
        sp();
        if (s >= e || *s != '{') fail(GPC_ERR_PARSE, "expected '{' after REPEAT count");
        ++s;
        std::vector<Instr> body;
        block(body, true, depth + 1);
        if ((uint64_t)reps * body.size() + dst.size() > (1ull << 31)) fail(GPC_ERR_CAPACITY, "circuit too long");
        dst.reserve(dst.size() + (size_t)reps * body.size());
        for (uint32_t r = 0; r < reps; ++r) dst.insert(dst.end(), body.begin(), body.end());
        continue;
      }
      int gi;
      if (n == last_len && last_gate >= 0 && memcmp(name, last_name, n) == 0) {
        gi = last_gate;
      } else {
        auto it = gateIndex().find(nv);
        if (it == gateIndex().end()) fail(GPC_ERR_UNSUPPORTED, "unsupported instruction " + std::string(nv));
        gi = it->second;
        memcpy(last_name, name, n);
        last_len = n;
        last_gate = gi;
      }
      const Gate &g = kGates[gi];
      Instr in{};
      in.gate = (uint16_t)gi;
      double args[3];
      int na = 0;
      if (s < e && *s == '(') {
        ++s;
        while (true) {
          sp();
          char *endp = nullptr;
          double v = strtod(s, &endp);
          if (endp == s) fail(GPC_ERR_PARSE, "bad argument");
          s = endp;
          if (na < 3) args[na] = v;
          ++na;
          sp();
          if (s < e && *s == ',') {
            ++s;
            continue;
          }
          if (s < e && *s == ')') {
            ++s;
            break;
          }
          fail(GPC_ERR_PARSE, "bad argument list");
        }
      }
      if (g.nargs_max != 255 && (na < g.nargs_min || na > g.nargs_max))
        fail(GPC_ERR_PARSE, std::string(g.name) + ": wrong number of arguments");
      in.nargs = (uint8_t)std::min(na, 3);
      for (int i = 0; i < in.nargs; ++i) in.args[i] = args[i];
      uint32_t *const t0 = tw;
      in.t0 = (uint32_t)(t0 - out->pool.data());
      // plain qubit indices and record targets (most targets), with the
      // cursors in locals the compiler keeps in registers; the loop below, on
      // the members, takes over at the first target of another kind (or one
      // it must report)
      uint32_t orf = 0, andf = 0xFFFFFFFFu, mx = 0;  // kind bits ORed and ANDed, the largest index
      {
        const char *p = s, *const end = e;
        uint32_t *w = tw;
        while (true) {
          while (p < end && (*p == ' ' || *p == '\t')) ++p;
          if (p >= end) break;
          unsigned d = (unsigned)(*p - '0');
          if (d < 10u) {
            const char *const d0 = p++;
            uint64_t q = d;
            while (p < end && (d = (unsigned)(*p - '0')) < 10u) {
              q = q * 10u + d;
              ++p;
            }
            if (p - d0 > 9 || q >= kMaxQubit) {
              s = p;
              tw = w;
              fail(GPC_ERR_CAPACITY, "qubit index too large");
            }
            *w++ = (uint32_t)q;
            andf = 0;
            mx = std::max(mx, (uint32_t)q);
            continue;
          }
          if (end - p < 7 || memcmp(p, "rec[-", 5) != 0) break;
          const char *r = p + 5, *const k0 = r;
          uint64_t k = 0;
          while (r < end && (d = (unsigned)(*r - '0')) < 10u && r - k0 < 9) {
            k = k * 10u + d;
            ++r;
          }
          if (r >= end || *r != ']' || k == 0 || k > 0xFFFFFFFull) break;
          p = r + 1;
          *w++ = kRec | (uint32_t)k;
          orf |= kRec;
          andf &= kRec;
          mx = std::max(mx, (uint32_t)k & 0xFFFFFFu);
        }
        s = p;
        tw = w;
      }
      uint32_t *const t1 = tw;  // (targets past t1 came from the general loop)
      while (true) {
        while (s < e && (*s == ' ' || *s == '\t')) ++s;
        if (s >= e) break;
        const char c0 = *s;
        if (is_digit(c0)) {  // fast path: a plain qubit index
          const char *d0 = s;
          uint64_t q = (uint32_t)(c0 - '0');
          ++s;
          while (s < e && is_digit(*s)) q = q * 10u + (uint32_t)(*s++ - '0');
          if (s - d0 > 9 || q >= kMaxQubit) fail(GPC_ERR_CAPACITY, "qubit index too large");
          *tw++ = (uint32_t)q;
          continue;
        }
        if (c0 == '\n' || c0 == '#' || c0 == '\r') break;
        if (*s == '!') ++s;  // inverted measurement result: no effect on sensitivities
        if (s >= e) fail(GPC_ERR_PARSE, "bad target");
        if (*s == '*') fail(GPC_ERR_UNSUPPORTED, "combiner targets are not supported");
        if (e - s >= 4 && memcmp(s, "rec[", 4) == 0) {
          s += 4;
          if (s >= e || *s != '-') fail(GPC_ERR_PARSE, "expected rec[-k]");
          ++s;
          uint32_t k = uint();
          if (s >= e || *s != ']' || k == 0) fail(GPC_ERR_PARSE, "bad record target");
          ++s;
          *tw++ = kRec | k;
        } else if (*s == 'X' || *s == 'Y' || *s == 'Z' || *s == 'x' || *s == 'y' || *s == 'z') {
          char p = to_upper(*s++);
          uint32_t q = uint();
          if (q >= kMaxQubit) fail(GPC_ERR_CAPACITY, "qubit index too large");
          *tw++ = kPau | ((uint32_t)(p == 'X' ? 1 : p == 'Z' ? 2 : 3) << 24) | q;
        } else if ((unsigned)(*s - '0') < 10u) {
          uint32_t q = uint();
          if (q >= kMaxQubit) fail(GPC_ERR_CAPACITY, "qubit index too large");
          *tw++ = q;
        } else if (e - s >= 6 && memcmp(s, "sweep[", 6) == 0) {
          fail(GPC_ERR_UNSUPPORTED, "sweep targets are not supported");
        } else {
          fail(GPC_ERR_PARSE, "bad target");
        }
      }
      in.tn = (uint32_t)(tw - t0);
      // the target checks of the lowering, made here while the targets are in
      // cache (those of the register loop above summed up as it went)
      uint32_t orv = orf, andv = andf, maxq = mx;
      for (const uint32_t *p = t1; p < tw; ++p) {
        orv |= *p;
        andv &= *p;
        maxq = std::max(maxq, *p & 0xFFFFFFu);
      }
      in.maxq = maxq;
      in.kinds = (uint8_t)((orv & kRec ? kAnyRec : 0) | (in.tn && (andv & kRec) ? kAllRec : 0) |
                           (orv & kPau ? kAnyPau : 0) | (in.tn && (andv & kPau) ? kAllPau : 0));
      if ((g.kind == G_C2 || g.kind == G_N2) && in.tn % 2 == 0)
        for (uint32_t k = 0; k < in.tn; k += 2)
          if (t0[k] == t0[k + 1]) fail(GPC_ERR_PARSE, std::string(g.name) + " on a single qubit");
      dst.push_back(in);
    }
  }
};


// Independent X, Y, Z probabilities equivalent to the disjoint channel
// (px, py, pz): with lambda_P = 1 - 2 P(anticommuting with P), independent
// channels give lambda_X = (1-2qy)(1-2qz), so 1-2qx = sqrt(lambda_Y lambda_Z / lambda_X).
bool pc1_independent(double px, double py, double pz, double q[3]) {
  double lx = 1 - 2 * (py + pz), ly = 1 - 2 * (px + pz), lz = 1 - 2 * (px + py);
  if (lx <= 0 || ly <= 0 || lz <= 0) return false;
  q[0] = 0.5 - 0.5 * std::sqrt(ly * lz / lx);
  q[1] = 0.5 - 0.5 * std::sqrt(lx * lz / ly);
  q[2] = 0.5 - 0.5 * std::sqrt(lx * ly / lz);
  return q[0] >= 0 && q[1] >= 0 && q[2] >= 0;
}

// Swaps the qubit halves of a two-qubit mask (Xa,Za,Xb,Zb) -> (Xb,Zb,Xa,Za).
uint32_t swap_halves(uint32_t m) { return ((m >> 2) & 3u) | ((m & 3u) << 2); }

// A two-qubit Clifford update for one side, as a single-XOR opcode when the
// masks allow (bits: 0 self X, 1 self Z, 2 partner X, 3 partner Z; newX in
// the low nibble, newZ in the high nibble).
uint64_t c2_op(uint32_t sub, uint32_t partner) {
  const uint32_t nx = sub & 15u, nz = sub >> 4;
  if (nz == 2u && nx == (1u | 4u)) return make_op(OP_XPX, 0, partner);
  if (nx == 1u && nz == (2u | 8u)) return make_op(OP_ZPZ, 0, partner);
  if (nz == 2u && nx == (1u | 8u)) return make_op(OP_XPZ, 0, partner);
  return make_op(OP_C2, sub, partner);
}

// One tape entry placed by the backward scheduler: qubit, epoch, slot, op.
struct Entry {
  uint32_t qk;  // qubit | slot << 24
  uint32_t e;
  uint64_t op;
  uint32_t q() const { return qk & 0xFFFFFFu; }
  uint32_t k() const { return qk >> 24; }
};

constexpr uint64_t kFnvBasis = 0xcbf29ce484222325ull, kFnvPrime = 0x100000001b3ull;  // FNV-1a 64

struct QState {
  int64_t last = -1;      // epoch of the latest entry
  uint32_t cnt = 0;       // entries in that epoch
  uint32_t open = kNone;  // point holding the current rows (until a row-changing op)
  // the qubit's op signatures in this segment (see the qubit packing), hashed
  // as its entries are placed: op kinds, and op kinds with their epochs
  uint64_t coarse = kFnvBasis, fine = kFnvBasis;
  void sign(uint64_t op, uint32_t e) {
    const uint32_t opc = (uint32_t)(op & 0xFF);
    if (opc == OP_INJ || opc == OP_SNAPD) return;  // vary with detector membership only
    coarse = (coarse ^ opc) * kFnvPrime;
    fine = (fine ^ (opc | ((uint64_t)e << 8))) * kFnvPrime;
  }
};

// Counts of a run of instructions (the forward pass's first pass), or the
// counts before an instruction (its starting counts).
struct FwdCount {
  uint64_t occ = 0, ndp = 0, nop = 0;  // target occurrences, detector pairs, observable pairs
  uint32_t m = 0, ndet = 0, nobs = 0, nq = 0;
};

// A run of equal lines of two texts: a[a, a + n) equals b[b, b + n).
struct Run {
  size_t a, b, n;
};

// Memoises the last split so uniform noise costs one sqrt/pow per distinct p.
struct SplitCache {
  double p1 = -1, s1 = 0, p2 = -1, s2 = 0;
  double dep1(double p) {
    if (p != p1) {
      p1 = p;
      s1 = split_dep1(p);
    }
    return s1;
  }
  double dep2(double p) {
    if (p != p2) {
      p2 = p;
      s2 = split_dep2(p);
    }
    return s2;
  }
};

}  // namespace

bool walk_clean_cut(const Tape &T, uint32_t e) {
  if (e == 0 || e >= T.n_epochs) return false;
  const uint64_t *op = T.ops.data() + T.ep_opoff[e];  // slot 0 of epoch e
  for (uint32_t s = 0; s < T.qpad; ++s) {
    const uint32_t opc = (uint32_t)op[s] & 0xFFu;
    if (opc == OP_INJ || opc == OP_M || opc == OP_SNAPD) return false;
  }
  return true;
}

void walk_segment_bounds(const Tape &T, uint32_t target, std::vector<uint32_t> &bounds) {
  const uint32_t nE = T.n_epochs;
  bounds.clear();
  bounds.push_back(0);
  if (nE == 0) return;
  target = std::max(1u, target);
  uint64_t acc = 0;
  for (uint32_t e = 0; e < nE; ++e) {
    if (acc >= target && walk_clean_cut(T, e)) {
      bounds.push_back(e);
      acc = 0;
    }
    acc += walk_epoch_cost(T.ep_k[e]);
  }
  if (bounds.size() > 1 && acc * 2 < target) bounds.pop_back();
  bounds.push_back(nE);
}

double split_dep1(double p) { return 0.5 - 0.5 * std::sqrt(1.0 - (4.0 * p) / 3.0); }
double split_dep2(double p) { return 0.5 - 0.5 * std::pow(1.0 - (16.0 * p) / 15.0, 0.125); }

void parse_stim_into(const char *text, size_t len, Parsed &p) {
  p.ins.clear();
  p.marks.clear();
  if (!text && len) throw Error(GPC_ERR_INVALID, "null circuit text");
  p.pool.resize(len / 2 + 16);  // the most targets a text of len bytes holds (not initialised)
  p.ins.reserve(len / 64 + 16);
  TextParser tp{text, text + len, 1, &p};
  tp.s0 = tp.ls = text;
  tp.tw = p.pool.data();
  try {
    tp.block(p.ins, false, 0);
  } catch (...) {
    p.pool.clear();
    throw;
  }
  p.pool.resize((size_t)(tp.tw - p.pool.data()));
  p.end_line = tp.line;
}

Parsed parse_stim(const char *text, size_t len) {
  Parsed p;
  parse_stim_into(text, len, p);
  return p;
}

void Tape::reset() {
  nq = qpad = nmeas = ndet = nobs = nbits = w = 0;
  n_epochs = kmax = 0;
  for (auto *v : {&ep_opoff, &ep_k, &ep_ptoff, &ep_chunk, &ch_off, &ch_bytes, &inj_lo, &inj_hi, &rec_moff})
    v->clear();
  ops.clear();
  rec.clear();
  rec_p.clear();
  rec_src.clear();
  chunk_cap = 0;
  npoints = 0;
  M = 0;
  n_ticks = 1;
}

// A grow-only array whose elements are left uninitialised (filled before use).
template <typename T>
struct RawArray {
  std::unique_ptr<T[]> p;
  size_t cap = 0;
  T *get(size_t n) {
    if (n > cap) {
      p.reset(new T[n]);
      cap = n;
    }
    return p.get();
  }
};

struct LowerScratch::Buffers {
  std::vector<uint32_t> measBase, occBase, tsrc, moff, mbits, measLo, measHi, slotOf, order, remap, ep_np;
  std::vector<std::pair<uint32_t, uint32_t>> detPairs, obsPairs, groups;
  std::vector<uint8_t> lastReset;
  // one time segment of the backward pass (its entries, epochs, points and records)
  struct Segment {
    RawArray<Entry> ent;
    size_t nent = 0;
    std::vector<QState> st;
    std::vector<uint32_t> ep_k, ep_np;
    HostArray<uint64_t> rec;
    HostArray<double> rec_p;
    HostArray<uint32_t> rec_src;
    size_t nrec = 0, roff = 0;
    uint64_t ncomp = 0, moff0 = 0;  // the segment's mechanisms, and those of the records before it
    uint32_t nprov = 0, eoff = 0, poff = 0;
    std::vector<uint64_t> fine, coarse;  // per-qubit op signatures of the segment (qubit packing)
    std::vector<uint64_t> snapbits;      // bit i: op oa + i of the segment's tape range is a snapshot
    std::vector<uint32_t> mlo, mhi;      // its measurements' first/last epochs (segment-local; incremental)
  };
  std::vector<Segment> segs;
  std::vector<size_t> cut;
  std::vector<uint64_t> fine, coarse;

  // ---- incremental lowering ----
  // The previous circuit of this scratch: its text, and (swapped out of the
  // arrays above when the next circuit is lowered against it) its forward-pass
  // arrays, cuts and segments.
  struct Prev {
    bool valid = false;
    std::string text;
    std::vector<uint32_t> measBase, occBase, tsrc, moff, mbits;
    std::vector<size_t> cut;
    std::vector<Segment> segs;
    size_t n_ins = 0, nocc = 0;
    uint32_t nmeas = 0, nq = 0, kcap = 0;
    int level = -1;
    bool sources = false;
  } prev;
  // Set by the planner for the next lower_into: the cuts, and for each new
  // segment the previous segment over the same statements (or -1).
  struct Plan {
    bool active = false;
    std::vector<size_t> cut;
    std::vector<int32_t> from;
  } plan;
  Parsed next;               // the new parse, assembled
  std::vector<Parsed> gaps;  // the statements parsed again
  std::vector<size_t> la, lb;
  std::vector<long> vbuf, trace;
  std::vector<Run> runs_;
  std::vector<uint32_t> runs;  // segments scheduled by this lowering
  std::vector<int64_t> dbits, dsrc;  // per reused segment: shift of its detector bits and sources
  // The forward pass done beside a parse in pieces (its arrays above), for
  // the parse `fwd_of` of fwd_ins instructions: totals in fwd.
  const Parsed *fwd_of = nullptr;
  size_t fwd_ins = 0;
  FwdCount fwd;
  std::vector<FwdCount> fwd_pc;
};

LowerScratch::LowerScratch() : b(new Buffers) {}
LowerScratch::~LowerScratch() = default;
LowerScratch::LowerScratch(LowerScratch &&) noexcept = default;
LowerScratch &LowerScratch::operator=(LowerScratch &&) noexcept = default;
const std::vector<size_t> &LowerScratch::last_cuts() const { return b->cut; }
void LowerScratch::forget() {
  b->prev.valid = false;
  b->plan.active = false;
}

namespace {

// ---- the forward pass over a run of instructions ----------------------------
// Checks that need no running count: an instruction's targets' kinds
// (summarised by the parser) and, after the counts, its arguments.
void check_targets(const Instr &in, const Gate &g) {
  if (!in.tn) return;
  if (g.kind == G_DET || g.kind == G_OBS) {
    if (!(in.kinds & kAllRec)) throw Error(GPC_ERR_PARSE, std::string(g.name) + " takes record targets only");
  } else if (in.kinds & kAnyRec) {
    throw Error(GPC_ERR_UNSUPPORTED, std::string("record targets are not supported on ") + g.name);
  } else if (g.kind == G_MPAD) {
    if (in.maxq > 1 || (in.kinds & kAnyPau)) throw Error(GPC_ERR_PARSE, "MPAD targets must be 0 or 1");
  } else if (g.kind == G_CORR) {
    if (!(in.kinds & kAllPau)) throw Error(GPC_ERR_PARSE, "E takes Pauli targets");
  } else if (in.kinds & kAnyPau) {
    throw Error(GPC_ERR_PARSE, std::string("Pauli targets are not allowed on ") + g.name);
  }
}
// qubits: the targets of every instruction but detectors, observables and MPAD
bool counts_qubits(const Instr &in, const Gate &g) {
  return in.tn && g.kind != G_DET && g.kind != G_OBS && g.kind != G_MPAD;
}
uint32_t obs_index(const Instr &in) {
  const double a = in.args[0];
  if (!(a >= 0) || a != std::floor(a) || a > 1e6) throw Error(GPC_ERR_PARSE, "bad observable index");
  return (uint32_t)a;
}
void check_pairs(const Instr &in, const Gate &g) {  // (the parser checked that no pair names one qubit twice)
  if ((g.kind == G_C2 || g.kind == G_N2) && in.tn % 2)
    throw Error(GPC_ERR_PARSE, std::string(g.name) + " needs an even number of targets");
}
void check_args(const Instr &in, const Gate &g) {
  auto prob = [&](double p) {
    if (!(p >= 0 && p <= 1)) throw Error(GPC_ERR_PARSE, std::string(g.name) + ": probability out of range");
  };
  if (g.kind == G_N1 || g.kind == G_N2 || g.kind == G_CORR || ((g.kind == G_M || g.kind == G_MR || g.kind == G_MPAD) && in.nargs))
    for (int k = 0; k < in.nargs; ++k) prob(in.args[k]);
  if (g.kind == G_N1 && g.a == N1_DEP1 && in.args[0] > 0.75) throw Error(GPC_ERR_PARSE, "DEPOLARIZE1 p > 0.75");
  if (g.kind == G_N2 && in.args[0] > 0.9375) throw Error(GPC_ERR_PARSE, "DEPOLARIZE2 p > 0.9375");
  if (g.kind == G_N1 && g.a == N1_PC1) {
    double q[3];
    if (!pc1_independent(in.args[0], in.args[1], in.args[2], q))
      throw Error(GPC_ERR_UNSUPPORTED, "PAULI_CHANNEL_1 is not a product of independent X, Y, Z channels");
  }
  if (g.kind == G_MPAD && in.nargs && in.args[0] > 0) throw Error(GPC_ERR_UNSUPPORTED, "noisy MPAD is not supported");
}

// First pass over ins[0, n): counts and checks (throws on a failed check;
// the lookbacks are checked by the second pass).
void forward_count(const Instr *ins, size_t n, FwdCount &c) {
  for (size_t i = 0; i < n; ++i) {
    const Instr &in = ins[i];
    const Gate &g = kGates[in.gate];
    c.occ += in.tn;
    check_targets(in, g);
    if (counts_qubits(in, g)) c.nq = std::max(c.nq, in.maxq + 1);
    switch (g.kind) {
      case G_M:
      case G_MR:
      case G_MPAD:
        c.m += in.tn;
        break;
      case G_DET:
        c.ndp += in.tn;
        ++c.ndet;
        break;
      case G_OBS:
        c.nop += in.tn;
        c.nobs = std::max(c.nobs, obs_index(in) + 1);
        break;
      default:
        check_pairs(in, g);
        break;
    }
    check_args(in, g);
  }
}

// Second pass over ins[0, n) (targets at tp[t0]) from the starting counts c:
// measurement and occurrence bases at mb and ob, pairs at dp and op (throws
// on a lookback beyond the start of the circuit).
void forward_write(const Instr *ins, size_t n, const uint32_t *tp, const FwdCount &c, uint32_t *mb, uint32_t *ob,
                   std::pair<uint32_t, uint32_t> *dp, std::pair<uint32_t, uint32_t> *op) {
  uint32_t mm = c.m, nd = c.ndet;
  uint64_t oc = c.occ;
  for (size_t i = 0; i < n; ++i) {
    const Instr &in = ins[i];
    const Gate &g = kGates[in.gate];
    const uint32_t *t = tp + in.t0;
    mb[i] = mm;
    ob[i] = (uint32_t)oc;
    oc += in.tn;
    if (g.kind == G_M || g.kind == G_MR || g.kind == G_MPAD) {
      mm += in.tn;
    } else if (g.kind == G_DET || g.kind == G_OBS) {
      const bool det = g.kind == G_DET;
      const uint32_t id = det ? nd++ : (uint32_t)in.args[0];
      std::pair<uint32_t, uint32_t> *&at = det ? dp : op;
      for (uint32_t k = 0; k < in.tn; ++k) {
        const uint32_t back = t[k] & ~kRec;
        if (back > mm) throw Error(GPC_ERR_PARSE, "record lookback beyond the start of the circuit");
        *at++ = {mm - back, id};
      }
    }
  }
}

// Running counts: pc[k + 1] holds run k's own counts; afterwards pc[k] holds
// the counts before run k and pc[n] the totals (nq and nobs as maxima).
void forward_prefix(std::vector<FwdCount> &pc, size_t n) {
  for (size_t k = 0; k < n; ++k) {
    FwdCount &a = pc[k + 1];
    const FwdCount &b = pc[k];
    a.occ += b.occ;
    a.ndp += b.ndp;
    a.nop += b.nop;
    a.m += b.m;
    a.ndet += b.ndet;
    a.nq = std::max(a.nq, b.nq);
    a.nobs = std::max(a.nobs, b.nobs);
  }
}

// A text parsed in pieces on the pool (see parse_stim_pieces); with `fw`,
// the forward pass runs beside it: each piece is counted and checked right
// after it is parsed and written out beside its concatenation.  A failed
// forward check leaves fw->fwd_of null (the lowering then reports it).
void parse_pieces(const char *text, size_t len, Parsed &out, std::vector<Parsed> &pieces, HostPool &pool,
                  LowerScratch::Buffers *fw);

}  // namespace

void parse_stim_pieces(const char *text, size_t len, Parsed &out, std::vector<Parsed> &pieces, HostPool &pool) {
  parse_pieces(text, len, out, pieces, pool, nullptr);
}

namespace {
void parse_pieces(const char *text, size_t len, Parsed &out, std::vector<Parsed> &pieces, HostPool &pool,
                  LowerScratch::Buffers *fw) {
  if (fw) fw->fwd_of = nullptr;
  constexpr size_t kPieceMin = 16 * 1024;
  const size_t want = std::min<size_t>({(size_t)pool.workers() + 1, 16, len / kPieceMin});
  // a REPEAT block may not be cut: such texts (short ones, usually) parse whole
  if (want < 2 || !text || memchr(text, '{', len)) {
    parse_stim_into(text, len, out);
    return;
  }
  std::vector<size_t> cut{0};
  for (size_t i = 1; i < want; ++i) {
    size_t c = std::max(cut.back(), len * i / want);
    const void *nl = memchr(text + c, '\n', len - c);
    c = nl ? (size_t)(static_cast<const char *>(nl) - text) + 1 : len;
    if (c > cut.back() && c < len) cut.push_back(c);
  }
  cut.push_back(len);
  const uint32_t np = (uint32_t)cut.size() - 1;
  if (pieces.size() < np) pieces.resize(np);
  for (uint32_t i = 0; i < np; ++i) pieces[i].want_marks = out.want_marks;
  std::atomic<bool> fw_ok{fw != nullptr};
  if (fw) fw->fwd_pc.assign(np + 1, FwdCount{});
  try {
    pool.run(np, [&](uint32_t i, uint32_t) {
      parse_stim_into(text + cut[i], cut[i + 1] - cut[i], pieces[i]);
      if (fw_ok) try {
          forward_count(pieces[i].ins.data(), pieces[i].ins.size(), fw->fwd_pc[i + 1]);
        } catch (const Error &) {
          fw_ok = false;
        }
    });
  } catch (const Error &) {
    parse_stim_into(text, len, out);  // the error again, with its line number in the whole text
    return;
  }
  // the pieces' instructions and targets, concatenated (each piece on the pool)
  std::vector<size_t> ioff(np + 1, 0), toff(np + 1, 0);
  for (uint32_t i = 0; i < np; ++i) {
    ioff[i + 1] = ioff[i] + pieces[i].ins.size();
    toff[i + 1] = toff[i] + pieces[i].pool.size();
  }
  if (toff[np] > 0xFFFFFFFFull) throw Error(GPC_ERR_CAPACITY, "circuit too long");
  out.ins.resize(ioff[np]);
  out.pool.resize(toff[np]);
  out.marks.clear();
  size_t line0 = 0;
  for (uint32_t i = 0; i < np; ++i) {
    for (const ParseMark &k : pieces[i].marks)
      out.marks.push_back({k.off + cut[i], k.line + line0, k.ins + ioff[i], k.tpos + toff[i]});
    line0 += pieces[i].end_line - 1;
  }
  out.end_line = line0 + 1;
  if (fw_ok) {
    forward_prefix(fw->fwd_pc, np);
    const FwdCount &tot = fw->fwd_pc[np];
    if (tot.occ > 0xFFFFFFFFull / 4) {
      fw_ok = false;
    } else {
      fw->measBase.resize(ioff[np]);
      fw->occBase.resize(ioff[np]);
      fw->detPairs.resize(tot.ndp);
      fw->obsPairs.resize(tot.nop);
    }
  }
  pool.run(np, [&](uint32_t i, uint32_t) {
    const Parsed &pc = pieces[i];
    if (fw_ok) try {
        const FwdCount &c = fw->fwd_pc[i];
        forward_write(pc.ins.data(), pc.ins.size(), pc.pool.data(), c, fw->measBase.data() + ioff[i],
                      fw->occBase.data() + ioff[i], fw->detPairs.data() + c.ndp, fw->obsPairs.data() + c.nop);
      } catch (const Error &) {
        fw_ok = false;
      }
    if (!pc.pool.empty()) memcpy(out.pool.data() + toff[i], pc.pool.data(), pc.pool.size() * 4);
    Instr *dst = out.ins.data() + ioff[i];
    for (const Instr &in : pc.ins) {
      *dst = in;
      dst->t0 += (uint32_t)toff[i];
      ++dst;
    }
  });
  if (fw_ok) {
    fw->fwd = fw->fwd_pc[np];
    fw->fwd_of = &out;
    fw->fwd_ins = ioff[np];
  }
}
}  // namespace

namespace {

// Line starts of text[a, b) (b is a line start or the end of the text), plus b.
void line_starts(const char *text, size_t a, size_t b, std::vector<size_t> &out) {
  out.clear();
  for (size_t x = a; x < b;) {
    out.push_back(x);
    const void *nl = memchr(text + x, '\n', b - x);
    x = nl ? (size_t)(static_cast<const char *>(nl) - text) + 1 : b;
  }
  out.push_back(b);
}

// The common runs of the sequences a[0, n) and b[0, m) (eq(x, y): a[x]
// equals b[y]) along a shortest edit script (Myers' greedy O((n + m) D)
// algorithm, "An O(ND) difference algorithm and its variations", 1986), in
// order.  False when the script needs more than dmax insertions and
// deletions, or the search more than `budget` steps (texts that differ
// throughout are given up on early).  Round d's furthest reaching x on
// diagonals -d..d is kept at trace[d * d + d + k] for the walk back.
template <typename Eq>
bool diff_runs(Eq &&eq, long n, long m, long dmax, long budget, std::vector<long> &vbuf, std::vector<long> &trace,
               std::vector<Run> &runs) {
  const long off = dmax + 1;
  long work = 0;
  vbuf.assign((size_t)(2 * dmax + 3), 0);
  long *V = vbuf.data();
  trace.clear();
  long dfound = -1;
  for (long d = 0; d <= dmax && dfound < 0; ++d) {
    for (long k = -d; k <= d; k += 2) {
      long x = (k == -d || (k != d && V[off + k - 1] < V[off + k + 1])) ? V[off + k + 1] : V[off + k - 1] + 1;
      long y = x - k;
      const long x0 = x;
      while (x < n && y < m && eq(x, y)) {
        ++x;
        ++y;
      }
      work += 1 + (x - x0);
      if (work > budget) return false;
      V[off + k] = x;
      if (x >= n && y >= m) {
        dfound = d;
        break;
      }
    }
    trace.insert(trace.end(), V + off - d, V + off + d + 1);
  }
  if (dfound < 0) return false;
  runs.clear();
  long x = n, y = m;
  for (long d = dfound; d > 0; --d) {
    const long *P = trace.data() + (d - 1) * (d - 1) + (d - 1);  // P[k]: round d - 1, diagonal k
    const long k = x - y;
    const long pk = (k == -d || (k != d && P[k - 1] < P[k + 1])) ? k + 1 : k - 1;
    const long px = P[pk], py = px - pk;
    const long xs = pk == k + 1 ? px : px + 1;  // after the insertion (down) or the deletion (right)
    if (x > xs) runs.push_back({(size_t)xs, (size_t)(xs - k), (size_t)(x - xs)});
    x = px;
    y = py;
  }
  if (x > 0) runs.push_back({0, 0, (size_t)x});
  std::reverse(runs.begin(), runs.end());
  return true;
}

// Lowers `text` against the previous circuit of S (incremental lowering).
// The two texts are compared line by line (their common prefix and suffix
// first, then a shortest edit script of the lines between).  Runs of equal
// lines, shrunk to whole top-level statements, keep their parsed
// instructions; the statements between them are parsed again; S.parsed
// becomes the new circuit's parse.  The backward pass keeps the previous
// cuts of every segment that lies within one unchanged run (its
// instructions shifted) and cuts the rest afresh.  Returns false (S.parsed
// untouched) when a full lowering is the better way.
bool plan_incremental(const char *text, size_t len, const LowerOptions &opt, LowerScratch &S) {
  LowerScratch::Buffers &B = *S.b;
  const LowerScratch::Buffers::Prev &V = B.prev;
  Parsed &P = S.parsed;
  if (!V.valid || opt.cuts || !text || P.marks.empty() || B.cut.size() < 2 || B.cut.front() != P.ins.size())
    return false;
  const char *o = V.text.data();
  const size_t on = V.text.size(), mn = std::min(on, len);
  const size_t nI0 = P.ins.size(), nT0 = P.pool.size();
  if (2 * mn < std::max(on, len)) return false;  // one text more than twice the other: not a branch of it
  size_t lp = 0;
  while (lp < mn && o[lp] == text[lp]) ++lp;
  size_t ls = 0;
  while (ls < mn - lp && o[on - 1 - ls] == text[len - 1 - ls]) ++ls;

  // regions of equal bytes: old [o0, o1) == new [n0, n0 + o1 - o0), in order
  struct Region {
    size_t o0, o1, n0;
  };
  std::vector<Region> reg;
  if (lp == on && lp == len) {
    reg.push_back({0, on, 0});
  } else {
    // the lines between the common prefix and suffix (whole lines, so the
    // first changed line and the last are in it)
    size_t p0 = lp;
    while (p0 > 0 && o[p0 - 1] != '\n') --p0;
    size_t xo = on - ls;  // the first line start inside the common suffix (its newline common too)
    if (ls == 0) {
      xo = on;
    } else {
      const void *nl = memchr(o + xo, '\n', on - xo);
      xo = nl ? (size_t)(static_cast<const char *>(nl) - o) + 1 : on;
    }
    if (xo < p0) xo = p0;
    const size_t xn = xo + len - on;
    if (xn < p0 || xn > len) return false;
    reg.push_back({0, p0, 0});
    // Texts of one length whose changes keep every line after them in place
    // (lines changed or reordered within a span of the same bytes): compared
    // in step, 64 bytes at a time.  A changed span runs from the start of the
    // line of its first differing byte to a newline both texts share and
    // after which 64 more bytes agree.
    if (len == on) {
      size_t x = p0, i = p0, changed = 0;
      while (i < xo) {
        const size_t n = std::min<size_t>(64, xo - i);
        if (memcmp(o + i, text + i, n) == 0) {
          i += n;
          continue;
        }
        size_t d = i;
        while (o[d] == text[d]) ++d;
        size_t a = d;
        while (a > x && o[a - 1] != '\n') --a;
        size_t e = d;
        for (;;) {
          const void *nl = memchr(o + e, '\n', xo - e);
          if (!nl) {
            e = xo;
            break;
          }
          const size_t q = (size_t)(static_cast<const char *>(nl) - o);
          e = q + 1;
          if (text[q] == '\n' && memcmp(o + e, text + e, std::min<size_t>(64, xo - e)) == 0) break;
        }
        if (a > x) reg.push_back({x, a, x});
        changed += e - a;
        x = i = e;
      }
      if (2 * changed <= xo - p0) {  // (else a shortest edit script may find more in common)
        if (xo > x) reg.push_back({x, xo, x});
        reg.push_back({xo, on, xn});
      } else {
        reg.resize(1);
      }
    }
  }
  if (reg.empty() || reg.back().o1 != on) {
    size_t p0 = reg.back().o1;  // (the common prefix's lines)
    size_t xo = on - ls;
    if (ls == 0) {
      xo = on;
    } else {
      const void *nl = memchr(o + xo, '\n', on - xo);
      xo = nl ? (size_t)(static_cast<const char *>(nl) - o) + 1 : on;
    }
    if (xo < p0) xo = p0;
    const size_t xn = xo + len - on;
    std::vector<size_t> &la = B.la, &lb = B.lb;
    line_starts(o, p0, xo, la);
    line_starts(text, p0, xn, lb);
    const long na = (long)la.size() - 1, nb = (long)lb.size() - 1;
    // when the lines between the common prefix and suffix are most of the
    // text: a sample of the new ones, each looked for near its place among
    // the old ones (when most are missing the texts differ throughout)
    if (2 * (xn - p0) > len) {
      const long ns = std::min<long>(nb, 64), win = 64 + std::labs(na - nb);
      long hits = 0;
      for (long t = 0; t < ns; ++t) {
        const long j = (long)(((double)t + 0.5) * (double)nb / (double)ns);
        const long c = (long)((double)j * (double)na / (double)std::max<long>(nb, 1));
        const size_t lj = lb[j + 1] - lb[j];
        for (long i = std::max<long>(0, c - win); i < std::min<long>(na, c + win + 1); ++i)
          if (la[i + 1] - la[i] == lj && memcmp(o + la[i], text + lb[j], lj) == 0) {
            ++hits;
            break;
          }
      }
      if (2 * hits < ns) return false;
    }
    auto same_line = [&](long x, long y) {
      const size_t n = la[x + 1] - la[x];
      return lb[y + 1] - lb[y] == n && memcmp(o + la[x], text + lb[y], n) == 0;
    };
    std::vector<Run> &runs = B.runs_;
    // a search of some tens of steps per line (about 0.2 ms for a text of
    // 5,000 lines): a bound on the time spent on texts that differ throughout
    if (!diff_runs(same_line, na, nb, std::min<long>(2048, na + nb), 32 * (na + nb) + 131072, B.vbuf, B.trace, runs))
      return false;
    for (const Run &r : runs) reg.push_back({la[r.a], la[r.a + r.n], lb[r.b]});
    reg.push_back({xo, on, xn});
  }
  // merge touching regions with the same shift; shrink each to whole
  // top-level statements: from the first statement boundary at or after its
  // start to the last at or before its end (boundaries: 0, the marks, the end)
  const std::vector<ParseMark> &mk = P.marks;
  auto bnd_at_or_after = [&](size_t x) -> ParseMark {
    if (x == 0) return ParseMark{0, 1, 0, 0};
    auto it = std::lower_bound(mk.begin(), mk.end(), x, [](const ParseMark &m, size_t v) { return m.off < v; });
    return it == mk.end() ? ParseMark{on, P.end_line, nI0, nT0} : *it;
  };
  auto bnd_at_or_before = [&](size_t x) -> ParseMark {
    if (x >= on) return ParseMark{on, P.end_line, nI0, nT0};
    auto it = std::upper_bound(mk.begin(), mk.end(), x, [](size_t v, const ParseMark &m) { return v < m.off; });
    return it == mk.begin() ? ParseMark{0, 1, 0, 0} : *(it - 1);
  };
  struct Keep {
    ParseMark s, e;  // statement boundaries in the old text
    size_t n0;       // new offset of s
  };
  std::vector<Keep> keep;
  for (size_t i = 0; i < reg.size();) {
    Region r = reg[i++];
    while (i < reg.size() && reg[i].o0 == r.o1 && reg[i].n0 == r.n0 + (r.o1 - r.o0)) r.o1 = reg[i++].o1;
    if (r.o1 <= r.o0) continue;
    const ParseMark s = bnd_at_or_after(r.o0), e = bnd_at_or_before(r.o1);
    // (a run of fewer than 16 instructions between two changes is parsed again
    // with them: lines swapped around it then make one span of unchanged size)
    if (s.off >= e.off || e.off > r.o1 || e.ins - s.ins < 16) continue;
    if (!keep.empty() && (s.off < keep.back().e.off || r.n0 + (s.off - r.o0) < keep.back().n0 + (keep.back().e.off - keep.back().s.off)))
      return false;
    keep.push_back({s, e, r.n0 + (s.off - r.o0)});
  }
  // the statements between kept runs, parsed again
  size_t gap_bytes = 0;
  {
    size_t nprev = 0;
    for (const Keep &k : keep) {
      if (k.n0 < nprev) return false;
      gap_bytes += k.n0 - nprev;
      nprev = k.n0 + (k.e.off - k.s.off);
    }
    if (nprev > len) return false;
    gap_bytes += len - nprev;
  }
  if (2 * gap_bytes > len) return false;  // mostly changed: parse and lower it whole
  const size_t ngap = keep.size() + 1;
  if (B.gaps.size() < ngap) B.gaps.resize(ngap);
  {
    size_t nprev = 0;
    for (size_t g = 0; g < ngap; ++g) {
      const size_t gend = g < keep.size() ? keep[g].n0 : len;
      Parsed &G = B.gaps[g];
      G.want_marks = true;
      try {
        parse_stim_into(text + nprev, gend - nprev, G);
      } catch (const Error &) {
        return false;  // (a full parse reports the error with its line in the whole text)
      }
      if (g < keep.size()) nprev = keep[g].n0 + (keep[g].e.off - keep[g].s.off);
    }
  }
  // the new parse: gap 0, kept run 0, gap 1, ...  When every gap parses to
  // as many instructions and targets as the old statements it replaces
  // (lines changed or reordered in place), the kept runs stay where they are
  // and the gaps are written over in S.parsed itself; otherwise the new parse
  // is assembled in a second buffer (the old index range of each kept run,
  // and where it lands, go to the cuts)
  bool inplace = true;
  {
    size_t pi = 0, pt = 0;
    for (size_t g = 0; g < ngap && inplace; ++g) {
      const size_t ei = g < keep.size() ? keep[g].s.ins : nI0, et = g < keep.size() ? keep[g].s.tpos : nT0;
      inplace = B.gaps[g].ins.size() == ei - pi && B.gaps[g].pool.size() == et - pt;
      if (g < keep.size()) {
        pi = keep[g].e.ins;
        pt = keep[g].e.tpos;
      }
    }
  }
  Parsed &N = B.next;
  N.marks.clear();
  if (!inplace) {
    size_t ti = 0, tt = 0;
    for (size_t g = 0; g < ngap; ++g) {
      ti += B.gaps[g].ins.size();
      tt += B.gaps[g].pool.size();
    }
    for (const Keep &k : keep) {
      ti += k.e.ins - k.s.ins;
      tt += k.e.tpos - k.s.tpos;
    }
    if (tt > 0xFFFFFFFFull) return false;
    N.ins.clear();
    N.ins.reserve(ti);
    N.pool.resize(tt);
  }
  Parsed &W = inplace ? P : N;  // where the new parse is written
  struct Moved {
    size_t o0, o1, n0;  // old instructions [o0, o1) are new [n0, n0 + o1 - o0)
  };
  std::vector<Moved> moved;
  size_t ni = 0, tp = 0, line = 1, noff = 0;
  for (size_t g = 0; g < ngap; ++g) {
    const Parsed &G = B.gaps[g];
    if (inplace) {
      for (size_t i = 0; i < G.ins.size(); ++i) {
        P.ins[ni + i] = G.ins[i];
        P.ins[ni + i].t0 += (uint32_t)tp;
      }
    } else {
      for (const Instr &in : G.ins) {
        N.ins.push_back(in);
        N.ins.back().t0 += (uint32_t)tp;
      }
    }
    if (!G.pool.empty()) memcpy(W.pool.data() + tp, G.pool.data(), G.pool.size() * 4);
    for (const ParseMark &x : G.marks) N.marks.push_back({x.off + noff, x.line + line - 1, x.ins + ni, x.tpos + tp});
    ni += G.ins.size();
    tp += G.pool.size();
    line += G.end_line - 1;
    if (g == keep.size()) break;
    const Keep &k = keep[g];
    moved.push_back({k.s.ins, k.e.ins, ni});
    if (!inplace) {
      const int64_t dt = (int64_t)tp - (int64_t)k.s.tpos;
      for (size_t i = k.s.ins; i < k.e.ins; ++i) {
        N.ins.push_back(P.ins[i]);
        N.ins.back().t0 = (uint32_t)((int64_t)N.ins.back().t0 + dt);
      }
      if (k.e.tpos > k.s.tpos) memcpy(N.pool.data() + tp, P.pool.data() + k.s.tpos, (k.e.tpos - k.s.tpos) * 4);
    }
    auto m0 = std::lower_bound(mk.begin(), mk.end(), k.s.off, [](const ParseMark &m, size_t v) { return m.off < v; });
    for (auto it = m0; it != mk.end() && it->off < k.e.off; ++it)
      N.marks.push_back({it->off - k.s.off + k.n0, it->line - k.s.line + line, it->ins - k.s.ins + ni,
                         it->tpos - k.s.tpos + tp});
    ni += k.e.ins - k.s.ins;
    tp += k.e.tpos - k.s.tpos;
    line += k.e.line - k.s.line;
    noff = k.n0 + (k.e.off - k.s.off);
  }
  if (tp != W.pool.size() || ni != W.ins.size()) return false;
  const size_t nI = ni;
  const Instr *const NI = W.ins.data();

  // cuts: the previous segments that lie within one kept run, moved with it.
  // The instructions between them are cut where the previous circuit was
  // cut when they are as many as the previous instructions between the same
  // segments (statements changed in place: the schedule keeps its shape),
  // else afresh into pieces of about segment_occ occurrences.
  const std::vector<size_t> &oc = B.cut;
  std::vector<size_t> &nc = B.plan.cut;
  std::vector<int32_t> &from = B.plan.from;
  nc.assign(1, nI);
  from.clear();
  const size_t so = std::max<uint32_t>(1024, opt.segment_occ);
  // segments over new instructions [lo, nc.back()), which were old [olo, ohi)
  auto fresh = [&](size_t lo, size_t olo, size_t ohi) {
    const size_t hi = nc.back();
    if (hi <= lo) return;
    if (hi - lo == ohi - olo) {
      for (size_t c : oc)
        if (c > olo && c < ohi) {
          nc.push_back(c - olo + lo);
          from.push_back(-1);
        }
      nc.push_back(lo);
      from.push_back(-1);
      return;
    }
    size_t acc = 0;
    for (size_t ii = hi; ii-- > lo + 1;) {
      acc += NI[ii].tn;
      if (acc >= so) {
        nc.push_back(ii);
        from.push_back(-1);
        acc = 0;
      }
    }
    nc.push_back(lo);
    from.push_back(-1);
  };
  size_t r = moved.size();
  size_t ohi = nI0;  // old index of nc.back()
  for (size_t s = 0; s + 1 < oc.size(); ++s) {
    const size_t j0 = oc[s + 1], j1 = oc[s];
    while (r > 0 && moved[r - 1].o0 > j0) --r;
    if (r == 0 || j0 < moved[r - 1].o0 || j1 > moved[r - 1].o1 || j1 == j0) continue;
    const Moved &m = moved[r - 1];
    const size_t a = j0 - m.o0 + m.n0, b = j1 - m.o0 + m.n0;
    if (b > nc.back() || j1 > ohi) return false;
    fresh(b, j1, ohi);
    nc.push_back(a);
    from.push_back((int32_t)s);
    ohi = j0;
  }
  fresh(0, 0, ohi);
  if (nc.back() != 0 || from.size() + 1 != nc.size()) return false;
  if (!inplace) {
    P.ins.swap(N.ins);
    P.pool.swap(N.pool);
  }
  P.marks.swap(N.marks);
  P.end_line = line;
  S.stats.parsed_bytes = gap_bytes;
  B.plan.active = true;
  return true;
}

}  // namespace

void lower_text(const char *text, size_t len, const LowerOptions &opt, Tape &T, LowerScratch &S, HostPool *pool) {
  LowerScratch::Buffers &B = *S.b;
  S.stats = LowerScratch::Stats{};
  S.parsed.want_marks = opt.incremental;
  B.plan.active = false;
  B.fwd_of = nullptr;
  if (!opt.incremental || !plan_incremental(text, len, opt, S)) {
    B.prev.valid = false;  // (a parse that fails leaves S.parsed half written)
    if (pool)
      parse_pieces(text, len, S.parsed, S.pieces, *pool, &B);  // (with the forward pass beside it)
    else
      parse_stim_into(text, len, S.parsed);
  }
  const size_t parsed = B.plan.active ? S.stats.parsed_bytes : len;
  B.prev.valid = false;
  lower_into(S.parsed, opt, T, S, pool);
  S.stats.parsed_bytes = parsed;
  if (opt.incremental) {
    B.prev.text.assign(text, len);
    B.prev.valid = true;
  }
}

Tape lower(const Parsed &P, const LowerOptions &opt) {
  Tape T;
  LowerScratch S;
  lower_into(P, opt, T, S);
  return T;
}

void lower_into(const Parsed &P, const LowerOptions &opt, Tape &T, LowerScratch &S, HostPool *pool) {
  if (opt.level < 0 || opt.level > 2) throw Error(GPC_ERR_INVALID, "correlation level must be 0, 1 or 2");
  T.reset();
  LowerScratch::Buffers &B = *S.b;
  uint32_t kcap = std::max<uint32_t>(1, opt.kcap);
  // Lowered against the previous circuit (a plan from lower_text): its arrays
  // move aside, readable while this circuit's are built, and its segments
  // are taken over where they still apply.
  const bool reuse = opt.incremental && B.plan.active;
  B.plan.active = false;
  B.prev.valid = false;  // lower_text marks the state valid once this lowering is done
  if (reuse) {
    std::swap(B.measBase, B.prev.measBase);
    std::swap(B.occBase, B.prev.occBase);
    std::swap(B.tsrc, B.prev.tsrc);
    std::swap(B.moff, B.prev.moff);
    std::swap(B.mbits, B.prev.mbits);
    std::swap(B.cut, B.prev.cut);
    std::swap(B.segs, B.prev.segs);
  }
  S.stats = LowerScratch::Stats{};
  S.stats.incremental = reuse;

  // ---- forward pass: qubits, measurements, detectors, observables --------
  std::vector<uint32_t> &measBase = B.measBase;
  measBase.resize(P.ins.size());
  // target occurrences: a REPEAT body's targets are stored once and occur once per repetition
  std::vector<uint32_t> &occBase = B.occBase;
  occBase.resize(P.ins.size());
  size_t occ = 0;
  std::vector<std::pair<uint32_t, uint32_t>> &detPairs = B.detPairs;  // (measurement, detector)
  std::vector<std::pair<uint32_t, uint32_t>> &obsPairs = B.obsPairs;  // (measurement, observable)
  uint32_t m = 0, ndet = 0, nobs = 0;
  uint32_t nq = 0;
  // the pass on one thread; it throws the first error in instruction order
  auto forward_serial = [&] {
    occ = 0;
    m = ndet = nobs = nq = 0;
    detPairs.clear();
    obsPairs.clear();
    for (size_t i = 0; i < P.ins.size(); ++i) {
      const Instr &in = P.ins[i];
      const Gate &g = kGates[in.gate];
      const uint32_t *t = P.pool.data() + in.t0;
      measBase[i] = m;
      occBase[i] = (uint32_t)occ;
      occ += in.tn;
      if (occ > 0xFFFFFFFFull / 4) throw Error(GPC_ERR_CAPACITY, "circuit too long");
      check_targets(in, g);
      if (counts_qubits(in, g)) nq = std::max(nq, in.maxq + 1);
      switch (g.kind) {
        case G_M:
        case G_MR:
        case G_MPAD:
          m += in.tn;
          break;
        case G_DET:
          for (uint32_t k = 0; k < in.tn; ++k) {
            uint32_t back = t[k] & ~kRec;
            if (back > m) throw Error(GPC_ERR_PARSE, "record lookback beyond the start of the circuit");
            detPairs.push_back({m - back, ndet});
          }
          ++ndet;
          break;
        case G_OBS: {
          const uint32_t kk = obs_index(in);
          for (uint32_t k = 0; k < in.tn; ++k) {
            uint32_t back = t[k] & ~kRec;
            if (back > m) throw Error(GPC_ERR_PARSE, "record lookback beyond the start of the circuit");
            obsPairs.push_back({m - back, kk});
          }
          nobs = std::max(nobs, kk + 1);
          break;
        }
        default:
          check_pairs(in, g);
          break;
      }
      check_args(in, g);
    }
  };
  // A long circuit on the pool: its instructions in pieces, counted (and
  // checked) in a first pass, written from the pieces' starting counts in a
  // second (done beside the parse when the text was parsed in pieces).  Any
  // error sends it back to the serial pass, which reports the first error in
  // instruction order.
  bool done = false;
  const size_t nins = P.ins.size();
  if (B.fwd_of == &P && B.fwd_ins == nins) {
    done = true;
  } else if (pool && nins >= 1024) {
    const uint32_t np = (uint32_t)std::min<size_t>({(size_t)pool->workers() + 1, 16, nins / 128});
    std::vector<FwdCount> &pc = B.fwd_pc;
    pc.assign(np + 1, FwdCount{});
    auto lo_of = [&](uint32_t p) { return nins * p / np; };
    bool ok = true;
    try {
      pool->run(np, [&](uint32_t p, uint32_t) { forward_count(P.ins.data() + lo_of(p), lo_of(p + 1) - lo_of(p), pc[p + 1]); });
    } catch (const Error &) {
      ok = false;
    }
    if (ok) {
      forward_prefix(pc, np);
      ok = pc[np].occ <= 0xFFFFFFFFull / 4;
    }
    if (ok) {
      detPairs.resize(pc[np].ndp);
      obsPairs.resize(pc[np].nop);
      try {
        pool->run(np, [&](uint32_t p, uint32_t) {
          const size_t i0 = lo_of(p);
          forward_write(P.ins.data() + i0, lo_of(p + 1) - i0, P.pool.data(), pc[p], measBase.data() + i0,
                        occBase.data() + i0, detPairs.data() + pc[p].ndp, obsPairs.data() + pc[p].nop);
        });
      } catch (const Error &) {
        ok = false;
      }
    }
    if (ok) {
      B.fwd = pc[np];
      done = true;
    }
  }
  B.fwd_of = nullptr;
  if (done) {
    occ = B.fwd.occ;
    m = B.fwd.m;
    ndet = B.fwd.ndet;
    nobs = B.fwd.nobs;
    nq = B.fwd.nq;
  }
  if (!done) forward_serial();
  // sources of the noise targets: tick and class (see Tape::rec_src)
  std::vector<uint32_t> &tsrc = B.tsrc;
  if (opt.sources) {
    tsrc.assign(occ, kNone);  // by target occurrence
    uint32_t tick = 0;
    std::vector<uint8_t> &lastReset = B.lastReset;  // the qubit's last operation was a reset
    lastReset.assign(nq, 0);
    for (size_t i = 0; i < P.ins.size(); ++i) {
      const Instr &in = P.ins[i];
      const Gate &g = kGates[in.gate];
      const uint32_t *t = P.pool.data() + in.t0;
      switch (g.kind) {
        case G_TICK:
          ++tick;
          break;
        case G_N2:
          for (uint32_t k = 0; k < in.tn; ++k) tsrc[occBase[i] + k] = tick * SRC_CLASSES + SRC_DEP2;
          break;
        case G_N1:
          for (uint32_t k = 0; k < in.tn; ++k) {
            if (g.a == N1_DEP1)
              tsrc[occBase[i] + k] = tick * SRC_CLASSES + SRC_DEP1;
            else if (g.a != N1_PC1)
              tsrc[occBase[i] + k] = tick * SRC_CLASSES + (lastReset[t[k]] ? SRC_RESET_FLIP : SRC_MEAS_FLIP);
          }
          break;
        case G_M:
        case G_MR:
          for (uint32_t k = 0; k < in.tn; ++k) {
            tsrc[occBase[i] + k] = tick * SRC_CLASSES + SRC_MEAS_FLIP;
            lastReset[t[k]] = g.kind == G_MR;
          }
          break;
        case G_R:
          for (uint32_t k = 0; k < in.tn; ++k) lastReset[t[k]] = 1;
          break;
        case G_C1:
        case G_C2:
        case G_PAULI:
          for (uint32_t k = 0; k < in.tn; ++k) lastReset[t[k]] = 0;
          break;
        default:
          break;
      }
    }
    T.n_ticks = tick + 1;
  } else {
    tsrc.clear();
    T.n_ticks = 1;
    for (const Instr &in : P.ins) T.n_ticks += kGates[in.gate].kind == G_TICK;
  }
  T.nq = nq;
  T.nmeas = m;
  T.ndet = ndet;
  T.nobs = nobs;
  T.nbits = ndet + nobs;
  T.w = std::max<uint32_t>(1, (T.nbits + 63) / 64);
  if (nq > 4096) throw Error(GPC_ERR_CAPACITY, "more than 4096 qubits");
  if (T.nbits >= (1u << 24)) throw Error(GPC_ERR_CAPACITY, "more than 2^24 detectors and observables");
  {
    uint32_t qpt = nq <= 1024 ? 1 : nq <= 2048 ? 2 : 4;
    uint32_t per = (nq + qpt - 1) / qpt;
    uint32_t threads = std::max<uint32_t>(32, (per + 31) / 32 * 32);
    T.qpad = threads * qpt;
    // an epoch (kcap slots x qpad ops) must fit one shared-memory chunk buffer
    T.chunk_cap = walk_chunk_cap(T.qpad);
    if (T.chunk_cap < T.qpad * 8u) throw Error(GPC_ERR_CAPACITY, "too many qubits for the walk's shared memory");
    kcap = std::min<uint32_t>(kcap, T.chunk_cap / (T.qpad * 8u));
  }

  // measurement -> bits (XOR: a measurement listed twice in one detector cancels),
  // bits ascending per measurement: a counting sort by measurement, then a
  // small sort of each measurement's bits
  std::vector<uint32_t> &moff = B.moff, &mbits = B.mbits;
  moff.assign(m + 1, 0);
  {
    for (auto &d : detPairs) moff[d.first + 1]++;
    for (auto &o : obsPairs) moff[o.first + 1]++;
    for (uint32_t i = 0; i < m; ++i) moff[i + 1] += moff[i];
    std::vector<uint32_t> &cur = B.order;
    cur.assign(moff.begin(), moff.end() - 1);
    mbits.resize(moff[m]);
    for (auto &d : detPairs) mbits[cur[d.first]++] = d.second;
    for (auto &o : obsPairs) mbits[cur[o.first]++] = ndet + o.second;
    uint32_t w = 0, lo = 0;
    for (uint32_t i = 0; i < m; ++i) {
      const uint32_t hi = moff[i + 1];
      moff[i] = w;
      if (hi - lo == 1) {
        mbits[w++] = mbits[lo];
        lo = hi;
        continue;
      }
      // detector bits arrive in ascending order (detectors are numbered as they
      // appear); only observable bits can be out of order
      if (!std::is_sorted(mbits.begin() + lo, mbits.begin() + hi)) std::sort(mbits.begin() + lo, mbits.begin() + hi);
      for (uint32_t a = lo; a < hi;) {
        uint32_t b = a;
        while (b < hi && mbits[b] == mbits[a]) ++b;
        if ((b - a) & 1) mbits[w++] = mbits[a];
        a = b;
      }
      lo = hi;
    }
    moff[m] = w;
    mbits.resize(w);
  }

  // ---- backward pass: epoch scheduling and noise records -----------------
  // The circuit is cut into time segments of a fixed number of target
  // occurrences (the cut depends on the circuit alone).  Each segment is
  // scheduled backwards from a fresh qubit state -- its first epoch starts
  // empty for every qubit -- and the segments are stitched in walk order:
  // a segment's epochs, points and records follow those of the segments after
  // it in time.  Every qubit keeps its op order and the records keep theirs,
  // so the DEM is that of one uncut pass; the schedule gains at most about one
  // epoch per cut.  Segments run on the pool when one is given.
  std::vector<size_t> &cut = B.cut;  // segment s covers instructions [cut[s + 1], cut[s])
  if (reuse) {
    cut.swap(B.plan.cut);
  } else if (opt.cuts) {
    cut = *opt.cuts;
    bool ok = cut.size() >= 2 && cut.front() == P.ins.size() && cut.back() == 0;
    for (size_t i = 0; ok && i + 1 < cut.size(); ++i) ok = cut[i] > cut[i + 1] || (P.ins.empty() && cut.size() == 2);
    if (!ok) throw Error(GPC_ERR_INVALID, "segment cuts must descend from the instruction count to 0");
  } else {
    cut.clear();
    cut.push_back(P.ins.size());
    // at most 8 segments of equal size, about opt.segment_occ occurrences or fewer each
    const size_t so = std::max<uint32_t>(1024, opt.segment_occ);
    const size_t nsegw = std::max<size_t>(1, std::min<size_t>(8, (occ + so - 1) / so));
    const size_t per = (occ + nsegw - 1) / nsegw;
    size_t acc = 0;
    for (size_t ii = P.ins.size(); ii-- > 1;) {
      acc += P.ins[ii].tn;
      if (acc >= per) {
        cut.push_back(ii);
        acc = 0;
      }
    }
    cut.push_back(0);
  }
  const uint32_t nseg = (uint32_t)cut.size() - 1;
  if (B.segs.size() < nseg) B.segs.resize(nseg);
  // one segment writes its records in place (unless the segment is kept for
  // the next circuit of an incremental lowering)
  const bool direct = nseg == 1 && !opt.incremental;
  std::vector<uint32_t> &measLo = B.measLo, &measHi = B.measHi;
  measLo.assign(m, kNone);
  measHi.assign(m, kNone);
  const uint32_t dep1Type = opt.level == 0 ? REC_DEP1_L0 : REC_DEP1_L12;
  const uint32_t dep2Type = opt.level == 0 ? REC_DEP2_L0 : opt.level == 1 ? REC_DEP2_L1 : REC_DEP2_L2;
  auto occ_at = [&](size_t i) -> size_t { return i < P.ins.size() ? occBase[i] : occ; };
  auto meas_at = [&](size_t i) -> uint32_t { return i < P.ins.size() ? measBase[i] : m; };

  // Segments taken over from the previous circuit.  A previous segment over
  // the same statements scheduled exactly these ops, except that its
  // measurements' detector bits and its noise targets' sources came from the
  // rest of that circuit: it is taken over when both differ from this
  // circuit's by one shift each (detectors numbered after a changed span,
  // ticks counted after it), and its bits and sources are shifted.
  std::vector<uint32_t> &runs = B.runs;  // 1: schedule the segment, 0: take it over
  runs.assign(nseg, 1);
  B.dbits.assign(nseg, 0);
  B.dsrc.assign(nseg, 0);
  if (reuse && B.prev.nq == nq && B.prev.kcap == kcap && B.prev.level == opt.level &&
      B.prev.sources == opt.sources && B.plan.from.size() == nseg) {
    const LowerScratch::Buffers::Prev &V = B.prev;
    auto pocc_at = [&](size_t i) -> size_t { return i < V.n_ins ? V.occBase[i] : V.nocc; };
    auto pmeas_at = [&](size_t i) -> uint32_t { return i < V.n_ins ? V.measBase[i] : V.nmeas; };
    for (uint32_t sg = 0; sg < nseg; ++sg) {
      const int32_t f = B.plan.from[sg];
      if (f < 0 || (size_t)f + 1 >= V.cut.size()) continue;
      const size_t i0 = cut[sg + 1], i1 = cut[sg], j0 = V.cut[f + 1], j1 = V.cut[f];
      if (i1 - i0 != j1 - j0) continue;
      const uint32_t m0 = meas_at(i0), m1 = meas_at(i1), pm0 = pmeas_at(j0), pm1 = pmeas_at(j1);
      if (m1 - m0 != pm1 - pm0) continue;
      bool ok = true;
      int64_t db = 0;
      bool have = false;
      for (uint32_t k = 0; ok && k < m1 - m0; ++k) {
        const uint32_t a0 = moff[m0 + k], a1 = moff[m0 + k + 1];
        const uint32_t b0 = V.moff[pm0 + k], b1 = V.moff[pm0 + k + 1];
        if (a1 - a0 != b1 - b0) {
          ok = false;
          break;
        }
        for (uint32_t i = 0; i < a1 - a0; ++i) {
          const int64_t d = (int64_t)mbits[a0 + i] - (int64_t)V.mbits[b0 + i];
          if (!have) {
            db = d;
            have = true;
          } else if (d != db) {
            ok = false;
            break;
          }
        }
      }
      int64_t ds = 0;
      if (ok && opt.sources) {
        const size_t o0 = occ_at(i0), o1 = occ_at(i1), po0 = pocc_at(j0);
        if (o1 - o0 != pocc_at(j1) - po0) ok = false;
        bool hs = false;
        for (size_t o = 0; ok && o < o1 - o0; ++o) {
          const uint32_t x = tsrc[o0 + o], y = V.tsrc[po0 + o];
          if ((x == kNone) != (y == kNone)) {
            ok = false;
          } else if (x != kNone) {
            const int64_t d = (int64_t)x - (int64_t)y;
            if (!hs) {
              ds = d;
              hs = true;
            } else if (d != ds) {
              ok = false;
            }
          }
        }
      }
      if (!ok) continue;
      std::swap(B.segs[sg], B.prev.segs[f]);
      runs[sg] = 0;
      B.dbits[sg] = db;
      B.dsrc[sg] = ds;
      ++S.stats.reused;
    }
  }
  S.stats.segments = nseg;

  auto run_segment = [&](uint32_t sg) {
    LowerScratch::Buffers::Segment &G = B.segs[sg];
    const size_t i0 = cut[sg + 1], i1 = cut[sg];
    const size_t socc = occ_at(i1) - occ_at(i0);
    const size_t sbits = moff[meas_at(i1)] - moff[meas_at(i0)];
    // tape entries: at most one per target occurrence, plus two per
    // measurement and one per further bit of a measurement (OP_M, OP_SNAPD, OP_INJ)
    Entry *const ent0 = G.ent.get(socc * 3 + sbits + 16);
    Entry *ent1 = ent0;
    std::vector<QState> &st = G.st;
    st.assign(nq, QState{});
    std::vector<uint32_t> &ep_k = G.ep_k, &ep_np = G.ep_np;  // slots and points per epoch, grown on demand
    ep_k.clear();
    ep_np.clear();
    uint32_t nprov = 0;  // provisional point ids (creation order)
    // records: at most three per target occurrence (PAULI_CHANNEL_1), written
    // through pointers into arrays sized to that bound and cut to size after
    const size_t rec_max = socc * 3 + 16;
    HostArray<uint64_t> &RD = direct ? T.rec : G.rec;
    HostArray<double> &RP = direct ? T.rec_p : G.rec_p;
    HostArray<uint32_t> &RS = direct ? T.rec_src : G.rec_src;
    RD.resize(rec_max);
    RP.resize(rec_max);
    RS.resize(opt.sources ? rec_max : 0);
    uint64_t *const rec_d = RD.data();
    double *const rec_pp = RP.data();
    uint32_t *const rec_s = opt.sources ? RS.data() : nullptr;
    size_t nrec = 0;
    uint64_t ncomp = 0;
    SplitCache split;

    auto place1 = [&](uint32_t q, uint64_t op) -> uint32_t {
      QState &s = st[q];
      uint32_t e;
      if (s.last < 0) {
        e = 0;
        s.cnt = 0;
      } else if (s.cnt >= kcap) {
        e = (uint32_t)s.last + 1;
        s.cnt = 0;
      } else {
        e = (uint32_t)s.last;
      }
      *ent1++ = {q | (s.cnt << 24), e, op};
      s.sign(op, e);
      if (e >= ep_k.size()) {
        ep_k.resize((size_t)e + 1, 0);
        ep_np.resize((size_t)e + 1, 0);
      }
      ep_k[e] = std::max(ep_k[e], s.cnt + 1);
      s.last = e;
      s.cnt++;
      return e;
    };
    auto point = [&](uint32_t q) -> uint32_t {
      QState &s = st[q];
      if (s.open != kNone) return s.open;
      uint32_t id = nprov++;
      ++ep_np[place1(q, make_op(OP_SNAP, 0, id))];
      s.open = id;
      return id;
    };
    // `at`: the target occurrence whose (tick, class) source the record takes, or kNone
    auto record = [&](uint32_t pa, uint32_t pb, uint32_t type, uint32_t Pa, uint32_t Pb, double p, uint32_t at) {
      rec_d[nrec] = make_rec(pa, pb, type, Pa, Pb);
      rec_pp[nrec] = p;
      if (rec_s) rec_s[nrec] = at == kNone ? kNone : tsrc[at];
      ncomp += kRecComps[type];
      ++nrec;
    };

    for (size_t ii = i1; ii-- > i0;) {
      const Instr &in = P.ins[ii];
      const Gate &g = kGates[in.gate];
      const uint32_t *t = P.pool.data() + in.t0;
      switch (g.kind) {
        case G_C1:
          for (uint32_t k = in.tn; k-- > 0;) {
            uint32_t q = t[k];
            place1(q, make_op(OP_C1, (uint32_t)g.a | ((uint32_t)g.b << 2), 0));
            st[q].open = kNone;
          }
          break;
        case G_C2:
          for (uint32_t k = in.tn; k >= 2; k -= 2) {
            uint32_t a = t[k - 2], b = t[k - 1];
            uint32_t E = (uint32_t)(std::max(st[a].last, st[b].last) + 1);
            uint32_t subA = (uint32_t)g.img[0] | ((uint32_t)g.img[1] << 4);
            uint32_t subB = swap_halves(g.img[2]) | (swap_halves(g.img[3]) << 4);
            const uint64_t opA = c2_op(subA, b), opB = c2_op(subB, a);
            *ent1++ = {a, E, opA};  // partner operands become slots below
            *ent1++ = {b, E, opB};
            st[a].sign(opA, E);
            st[b].sign(opB, E);
            if (E >= ep_k.size()) {
              ep_k.resize((size_t)E + 1, 0);
              ep_np.resize((size_t)E + 1, 0);
            }
            ep_k[E] = std::max<uint32_t>(ep_k[E], 1);
            st[a].last = st[b].last = E;
            st[a].cnt = st[b].cnt = 1;
            st[a].open = st[b].open = kNone;
          }
          break;
        case G_R:
          for (uint32_t k = in.tn; k-- > 0;) {
            place1(t[k], make_op(OP_R, 0, 0));
            st[t[k]].open = kNone;
          }
          break;
        case G_M:
        case G_MR: {
          double p = in.nargs ? in.args[0] : 0.0;
          uint32_t sub = (uint32_t)g.a | (g.kind == G_MR ? 4u : 0u);
          for (uint32_t k = in.tn; k-- > 0;) {
            uint32_t q = t[k];
            uint32_t meas = measBase[ii] + k;
            const uint32_t b0 = moff[meas], b1 = moff[meas + 1];
            // bits beyond the first ride on OP_INJ slots placed before the OP_M
            uint32_t first = b0 < b1 ? mbits[b0] : kNone;
            uint32_t lo = kNone;
            for (uint32_t b = b0 + 1; b < b1; b += 2) {
              uint32_t e = place1(q, make_inj(mbits[b], b + 1 < b1 ? mbits[b + 1] : 0xFFFFFFu));
              if (lo == kNone) lo = e;
            }
            uint32_t e = place1(q, make_op(OP_M, sub, first));
            measLo[meas] = lo == kNone ? e : lo;
            measHi[meas] = e;
            st[q].open = kNone;
            if (p > 0 && b1 > b0) {
              uint32_t id = nprov++;
              ++ep_np[place1(q, make_op(OP_SNAPD, 0, id))];
              record(id, 0, REC_PAULI, 1, 0, p, occBase[ii] + k);
            }
          }
          break;
        }
        case G_N1: {
          for (uint32_t k = in.tn; k-- > 0;) {
            uint32_t q = t[k];
            switch (g.a) {
              case N1_X:
              case N1_Y:
              case N1_Z:
                if (in.args[0] > 0)
                  record(point(q), 0, REC_PAULI, g.a == N1_X ? 1 : g.a == N1_Z ? 2 : 3, 0, in.args[0], occBase[ii] + k);
                break;
              case N1_DEP1:
                if (in.args[0] > 0) record(point(q), 0, dep1Type, 0, 0, split.dep1(in.args[0]), occBase[ii] + k);
                break;
              case N1_PC1: {
                double qq[3];
                pc1_independent(in.args[0], in.args[1], in.args[2], qq);
                if (qq[0] > 0 || qq[1] > 0 || qq[2] > 0) {
                  uint32_t pt = point(q);
                  if (qq[0] > 0) record(pt, 0, REC_PAULI, 1, 0, qq[0], kNone);
                  if (qq[1] > 0) record(pt, 0, REC_PAULI, 3, 0, qq[1], kNone);
                  if (qq[2] > 0) record(pt, 0, REC_PAULI, 2, 0, qq[2], kNone);
                }
                break;
              }
            }
          }
          break;
        }
        case G_N2: {
          if (!(in.args[0] > 0)) break;
          const double sp = split.dep2(in.args[0]);
          for (uint32_t k = in.tn; k >= 2; k -= 2) {
            uint32_t a = t[k - 2], b = t[k - 1];
            uint32_t pa = point(a), pb = point(b);
            record(pa, pb, dep2Type, 0, 0, sp, occBase[ii] + k - 2);
          }
          break;
        }
        case G_CORR: {
          double p = in.args[0];
          if (!(p > 0)) break;
          uint32_t q0 = kNone, q1 = kNone, P0 = 0, P1 = 0;
          for (uint32_t k = 0; k < in.tn; ++k) {
            uint32_t q = t[k] & 0xFFFFFFu, Pv = (t[k] >> 24) & 3u;
            if (q0 == kNone || q0 == q) {
              q0 = q;
              P0 ^= Pv;
            } else if (q1 == kNone || q1 == q) {
              q1 = q;
              P1 ^= Pv;
            } else {
              throw Error(GPC_ERR_UNSUPPORTED, "correlated errors on more than two qubits are not supported");
            }
          }
          if (P0 && P1)
            record(point(q0), point(q1), REC_PAULI, P0, P1, p, kNone);
          else if (P0)
            record(point(q0), 0, REC_PAULI, P0, 0, p, kNone);
          else if (P1)
            record(point(q1), 0, REC_PAULI, P1, 0, p, kNone);
          break;
        }
        default:
          break;
      }
    }

    RD.resize(nrec);
    RP.resize(nrec);
    RS.resize(opt.sources ? nrec : 0);
    G.nent = (size_t)(ent1 - ent0);
    G.nrec = nrec;
    G.ncomp = ncomp;
    G.nprov = nprov;
    // the segment's share of each qubit's signatures (see the qubit packing):
    // op kinds, and op kinds with their (segment-local) epochs
    G.fine.resize(nq);
    G.coarse.resize(nq);
    for (uint32_t q = 0; q < nq; ++q) {
      G.fine[q] = st[q].fine;
      G.coarse[q] = st[q].coarse;
    }
    if (opt.incremental) {  // kept for a later circuit that takes this segment over
      G.mlo.assign(measLo.begin() + meas_at(i0), measLo.begin() + meas_at(i1));
      G.mhi.assign(measHi.begin() + meas_at(i0), measHi.begin() + meas_at(i1));
    }
  };
  // A segment taken over: shift its detector bits (the OP_M operand and the
  // OP_INJ bits) and its sources, and place its measurements' epochs.
  auto take_segment = [&](uint32_t sg) {
    LowerScratch::Buffers::Segment &G = B.segs[sg];
    const int64_t db = B.dbits[sg], ds = B.dsrc[sg];
    if (db) {
      Entry *const ent0 = G.ent.p.get();
      for (size_t i = 0; i < G.nent; ++i) {
        uint64_t &op = ent0[i].op;
        const uint32_t opc = (uint32_t)(op & 0xFF);
        if (opc == OP_M) {
          const uint32_t b = (uint32_t)(op >> 32);
          if (b != kNone) op = (op & 0xFFFFFFFFull) | ((uint64_t)(uint32_t)((int64_t)b + db) << 32);
        } else if (opc == OP_INJ) {
          const uint32_t b1 = (uint32_t)(op >> 32), b2 = (uint32_t)(op >> 8) & 0xFFFFFFu;
          op = make_inj((uint32_t)((int64_t)b1 + db), b2 == 0xFFFFFFu ? b2 : (uint32_t)((int64_t)b2 + db));
        }
      }
    }
    if (ds && opt.sources)
      for (size_t i = 0; i < G.nrec; ++i)
        if (G.rec_src[i] != kNone) G.rec_src[i] = (uint32_t)((int64_t)G.rec_src[i] + ds);
    const uint32_t a = meas_at(cut[sg + 1]);
    std::copy(G.mlo.begin(), G.mlo.end(), measLo.begin() + a);
    std::copy(G.mhi.begin(), G.mhi.end(), measHi.begin() + a);
  };
  auto segment_job = [&](uint32_t sg) {
    if (runs[sg])
      run_segment(sg);
    else
      take_segment(sg);
  };
  if (pool && nseg > 1)
    pool->run(nseg, [&](uint32_t sg, uint32_t) { segment_job(sg); });
  else
    for (uint32_t sg = 0; sg < nseg; ++sg) segment_job(sg);

  // stitch: offsets of each segment's epochs, points and records in walk order
  std::vector<uint32_t> &ep_k = T.ep_k;
  std::vector<uint32_t> &ep_np = B.ep_np;
  ep_k.clear();
  ep_np.clear();
  uint32_t nprov = 0;
  size_t nrec_all = 0;
  for (uint32_t sg = 0; sg < nseg; ++sg) {
    LowerScratch::Buffers::Segment &G = B.segs[sg];
    G.eoff = (uint32_t)ep_k.size();
    G.poff = nprov;
    G.roff = nrec_all;
    ep_k.insert(ep_k.end(), G.ep_k.begin(), G.ep_k.end());
    ep_np.insert(ep_np.end(), G.ep_np.begin(), G.ep_np.end());
    nprov += G.nprov;
    nrec_all += G.nrec;
    if (G.eoff)
      for (uint32_t k = meas_at(cut[sg + 1]); k < meas_at(cut[sg]); ++k)
        if (measLo[k] != kNone) {
          measLo[k] += G.eoff;
          measHi[k] += G.eoff;
        }
  }

  // ---- warp-uniform qubit packing -------------------------------------
  // Qubits with the same sequence of op kinds (data, X-check, Z-check qubits
  // of a code) take the same branches in the walk.  Group them, and start
  // each group on a warp boundary when that costs at most half again as many
  // slots, so a warp does not mix roles.
  std::vector<uint32_t> &slotOf = B.slotOf;
  slotOf.assign(nq, 0);
  {
    // fine signature: op kinds with their epochs; coarse: op kinds only.
    // Each segment hashed its own ops; the segments' hashes are chained in
    // segment order (segments are time ranges common to every qubit, so equal
    // fine signatures still mean equal op kinds at equal epochs)
    std::vector<uint64_t> &fine = B.fine, &coarse = B.coarse;
    fine.assign(nq, kFnvBasis);
    coarse.assign(nq, kFnvBasis);
    for (uint32_t sg = 0; sg < nseg; ++sg) {
      const LowerScratch::Buffers::Segment &G = B.segs[sg];
      for (uint32_t q = 0; q < nq; ++q) {
        coarse[q] = (coarse[q] ^ G.coarse[q]) * kFnvPrime;
        fine[q] = (fine[q] ^ G.fine[q]) * kFnvPrime;
      }
    }
    const uint32_t qptBase = T.qpad <= 1024 ? 1u : T.qpad <= 2048 ? 2u : 4u;
    // Orders qubits by group (groups in order of their first qubit); returns the
    // padded slot count, or 0 if padding does not fit.
    auto plan = [&](const std::vector<uint64_t> &sig, std::vector<uint32_t> &order,
                    std::vector<std::pair<uint32_t, uint32_t>> &groups) -> uint32_t {
      order.resize(nq);
      for (uint32_t q = 0; q < nq; ++q) order[q] = q;
      std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
        return sig[a] != sig[b] ? sig[a] < sig[b] : a < b;
      });
      groups.clear();
      for (uint32_t i = 0; i < nq;) {
        uint32_t k = i;
        while (k < nq && sig[order[k]] == sig[order[i]]) ++k;
        groups.push_back({i, k - i});
        i = k;
      }
      std::sort(groups.begin(), groups.end(),
                [&](const std::pair<uint32_t, uint32_t> &a, const std::pair<uint32_t, uint32_t> &b) {
                  return order[a.first] < order[b.first];
                });
      uint32_t padded = 0;
      for (auto &g : groups) padded += (g.second + 31) / 32 * 32;
      const uint32_t qptP = padded <= 1024 ? 1u : padded <= 2048 ? 2u : 4u;
      const uint32_t qpadP = std::max<uint32_t>(32, (padded + 31) / 32 * 32);
      const bool ok = qptP == qptBase && padded <= 4096 && 2 * (uint64_t)padded <= 3 * (uint64_t)T.qpad &&
                      (uint64_t)kcap * qpadP * 8 <= walk_chunk_cap(qpadP);
      return ok ? qpadP : 0u;
    };
    std::vector<uint32_t> &order = B.order;
    std::vector<std::pair<uint32_t, uint32_t>> &groups = B.groups;
    uint32_t qpadP = plan(fine, order, groups);
    if (!qpadP) qpadP = plan(coarse, order, groups);
    uint32_t next = 0;
    for (auto &g : groups) {
      for (uint32_t i = 0; i < g.second; ++i) slotOf[order[g.first + i]] = next++;
      if (qpadP) next = (next + 31) / 32 * 32;
    }
    if (qpadP) {
      T.qpad = qpadP;
      T.chunk_cap = walk_chunk_cap(T.qpad);
    }
  }

  // ---- assemble epochs -------------------------------------------------
  const uint32_t nE = (uint32_t)ep_k.size();
  T.n_epochs = nE;
  for (auto &k : ep_k) k = std::max<uint32_t>(k, 1);  // every epoch copies at least one slot
  T.ep_opoff.assign(nE, 0);
  uint64_t total = 0;
  for (uint32_t e = 0; e < nE; ++e) {
    T.ep_opoff[e] = (uint32_t)total;
    total += (uint64_t)T.ep_k[e] * T.qpad;
    T.kmax = std::max(T.kmax, T.ep_k[e]);
    if (total > 0xFFFFFFFFull) throw Error(GPC_ERR_CAPACITY, "tape too long");
  }
  // points are numbered in walk order (epoch, slot, qubit slot), so each
  // epoch owns a contiguous range.  Segments own disjoint epoch ranges (so
  // disjoint ops and points): a large tape is zeroed, scattered and
  // renumbered segment by segment on the pool.
  T.ops.resize(total);
  T.ep_ptoff.assign(nE + 1, 0);
  for (uint32_t e = 0; e < nE; ++e) T.ep_ptoff[e + 1] = T.ep_ptoff[e] + ep_np[e];
  std::vector<uint32_t> &remap = B.remap;
  remap.assign(nprov, kNone);
  // records in walk order: each segment's records go to their place with their
  // points renumbered (its own points, numbered by its own assembly just
  // before), beside the first mechanism of each record
  const size_t R = nrec_all;
  uint64_t mm = 0;
  for (uint32_t s = 0; s < nseg; ++s) {
    B.segs[s].moff0 = mm;
    mm += B.segs[s].ncomp;
  }
  if (mm >= 0xFFFFFFFFull) throw Error(GPC_ERR_CAPACITY, "too many error mechanisms");
  if (!direct) {  // (one segment wrote its records in place)
    T.rec.resize(R);
    T.rec_p.resize(R);
    T.rec_src.resize(opt.sources ? R : 0);
  }
  T.rec_moff.resize(R + 1);
  auto place_records = [&](uint32_t sg, uint32_t) {
    const LowerScratch::Buffers::Segment &G = B.segs[sg];
    const uint64_t *const src = direct ? T.rec.data() : G.rec.data();
    uint64_t *const dst = T.rec.data() + G.roff;
    uint32_t *const mo = T.rec_moff.data() + G.roff;
    uint64_t m0 = G.moff0;
    for (size_t i = 0; i < G.nrec; ++i) {
      uint64_t d = src[i];
      const uint32_t pa = (uint32_t)(d & kMaxPoint28) + G.poff, pb = (uint32_t)((d >> 28) & kMaxPoint28) + G.poff;
      const uint32_t type = (uint32_t)((d >> 56) & 15u), Pb = (uint32_t)(d >> 62);
      const bool hasB = type >= REC_DEP2_L0 || Pb != 0;
      d = (d & ~(((uint64_t)kMaxPoint28) | ((uint64_t)kMaxPoint28 << 28))) | (uint64_t)remap[pa] |
          ((uint64_t)(hasB ? remap[pb] : 0) << 28);
      dst[i] = d;
      mo[i] = (uint32_t)m0;
      m0 += kRecComps[type];
    }
    if (!direct && G.nrec) {
      memcpy(T.rec_p.data() + G.roff, G.rec_p.data(), G.nrec * 8);
      if (opt.sources) memcpy(T.rec_src.data() + G.roff, G.rec_src.data(), G.nrec * 4);
    }
  };

  std::atomic<bool> miscount{false};
  auto assemble = [&](uint32_t sg, uint32_t) {
    LowerScratch::Buffers::Segment &G = B.segs[sg];
    const uint32_t ea = G.eoff, eb = G.eoff + (uint32_t)G.ep_k.size();
    const size_t oa = ea < nE ? T.ep_opoff[ea] : total, ob = eb < nE ? T.ep_opoff[eb] : total;
    if (ob > oa) memset(T.ops.data() + oa, 0, (ob - oa) * 8);
    std::vector<uint64_t> &bits = G.snapbits;
    bits.assign((ob - oa + 63) / 64, 0);
    const Entry *const ent0 = G.ent.p.get();
    for (size_t i = 0; i < G.nent; ++i) {
      const Entry &x = ent0[i];
      uint64_t op = x.op;
      const uint32_t opc = (uint32_t)(op & 0xFF);
      const size_t at = (size_t)T.ep_opoff[x.e + G.eoff] + (size_t)x.k() * T.qpad + slotOf[x.q()];
      if (opc == OP_C2 || opc >= OP_XPX) {  // partner qubit -> partner slot
        op = (op & 0xFFFFFFFFull) | ((uint64_t)slotOf[(uint32_t)(op >> 32)] << 32);
      } else if (opc == OP_SNAP || opc == OP_SNAPD) {  // segment-local point -> provisional point
        op += (uint64_t)G.poff << 32;
        bits[(at - oa) >> 6] |= 1ull << ((at - oa) & 63);
      }
      T.ops[at] = op;
    }
    // points in walk order = snapshot ops in tape order: number them by
    // walking the set bits (the segment's epochs are consecutive in the tape)
    uint32_t next = T.ep_ptoff[ea];
    uint64_t *const base = T.ops.data() + oa;
    for (size_t w = 0; w < bits.size(); ++w) {
      for (uint64_t m = bits[w]; m; m &= m - 1) {
        uint64_t &op = base[w * 64 + (size_t)__builtin_ctzll(m)];
        remap[(uint32_t)(op >> 32)] = next;
        op = (op & 0xFFFFFFFFull) | ((uint64_t)next << 32);
        ++next;
      }
    }
    if (next != T.ep_ptoff[eb]) miscount = true;
  };
  // each segment's epochs, then its records, in one task per segment
  auto assemble_and_place = [&](uint32_t sg, uint32_t slot) {
    assemble(sg, slot);
    place_records(sg, slot);
  };
  if (pool && nseg > 1)
    pool->run(nseg, assemble_and_place);
  else
    for (uint32_t sg = 0; sg < nseg; ++sg) assemble_and_place(sg, 0);
  if (miscount) throw Error(GPC_ERR_INVALID, "internal: points per epoch miscounted");
  const uint32_t next = T.ep_ptoff[nE];
  T.npoints = next;
  // copy chunks: runs of whole epochs of at most chunk_cap bytes, chunk_cap
  // sized from the largest epoch (and at least opt.chunk_min)
  {
    uint64_t big = 0;
    for (uint32_t e = 0; e < nE; ++e) big = std::max<uint64_t>(big, (uint64_t)T.ep_k[e] * T.qpad * 8);
    const uint64_t want = std::max<uint64_t>((big + 255) & ~(uint64_t)255, opt.chunk_min);
    T.chunk_cap = (uint32_t)std::min<uint64_t>(walk_chunk_cap(T.qpad), want);
  }
  T.ep_chunk.assign(nE, 0);
  for (uint32_t e = 0; e < nE;) {
    const uint32_t c = (uint32_t)T.ch_off.size();
    uint64_t bytes = 0;
    uint32_t f = e;
    while (f < nE && bytes + (uint64_t)T.ep_k[f] * T.qpad * 8 <= T.chunk_cap) {
      bytes += (uint64_t)T.ep_k[f] * T.qpad * 8;
      T.ep_chunk[f] = c;
      ++f;
    }
    T.ch_off.push_back(T.ep_opoff[e]);
    T.ch_bytes.push_back((uint32_t)bytes);
    e = f;
  }
  if (next > kMaxPoint28) throw Error(GPC_ERR_CAPACITY, "too many snapshot points");
  T.rec_moff[R] = (uint32_t)mm;
  T.M = (uint32_t)mm;
  // injection range of each word
  T.inj_lo.assign(T.w, kNone);
  T.inj_hi.assign(T.w, kNone);
  for (uint32_t k = 0; k < m; ++k) {
    if (measLo[k] == kNone) continue;
    for (uint32_t i = moff[k]; i < moff[k + 1]; ++i) {
      uint32_t j = mbits[i] >> 6;
      if (T.inj_lo[j] == kNone || measLo[k] < T.inj_lo[j]) T.inj_lo[j] = measLo[k];
      if (T.inj_hi[j] == kNone || measHi[k] > T.inj_hi[j]) T.inj_hi[j] = measHi[k];
    }
  }
  if (opt.incremental) {
    LowerScratch::Buffers::Prev &V = B.prev;
    V.n_ins = P.ins.size();
    V.nocc = occ;
    V.nmeas = m;
    V.nq = nq;
    V.kcap = kcap;
    V.level = opt.level;
    V.sources = opt.sources;
  }
}

}  // namespace gpc
