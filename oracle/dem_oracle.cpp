// dem_oracle.cpp -- CPU FP64 oracle for detector-error-model compilation.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker that the CUDA path is
// compared against.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline may load it; the product library never links or calls it.
//
// What it computes (the same function as GreenPeas'
// `Driver::compileDetectorErrorModel`, QEC/ErrorAnalysis/Driver.hpp:199-204,
// under stim's circuit semantics):
//   * parse stim circuit text (its own small parser, independent of the
//     product's parser), flatten REPEAT blocks;
//   * a forward pass numbers measurements and builds, per measurement, the
//     set of detector/observable bits that contain it (detector d -> bit d,
//     observable k -> bit numDetectors + k, as in Driver.hpp:181-183);
//   * a backward pass over the instruction list keeps, per qubit, the set of
//     detector/observable bits flipped by an X error (row X_q) and by a Z
//     error (row Z_q) at the current point in time.  Clifford gates map the
//     rows through the gate's Pauli images, measurements inject their bits,
//     resets clear both rows;
//   * each noise channel is split into independent Pauli components with the
//     reference's split formulas (DEPOLARIZE1: 0.5 - 0.5*sqrt(1 - 4p/3),
//     Mixer.hpp:164; DEPOLARIZE2: 0.5 - 0.5*(1 - 16p/15)^(1/8) over 15
//     Paulis, Mixer.hpp:184-200).  A component's symptom is the XOR of the
//     rows its Pauli touches; a measurement flip M(p) has the constant
//     symptom of its measurement;
//   * components with equal symptoms are merged with the XOR-merge
//     p <- p1(1-p2) + p2(1-p1) (STEPG.hpp:128-131, CUDAHandlers.hpp:124-139),
//     folded in emission order; empty symptoms and p == 0 are dropped
//     (Driver.hpp:185).
//   * CorrelationLevel L0/L1/L2 keep the Pauli component sets listed at
//     Mixer.hpp:13-20 (X,Z,IX,IZ,XI,XX,ZI,ZZ / + Y,IY,XZ,YI,ZX / all), with no
//     renormalisation, exactly as the reference drops them.
//
// Parallelism: the backward pass is independent per 64-bit word of the
// detector bitset, so `threads` workers each walk the circuit for a slice of
// words and fill a dense symptom matrix; merging is a hash sort on one thread.
#include <algorithm>
#include <atomic>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

namespace {

thread_local std::string g_err;

enum Kind : uint8_t {
  K_NOP,
  K_TICK,
  K_DETECTOR,
  K_OBSERVABLE,
  K_C1,     // single-qubit Clifford
  K_C2,     // two-qubit Clifford
  K_MEAS,   // measurement (basis in a)
  K_MR,     // measure + reset
  K_RESET,  // reset (any basis)
  K_N1,     // single-qubit noise
  K_N2,     // two-qubit noise
  K_CORR,   // correlated error on Pauli targets
  K_MPAD,
};

// Pauli encoding used throughout: bit0 = X part, bit1 = Z part (Y = 3).
struct GateDef {
  const char *name;
  Kind kind;
  uint8_t a;       // C1: image of X;  MEAS/MR/RESET: basis (0=Z,1=X,2=Y); N1: channel
  uint8_t b;       // C1: image of Z
  uint16_t c2[4];  // C2: images of Xa, Za, Xb, Zb as 4-bit (xa,za,xb,zb)
};

enum { N1_X = 0, N1_Y, N1_Z, N1_DEP1, N1_PC1 };
enum { N2_DEP2 = 0 };

// Two-qubit Pauli as 4 bits: bit0 Xa, bit1 Za, bit2 Xb, bit3 Zb.
constexpr uint16_t XA = 1, ZA = 2, XB = 4, ZB = 8;

const GateDef kGates[] = {
    {"TICK", K_TICK, 0, 0, {}},
    {"DETECTOR", K_DETECTOR, 0, 0, {}},
    {"OBSERVABLE_INCLUDE", K_OBSERVABLE, 0, 0, {}},
    {"QUBIT_COORDS", K_NOP, 0, 0, {}},
    {"SHIFT_COORDS", K_NOP, 0, 0, {}},
    {"MPAD", K_MPAD, 0, 0, {}},
    // single-qubit Cliffords: (image of X, image of Z), signs dropped
    {"I", K_C1, 1, 2, {}},
    {"X", K_C1, 1, 2, {}},
    {"Y", K_C1, 1, 2, {}},
    {"Z", K_C1, 1, 2, {}},
    {"H", K_C1, 2, 1, {}},
    {"H_XZ", K_C1, 2, 1, {}},
    {"H_XY", K_C1, 3, 2, {}},
    {"H_YZ", K_C1, 1, 3, {}},
    {"S", K_C1, 3, 2, {}},
    {"SQRT_Z", K_C1, 3, 2, {}},
    {"S_DAG", K_C1, 3, 2, {}},
    {"SQRT_Z_DAG", K_C1, 3, 2, {}},
    {"SQRT_X", K_C1, 1, 3, {}},
    {"SQRT_X_DAG", K_C1, 1, 3, {}},
    {"SQRT_Y", K_C1, 2, 1, {}},
    {"SQRT_Y_DAG", K_C1, 2, 1, {}},
    {"C_XYZ", K_C1, 3, 1, {}},
    {"C_ZYX", K_C1, 2, 3, {}},
    // two-qubit Cliffords: images of Xa, Za, Xb, Zb
    {"CX", K_C2, 0, 0, {XA | XB, ZA, XB, ZA | ZB}},
    {"CNOT", K_C2, 0, 0, {XA | XB, ZA, XB, ZA | ZB}},
    {"ZCX", K_C2, 0, 0, {XA | XB, ZA, XB, ZA | ZB}},
    {"CZ", K_C2, 0, 0, {XA | ZB, ZA, ZA | XB, ZB}},
    {"ZCZ", K_C2, 0, 0, {XA | ZB, ZA, ZA | XB, ZB}},
    {"CY", K_C2, 0, 0, {XA | XB | ZB, ZA, ZA | XB, ZA | ZB}},
    {"ZCY", K_C2, 0, 0, {XA | XB | ZB, ZA, ZA | XB, ZA | ZB}},
    {"XCZ", K_C2, 0, 0, {XA, ZA | ZB, XA | XB, ZB}},
    {"XCX", K_C2, 0, 0, {XA, ZA | XB, XB, XA | ZB}},
    {"SWAP", K_C2, 0, 0, {XB, ZB, XA, ZA}},
    // measurements / resets
    {"M", K_MEAS, 0, 0, {}},
    {"MZ", K_MEAS, 0, 0, {}},
    {"MX", K_MEAS, 1, 0, {}},
    {"MY", K_MEAS, 2, 0, {}},
    {"MR", K_MR, 0, 0, {}},
    {"MRZ", K_MR, 0, 0, {}},
    {"MRX", K_MR, 1, 0, {}},
    {"MRY", K_MR, 2, 0, {}},
    {"R", K_RESET, 0, 0, {}},
    {"RZ", K_RESET, 0, 0, {}},
    {"RX", K_RESET, 1, 0, {}},
    {"RY", K_RESET, 2, 0, {}},
    // noise
    {"X_ERROR", K_N1, N1_X, 0, {}},
    {"Y_ERROR", K_N1, N1_Y, 0, {}},
    {"Z_ERROR", K_N1, N1_Z, 0, {}},
    {"DEPOLARIZE1", K_N1, N1_DEP1, 0, {}},
    {"PAULI_CHANNEL_1", K_N1, N1_PC1, 0, {}},
    {"DEPOLARIZE2", K_N2, N2_DEP2, 0, {}},
    {"E", K_CORR, 0, 0, {}},
    {"CORRELATED_ERROR", K_CORR, 0, 0, {}},
};

const GateDef *findGate(const std::string &name) {
  for (const auto &g : kGates)
    if (name == g.name) return &g;
  return nullptr;
}

// Target encoding: qubit q -> q; rec[-k] -> kRec | k; Pauli target -> kPauli | (p<<24) | q.
constexpr uint32_t kRec = 0x80000000u;
constexpr uint32_t kPauli = 0x40000000u;

struct Op {
  const GateDef *g;
  std::vector<double> args;
  std::vector<uint32_t> t;
};

struct Parser {
  const char *s;
  const char *e;
  size_t line = 1;

  [[noreturn]] void fail(const std::string &msg) {
    throw std::runtime_error("line " + std::to_string(line) + ": " + msg);
  }
  void skipSpace() {
    while (s < e && (*s == ' ' || *s == '\t' || *s == '\r')) ++s;
  }
  void skipToEol() {
    while (s < e && *s != '\n') ++s;
  }
  uint64_t readUint() {
    if (s >= e || !isdigit((unsigned char)*s)) fail("expected an integer");
    uint64_t v = 0;
    while (s < e && isdigit((unsigned char)*s)) {
      v = v * 10 + (uint64_t)(*s - '0');
      if (v > 0xFFFFFFFFull) fail("integer out of range");
      ++s;
    }
    return v;
  }

  // Parses statements until '}' (inside a block) or end of input.
  void parseBlock(std::vector<Op> &out, bool inBlock, int depth) {
    if (depth > 64) fail("REPEAT nesting too deep");
    while (true) {
      skipSpace();
      if (s >= e) {
        if (inBlock) fail("unterminated REPEAT block");
        return;
      }
      char c = *s;
      if (c == '\n') {
        ++s;
        ++line;
        continue;
      }
      if (c == '#') {
        skipToEol();
        continue;
      }
      if (c == '}') {
        if (!inBlock) fail("unmatched '}'");
        ++s;
        return;
      }
      std::string name;
      while (s < e && (isalnum((unsigned char)*s) || *s == '_')) name += (char)toupper((unsigned char)*s++);
      if (name.empty()) fail(std::string("unexpected character '") + c + "'");
      if (s < e && *s == '[') {  // instruction tag: ignored
        while (s < e && *s != ']' && *s != '\n') ++s;
        if (s >= e || *s != ']') fail("unterminated tag");
        ++s;
      }
      if (name == "REPEAT") {
        skipSpace();
        uint64_t n = readUint();
        skipSpace();
        if (s >= e || *s != '{') fail("expected '{' after REPEAT count");
        ++s;
        std::vector<Op> body;
        parseBlock(body, true, depth + 1);
        for (uint64_t i = 0; i < n; ++i) out.insert(out.end(), body.begin(), body.end());
        continue;
      }
      const GateDef *g = findGate(name);
      if (!g) fail("unsupported instruction " + name);
      Op op;
      op.g = g;
      if (s < e && *s == '(') {
        ++s;
        while (true) {
          skipSpace();
          char *endp = nullptr;
          double v = strtod(s, &endp);
          if (endp == s) fail("bad argument");
          s = endp;
          op.args.push_back(v);
          skipSpace();
          if (s < e && *s == ',') {
            ++s;
            continue;
          }
          if (s < e && *s == ')') {
            ++s;
            break;
          }
          fail("bad argument list");
        }
      }
      while (true) {
        skipSpace();
        if (s >= e || *s == '\n' || *s == '#') break;
        if (*s == '{') fail("unexpected '{'");
        if (*s == '!') ++s;  // inverted result: no effect on sensitivities
        if (*s == '*') {     // Pauli product combiner: not supported here
          fail("combiner targets are not supported");
        }
        if (e - s >= 4 && strncmp(s, "rec[", 4) == 0) {
          s += 4;
          if (s >= e || *s != '-') fail("expected rec[-k]");
          ++s;
          uint64_t k = readUint();
          if (s >= e || *s != ']' || k == 0) fail("bad record target");
          ++s;
          op.t.push_back(kRec | (uint32_t)k);
        } else if (*s == 'X' || *s == 'Y' || *s == 'Z' || *s == 'x' || *s == 'y' || *s == 'z') {
          char p = (char)toupper((unsigned char)*s++);
          uint64_t q = readUint();
          if (q >= (1u << 24)) fail("qubit index too large");
          uint32_t pb = p == 'X' ? 1 : p == 'Z' ? 2 : 3;
          op.t.push_back(kPauli | (pb << 24) | (uint32_t)q);
        } else if (isdigit((unsigned char)*s)) {
          uint64_t q = readUint();
          if (q >= (1u << 24)) fail("qubit index too large");
          op.t.push_back((uint32_t)q);
        } else {
          fail("bad target");
        }
      }
      out.push_back(std::move(op));
    }
  }
};

struct Mech {
  uint32_t begin;  // offset into the dense symptom matrix row index space
  double p;
};

struct Result {
  uint32_t numDetectors = 0;
  uint32_t numObservables = 0;
  uint32_t numQubits = 0;
  uint64_t numRaw = 0;  // emitted components before merging (incl. empty)
  std::vector<double> probs;
  std::vector<uint32_t> offsets;  // CSR over targets, size probs.size()+1
  std::vector<uint32_t> targets;  // detector d -> d, observable k -> numDetectors+k
  // provenance of every raw component (for the noise-rate gradient)
  uint32_t numTicks = 1;
  std::vector<int32_t> rawGroup;  // merged error holding the component, -1 if dropped
  std::vector<double> rawProb;    // the component's probability
  std::vector<uint32_t> rawSrc;   // tick * 4 + class, 0xFFFFFFFF if none
  std::vector<uint8_t> rawChan;   // 0 X/Y/Z error or measurement flip, 1 DEPOLARIZE1, 2 DEPOLARIZE2, 3 other
  std::vector<double> rawArg;     // the instruction's probability argument
};

// Component lists for the correlation levels (Mixer.hpp:13-20).  Paulis are
// (P_a, P_b) with 0 = I, 1 = X, 2 = Z, 3 = Y in the X|Z bit encoding.
struct Comp2 {
  uint8_t pa, pb;
};
// stim's order of the 15 two-qubit Paulis: IX IY IZ XI XX XY XZ YI YX YY YZ ZI ZX ZY ZZ
const Comp2 kDep2All[15] = {{0, 1}, {0, 3}, {0, 2}, {1, 0}, {1, 1}, {1, 3}, {1, 2}, {3, 0},
                            {3, 1}, {3, 3}, {3, 2}, {2, 0}, {2, 1}, {2, 3}, {2, 2}};
bool dep2Kept(int level, Comp2 c) {
  if (level >= 2) return true;
  bool hasY = c.pa == 3 || c.pb == 3;
  bool l0 = !hasY && !((c.pa == 1 && c.pb == 2) || (c.pa == 2 && c.pb == 1));
  if (level == 0) return l0;
  // L1 adds IY, YI, XZ, ZX.
  bool l1extra = (c.pa == 0 && c.pb == 3) || (c.pa == 3 && c.pb == 0) || (c.pa == 1 && c.pb == 2) ||
                 (c.pa == 2 && c.pb == 1);
  return l0 || l1extra;
}

double splitDep1(double p) { return 0.5 - 0.5 * std::sqrt(1.0 - (4.0 * p) / 3.0); }
double splitDep2(double p) { return 0.5 - 0.5 * std::pow(1.0 - (16.0 * p) / 15.0, 0.125); }

// Exact conversion of a disjoint single-qubit Pauli channel (px, py, pz) into
// independent X, Y, Z channels via the channel's Pauli eigenvalues:
// lambda_P = 1 - 2 * (probability of the Paulis anticommuting with P), and for
// independent channels lambda_X = (1-2qy)(1-2qz) etc.
bool pc1ToIndependent(double px, double py, double pz, double out[3]) {
  double lx = 1 - 2 * (py + pz), ly = 1 - 2 * (px + pz), lz = 1 - 2 * (px + py);
  if (lx <= 0 || ly <= 0 || lz <= 0) return false;
  double ax = std::sqrt(ly * lz / lx), ay = std::sqrt(lx * lz / ly), az = std::sqrt(lx * ly / lz);
  out[0] = 0.5 - 0.5 * ax;
  out[1] = 0.5 - 0.5 * ay;
  out[2] = 0.5 - 0.5 * az;
  for (int i = 0; i < 3; ++i)
    if (!(out[i] >= 0)) return false;
  return true;
}

struct Circuit {
  std::vector<Op> ops;
  uint32_t nq = 0, nmeas = 0, ndet = 0, nobs = 0;
  // per measurement: bits it belongs to (XOR semantics)
  std::vector<std::vector<uint32_t>> measBits;
  // per op: index of its first measurement
  std::vector<uint32_t> measBase;
};

void analyse(Circuit &c) {
  // forward pass: number measurements, collect detectors and observables.
  std::vector<std::vector<uint32_t>> detMeas;
  std::vector<std::pair<uint32_t, uint32_t>> obsRefs;  // (k, meas)
  c.measBase.resize(c.ops.size());
  uint32_t m = 0;
  uint32_t maxQ = 0;
  bool anyQ = false;
  for (size_t i = 0; i < c.ops.size(); ++i) {
    const Op &op = c.ops[i];
    c.measBase[i] = m;
    Kind k = op.g->kind;
    for (uint32_t t : op.t) {
      if (t & kRec) {
        if (k != K_DETECTOR && k != K_OBSERVABLE)
          throw std::runtime_error(std::string("record targets not supported on ") + op.g->name);
        continue;
      }
      uint32_t q = (t & kPauli) ? (t & 0xFFFFFF) : t;
      if (k == K_DETECTOR || k == K_OBSERVABLE)
        throw std::runtime_error(std::string("only record targets are supported on ") + op.g->name);
      if (k == K_MPAD) {  // MPAD targets are result values, not qubits
        if (t > 1) throw std::runtime_error("MPAD targets must be 0 or 1");
        continue;
      }
      if ((t & kPauli) && k != K_CORR) throw std::runtime_error(std::string("Pauli targets not supported on ") + op.g->name);
      if (!(t & kPauli) && k == K_CORR) throw std::runtime_error("E needs Pauli targets");
      maxQ = std::max(maxQ, q);
      anyQ = true;
    }
    switch (k) {
      case K_MEAS:
      case K_MR:
        if (op.args.size() > 1) throw std::runtime_error("measurement takes at most one argument");
        m += (uint32_t)op.t.size();
        break;
      case K_MPAD:
        m += (uint32_t)op.t.size();
        break;
      case K_DETECTOR: {
        std::vector<uint32_t> ms;
        for (uint32_t t : op.t) {
          uint32_t back = t & ~kRec;
          if (back > m) throw std::runtime_error("record lookback beyond the start of the circuit");
          ms.push_back(m - back);
        }
        detMeas.push_back(std::move(ms));
        break;
      }
      case K_OBSERVABLE: {
        if (op.args.size() != 1) throw std::runtime_error("OBSERVABLE_INCLUDE needs an index");
        double a = op.args[0];
        if (a < 0 || a != std::floor(a) || a > 1e6) throw std::runtime_error("bad observable index");
        uint32_t kidx = (uint32_t)a;
        for (uint32_t t : op.t) {
          uint32_t back = t & ~kRec;
          if (back > m) throw std::runtime_error("record lookback beyond the start of the circuit");
          obsRefs.push_back({kidx, m - back});
        }
        c.nobs = std::max(c.nobs, kidx + 1);
        break;
      }
      case K_C2:
      case K_N2:
        if (op.t.size() % 2) throw std::runtime_error(std::string("odd number of targets for ") + op.g->name);
        for (size_t j = 0; j < op.t.size(); j += 2)
          if (op.t[j] == op.t[j + 1]) throw std::runtime_error("two-qubit gate on a single qubit");
        break;
      default:
        break;
    }
  }
  c.nq = anyQ ? maxQ + 1 : 0;
  c.nmeas = m;
  c.ndet = (uint32_t)detMeas.size();
  c.measBits.assign(m, {});
  auto toggle = [&](uint32_t meas, uint32_t bit) {
    auto &v = c.measBits[meas];
    auto it = std::find(v.begin(), v.end(), bit);
    if (it == v.end())
      v.push_back(bit);
    else
      v.erase(it);
  };
  for (uint32_t d = 0; d < c.ndet; ++d)
    for (uint32_t ms : detMeas[d]) toggle(ms, d);
  for (auto &r : obsRefs) toggle(r.second, c.ndet + r.first);
}

// Emission sink: either counts components (pass 0) or writes symptom words.
struct Walker {
  const Circuit &c;
  int level;
  uint32_t w0, w1;  // word slice [w0, w1)
  uint32_t ww;      // words in slice
  uint32_t wTotal;
  std::vector<uint64_t> X, Z;
  std::vector<uint64_t> tmp, inj;
  // outputs
  bool counting;
  std::vector<double> *probs;  // filled when counting
  std::vector<uint64_t> *origin = nullptr;  // (op << 32 | target) of each component, filled when counting
  uint64_t curOp = 0, curT = 0;
  uint64_t *dense;              // [raw][wTotal] when writing
  uint64_t next = 0;

  Walker(const Circuit &c_, int level_, uint32_t w0_, uint32_t w1_, uint32_t wTotal_)
      : c(c_), level(level_), w0(w0_), w1(w1_), ww(w1_ - w0_), wTotal(wTotal_) {
    X.assign((size_t)c.nq * ww, 0);
    Z.assign((size_t)c.nq * ww, 0);
    tmp.assign(ww, 0);
    inj.assign(ww, 0);
  }

  uint64_t *xr(uint32_t q) { return &X[(size_t)q * ww]; }
  uint64_t *zr(uint32_t q) { return &Z[(size_t)q * ww]; }

  void injection(uint32_t meas) {
    std::fill(inj.begin(), inj.end(), 0);
    for (uint32_t bit : c.measBits[meas]) {
      uint32_t wd = bit >> 6;
      if (wd >= w0 && wd < w1) inj[wd - w0] ^= 1ull << (bit & 63);
    }
  }
  // accumulate sensitivity of Pauli p (X|Z bits) on qubit q into tmp
  void acc(uint32_t q, uint32_t p) {
    if (p & 1)
      for (uint32_t i = 0; i < ww; ++i) tmp[i] ^= xr(q)[i];
    if (p & 2)
      for (uint32_t i = 0; i < ww; ++i) tmp[i] ^= zr(q)[i];
  }
  void clearTmp() { std::fill(tmp.begin(), tmp.end(), 0); }
  void emit(double p) {
    if (counting) {
      probs->push_back(p);
      if (origin) origin->push_back(curOp << 32 | curT);
    } else {
      uint64_t *row = dense + next * wTotal + w0;
      for (uint32_t i = 0; i < ww; ++i) row[i] = tmp[i];
    }
    ++next;
  }
  void emitPauli1(uint32_t q, uint32_t p, double prob) {
    clearTmp();
    acc(q, p);
    emit(prob);
  }

  void run() {
    for (size_t oi = c.ops.size(); oi-- > 0;) {
      const Op &op = c.ops[oi];
      const GateDef *g = op.g;
      size_t nt = op.t.size();
      curOp = oi;
      curT = 0;
      switch (g->kind) {
        case K_C1:
          for (size_t ti = nt; ti-- > 0;) {
            uint32_t q = op.t[ti];
            for (uint32_t i = 0; i < ww; ++i) {
              uint64_t x = xr(q)[i], z = zr(q)[i];
              uint64_t nx = ((g->a & 1) ? x : 0) ^ ((g->a & 2) ? z : 0);
              uint64_t nz = ((g->b & 1) ? x : 0) ^ ((g->b & 2) ? z : 0);
              xr(q)[i] = nx;
              zr(q)[i] = nz;
            }
          }
          break;
        case K_C2:
          for (size_t ti = nt; ti >= 2; ti -= 2) {
            uint32_t a = op.t[ti - 2], b = op.t[ti - 1];
            for (uint32_t i = 0; i < ww; ++i) {
              uint64_t v[4] = {xr(a)[i], zr(a)[i], xr(b)[i], zr(b)[i]};
              uint64_t nv[4];
              for (int k = 0; k < 4; ++k) {
                uint64_t s = 0;
                for (int bit = 0; bit < 4; ++bit)
                  if (g->c2[k] & (1u << bit)) s ^= v[bit];
                nv[k] = s;
              }
              xr(a)[i] = nv[0];
              zr(a)[i] = nv[1];
              xr(b)[i] = nv[2];
              zr(b)[i] = nv[3];
            }
          }
          break;
        case K_MEAS:
        case K_MR: {
          double p = op.args.empty() ? 0.0 : op.args[0];
          for (size_t ti = nt; ti-- > 0;) {
            uint32_t q = op.t[ti];
            uint32_t meas = c.measBase[oi] + (uint32_t)ti;
            curT = ti;
            if (g->kind == K_MR) {
              std::fill(xr(q), xr(q) + ww, 0);
              std::fill(zr(q), zr(q) + ww, 0);
            }
            injection(meas);
            if (p > 0) {
              for (uint32_t i = 0; i < ww; ++i) tmp[i] = inj[i];
              emit(p);
            }
            if (g->a == 0 || g->a == 2)
              for (uint32_t i = 0; i < ww; ++i) xr(q)[i] ^= inj[i];
            if (g->a == 1 || g->a == 2)
              for (uint32_t i = 0; i < ww; ++i) zr(q)[i] ^= inj[i];
          }
          break;
        }
        case K_MPAD: {
          double p = op.args.empty() ? 0.0 : op.args[0];
          if (p > 0)
            for (size_t ti = nt; ti-- > 0;) {
              injection(c.measBase[oi] + (uint32_t)ti);
              for (uint32_t i = 0; i < ww; ++i) tmp[i] = inj[i];
              emit(p);
            }
          break;
        }
        case K_RESET:
          for (size_t ti = nt; ti-- > 0;) {
            uint32_t q = op.t[ti];
            std::fill(xr(q), xr(q) + ww, 0);
            std::fill(zr(q), zr(q) + ww, 0);
          }
          break;
        case K_N1: {
          for (size_t ti = nt; ti-- > 0;) {
            uint32_t q = op.t[ti];
            curT = ti;
            switch (g->a) {
              case N1_X:
                emitPauli1(q, 1, op.args.at(0));
                break;
              case N1_Y:
                emitPauli1(q, 3, op.args.at(0));
                break;
              case N1_Z:
                emitPauli1(q, 2, op.args.at(0));
                break;
              case N1_DEP1: {
                double ps = splitDep1(op.args.at(0));
                emitPauli1(q, 1, ps);
                if (level >= 1) emitPauli1(q, 3, ps);
                emitPauli1(q, 2, ps);
                break;
              }
              case N1_PC1: {
                double ind[3];
                pc1ToIndependent(op.args.at(0), op.args.at(1), op.args.at(2), ind);
                emitPauli1(q, 1, ind[0]);
                emitPauli1(q, 3, ind[1]);
                emitPauli1(q, 2, ind[2]);
                break;
              }
            }
          }
          break;
        }
        case K_N2: {
          double ps = splitDep2(op.args.at(0));
          for (size_t ti = nt; ti >= 2; ti -= 2) {
            uint32_t a = op.t[ti - 2], b = op.t[ti - 1];
            curT = ti - 2;
            for (const Comp2 &cc : kDep2All) {
              if (!dep2Kept(level, cc)) continue;
              clearTmp();
              acc(a, cc.pa);
              acc(b, cc.pb);
              emit(ps);
            }
          }
          break;
        }
        case K_CORR: {
          clearTmp();
          for (uint32_t t : op.t) acc(t & 0xFFFFFF, (t >> 24) & 3);
          emit(op.args.at(0));
          break;
        }
        default:
          break;
      }
    }
  }
};

void validateArgs(const Circuit &c) {
  for (const Op &op : c.ops) {
    const GateDef *g = op.g;
    auto need = [&](size_t n) {
      if (op.args.size() != n)
        throw std::runtime_error(std::string(g->name) + " takes " + std::to_string(n) + " argument(s)");
    };
    auto prob = [&](double p) {
      if (!(p >= 0 && p <= 1)) throw std::runtime_error(std::string(g->name) + ": probability out of range");
    };
    switch (g->kind) {
      case K_N1:
        if (g->a == N1_PC1) {
          need(3);
          for (double p : op.args) prob(p);
          double ind[3];
          if (!pc1ToIndependent(op.args[0], op.args[1], op.args[2], ind))
            throw std::runtime_error("PAULI_CHANNEL_1 cannot be written as independent X, Y, Z channels");
        } else {
          need(1);
          prob(op.args[0]);
          if (g->a == N1_DEP1 && op.args[0] > 0.75) throw std::runtime_error("DEPOLARIZE1 p > 0.75");
        }
        break;
      case K_N2:
        need(1);
        prob(op.args[0]);
        if (op.args[0] > 0.9375) throw std::runtime_error("DEPOLARIZE2 p > 0.9375");
        break;
      case K_CORR:
        need(1);
        prob(op.args[0]);
        break;
      case K_MEAS:
      case K_MR:
      case K_MPAD:
        if (!op.args.empty()) prob(op.args[0]);
        break;
      default:
        break;
    }
  }
}

inline uint64_t mix64(uint64_t x) {
  x ^= x >> 30;
  x *= 0xbf58476d1ce4e5b9ull;
  x ^= x >> 27;
  x *= 0x94d049bb133111ebull;
  x ^= x >> 31;
  return x;
}

// Source of each raw component for the noise-rate gradient: the tick of its
// instruction (TICKs before it) and its class -- 0 DEPOLARIZE2, 1
// DEPOLARIZE1, 2 measurement flip (X/Y/Z_ERROR on a qubit whose last
// operation was not a reset, or a measurement's flip argument), 3 reset flip
// (X/Y/Z_ERROR on a qubit whose last operation was a reset).
void provenance(const Circuit &c, const std::vector<uint64_t> &origin, const std::vector<double> &probs, Result &r) {
  std::vector<std::vector<uint32_t>> src(c.ops.size());
  std::vector<uint8_t> chan(c.ops.size(), 3);
  std::vector<bool> afterReset(c.nq, false);
  uint32_t tick = 0;
  for (size_t i = 0; i < c.ops.size(); ++i) {
    const Op &op = c.ops[i];
    const GateDef *g = op.g;
    src[i].assign(op.t.size(), 0xFFFFFFFFu);
    if (g->kind == K_TICK) {
      ++tick;
      continue;
    }
    switch (g->kind) {
      case K_N2:
        chan[i] = 2;
        for (size_t k = 0; k < op.t.size(); ++k) src[i][k] = tick * 4 + 0;
        break;
      case K_N1:
        if (g->a == N1_DEP1) {
          chan[i] = 1;
          for (size_t k = 0; k < op.t.size(); ++k) src[i][k] = tick * 4 + 1;
        } else if (g->a != N1_PC1) {
          chan[i] = 0;
          for (size_t k = 0; k < op.t.size(); ++k) src[i][k] = tick * 4 + (afterReset[op.t[k]] ? 3 : 2);
        }
        break;
      case K_MEAS:
      case K_MR:
        chan[i] = 0;
        for (size_t k = 0; k < op.t.size(); ++k) {
          src[i][k] = tick * 4 + 2;
          afterReset[op.t[k]] = g->kind == K_MR;
        }
        break;
      case K_RESET:
        for (uint32_t q : op.t) afterReset[q] = true;
        break;
      case K_C1:
      case K_C2:
        for (uint32_t q : op.t) afterReset[q] = false;
        break;
      default:
        break;
    }
  }
  r.numTicks = tick + 1;
  const size_t raw = origin.size();
  r.rawProb = probs;
  r.rawSrc.resize(raw);
  r.rawChan.resize(raw);
  r.rawArg.resize(raw);
  for (size_t i = 0; i < raw; ++i) {
    const uint32_t oi = (uint32_t)(origin[i] >> 32), ti = (uint32_t)origin[i];
    const Op &op = c.ops[oi];
    r.rawSrc[i] = ti < src[oi].size() ? src[oi][ti] : 0xFFFFFFFFu;
    r.rawChan[i] = chan[oi];
    r.rawArg[i] = op.args.empty() ? 0.0 : op.args[0];
  }
}

Result compile(const char *text, size_t len, int level, int threads) {
  Circuit c;
  Parser ps{text, text + len};
  ps.parseBlock(c.ops, false, 0);
  validateArgs(c);
  analyse(c);
  const uint32_t nbits = c.ndet + c.nobs;
  const uint32_t w = std::max<uint32_t>(1, (nbits + 63) / 64);

  // pass 0: enumerate components and their probabilities (word-independent)
  std::vector<double> probs;
  std::vector<uint64_t> origin;
  {
    Walker wk(c, level, 0, 0, w);
    wk.counting = true;
    wk.probs = &probs;
    wk.origin = &origin;
    wk.dense = nullptr;
    wk.run();
  }
  const uint64_t raw = probs.size();
  std::vector<uint64_t> dense((size_t)raw * w, 0);

  // pass 1: fill symptoms, word slices in parallel
  int nt = std::max(1, std::min<int>(threads, (int)w));
  auto work = [&](int t) {
    uint32_t a = (uint32_t)((uint64_t)w * t / nt), b = (uint32_t)((uint64_t)w * (t + 1) / nt);
    if (a == b) return;
    Walker wk(c, level, a, b, w);
    wk.counting = false;
    wk.probs = nullptr;
    wk.dense = dense.data();
    wk.run();
  };
  if (nt == 1) {
    work(0);
  } else {
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t) th.emplace_back(work, t);
    for (auto &x : th) x.join();
  }

  // pass 2: group equal symptoms (hash, then exact compare), fold in emission order
  std::vector<uint64_t> h(raw);
  std::vector<uint32_t> idx;
  idx.reserve(raw);
  for (uint64_t i = 0; i < raw; ++i) {
    const uint64_t *row = &dense[i * w];
    uint64_t acc = 0;
    bool nz = false;
    for (uint32_t j = 0; j < w; ++j) {
      if (row[j]) {
        nz = true;
        acc ^= mix64(row[j] + 0x9e3779b97f4a7c15ull * (j + 1));
      }
    }
    h[i] = acc;
    if (nz && probs[i] != 0) idx.push_back((uint32_t)i);
  }
  std::stable_sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) {
    if (h[a] != h[b]) return h[a] < h[b];
    int cmp = memcmp(&dense[(size_t)a * w], &dense[(size_t)b * w], w * 8);
    if (cmp != 0) return cmp < 0;
    return a < b;
  });
  Result r;
  r.numDetectors = c.ndet;
  r.numObservables = c.nobs;
  r.numQubits = c.nq;
  r.numRaw = raw;
  r.offsets.push_back(0);
  provenance(c, origin, probs, r);
  r.rawGroup.assign(raw, -1);
  size_t i = 0;
  while (i < idx.size()) {
    size_t j = i + 1;
    while (j < idx.size() && h[idx[j]] == h[idx[i]] &&
           memcmp(&dense[(size_t)idx[j] * w], &dense[(size_t)idx[i] * w], w * 8) == 0)
      ++j;
    double p = 0;
    for (size_t k = i; k < j; ++k) {
      double q = probs[idx[k]];
      p = p * (1 - q) + q * (1 - p);
      r.rawGroup[idx[k]] = (int32_t)r.probs.size();
    }
    const uint64_t *row = &dense[(size_t)idx[i] * w];
    for (uint32_t wd = 0; wd < w; ++wd) {
      uint64_t v = row[wd];
      while (v) {
        int b = __builtin_ctzll(v);
        r.targets.push_back(wd * 64 + (uint32_t)b);
        v &= v - 1;
      }
    }
    r.probs.push_back(p);
    r.offsets.push_back((uint32_t)r.targets.size());
    i = j;
  }
  return r;
}

}  // namespace

extern "C" {

struct oracle_result;

const char *oracle_last_error(void) { return g_err.c_str(); }

// Compiles stim circuit text; returns 0 on success and a handle in *out.
int oracle_compile(const char *text, size_t len, int level, int threads, oracle_result **out) {
  try {
    if (!text || !out) throw std::runtime_error("null argument");
    if (level < 0 || level > 2) throw std::runtime_error("correlation level must be 0, 1 or 2");
    auto *r = new Result(compile(text, len, level, threads));
    *out = reinterpret_cast<oracle_result *>(r);
    return 0;
  } catch (const std::exception &e) {
    g_err = e.what();
    return -1;
  }
}

void oracle_info(const oracle_result *h, uint32_t *num_errors, uint32_t *num_targets, uint32_t *num_detectors,
                 uint32_t *num_observables, uint64_t *num_raw, uint32_t *num_qubits) {
  const Result *r = reinterpret_cast<const Result *>(h);
  *num_errors = (uint32_t)r->probs.size();
  *num_targets = (uint32_t)r->targets.size();
  *num_detectors = r->numDetectors;
  *num_observables = r->numObservables;
  *num_raw = r->numRaw;
  *num_qubits = r->numQubits;
}

void oracle_arrays(const oracle_result *h, double *probs, uint32_t *offsets, uint32_t *targets) {
  const Result *r = reinterpret_cast<const Result *>(h);
  memcpy(probs, r->probs.data(), r->probs.size() * sizeof(double));
  memcpy(offsets, r->offsets.data(), r->offsets.size() * sizeof(uint32_t));
  memcpy(targets, r->targets.data(), r->targets.size() * sizeof(uint32_t));
}

void oracle_free(oracle_result *h) { delete reinterpret_cast<Result *>(h); }

uint32_t oracle_num_ticks(const oracle_result *h) { return reinterpret_cast<const Result *>(h)->numTicks; }

// Provenance of the raw components (num_raw entries each, see oracle_info).
void oracle_raw(const oracle_result *h, int32_t *group, double *prob, uint32_t *src, uint8_t *chan, double *arg) {
  const Result *r = reinterpret_cast<const Result *>(h);
  const size_t n = r->rawGroup.size();
  memcpy(group, r->rawGroup.data(), n * sizeof(int32_t));
  memcpy(prob, r->rawProb.data(), n * sizeof(double));
  memcpy(src, r->rawSrc.data(), n * sizeof(uint32_t));
  memcpy(chan, r->rawChan.data(), n * sizeof(uint8_t));
  memcpy(arg, r->rawArg.data(), n * sizeof(double));
}

double oracle_split_dep1(double p) { return splitDep1(p); }
double oracle_split_dep2(double p) { return splitDep2(p); }
double oracle_xor_merge(double a, double b) { return a * (1 - b) + b * (1 - a); }
}
