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
#include <stdexcept>
#include <string>
#include <vector>

namespace gpc {

// Errors thrown by the lowering carry a gpc_status code.
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

// ---- tape op encoding (u64) ----------------------------------------------
// bits 0-7 opcode, bits 8-15 sub, bits 32-63 operand.
enum : uint32_t {
  OP_NOP = 0,
  OP_C1 = 1,     // sub: newX mask (bits 0-1 over X,Z) | newZ mask << 2
  OP_C2 = 2,     // sub: newX mask (4 bits over selfX,selfZ,partX,partZ) | newZ mask << 4; operand: partner qubit
  OP_R = 3,      // clear both rows
  OP_M = 4,      // sub: basis 0=Z 1=X 2=Y; operand: measurement index; rows ^= bits of that measurement
  OP_MR = 5,     // clear, then as OP_M
  OP_SNAP = 6,   // operand: point; point <- (X, Z)
  OP_SNAPD = 7,  // operand: point; point <- (bits of the last measurement, 0)
};

inline uint64_t make_op(uint32_t opc, uint32_t sub, uint32_t operand) {
  return (uint64_t)opc | ((uint64_t)(sub & 0xFF) << 8) | ((uint64_t)operand << 32);
}

// Mechanism descriptor: point a (30 bits) | Pauli a (2 bits) | point b | Pauli b.
// Pauli: 0 none, 1 X, 2 Z, 3 Y (X|Z).
inline uint64_t make_desc(uint32_t pa, uint32_t Pa, uint32_t pb, uint32_t Pb) {
  return (uint64_t)(pa & 0x3FFFFFFFu) | ((uint64_t)(Pa & 3) << 30) | ((uint64_t)(pb & 0x3FFFFFFFu) << 32) |
         ((uint64_t)(Pb & 3) << 62);
}

constexpr uint32_t kNone = 0xFFFFFFFFu;

// Parsed instruction: gate id, args, a span of targets in a shared pool.
struct Instr {
  uint16_t gate;
  uint8_t nargs;
  double args[3];
  uint32_t t0, tn;
};

struct Parsed {
  std::vector<Instr> ins;
  std::vector<uint32_t> pool;
};

// Parses stim circuit text, flattening REPEAT blocks.  Throws gpc::Error.
Parsed parse_stim(const char *text, size_t len);

// A lowered circuit: everything the device pipeline needs.
struct Tape {
  uint32_t nq = 0, qpad = 0, nmeas = 0, ndet = 0, nobs = 0, nbits = 0, w = 0;
  uint32_t n_epochs = 0, kmax = 0;
  std::vector<uint64_t> ops;        // sum_e K_e * qpad
  std::vector<uint32_t> ep_opoff;   // [n_epochs]     first op of epoch e
  std::vector<uint32_t> ep_k;       // [n_epochs]     slots in epoch e
  std::vector<uint32_t> ep_ptoff;   // [n_epochs + 1] first point of epoch e
  std::vector<uint32_t> meas_off;   // [nmeas + 1]
  std::vector<uint32_t> meas_bits;  // bits of each measurement
  std::vector<uint32_t> inj_lo;     // [w] first epoch (walk order) injecting into word j, kNone if none
  std::vector<uint32_t> inj_hi;     // [w] last such epoch
  uint32_t npoints = 0;
  std::vector<uint64_t> desc;  // [M] mechanism descriptors
  std::vector<double> prob;    // [M] mechanism probabilities
};

struct LowerOptions {
  int level = 2;     // correlation level 0/1/2
  uint32_t kcap = 8; // max slots per epoch
};

Tape lower(const Parsed &p, const LowerOptions &opt);

}  // namespace gpc
