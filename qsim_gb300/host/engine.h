// Host-side engine: circuit IR, gate library, text parser, synthetic circuit
// generators, the fusion planner and the plan runner.  Everything here is
// plain C++17 on the host; device work goes through the C ABI of
// include/qsim_gb300.h.
#pragma once

#include <complex>
#include <cstdint>
#include <random>
#include <string>
#include <vector>

#include "qsim_gb300.h"

namespace qsg {
namespace host {

using cplx = std::complex<double>;

enum class OpKind : int { kGate = 0, kControlled = 1, kMeasure = 2 };

// One circuit operation.  `qs` is sorted ascending and `m` is the
// 2^k x 2^k row-major matrix whose row/column bit j is qs[j] (the layout of
// the reference's lib/gate.h:266-290 after qubit sorting).  `cvals` bit i is
// the required value of cqs[i] (lib/gate.h:37-70).
struct Op {
  OpKind kind = OpKind::kGate;
  unsigned time = 0;
  std::vector<unsigned> qs;
  std::vector<unsigned> cqs;
  uint64_t cvals = 0;
  std::vector<cplx> m;
  // Two-qubit named gates: operator Schmidt terms, U = sum_t A_t (x) B_t,
  // 8 values per term: A_t on qs[0] then B_t on qs[1] (2x2 row-major).
  // Empty for other gates.  Used by the hybrid simulator (hybrid.cc).
  std::vector<cplx> schmidt;
};

struct Circuit {
  unsigned num_qubits = 0;
  std::vector<Op> ops;
};

// ---- gate library (gates.cc) -------------------------------------------
// Creates a matrix gate on `qubits` given in any order; `m` uses bit j <->
// qubits[j].  Qubits are sorted and the matrix permuted to match.
Op make_gate(unsigned time, std::vector<unsigned> qubits, std::vector<cplx> m);
// Named gates of the reference's gate set (lib/gates_qsim.h) and U3.
// Returns false for an unknown name or wrong parameter count.
bool named_gate(const std::string& name, unsigned time,
                const std::vector<unsigned>& qubits,
                const std::vector<double>& params, Op* out);
std::vector<cplx> u3_matrix(double theta, double phi, double lambda);
// Operator Schmidt terms of a two-qubit named gate with the qubits in the
// given order (8 values per term, first the factor on qubits[0]); empty for
// names without a decomposition.
std::vector<cplx> schmidt_terms(const std::string& name,
                                const std::vector<double>& params);
// Kronecker product of Pauli letters; letter j acts on sorted qubit j.
std::vector<cplx> pauli_string_matrix(const std::string& letters);

// ---- text format (parser.cc) -------------------------------------------
// The reference's circuit text format (docs/input_format.md,
// lib/circuit_qsim_parser.h:52-153).  Returns false and sets `err` on
// malformed input; operations with time > maxtime are dropped.
bool parse_qsim_text(const std::string& text, unsigned maxtime, Circuit* out,
                     std::string* err);

// ---- synthetic workloads (generate.cc) ---------------------------------
// Grid random circuit: rows x cols (+ extra qubits on a last ragged row),
// `cycles` cycles of {sqrt(X), sqrt(Y), sqrt(W)} single-qubit layers (never
// repeating a qubit's previous gate) and fSim(pi/2, pi/6) on coupler
// patterns A,B,C,D,C,D,A,B.
Circuit grid_random_circuit(unsigned rows, unsigned cols, unsigned extra,
                            unsigned cycles, uint64_t seed);
// Same gate set on a linear chain of n qubits (alternating even/odd pairs).
Circuit chain_random_circuit(unsigned n, unsigned cycles, uint64_t seed);
// Layered circuit: U3 on every qubit, CZ or CNOT on random disjoint pairs,
// and `num_controlled` U3 gates with 1-2 controls per layer.
Circuit layered_u3_circuit(unsigned n, unsigned layers,
                           unsigned num_controlled, uint64_t seed);
// Random Pauli strings of weight 1..max_weight with U[-1,1] coefficients.
struct PauliTerm {
  std::vector<unsigned> qs;
  std::string letters;
  double coeff;
};
std::vector<PauliTerm> random_pauli_sum(unsigned n, unsigned count,
                                        unsigned max_weight, uint64_t seed);

// ---- fusion plan (fuser.cc) --------------------------------------------
enum class Path : int { kCudaCore = 0, kTensor = 1 };

struct PlanOp {
  OpKind kind = OpKind::kGate;
  unsigned time = 0;
  std::vector<unsigned> qs, cqs;
  uint64_t cvals = 0;
  std::vector<cplx> m;          // fused matrix, FP64
  std::vector<float> m32;       // interleaved FP32 copy used for launches
  std::vector<int> members;     // indices of the circuit ops it contains
  Path path = Path::kCudaCore;
  // Tensor-core ops only: this op and the next one run as one two-gate
  // tensor-core pass (one read and one write of the state).
  bool tc_pair_next = false;
  // Every member gate is unitary (M^dagger M = 1 within 1e-5 per entry),
  // so the block is: set when the op is built from its members; the
  // runner's norm carry needs it.
  bool unitary = false;
};

struct Plan {
  unsigned num_qubits = 0;
  std::vector<PlanOp> ops;
  unsigned max_k() const;
};

// Cost of applying one fused block, in microseconds, for the planner.
struct CostModel {
  virtual ~CostModel() = default;
  virtual double cost_us(unsigned n, const std::vector<unsigned>& qs,
                         unsigned ncontrols, Path path) const = 0;
};

struct FuseOptions {
  unsigned max_fused_size = 4;  // 1..6 (reference Parameter, 2..6)
  unsigned seeds = 12;          // front gates tried as block seeds
  bool tensor_path = false;     // route k >= tc_min_k blocks to tcgen05
  unsigned tc_min_k = 5;
  const CostModel* cost = nullptr;  // null: maximise gates per block
  // Two-gate tensor-core passes: consecutive tensor-core blocks whose
  // 12-qubit tile has at least this many run bits (contiguous low qubits)
  // share one pass; 0: one pass per block.
  unsigned tc_pair_bits = 0;
};

// Measured cost of a two-gate tensor-core pass relative to the two one-gate
// passes it replaces, by the shape of its 12-qubit tile (`tile`: the mask of
// its qubits; GB300, 30 and 32 qubits, CUDA events, best of several runs).
// With run bits b (tile qubits 0..b-1) of 4 or more: 0.78-0.82.  Shorter
// runs depend on the tile's other low qubits, `near` = those in [b, 12):
// b = 3 with near >= 1 0.87-0.88, with near = 0 1.28; b = 2 with near >= 2,
// or near = 1 and >= 2 tile qubits in [12, 21), 0.84-1.03 (0.95 taken),
// near = 1 and the rest of the tile above 20 1.28, near = 0 2.0-2.5; b = 1
// 1.11.
inline double tc_pair_cost_factor(uint64_t tile) {
  int b = 0;
  while (b < 64 && ((tile >> b) & 1)) ++b;
  if (b >= 4) return 0.80;
  const uint64_t low12 = (uint64_t{1} << 12) - 1;
  const int near = __builtin_popcountll(tile & low12 & ~((uint64_t{1} << b) - 1));
  const int mid = __builtin_popcountll(tile & (((uint64_t{1} << 21) - 1) & ~low12));
  if (b == 3) return near >= 1 ? 0.87 : 1.28;
  if (b == 2) {
    if (near >= 2 || (near == 1 && mid >= 2)) return 0.95;
    return near == 1 ? 1.28 : 2.49;
  }
  return b == 1 ? 1.11 : 2.49;
}
// Marks pairs of consecutive tensor-core ops (tc_pair_next) that fit a
// two-gate pass with >= `bits` run bits and are predicted faster than two
// passes, choosing the set of pairs with the largest predicted saving;
// returns their number.
size_t pair_tensor_ops(Plan& plan, unsigned bits);

Plan fuse(const Circuit& c, const FuseOptions& opt);
// Unfused plan: one plan op per circuit op (matrices as given).
Plan unfused(const Circuit& c);
// Matrix of a block: product of the member gates (in order) on the sorted
// qubit set `qs`.
std::vector<cplx> block_matrix(const Circuit& c, const std::vector<int>& members,
                               const std::vector<unsigned>& qs);
// Same product for gates given by pointer (qubits of each within `qs`).
std::vector<cplx> block_matrix_ops(const std::vector<const Op*>& ops,
                                   const std::vector<unsigned>& qs);

}  // namespace host
}  // namespace qsg
