// Drop-in check: the reference's gate_appl.h ApplyGate template and its
// text-format parser driving the GB300 unitary calculator
// (include/qsim_gb300/unitary_gb300.h).  Built against a qsim checkout's
// headers (-I<qsim>/lib) and include/.
//
// Usage: dropin_unitary <circuit.txt> <out>
// Writes <out>: the unitary of the circuit (complex64, entry (i, j) at
// i * 2^n + j, the reference's layout).

#include <cstdio>
#include <vector>

#include "circuit.h"
#include "circuit_qsim_parser.h"
#include "gate_appl.h"
#include "io_file.h"
#include "operation.h"

#include "qsim_gb300/unitary_gb300.h"

int main(int argc, char** argv) {
  using namespace qsim;
  if (argc < 3) return 2;
  Circuit<Operation<float>> circuit;
  if (!CircuitQsimParser<IOFile>::FromFile(~0u, argv[1], circuit)) return 1;
  using Calc = qsim_gb300::UnitaryCalculatorGB300<float>;
  Calc::UnitarySpace us;
  Calc calc;
  auto u = us.CreateUnitary(circuit.num_qubits);
  if (us.IsNull(u)) return 3;
  us.SetIdentity(u);
  for (const auto& op : circuit.ops) ApplyGate(calc, op, u);
  const uint64_t dim = Calc::UnitarySpace::Size(circuit.num_qubits);
  std::vector<float> host(2 * dim * dim);
  for (uint64_t i = 0; i < dim; ++i)
    for (uint64_t j = 0; j < dim; ++j) {
      const auto v = us.GetEntry(u, i, j);
      host[2 * (i * dim + j)] = v.real();
      host[2 * (i * dim + j) + 1] = v.imag();
    }
  FILE* f = std::fopen(argv[2], "wb");
  if (!f) return 4;
  std::fwrite(host.data(), sizeof(float), host.size(), f);
  std::fclose(f);
  return 0;
}
