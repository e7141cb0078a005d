// Drop-in check: qsim's text-format parser and circuit types driving the
// GB300 hybrid runner (include/qsim_gb300/hybrid_gb300.h) with the
// Parameter fields apps/qsimh_base.cc sets.  Built against a qsim
// checkout's headers (-I<qsim>/lib) and include/.
//
// Usage: dropin_hybrid <circuit.txt> <out> <num_prefix> <num_root> <prefix>
//                      <parts as 0/1 string, qubit 0 first>
// Writes <out>: the amplitudes of bitstrings 0 .. min(8, 2^n) - 1 (complex
// float).
//        dropin_hybrid --check <circuit.txt> <parts>
// No GPU: converts the circuit through the adapter and compares it with the
// reference's own SplitLattice counts and gate matrices; prints "ok".

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <string>
#include <vector>

#include "circuit.h"
#include "circuit_qsim_parser.h"
#include "formux.h"
#include "gates_qsim.h"
#include "hybrid.h"
#include "io.h"
#include "io_file.h"
#include "operation.h"

#include "qsim_gb300/hybrid_gb300.h"

static int Check(const char* path, const char* parts_str) {
  using namespace qsim;
  Circuit<Operation<float>> circuit;
  if (!CircuitQsimParser<IOFile>::FromFile(~0u, path, circuit)) return 1;
  std::vector<unsigned> parts;
  for (const char* p = parts_str; *p; ++p) parts.push_back(unsigned(*p - '0'));
  using HS = HybridSimulator<IO, For>;
  HS::HybridData<float> hd;
  if (!HS::SplitLattice(parts, circuit.ops, hd)) return 5;
  qsg_circuit* c = qsim_gb300::QSimHRunnerGB300<IO>::ToCircuit(circuit);
  if (!c) return 6;
  qsg_hybrid_info info{};
  if (qsg_hybrid_split(c, parts.data(), unsigned(parts.size()), &info)) return 7;
  if (info.num_ops0 != hd.ops0.size() || info.num_ops1 != hd.ops1.size() ||
      info.num_gatexs != hd.num_gatexs || info.num_qubits0 != hd.num_qubits0 ||
      info.num_qubits1 != hd.num_qubits1) {
    std::printf("counts differ: %u %u %u vs %zu %zu %u\n", info.num_ops0,
                info.num_ops1, info.num_gatexs, hd.ops0.size(),
                hd.ops1.size(), hd.num_gatexs);
    return 8;
  }
  // Gate matrices: the engine's (double) against the reference's (float).
  double worst = 0;
  for (size_t i = 0; i < circuit.ops.size(); ++i) {
    const auto* g = OpGetAlternative<Gate<float>>(circuit.ops[i]);
    unsigned k = 0;
    qsg_circuit_get_op(c, i, nullptr, nullptr, &k, nullptr, nullptr, nullptr,
                       nullptr, nullptr);
    std::vector<unsigned> qs(k);
    std::vector<double> m(2u << (2 * k));
    qsg_circuit_get_op(c, i, nullptr, nullptr, nullptr, qs.data(), nullptr,
                       nullptr, nullptr, m.data());
    if (qs != g->qubits || m.size() != g->matrix.size()) return 9;
    for (size_t j = 0; j < m.size(); ++j)
      worst = std::max(worst, std::abs(m[j] - double(g->matrix[j])));
  }
  qsg_circuit_destroy(c);
  if (worst > 1e-6) {
    std::printf("matrices differ by %g\n", worst);
    return 10;
  }
  std::printf("ok\n");
  return 0;
}

int main(int argc, char** argv) {
  using namespace qsim;
  if (argc == 4 && std::string(argv[1]) == "--check")
    return Check(argv[2], argv[3]);
  if (argc < 7) return 2;
  Circuit<Operation<float>> circuit;
  if (!CircuitQsimParser<IOFile>::FromFile(~0u, argv[1], circuit)) return 1;
  std::vector<unsigned> parts;
  for (const char* p = argv[6]; *p; ++p) parts.push_back(unsigned(*p - '0'));
  const uint64_t m = std::min(uint64_t{8}, uint64_t{1} << circuit.num_qubits);
  std::vector<uint64_t> bitstrings;
  for (uint64_t i = 0; i < m; ++i) bitstrings.push_back(i);

  struct Factory {};  // the reference's runner takes one; unused here
  using Runner = qsim_gb300::QSimHRunnerGB300<IO>;
  Runner::Parameter param;
  param.prefix = std::stoull(argv[5]);
  param.num_prefix_gatexs = std::stoul(argv[3]);
  param.num_root_gatexs = std::stoul(argv[4]);
  param.num_threads = 1;
  param.verbosity = 0;
  std::vector<std::complex<float>> results(m, 0);
  if (!Runner::Run(param, Factory(), circuit, parts, bitstrings, results))
    return 3;
  FILE* f = std::fopen(argv[2], "wb");
  if (!f) return 4;
  std::fwrite(results.data(), sizeof(results[0]), results.size(), f);
  std::fclose(f);
  return 0;
}
