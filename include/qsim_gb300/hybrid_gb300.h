// hybrid_gb300.h — qsim's QSimHRunner (lib/run_qsimh.h:29-104) with the
// hybrid simulation on the GB300 engine (qsg_hybrid_run).
//
// Same Parameter fields and Run signature as
// QSimHRunner<IO, Fuser, HybridSimulator>, so a qsimh application changes one
// type (apps/qsimh_base.cc):
//
//   using Runner = qsim_gb300::QSimHRunnerGB300<IO>;
//   Runner::Parameter param;  // prefix, num_prefix_gatexs, num_root_gatexs,
//                             // num_threads, verbosity (+ max_fused_size...)
//   Runner::Run(param, factory, circuit, parts, bitstrings, results);
//
// The factory is accepted and unused (the engine owns its device states).
// Circuit operations are read through qsim's own operation accessors, so
// this header is included after the reference's headers (lib/ on the
// include path): one-qubit gates pass their matrices; two-qubit gates of the
// qsim gate set (lib/gates_qsim.h: id2, cz, cnot, sw, is, fs, cp) pass by
// name and parameters in their original qubit order, which gives the engine
// the same Schmidt terms as the reference; other two-qubit gates pass their
// matrices and may not sit on the cut (as in the reference, which has no
// Schmidt decomposition for them either).  Amplitudes are added to
// `results`, as the reference does.
#ifndef QSIM_GB300_HYBRID_GB300_H_
#define QSIM_GB300_HYBRID_GB300_H_

#include <complex>
#include <cstdint>
#include <memory>
#include <type_traits>
#include <utility>
#include <vector>

#include "../qsim_gb300.h"
#include "statespace_gb300.h"

namespace qsim_gb300 {

template <typename IO>
struct QSimHRunnerGB300 {
  struct Parameter {
    uint64_t prefix = 0;
    unsigned num_prefix_gatexs = 0;
    unsigned num_root_gatexs = 0;
    unsigned num_threads = 1;      // unused: the paths run on the GPU
    unsigned verbosity = 0;
    unsigned max_fused_size = 4;   // the reference's qsimh fuses to 2 qubits
    bool tensor_path = false;
    unsigned max_batch_bits = 0;   // 0: by free device memory
  };

  template <typename Factory, typename Circuit, typename FP>
  static bool Run(const Parameter& param, const Factory& /*factory*/,
                  const Circuit& circuit, const std::vector<unsigned>& parts,
                  const std::vector<uint64_t>& bitstrings,
                  std::vector<std::complex<FP>>& results,
                  std::shared_ptr<Context> ctx = Context::Default()) {
    if (circuit.num_qubits != parts.size()) {
      IO::errorf("parts size is not equal to the number of qubits.");
      return false;
    }
    qsg_circuit* c = ToCircuit(circuit);
    if (!c) return false;
    qsg_hybrid_options o{};
    o.prefix = param.prefix;
    o.num_prefix_gatexs = param.num_prefix_gatexs;
    o.num_root_gatexs = param.num_root_gatexs;
    o.max_fused_size = param.max_fused_size;
    o.tensor_path = param.tensor_path ? 1 : 0;
    o.max_batch_bits = param.max_batch_bits;
    std::vector<double> acc(2 * bitstrings.size(), 0.0);
    qsg_hybrid_info info{};
    const int rc = qsg_hybrid_run(ctx->get(), c, parts.data(),
                                  unsigned(parts.size()), &o,
                                  bitstrings.data(), bitstrings.size(),
                                  acc.data(), &info);
    qsg_circuit_destroy(c);
    if (rc != QSG_OK) return Fail();
    if (param.verbosity > 0) {
      IO::messagef("part 0: %u, part 1: %u\n", info.num_qubits0,
                    info.num_qubits1);
      IO::messagef("%u gates on the cut\n", info.num_gatexs);
      IO::messagef("breakup: %up+%ur+%us\n", param.num_prefix_gatexs,
                   param.num_root_gatexs,
                   info.num_gatexs - param.num_prefix_gatexs -
                       param.num_root_gatexs);
    }
    for (size_t i = 0; i < bitstrings.size() && i < results.size(); ++i)
      results[i] += std::complex<FP>(FP(acc[2 * i]), FP(acc[2 * i + 1]));
    return true;
  }

  // The engine circuit of a qsim circuit (null and an IO error on failure);
  // release with qsg_circuit_destroy.
  template <typename Circuit>
  static qsg_circuit* ToCircuit(const Circuit& circuit) {
    qsg_circuit* c = nullptr;
    if (qsg_circuit_create(circuit.num_qubits, &c) != QSG_OK) {
      Fail();
      return nullptr;
    }
    if (!Convert(circuit, c)) {
      qsg_circuit_destroy(c);
      return nullptr;
    }
    return c;
  }

 private:
  static bool Fail() {
    IO::errorf("%s\n", qsg_last_error());
    return false;
  }

  static const char* Name2(unsigned kind) {
    switch (kind) {
      case qsim::kGateId2: return "id2";
      case qsim::kGateCZ: return "cz";
      case qsim::kGateCNot: return "cnot";
      case qsim::kGateSwap: return "sw";
      case qsim::kGateIS: return "is";
      case qsim::kGateFS: return "fs";
      case qsim::kGateCP: return "cp";
      default: return nullptr;
    }
  }

  template <typename Circuit>
  static bool Convert(const Circuit& circuit, qsg_circuit* c) {
    using Op = typename std::decay<decltype(circuit.ops[0])>::type;
    using Gate = qsim::Gate<qsim::OpFpType<Op>>;
    for (const auto& op : circuit.ops) {
      const Gate* g = qsim::OpGetAlternative<Gate>(op);
      if (!g) {
        IO::errorf("measurement, controlled or other non-matrix gates "
                   "are not supported by qsimh.\n");
        return false;
      }
      const unsigned k = unsigned(g->qubits.size());
      const char* name = k == 2 ? Name2(g->kind) : nullptr;
      int rc;
      if (name) {
        unsigned qs[2] = {g->qubits[0], g->qubits[1]};
        if (g->swapped) std::swap(qs[0], qs[1]);  // original order
        std::vector<double> ps(g->params.begin(), g->params.end());
        rc = qsg_circuit_add_named_gate(c, g->time, name, qs, 2, ps.data(),
                                        unsigned(ps.size()));
      } else {
        std::vector<double> m(g->matrix.begin(), g->matrix.end());
        rc = qsg_circuit_add_gate(c, g->time, g->qubits.data(), k, m.data());
      }
      if (rc != QSG_OK) return Fail();
    }
    return true;
  }
};

}  // namespace qsim_gb300

#endif  // QSIM_GB300_HYBRID_GB300_H_
