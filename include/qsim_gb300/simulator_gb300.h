// simulator_gb300.h — header-only Simulator over the GB300 engine's C ABI,
// and the Factory that qsim's runners take.
//
// Drop-in for qsim's SimulatorCUDA<float> (lib/simulator_cuda.h:34-267):
// ApplyGate, ApplyControlledGate, ExpectationValue and SIMDRegisterSize keep
// their names, signatures and the reference's convention that qs (and cqs)
// are sorted ascending and the matrix is row-major interleaved complex with
// bit j of the row/column index <-> qs[j].  Gates of up to 6 target qubits
// are applied (the reference silently ignores larger ones; here they throw).
//
// With FactoryGB300 (below) the reference's QSimRunner (lib/run_qsim.h:33),
// MultiQubitGateFuser (lib/fuser_mqubit.h:39), QuantumTrajectorySimulator
// (lib/qtrajectory.h:35) and ExpectationValue (lib/expect.h:47,105) run on
// this engine unchanged, e.g.
//
//   using Runner = qsim::QSimRunner<qsim::IO, qsim::MultiQubitGateFuser<qsim::IO>,
//                                   qsim_gb300::FactoryGB300>;
#ifndef QSIM_GB300_SIMULATOR_GB300_H_
#define QSIM_GB300_SIMULATOR_GB300_H_

#include <complex>
#include <cstdint>
#include <memory>
#include <vector>

#include "../qsim_gb300.h"
#include "statespace_gb300.h"

namespace qsim_gb300 {

template <typename FP = float>
class SimulatorGB300 {
 public:
  using StateSpace = StateSpaceGB300<FP>;
  using State = typename StateSpace::State;
  using fp_type = typename StateSpace::fp_type;

  explicit SimulatorGB300(std::shared_ptr<Context> ctx = Context::Default())
      : ctx_(std::move(ctx)) {}

  // lib/simulator_cuda.h:70-125.
  void ApplyGate(const std::vector<unsigned>& qs, const fp_type* matrix,
                 State& state) const {
    check(qsg_apply_gate(ctx_->get(), state.get(), state.num_qubits(),
                         qs.data(), unsigned(qs.size()), matrix));
  }

  // lib/simulator_cuda.h:135-207.
  void ApplyControlledGate(const std::vector<unsigned>& qs,
                           const std::vector<unsigned>& cqs, uint64_t cvals,
                           const fp_type* matrix, State& state) const {
    check(qsg_apply_controlled_gate(ctx_->get(), state.get(),
                                    state.num_qubits(), qs.data(),
                                    unsigned(qs.size()), cqs.data(),
                                    unsigned(cqs.size()), cvals, matrix));
  }

  // lib/simulator_cuda.h:216-260.
  std::complex<double> ExpectationValue(const std::vector<unsigned>& qs,
                                        const fp_type* matrix,
                                        const State& state) const {
    double r[2];
    check(qsg_expectation_value(ctx_->get(), state.get(), state.num_qubits(),
                                qs.data(), unsigned(qs.size()), matrix, r));
    return {r[0], r[1]};
  }

  // lib/simulator_cuda.h:265-267.
  static unsigned SIMDRegisterSize() { return qsg_simd_register_size(); }

  // Tensor-core application (tcgen05, split FP16) of a gate on <= 6 qubits;
  // no counterpart in the reference.
  void ApplyGateTensor(const std::vector<unsigned>& qs, const fp_type* matrix,
                       State& state) const {
    check(qsg_apply_gate_tc(ctx_->get(), state.get(), state.num_qubits(),
                            qs.data(), unsigned(qs.size()), matrix));
  }

 private:
  std::shared_ptr<Context> ctx_;
};

// The Factory concept of apps/qsim_base_cuda.cu:123-138: a state space and a
// simulator sharing one context (stream).
struct FactoryGB300 {
  using Simulator = SimulatorGB300<float>;
  using StateSpace = Simulator::StateSpace;

  explicit FactoryGB300(std::shared_ptr<Context> ctx = Context::Default(),
                        StateSpace::Parameter param = StateSpace::Parameter())
      : ctx_(std::move(ctx)), param_(param) {}

  StateSpace CreateStateSpace() const { return StateSpace(param_, ctx_); }
  Simulator CreateSimulator() const { return Simulator(ctx_); }

 private:
  std::shared_ptr<Context> ctx_;
  StateSpace::Parameter param_;
};

}  // namespace qsim_gb300

#endif  // QSIM_GB300_SIMULATOR_GB300_H_
