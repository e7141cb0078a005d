// Drop-in check: the reference's own QSimRunner + MultiQubitGateFuser,
// ExpectationValue (lib/expect.h) and QuantumTrajectorySimulator templates
// instantiated with the GB300 Factory.  Built against a qsim checkout's
// headers (-I<qsim>/lib) and include/; runs only where a GPU is present.
//
// Usage: dropin_qsim_runner <circuit.txt> <max_fused_size> <out-prefix>
// Writes <out>.state (complex64, normal order), <out>.samples (uint64,
// 1000 samples with seed 7), <out>.ev (complex<double> of Z0 Z1 through the
// in-place and the copy variants of lib/expect.h) and <out>.traj (per
// repetition of 4 depolarizing-noise trajectories: norm of the final state).

#include <cstdio>
#include <string>
#include <vector>

#include "circuit.h"
#include "channels_cirq.h"
#include "circuit_noisy.h"
#include "circuit_qsim_parser.h"
#include "expect.h"
#include "gates_cirq.h"
#include "qtrajectory.h"
#include "fuser_mqubit.h"
#include "io_file.h"
#include "operation.h"
#include "run_qsim.h"

#include "qsim_gb300/simulator_gb300.h"

int main(int argc, char** argv) {
  using namespace qsim;
  if (argc < 4) return 2;
  Circuit<Operation<float>> circuit;
  if (!CircuitQsimParser<IOFile>::FromFile(~0u, argv[1], circuit)) return 1;
  using Factory = qsim_gb300::FactoryGB300;
  using Runner = QSimRunner<IO, MultiQubitGateFuser<IO>, Factory>;
  Factory factory;
  auto ss = factory.CreateStateSpace();
  auto state = ss.Create(circuit.num_qubits);
  if (ss.IsNull(state)) return 3;
  ss.SetStateZero(state);
  Runner::Parameter param;
  param.max_fused_size = std::atoi(argv[2]);
  param.seed = 1;
  param.verbosity = 0;
  if (!Runner::Run(param, factory, circuit, state)) return 4;
  std::vector<float> host(ss.MinSize(circuit.num_qubits));
  ss.Copy(state, host.data());
  std::string out = argv[3];
  FILE* f = std::fopen((out + ".state").c_str(), "wb");
  std::fwrite(host.data(), sizeof(float), size_t(2) << circuit.num_qubits, f);
  std::fclose(f);
  auto samples = ss.Sample(state, 1000, 7);
  f = std::fopen((out + ".samples").c_str(), "wb");
  std::fwrite(samples.data(), sizeof(uint64_t), samples.size(), f);
  std::fclose(f);
  // Expectation value of Z0 Z1 (lib/expect.h:105-151 and :47-91).
  using fp = float;
  std::vector<OpString<fp>> strings = {
      {{1.0, 0.0},
       {GateZ<fp>::Create(0, 0), GateZ<fp>::Create(0, 1)}}};
  auto sim = factory.CreateSimulator();
  auto ev1 = ExpectationValue<IO, MultiQubitGateFuser<IO>>(strings, sim, state);
  auto ket = ss.Null();
  MultiQubitGateFuser<IO>::Parameter fparam;
  auto ev2 = ExpectationValue<IO, MultiQubitGateFuser<IO>>(fparam, strings, ss,
                                                           sim, state, ket);
  double evs[4] = {ev1.real(), ev1.imag(), ev2.real(), ev2.imag()};
  f = std::fopen((out + ".ev").c_str(), "wb");
  std::fwrite(evs, sizeof(double), 4, f);
  std::fclose(f);

  // Noisy trajectories through QuantumTrajectorySimulator
  // (lib/qtrajectory.h:141-180): depolarizing p = 0.01 after every gate.
  auto noisy = MakeNoisy<fp>(circuit.num_qubits, circuit.ops.begin(),
                             circuit.ops.end(),
                             Cirq::DepolarizingChannel<fp>(0.01));
  using QTSim = QuantumTrajectorySimulator<IO, Runner>;
  QTSim::Parameter tparam;
  tparam.max_fused_size = param.max_fused_size;
  std::vector<double> norms;
  auto measure = [&](uint64_t r, const Factory::StateSpace::State& s,
                     const QTSim::Stat&) { norms.push_back(ss.Norm(s)); };
  if (!QTSim::RunBatch(tparam, noisy, 0, 4, ss, sim, measure)) return 5;
  f = std::fopen((out + ".traj").c_str(), "wb");
  std::fwrite(norms.data(), sizeof(double), norms.size(), f);
  std::fclose(f);
  std::printf("norm %.9f ev %.9f %.9f\n", ss.Norm(state), ev1.real(),
              ev2.real());
  return 0;
}
