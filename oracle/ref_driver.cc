// ref_driver.cc — TEST INFRASTRUCTURE ONLY (builds into oracle/_ref/).
//
// Runs the reference implementation (quantumlib/qsim, header-only C++) on
// gate lists written by tests/golden/make_golden.py and writes its outputs
// as raw binary files, which become the golden fixtures under tests/golden/.
// Compiled against the reference headers where they lie (-I<qsim>/lib); no
// reference source is copied.
//
// Gate-list format (one op per line, matrices as C99 hex floats, qubits
// sorted ascending and the matrix already in that order):
//   n <num_qubits>
//   g <time> <k> <q...> <2*4^k floats>                 matrix gate
//   c <time> <k> <q...> <c> <cq...> <cvals> <floats>   controlled gate
//   m <time> <k> <q...>                                measurement
//
// Commands:
//   mt <seed> <count> <out>
//       raw std::mt19937 outputs (uint32) then `count` draws of
//       uniform_real_distribution<double>(0,1) from a fresh mt19937(seed)
//       (.u01), and `count` draws of uniform_real_distribution<float>(0,
//       0.73) from another fresh mt19937(seed) (.f073).
//   run <gates> <out-prefix> <max_fused_size> <num_samples> <sample_seed>
//       [<ev-file>]
//       .f64  : final state of SimulatorBasic<For,double>, ops unfused
//       .f32  : final state of QSimRunner + MultiQubitGateFuser +
//               the host's SIMD simulator (float)
//       .s32  : Sample(f32 state, num_samples, seed)
//       .s64  : Sample(f64 state, num_samples, seed)
//       .ev   : per EV line: <k> <q...> <floats> -> complex<double> on the
//               f32 state (SIMD) then on the f64 state (basic)
//       .meta : norm, number of fused ops
//   unitary <gates> <out>
//       the full unitary of UnitaryCalculatorBasic<For,double> applied to
//       the identity (matrix and controlled gates, in order): 4^n complex
//       doubles, entry (i, j) at i * 2^n + j (the reference's layout).
//   text <circuit.txt> <out-prefix>
//       reference text format through CircuitQsimParser, FP64 state (.f64)
//   fuse <gates> <max_fused_size>
//       number of fused ops of MultiQubitGateFuser and their size histogram
//   traj <noisy> <out-prefix> <max_fused_size> <r0> <r1>
//       The gate list may also hold channels (one qubit each):
//         D|A|P|B|F <time> <q> <param>   depolarizing, amplitude damping,
//                                        phase damping, bit flip, phase flip
//         R <time> <q>                   reset
//         Q <time> <k> <q...> <p>        depolarizing on k qubits (the
//                                        reference's multi-qubit factory)
//       Runs QuantumTrajectorySimulator::RunBatch over repetitions [r0, r1)
//       with QSimRunner + MultiQubitGateFuser, collect_kop_stat and
//       collect_mea_stat on, in float (host SIMD simulator) and in double
//       (SimulatorBasic).  Writes per repetition the count and the
//       stat.samples (.stat32 / .stat64, uint64) and the final state in
//       normal order (.f32 / .f64).
//   hybrid <circuit.txt> <out> <num_prefix> <num_root> <prefix> <parts>
//          <bitstrings>
//       QSimHRunner<IO, BasicGateFuser, HybridSimulator>::Run on the text
//       circuit (CircuitQsimParser, double), parts as "0,1,1,...", the
//       bitstrings a raw uint64 file; writes the amplitudes as complex
//       doubles (each result starts from 0).
//   plan <gates> <max_fused_size> <out>
//       MultiQubitGateFuser's fused gates for the gate list (matrix gates
//       only), as QSimRunner applies them: per fused gate a uint32 k, k
//       uint32 qubits (ascending) and the 2*4^k floats of its matrix
//       (CalculateFusedMatrix, lib/fuser.h:149-179).
//   bench <gates> <max_fused_size> <reps> <threads>
//       QSimRunner<IO, MultiQubitGateFuser, host SIMD simulator>::Run on
//       the gate list from |0...0> in float with ParallelFor(threads),
//       `reps` times; prints one line per run: the wall seconds of Run
//       (fusion + every fused gate, the state synchronised), then the
//       seconds of FuseGates alone.
//   trajbench <gates> <max_fused_size> <reps> <threads>
//       QuantumTrajectorySimulator<IO, QSimRunner<IO, MultiQubitGateFuser,
//       host SIMD simulator>>::RunBatch over the noisy gate list (gates and
//       channels) in float with ParallelFor(threads): one warm-up
//       repetition (r = 10^6), then repetitions r = 0..reps-1, one line of
//       wall seconds each (each from |0...0>, lib/qtrajectory.h:141-180).
//   measure <gates> <out-prefix> <seed> <reps> <k> <q...>
//       From the f64 final state: `reps` rounds of Measure(qubits, rgen)
//       with one std::mt19937(seed); writes bits per round (.bits) and the
//       collapsed state after the last round (.f64).

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <random>
#include <sstream>
#include <string>
#include <vector>

#include "channel.h"
#include "channels_cirq.h"
#include "circuit.h"
#include "circuit_qsim_parser.h"
#include "io_file.h"
#include "formux.h"
#include "fuser_basic.h"
#include "fuser_mqubit.h"
#include "gate.h"
#include "gate_appl.h"
#include "gates_qsim.h"
#include "hybrid.h"
#include "io.h"
#include "operation.h"
#include "qtrajectory.h"
#include "run_qsim.h"
#include "run_qsimh.h"
#include "simmux.h"
#include "simulator_basic.h"
#include "statespace_basic.h"
#include "unitary_calculator_basic.h"
#include "unitaryspace_basic.h"

using namespace qsim;

struct GateSpec {
  char kind;
  unsigned time;
  std::vector<unsigned> qs, cqs;
  uint64_t cvals = 0;
  std::vector<float> m;
  double param = 0;  // channels
};

static bool IsChannel(char k) {
  return k == 'D' || k == 'A' || k == 'P' || k == 'B' || k == 'F' || k == 'R' ||
         k == 'Q';
}

static std::vector<GateSpec> ReadGates(const char* path, unsigned& n) {
  std::ifstream f(path);
  std::string line;
  std::vector<GateSpec> out;
  while (std::getline(f, line)) {
    std::istringstream ss(line);
    std::string tag;
    ss >> tag;
    if (tag == "n") {
      ss >> n;
      continue;
    }
    GateSpec g;
    g.kind = tag[0];
    if (g.kind == 'Q') {
      // Q <time> <k> <q...> <p>: multi-qubit depolarizing channel.
      unsigned k;
      ss >> g.time >> k;
      g.qs.resize(k);
      for (auto& q : g.qs) ss >> q;
      std::string t;
      ss >> t;
      g.param = std::strtod(t.c_str(), nullptr);
      out.push_back(std::move(g));
      continue;
    }
    if (IsChannel(g.kind)) {
      g.qs.resize(1);
      ss >> g.time >> g.qs[0];
      if (g.kind != 'R') {
        std::string t;
        ss >> t;
        g.param = std::strtod(t.c_str(), nullptr);
      }
      out.push_back(std::move(g));
      continue;
    }
    unsigned k;
    ss >> g.time >> k;
    g.qs.resize(k);
    for (auto& q : g.qs) ss >> q;
    if (g.kind == 'c') {
      unsigned c;
      ss >> c;
      g.cqs.resize(c);
      for (auto& q : g.cqs) ss >> q;
      ss >> g.cvals;
    }
    if (g.kind != 'm') {
      size_t cnt = 2u << (2 * k);
      g.m.resize(cnt);
      for (auto& x : g.m) {
        std::string t;
        ss >> t;
        x = std::strtof(t.c_str(), nullptr);
      }
    }
    out.push_back(std::move(g));
  }
  return out;
}

template <typename FP>
static Operation<FP> ToOp(const GateSpec& g) {
  if (g.kind == 'm') return CreateMeasurement(g.time, g.qs);
  const unsigned q = g.qs.empty() ? 0 : g.qs[0];
  switch (g.kind) {
    case 'D':
      return Cirq::DepolarizingChannel<FP>::Create(g.time, q, g.param);
    case 'Q':
      return Cirq::DepolarizingChannel<FP>::Create(g.time, g.qs, g.param);
    case 'A':
      return Cirq::AmplitudeDampingChannel<FP>::Create(g.time, q, g.param);
    case 'P':
      return Cirq::PhaseDampingChannel<FP>::Create(g.time, q, g.param);
    case 'B':
      return Cirq::BitFlipChannel<FP>::Create(g.time, q, g.param);
    case 'F':
      return Cirq::PhaseFlipChannel<FP>::Create(g.time, q, g.param);
    case 'R':
      return Cirq::ResetChannel<FP>::Create(g.time, q);
    default:
      break;
  }
  Gate<FP> gate;
  gate.kind = kGateMatrix1;
  gate.time = g.time;
  gate.qubits = g.qs;
  gate.matrix.assign(g.m.begin(), g.m.end());
  gate.swapped = false;
  if (g.kind == 'c') {
    return ControlledGate<FP>{gate, g.cqs, g.cvals};
  }
  return gate;
}

static void WriteRaw(const std::string& path, const void* p, size_t bytes) {
  FILE* f = std::fopen(path.c_str(), "wb");
  std::fwrite(p, 1, bytes, f);
  std::fclose(f);
}

static int CmdMt(int argc, char** argv) {
  unsigned seed = std::atoi(argv[2]);
  unsigned count = std::atoi(argv[3]);
  std::mt19937 g(seed);
  std::vector<uint32_t> raw(count);
  for (auto& x : raw) x = g();
  std::mt19937 g2(seed);
  std::uniform_real_distribution<double> d(0.0, 1.0);
  std::vector<double> u(count);
  for (auto& x : u) x = d(g2);
  std::mt19937 g3(seed);
  std::uniform_real_distribution<float> df(0.0f, 0.73f);
  std::vector<float> uf(count);
  for (auto& x : uf) x = df(g3);
  std::string out = argv[4];
  WriteRaw(out + ".raw", raw.data(), raw.size() * 4);
  WriteRaw(out + ".u01", u.data(), u.size() * 8);
  WriteRaw(out + ".f073", uf.data(), uf.size() * 4);
  return 0;
}

struct Factory32 {
  using Simulator = qsim::Simulator<For>;
  using StateSpace = Simulator::StateSpace;
  StateSpace CreateStateSpace() const { return StateSpace(1); }
  Simulator CreateSimulator() const { return Simulator(1); }
};

static int CmdRun(int argc, char** argv) {
  unsigned n = 0;
  auto specs = ReadGates(argv[2], n);
  std::string out = argv[3];
  unsigned fsize = std::atoi(argv[4]);
  uint64_t nsamples = std::strtoull(argv[5], nullptr, 10);
  unsigned sseed = std::atoi(argv[6]);

  // FP64, unfused: the reference's own FP64 oracle.
  using Sim64 = SimulatorBasic<For, double>;
  using SS64 = Sim64::StateSpace;
  SS64 ss64(1);
  Sim64 sim64(1);
  auto s64 = ss64.Create(n);
  ss64.SetStateZero(s64);
  for (const auto& g : specs) {
    auto op = ToOp<double>(g);
    ApplyGate(sim64, op, s64);
  }
  WriteRaw(out + ".f64", s64.get(), sizeof(double) * SS64::MinSize(n));

  // FP32 through QSimRunner + MultiQubitGateFuser + SIMD simulator.
  Circuit<Operation<float>> circuit;
  circuit.num_qubits = n;
  for (const auto& g : specs) circuit.ops.push_back(ToOp<float>(g));
  using Runner = QSimRunner<IO, MultiQubitGateFuser<IO>, Factory32>;
  Runner::Parameter param;
  param.max_fused_size = fsize;
  param.seed = 1;
  param.verbosity = 0;
  Factory32 factory;
  auto ss32 = factory.CreateStateSpace();
  auto sim32 = factory.CreateSimulator();
  auto s32 = ss32.Create(n);
  ss32.SetStateZero(s32);
  if (!Runner::Run(param, factory, circuit, s32)) {
    std::fprintf(stderr, "run failed\n");
    return 1;
  }
  ss32.InternalToNormalOrder(s32);
  WriteRaw(out + ".f32", s32.get(), sizeof(float) * 2 * (uint64_t{1} << n));
  ss32.NormalToInternalOrder(s32);

  auto fused = MultiQubitGateFuser<IO>::FuseGates(
      MultiQubitGateFuser<IO>::Parameter{fsize, 0}, n, circuit.ops);

  if (nsamples > 0) {
    auto b32 = ss32.Sample(s32, nsamples, sseed);
    WriteRaw(out + ".s32", b32.data(), b32.size() * 8);
    auto b64 = ss64.Sample(s64, nsamples, sseed);
    WriteRaw(out + ".s64", b64.data(), b64.size() * 8);
  }

  if (argc > 7) {
    std::ifstream f(argv[7]);
    std::string line;
    std::vector<double> evs;
    while (std::getline(f, line)) {
      std::istringstream ss(line);
      unsigned k;
      if (!(ss >> k)) continue;
      std::vector<unsigned> qs(k);
      for (auto& q : qs) ss >> q;
      std::vector<float> m32(2u << (2 * k));
      for (auto& x : m32) {
        std::string t;
        ss >> t;
        x = std::strtof(t.c_str(), nullptr);
      }
      std::vector<double> m64(m32.begin(), m32.end());
      auto e32 = sim32.ExpectationValue(qs, m32.data(), s32);
      auto e64 = sim64.ExpectationValue(qs, m64.data(), s64);
      evs.push_back(e32.real());
      evs.push_back(e32.imag());
      evs.push_back(e64.real());
      evs.push_back(e64.imag());
    }
    WriteRaw(out + ".ev", evs.data(), evs.size() * 8);
  }

  double meta[2] = {ss64.Norm(s64), double(fused.size())};
  WriteRaw(out + ".meta", meta, sizeof(meta));
  return 0;
}

static int CmdMeasure(int argc, char** argv) {
  unsigned n = 0;
  auto specs = ReadGates(argv[2], n);
  std::string out = argv[3];
  unsigned seed = std::atoi(argv[4]);
  unsigned reps = std::atoi(argv[5]);
  unsigned k = std::atoi(argv[6]);
  std::vector<unsigned> qs(k);
  for (unsigned i = 0; i < k; ++i) qs[i] = std::atoi(argv[7 + i]);

  using Sim64 = SimulatorBasic<For, double>;
  using SS64 = Sim64::StateSpace;
  SS64 ss64(1);
  Sim64 sim64(1);
  auto s64 = ss64.Create(n);
  ss64.SetStateZero(s64);
  for (const auto& g : specs) {
    auto op = ToOp<double>(g);
    ApplyGate(sim64, op, s64);
  }
  std::mt19937 rgen(seed);
  std::vector<uint64_t> bits;
  for (unsigned r = 0; r < reps; ++r) {
    auto res = ss64.Measure(qs, rgen, s64);
    bits.push_back(res.valid ? res.bits : ~uint64_t{0});
  }
  WriteRaw(out + ".bits", bits.data(), bits.size() * 8);
  WriteRaw(out + ".f64", s64.get(), sizeof(double) * SS64::MinSize(n));
  return 0;
}

struct Factory64 {
  using Simulator = SimulatorBasic<For, double>;
  using StateSpace = Simulator::StateSpace;
  StateSpace CreateStateSpace() const { return StateSpace(1); }
  Simulator CreateSimulator() const { return Simulator(1); }
};

template <typename FP, typename Factory>
static bool RunTraj(const std::vector<GateSpec>& specs, unsigned n,
                    unsigned fsize, uint64_t r0, uint64_t r1,
                    const std::string& out, const char* suffix) {
  Circuit<Operation<FP>> circuit;
  circuit.num_qubits = n;
  for (const auto& g : specs) circuit.ops.push_back(ToOp<FP>(g));
  using Runner = QSimRunner<IO, MultiQubitGateFuser<IO>, Factory>;
  using QTSim = QuantumTrajectorySimulator<IO, Runner>;
  typename QTSim::Parameter param;
  param.max_fused_size = fsize;
  param.verbosity = 0;
  param.collect_kop_stat = true;
  param.collect_mea_stat = true;
  Factory factory;
  auto ss = factory.CreateStateSpace();
  auto sim = factory.CreateSimulator();
  std::vector<uint64_t> stats;
  std::vector<FP> states;
  auto tmp = ss.Create(n);
  auto measure = [&](uint64_t, const typename Factory::StateSpace::State& st,
                     const typename QTSim::Stat& stat) {
    stats.push_back(stat.samples.size());
    stats.insert(stats.end(), stat.samples.begin(), stat.samples.end());
    ss.Copy(st, tmp);
    ss.InternalToNormalOrder(tmp);
    states.insert(states.end(), tmp.get(), tmp.get() + 2 * (uint64_t{1} << n));
  };
  if (!QTSim::RunBatch(param, circuit, r0, r1, ss, sim, measure)) return false;
  WriteRaw(out + ".stat" + suffix, stats.data(), stats.size() * 8);
  WriteRaw(out + ".f" + suffix, states.data(), states.size() * sizeof(FP));
  return true;
}

static int CmdTraj(int argc, char** argv) {
  unsigned n = 0;
  auto specs = ReadGates(argv[2], n);
  std::string out = argv[3];
  unsigned fsize = std::atoi(argv[4]);
  uint64_t r0 = std::strtoull(argv[5], nullptr, 10);
  uint64_t r1 = std::strtoull(argv[6], nullptr, 10);
  if (!RunTraj<float, Factory32>(specs, n, fsize, r0, r1, out, "32")) return 1;
  if (!RunTraj<double, Factory64>(specs, n, fsize, r0, r1, out, "64")) return 1;
  return 0;
}

// fuse <gates> <max_fused_size>: prints the number of fused operations
// MultiQubitGateFuser produces and the size histogram.
static int CmdFuse(int argc, char** argv) {
  unsigned n = 0;
  auto specs = ReadGates(argv[2], n);
  unsigned fsize = std::atoi(argv[3]);
  Circuit<Operation<float>> circuit;
  circuit.num_qubits = n;
  for (const auto& g : specs) circuit.ops.push_back(ToOp<float>(g));
  auto fused = MultiQubitGateFuser<IO>::FuseGates(
      MultiQubitGateFuser<IO>::Parameter{fsize, 0}, n, circuit.ops);
  unsigned hist[8] = {0};
  for (const auto& op : fused) {
    if (const auto* pg = OpGetAlternative<FusedGate<float>>(op)) {
      ++hist[std::min<size_t>(pg->qubits.size(), 7)];
    }
  }
  std::printf("%zu", fused.size());
  for (unsigned k = 0; k < 8; ++k) std::printf(" %u", hist[k]);
  std::printf("\n");
  return 0;
}

// text <circuit.txt> <out-prefix>: parses the reference text format with
// CircuitQsimParser (FP64 gates) and applies every gate, unfused, with
// SimulatorBasic<For,double>; measurements are skipped.  Writes .f64.
static int CmdText(int argc, char** argv) {
  Circuit<Operation<double>> circuit;
  if (!CircuitQsimParser<IOFile>::FromFile(~0u, argv[2], circuit)) return 1;
  unsigned n = circuit.num_qubits;
  using Sim64 = SimulatorBasic<For, double>;
  using SS64 = Sim64::StateSpace;
  SS64 ss64(1);
  Sim64 sim64(1);
  auto s64 = ss64.Create(n);
  ss64.SetStateZero(s64);
  for (const auto& op : circuit.ops) ApplyGate(sim64, op, s64);
  WriteRaw(std::string(argv[3]) + ".f64", s64.get(),
           sizeof(double) * SS64::MinSize(n));
  return 0;
}

static int CmdUnitary(int argc, char** argv) {
  if (argc < 4) return 2;
  unsigned n = 0;
  auto specs = ReadGates(argv[2], n);
  using UC = unitary::UnitaryCalculatorBasic<For, double>;
  using US = UC::UnitarySpace;
  US us(1);
  UC uc(1);
  auto u = us.CreateUnitary(n);
  us.SetIdentity(u);
  for (const auto& g : specs) {
    std::vector<double> m(g.m.begin(), g.m.end());
    if (g.kind == 'g') uc.ApplyGate(g.qs, m.data(), u);
    else if (g.kind == 'c')
      uc.ApplyControlledGate(g.qs, g.cqs, g.cvals, m.data(), u);
  }
  WriteRaw(argv[3], u.get(), sizeof(double) * US::MinSize(n));
  return 0;
}

struct HybridFactory {
  using Simulator = SimulatorBasic<For, double>;
  using StateSpace = Simulator::StateSpace;
  using fp_type = double;
  StateSpace CreateStateSpace() const { return StateSpace(1); }
  Simulator CreateSimulator() const { return Simulator(1); }
};

static int CmdHybrid(int argc, char** argv) {
  if (argc < 9) return 2;
  Circuit<Operation<double>> circuit;
  if (!CircuitQsimParser<IOFile>::FromFile(~0u, argv[2], circuit)) return 1;
  std::vector<unsigned> parts;
  {
    std::stringstream ss(argv[7]);
    std::string tok;
    while (std::getline(ss, tok, ',')) parts.push_back(std::stoul(tok));
  }
  std::vector<uint64_t> bitstrings;
  {
    std::ifstream in(argv[8], std::ios::binary);
    uint64_t b;
    while (in.read(reinterpret_cast<char*>(&b), sizeof(b))) bitstrings.push_back(b);
  }
  using HS = HybridSimulator<IO, For>;
  using Runner = QSimHRunner<IO, BasicGateFuser<IO>, HS>;
  Runner::Parameter param;
  param.num_prefix_gatexs = std::stoul(argv[4]);
  param.num_root_gatexs = std::stoul(argv[5]);
  param.prefix = std::stoull(argv[6]);
  param.num_threads = 1;
  param.verbosity = 0;
  std::vector<std::complex<double>> results(bitstrings.size(), 0);
  if (!Runner::Run(param, HybridFactory(), circuit, parts, bitstrings, results))
    return 1;
  WriteRaw(argv[3], results.data(), sizeof(std::complex<double>) * results.size());
  return 0;
}

struct Factory32T {
  using Simulator = qsim::Simulator<For>;
  using StateSpace = Simulator::StateSpace;
  unsigned threads = 1;
  StateSpace CreateStateSpace() const { return StateSpace(threads); }
  Simulator CreateSimulator() const { return Simulator(threads); }
};

static int CmdPlan(int argc, char** argv) {
  unsigned n = 0;
  auto specs = ReadGates(argv[2], n);
  unsigned fsize = std::atoi(argv[3]);
  Circuit<Operation<float>> circuit;
  circuit.num_qubits = n;
  for (const auto& g : specs) circuit.ops.push_back(ToOp<float>(g));
  auto fused = MultiQubitGateFuser<IO>::FuseGates(
      MultiQubitGateFuser<IO>::Parameter{fsize, 0}, n, circuit.ops);
  FILE* f = std::fopen(argv[4], "wb");
  if (!f) return 1;
  for (const auto& op : fused) {
    const auto* pg = OpGetAlternative<FusedGate<float>>(op);
    if (!pg) continue;
    const uint32_t k = pg->qubits.size();
    std::fwrite(&k, 4, 1, f);
    for (unsigned q : pg->qubits) {
      const uint32_t q32 = q;
      std::fwrite(&q32, 4, 1, f);
    }
    std::fwrite(pg->matrix.data(), sizeof(float), pg->matrix.size(), f);
  }
  std::fclose(f);
  return 0;
}

static int CmdBench(int argc, char** argv) {
  unsigned n = 0;
  auto specs = ReadGates(argv[2], n);
  unsigned fsize = std::atoi(argv[3]);
  unsigned reps = std::atoi(argv[4]);
  Circuit<Operation<float>> circuit;
  circuit.num_qubits = n;
  for (const auto& g : specs) circuit.ops.push_back(ToOp<float>(g));
  Factory32T factory;
  factory.threads = std::atoi(argv[5]);
  using Runner = QSimRunner<IO, MultiQubitGateFuser<IO>, Factory32T>;
  Runner::Parameter param;
  param.max_fused_size = fsize;
  param.seed = 1;
  param.verbosity = 0;
  auto ss = factory.CreateStateSpace();
  auto s = ss.Create(n);
  if (ss.IsNull(s)) return 1;
  for (unsigned r = 0; r < reps; ++r) {
    ss.SetStateZero(s);
    const double t0 = GetTime();
    if (!Runner::Run(param, factory, circuit, s)) return 1;
    ss.DeviceSync();
    const double t1 = GetTime();
    auto fused = MultiQubitGateFuser<IO>::FuseGates(
        MultiQubitGateFuser<IO>::Parameter{fsize, 0}, n, circuit.ops);
    const double t2 = GetTime();
    std::printf("%.6f %.6f %zu\n", t1 - t0, t2 - t1, fused.size());
    std::fflush(stdout);
  }
  return 0;
}

static int CmdTrajBench(int argc, char** argv) {
  if (argc < 6) return 2;
  unsigned n = 0;
  auto specs = ReadGates(argv[2], n);
  const unsigned fsize = std::atoi(argv[3]);
  const unsigned reps = std::atoi(argv[4]);
  Circuit<Operation<float>> circuit;
  circuit.num_qubits = n;
  for (const auto& g : specs) circuit.ops.push_back(ToOp<float>(g));
  Factory32T factory;
  factory.threads = std::atoi(argv[5]);
  using Runner = QSimRunner<IO, MultiQubitGateFuser<IO>, Factory32T>;
  using QTSim = QuantumTrajectorySimulator<IO, Runner>;
  typename QTSim::Parameter param;
  param.max_fused_size = fsize;
  param.verbosity = 0;
  auto ss = factory.CreateStateSpace();
  auto sim = factory.CreateSimulator();
  auto measure = [](uint64_t, const Factory32T::StateSpace::State&,
                    const typename QTSim::Stat&) {};
  if (!QTSim::RunBatch(param, circuit, 1000000, 1000001, ss, sim, measure))
    return 1;
  for (unsigned r = 0; r < reps; ++r) {
    const double t0 = GetTime();
    if (!QTSim::RunBatch(param, circuit, r, r + 1, ss, sim, measure)) return 1;
    std::printf("%.6f\n", GetTime() - t0);
    std::fflush(stdout);
  }
  return 0;
}

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  if (std::string(argv[1]) == "unitary") return CmdUnitary(argc, argv);
  std::string cmd = argv[1];
  if (cmd == "text") return CmdText(argc, argv);
  if (cmd == "hybrid") return CmdHybrid(argc, argv);
  if (cmd == "fuse") return CmdFuse(argc, argv);
  if (cmd == "mt") return CmdMt(argc, argv);
  if (cmd == "run") return CmdRun(argc, argv);
  if (cmd == "measure") return CmdMeasure(argc, argv);
  if (cmd == "traj") return CmdTraj(argc, argv);
  if (cmd == "plan") return CmdPlan(argc, argv);
  if (cmd == "bench") return CmdBench(argc, argv);
  if (cmd == "trajbench") return CmdTrajBench(argc, argv);
  return 2;
}
