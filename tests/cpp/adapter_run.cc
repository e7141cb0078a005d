// Adapter check without the reference: applies a gate list (the golden
// fixtures' text format, see tests/golden/make_golden.py) through
// qsim_gb300::SimulatorGB300 / StateSpaceGB300, then measures and samples.
//
// Usage: adapter_run <gates.txt> <out-prefix> <measure-seed> <q...>
// Writes <out>.state (complex64 after the gates), <out>.normal and
// <out>.internal (the state after InternalToNormalOrder, then after
// NormalToInternalOrder), <out>.bits (one Measure(qubits,
// std::mt19937(seed))), <out>.after (state after it), <out>.samples (1000
// samples, seed 7) and <out>.samples_f32 (the same with Sample<float>).

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <random>
#include <sstream>
#include <string>
#include <vector>

#include "qsim_gb300/simulator_gb300.h"

int main(int argc, char** argv) {
  if (argc < 5) return 2;
  using Factory = qsim_gb300::FactoryGB300;
  Factory factory;
  auto ss = factory.CreateStateSpace();
  auto sim = factory.CreateSimulator();
  std::ifstream in(argv[1]);
  std::string line, out = argv[2];
  unsigned n = 0;
  std::vector<std::vector<float>> mats;
  Factory::StateSpace::State state = Factory::StateSpace::Null();
  while (std::getline(in, line)) {
    std::istringstream ss_line(line);
    std::string tag;
    ss_line >> tag;
    if (tag == "n") {
      ss_line >> n;
      state = ss.Create(n);
      ss.SetStateZero(state);
      continue;
    }
    unsigned time, k;
    ss_line >> time >> k;
    std::vector<unsigned> qs(k), cqs;
    for (auto& q : qs) ss_line >> q;
    uint64_t cvals = 0;
    if (tag == "c") {
      unsigned c;
      ss_line >> c;
      cqs.resize(c);
      for (auto& q : cqs) ss_line >> q;
      ss_line >> cvals;
    }
    if (tag == "m") continue;
    std::vector<float> m(2u << (2 * k));
    for (auto& x : m) {
      std::string t;
      ss_line >> t;
      x = std::strtof(t.c_str(), nullptr);
    }
    if (tag == "c") sim.ApplyControlledGate(qs, cqs, cvals, m.data(), state);
    else sim.ApplyGate(qs, m.data(), state);
  }
  std::vector<float> host(ss.MinSize(n));
  auto dump = [&](const std::string& ext) {
    ss.Copy(state, host.data());
    FILE* f = std::fopen((out + ext).c_str(), "wb");
    std::fwrite(host.data(), sizeof(float), size_t(2) << n, f);
    std::fclose(f);
  };
  dump(".state");
  // The internal order is the normal order: both conversions leave the
  // state as it is.
  ss.InternalToNormalOrder(state);
  dump(".normal");
  ss.NormalToInternalOrder(state);
  dump(".internal");
  auto samples = ss.Sample(state, 1000, 7);
  FILE* f = std::fopen((out + ".samples").c_str(), "wb");
  std::fwrite(samples.data(), sizeof(uint64_t), samples.size(), f);
  std::fclose(f);
  // Sample<float>: uniforms drawn with uniform_real_distribution<float>.
  auto samples32 = ss.Sample<float>(state, 1000, 7);
  f = std::fopen((out + ".samples_f32").c_str(), "wb");
  std::fwrite(samples32.data(), sizeof(uint64_t), samples32.size(), f);
  std::fclose(f);
  std::vector<unsigned> mq;
  for (int i = 4; i < argc; ++i) mq.push_back(std::atoi(argv[i]));
  std::mt19937 rgen(std::atoi(argv[3]));
  auto res = ss.Measure(mq, rgen, state);
  f = std::fopen((out + ".bits").c_str(), "wb");
  uint64_t bits = res.valid ? res.bits : ~uint64_t{0};
  std::fwrite(&bits, sizeof(bits), 1, f);
  std::fclose(f);
  dump(".after");
  std::printf("ok %u %.9f\n", n, ss.Norm(state));
  return 0;
}
