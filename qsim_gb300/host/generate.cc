// Seeded synthetic workloads.  std::mt19937_64 drives every choice, so a
// (shape, seed) pair names one circuit on every platform.

#include <algorithm>
#include <cmath>
#include <numeric>

#include "engine.h"

namespace qsg {
namespace host {

namespace {

constexpr double kPi = 3.14159265358979323846;

// Uniform integer in [0, n) from a 64-bit engine (platform independent,
// unlike std::uniform_int_distribution).
unsigned draw(std::mt19937_64& g, unsigned n) {
  return unsigned(g() % n);
}

double draw01(std::mt19937_64& g) {
  return double(g() >> 11) * (1.0 / 9007199254740992.0);
}

const char* kSingle[3] = {"x_1_2", "y_1_2", "hz_1_2"};

// Single-qubit layer: for every qubit a gate from {sqrt X, sqrt Y, sqrt W}
// different from its previous one.
void single_layer(Circuit& c, unsigned time, std::vector<int>& prev,
                  std::mt19937_64& g) {
  for (unsigned q = 0; q < c.num_qubits; ++q) {
    int pick;
    if (prev[q] < 0) {
      pick = int(draw(g, 3));
    } else {
      pick = int(draw(g, 2));
      if (pick >= prev[q]) ++pick;
    }
    prev[q] = pick;
    Op op;
    named_gate(kSingle[pick], time, {q}, {}, &op);
    c.ops.push_back(std::move(op));
  }
}

void fsim(Circuit& c, unsigned time, unsigned a, unsigned b) {
  Op op;
  named_gate("fs", time, {a, b}, {kPi / 2, kPi / 6}, &op);
  c.ops.push_back(std::move(op));
}

}  // namespace

Circuit grid_random_circuit(unsigned rows, unsigned cols, unsigned extra,
                            unsigned cycles, uint64_t seed) {
  Circuit c;
  c.num_qubits = rows * cols + extra;
  std::mt19937_64 g(seed);
  // Qubit at (r, col) is r * cols + col; the extra qubits fill row `rows`
  // from column 0.
  auto id = [&](unsigned r, unsigned col) -> int {
    if (col >= cols) return -1;
    if (r < rows) return int(r * cols + col);
    if (r == rows && col < extra) return int(rows * cols + col);
    return -1;
  };
  const unsigned nrows = rows + (extra > 0 ? 1 : 0);
  // Coupler patterns: A/B horizontal (even/odd column), C/D vertical
  // (even/odd row); each qubit has at most one coupler per pattern.
  std::vector<std::vector<std::pair<unsigned, unsigned>>> pat(4);
  for (unsigned r = 0; r < nrows; ++r)
    for (unsigned col = 0; col < cols; ++col) {
      int a = id(r, col);
      if (a < 0) continue;
      int h = id(r, col + 1);
      if (h >= 0) pat[col % 2].push_back({unsigned(a), unsigned(h)});
      int v = id(r + 1, col);
      if (v >= 0) pat[2 + r % 2].push_back({unsigned(a), unsigned(v)});
    }
  const int seq[8] = {0, 1, 2, 3, 2, 3, 0, 1};  // A,B,C,D,C,D,A,B
  std::vector<int> prev(c.num_qubits, -1);
  for (unsigned cyc = 0; cyc < cycles; ++cyc) {
    single_layer(c, 2 * cyc, prev, g);
    for (auto& pr : pat[seq[cyc % 8]]) fsim(c, 2 * cyc + 1, pr.first, pr.second);
  }
  return c;
}

Circuit chain_random_circuit(unsigned n, unsigned cycles, uint64_t seed) {
  Circuit c;
  c.num_qubits = n;
  std::mt19937_64 g(seed);
  std::vector<int> prev(n, -1);
  for (unsigned cyc = 0; cyc < cycles; ++cyc) {
    single_layer(c, 2 * cyc, prev, g);
    for (unsigned q = cyc % 2; q + 1 < n; q += 2) fsim(c, 2 * cyc + 1, q, q + 1);
  }
  return c;
}

Circuit layered_u3_circuit(unsigned n, unsigned layers, unsigned num_controlled,
                           uint64_t seed) {
  Circuit c;
  c.num_qubits = n;
  std::mt19937_64 g(seed);
  std::vector<unsigned> perm(n);
  for (unsigned l = 0; l < layers; ++l) {
    const unsigned t0 = 3 * l;
    for (unsigned q = 0; q < n; ++q) {
      Op op;
      named_gate("u3", t0, {q},
                 {2 * kPi * draw01(g), 2 * kPi * draw01(g), 2 * kPi * draw01(g)},
                 &op);
      c.ops.push_back(std::move(op));
    }
    std::iota(perm.begin(), perm.end(), 0);
    for (unsigned i = n; i > 1; --i) std::swap(perm[i - 1], perm[draw(g, i)]);
    for (unsigned i = 0; i + 1 < n; i += 2) {
      Op op;
      named_gate(draw(g, 2) ? "cnot" : "cz", t0 + 1, {perm[i], perm[i + 1]}, {},
                 &op);
      c.ops.push_back(std::move(op));
    }
    // Controlled U3 gates on random distinct qubits; controls on |1> or |0>.
    for (unsigned j = 0; j < num_controlled; ++j) {
      const unsigned nc = 1 + draw(g, 2);
      std::iota(perm.begin(), perm.end(), 0);
      for (unsigned i = 0; i < nc + 1; ++i)
        std::swap(perm[i], perm[i + draw(g, n - i)]);
      Op op;
      named_gate("u3", t0 + 2, {perm[0]},
                 {2 * kPi * draw01(g), 2 * kPi * draw01(g), 2 * kPi * draw01(g)},
                 &op);
      op.kind = OpKind::kControlled;
      op.cqs.assign(perm.begin() + 1, perm.begin() + 1 + nc);
      std::sort(op.cqs.begin(), op.cqs.end());
      op.cvals = g() & ((uint64_t{1} << nc) - 1);
      op.time = t0 + 2;
      c.ops.push_back(std::move(op));
    }
  }
  // Controlled gates of one layer must not share qubits for the time order
  // to hold; give each its own time step instead.
  unsigned t = 0;
  std::vector<long long> last(n, -1);
  for (auto& op : c.ops) {
    long long need = 0;
    for (unsigned q : op.qs) need = std::max(need, last[q] + 1);
    for (unsigned q : op.cqs) need = std::max(need, last[q] + 1);
    op.time = unsigned(need);
    for (unsigned q : op.qs) last[q] = need;
    for (unsigned q : op.cqs) last[q] = need;
    t = std::max(t, op.time);
  }
  return c;
}

std::vector<PauliTerm> random_pauli_sum(unsigned n, unsigned count,
                                        unsigned max_weight, uint64_t seed) {
  std::mt19937_64 g(seed);
  std::vector<PauliTerm> out;
  std::vector<unsigned> perm(n);
  for (unsigned i = 0; i < count; ++i) {
    PauliTerm t;
    const unsigned w = 1 + draw(g, std::min(max_weight, n));
    std::iota(perm.begin(), perm.end(), 0);
    for (unsigned j = 0; j < w; ++j) std::swap(perm[j], perm[j + draw(g, n - j)]);
    t.qs.assign(perm.begin(), perm.begin() + w);
    std::sort(t.qs.begin(), t.qs.end());
    for (unsigned j = 0; j < w; ++j) t.letters.push_back("XYZ"[draw(g, 3)]);
    t.coeff = 2 * draw01(g) - 1;
    out.push_back(std::move(t));
  }
  return out;
}

}  // namespace host
}  // namespace qsg
