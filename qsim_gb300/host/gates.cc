// Gate library: the reference's qsim gate set (lib/gates_qsim.h; names as in
// docs/input_format.md) plus U3, written from the gates' definitions.
// Matrices are row-major with bit j of the row/column index <-> qubits[j].

#include <algorithm>
#include <cmath>
#include <numeric>

#include "engine.h"

namespace qsg {
namespace host {

namespace {

constexpr double kPi = 3.14159265358979323846;
const cplx I(0.0, 1.0);

std::vector<cplx> m1(cplx a, cplx b, cplx c, cplx d) { return {a, b, c, d}; }

// Diagonal 4x4 plus an off-diagonal block in rows/cols 1,2.
std::vector<cplx> m2(cplx d0, cplx a11, cplx a12, cplx a21, cplx a22, cplx d3) {
  std::vector<cplx> m(16, 0.0);
  m[0] = d0;
  m[5] = a11;
  m[6] = a12;
  m[9] = a21;
  m[10] = a22;
  m[15] = d3;
  return m;
}

}  // namespace

Op make_gate(unsigned time, std::vector<unsigned> qubits, std::vector<cplx> m) {
  const unsigned k = qubits.size();
  Op op;
  op.kind = OpKind::kGate;
  op.time = time;
  std::vector<unsigned> order(k);
  std::iota(order.begin(), order.end(), 0);
  std::sort(order.begin(), order.end(),
            [&](unsigned a, unsigned b) { return qubits[a] < qubits[b]; });
  bool sorted = true;
  for (unsigned j = 0; j < k; ++j) sorted &= order[j] == j;
  op.qs.resize(k);
  for (unsigned j = 0; j < k; ++j) op.qs[j] = qubits[order[j]];
  if (sorted) {
    op.m = std::move(m);
    return op;
  }
  // pos[j]: position of given qubit j in the sorted list.
  std::vector<unsigned> pos(k);
  for (unsigned j = 0; j < k; ++j) pos[order[j]] = j;
  const unsigned d = 1u << k;
  auto perm = [&](unsigned i) {
    unsigned r = 0;
    for (unsigned j = 0; j < k; ++j)
      if ((i >> j) & 1) r |= 1u << pos[j];
    return r;
  };
  op.m.assign(size_t(d) * d, 0.0);
  for (unsigned r = 0; r < d; ++r)
    for (unsigned c = 0; c < d; ++c) op.m[perm(r) * d + perm(c)] = m[r * d + c];
  return op;
}

std::vector<cplx> u3_matrix(double theta, double phi, double lambda) {
  const double c = std::cos(0.5 * theta), s = std::sin(0.5 * theta);
  return m1(c, -std::exp(I * lambda) * s, std::exp(I * phi) * s,
            std::exp(I * (phi + lambda)) * c);
}

std::vector<cplx> pauli_string_matrix(const std::string& letters) {
  std::vector<cplx> m{1.0};
  unsigned d = 1;
  for (char ch : letters) {
    cplx p[4];
    switch (ch) {
      case 'X': p[0] = 0; p[1] = 1; p[2] = 1; p[3] = 0; break;
      case 'Y': p[0] = 0; p[1] = -I; p[2] = I; p[3] = 0; break;
      case 'Z': p[0] = 1; p[1] = 0; p[2] = 0; p[3] = -1.0; break;
      default: p[0] = 1; p[1] = 0; p[2] = 0; p[3] = 1; break;
    }
    // New letter is the most significant bit: kron(p, m).
    const unsigned nd = 2 * d;
    std::vector<cplx> r(size_t(nd) * nd);
    for (unsigned a = 0; a < 2; ++a)
      for (unsigned b = 0; b < 2; ++b)
        for (unsigned i = 0; i < d; ++i)
          for (unsigned j = 0; j < d; ++j)
            r[(a * d + i) * nd + (b * d + j)] = p[a * 2 + b] * m[i * d + j];
    m.swap(r);
    d = nd;
  }
  return m;
}

bool named_gate(const std::string& name, unsigned time,
                const std::vector<unsigned>& q, const std::vector<double>& p,
                Op* out) {
  const double h = 0.5, is2 = std::sqrt(0.5);
  auto need = [&](size_t nq, size_t np) {
    return q.size() == nq && p.size() == np;
  };
  std::vector<cplx> m;
  if (name == "p" && need(0, 1)) {
    m = {std::exp(I * p[0])};
  } else if (name == "id1" && need(1, 0)) {
    m = m1(1, 0, 0, 1);
  } else if (name == "h" && need(1, 0)) {
    m = m1(is2, is2, is2, -is2);
  } else if (name == "t" && need(1, 0)) {
    m = m1(1, 0, 0, cplx(is2, is2));
  } else if (name == "x" && need(1, 0)) {
    m = m1(0, 1, 1, 0);
  } else if (name == "y" && need(1, 0)) {
    m = m1(0, -I, I, 0);
  } else if (name == "z" && need(1, 0)) {
    m = m1(1, 0, 0, -1.0);
  } else if (name == "x_1_2" && need(1, 0)) {  // sqrt(X)
    m = m1(cplx(h, h), cplx(h, -h), cplx(h, -h), cplx(h, h));
  } else if (name == "y_1_2" && need(1, 0)) {  // sqrt(Y)
    m = m1(cplx(h, h), cplx(-h, -h), cplx(h, h), cplx(h, h));
  } else if (name == "hz_1_2" && need(1, 0)) {  // sqrt(W), W = (X+Y)/sqrt2
    m = m1(cplx(h, h), cplx(0, -is2), cplx(is2, 0), cplx(h, h));
  } else if (name == "s" && need(1, 0)) {
    m = m1(1, 0, 0, I);
  } else if ((name == "rx" || name == "ry" || name == "rz") && need(1, 1)) {
    const double c = std::cos(-0.5 * p[0]), s = std::sin(-0.5 * p[0]);
    if (name == "rx") m = m1(c, cplx(0, s), cplx(0, s), c);
    if (name == "ry") m = m1(c, s, -s, c);
    if (name == "rz") m = m1(cplx(c, s), 0, 0, cplx(c, -s));
  } else if (name == "rxy" && need(1, 2)) {
    const double cp = std::cos(-0.5 * p[1]), sp = std::sin(-0.5 * p[1]);
    const double ct = std::cos(p[0]) * sp, st = std::sin(p[0]) * sp;
    m = m1(cp, cplx(st, ct), cplx(-st, ct), cp);
  } else if (name == "u3" && need(1, 3)) {
    m = u3_matrix(p[0], p[1], p[2]);
  } else if (name == "id2" && need(2, 0)) {
    m = m2(1, 1, 0, 0, 1, 1);
  } else if (name == "cz" && need(2, 0)) {
    m = m2(1, 1, 0, 0, 1, -1.0);
  } else if ((name == "cnot" || name == "cx") && need(2, 0)) {
    // Control qubits[0], target qubits[1]: flips bit 1 when bit 0 is set.
    m.assign(16, 0.0);
    m[0 * 4 + 0] = 1;
    m[1 * 4 + 3] = 1;
    m[2 * 4 + 2] = 1;
    m[3 * 4 + 1] = 1;
  } else if (name == "sw" && need(2, 0)) {
    m = m2(1, 0, 1, 1, 0, 1);
  } else if (name == "is" && need(2, 0)) {
    m = m2(1, 0, I, I, 0, 1);
  } else if (name == "fs" && need(2, 2)) {
    double phi = p[1];
    if (phi < 0) phi += 2 * kPi;
    const double ct = std::cos(p[0]), st = std::sin(p[0]);
    m = m2(1, ct, cplx(0, -st), cplx(0, -st), ct, std::exp(-I * phi));
  } else if (name == "cp" && need(2, 1)) {
    m = m2(1, 1, 0, 0, 1, std::exp(-I * p[0]));
  } else {
    return false;
  }
  *out = make_gate(time, q, std::move(m));
  return true;
}

}  // namespace host
}  // namespace qsg
