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
  if (q.size() == 2) {
    out->schmidt = schmidt_terms(name, p);
    if (q[0] > q[1]) {
      // make_gate sorted the qubits: the factors trade places.
      for (size_t t = 0; t + 8 <= out->schmidt.size(); t += 8)
        std::swap_ranges(out->schmidt.begin() + t, out->schmidt.begin() + t + 4,
                         out->schmidt.begin() + t + 4);
    }
  }
  return true;
}

// Operator Schmidt terms of the two-qubit gates (lib/gates_qsim.h:382-651
// lists the same decompositions).  A path of the hybrid simulator picks one
// term per gate on the cut, so partial sums over fixed path bits equal the
// reference's only with these terms, which is why they are the same.
//   id2        I (x) I
//   cz, cp     |0><0| (x) I + |1><1| (x) diag(1, e^{-i phi})   (cz: phi = pi)
//   cnot       |0><0| (x) I + |1><1| (x) X                     (control first)
//   sw         (I I + X X + Y Y + Z Z) / 2
//   is         (I I + Z Z) / 2 + i (X X + Y Y) / 2
//   fs         diagonal part D = A (x) A + E (x) E (rank 2) plus
//              -i sin(theta) (X X + Y Y) / 2 (rank 2)
std::vector<cplx> schmidt_terms(const std::string& name,
                                const std::vector<double>& p) {
  const double is2 = std::sqrt(0.5);
  const cplx P0[4] = {1, 0, 0, 0}, P1[4] = {0, 0, 0, 1};
  const cplx Id[4] = {1, 0, 0, 1}, X[4] = {0, 1, 1, 0};
  const cplx Y[4] = {0, -I, I, 0}, Z[4] = {1, 0, 0, -1.0};
  std::vector<cplx> t;
  auto term = [&](const cplx* a, cplx ca, const cplx* b, cplx cb) {
    for (int j = 0; j < 4; ++j) t.push_back(ca * a[j]);
    for (int j = 0; j < 4; ++j) t.push_back(cb * b[j]);
  };
  if (name == "id2") {
    term(Id, 1.0, Id, 1.0);
  } else if (name == "cz" || name == "cp") {
    const cplx ph = name == "cz" ? cplx(-1.0) : std::exp(-I * p.at(0));
    const cplx D[4] = {1, 0, 0, ph};
    term(P0, 1.0, Id, 1.0);
    term(P1, 1.0, D, 1.0);
  } else if (name == "cnot" || name == "cx") {
    term(P0, 1.0, Id, 1.0);
    term(P1, 1.0, X, 1.0);
  } else if (name == "sw") {
    term(Id, is2, Id, is2);
    term(X, is2, X, is2);
    term(Y, is2, Y, is2);
    term(Z, is2, Z, is2);
  } else if (name == "is") {
    const cplx c(0.5, 0.5);  // c^2 = i/2
    term(Id, is2, Id, is2);
    term(X, c, X, c);
    term(Y, c, Y, c);
    term(Z, is2, Z, is2);
  } else if (name == "fs") {
    const double theta = p.at(0);
    double phi = p.at(1);
    if (phi < 0) phi += 2 * kPi;
    const double ct = std::cos(theta), st = std::sin(theta);
    // D = diag(1, ct, ct, e^{-i phi}) = A (x) A + E (x) E with
    // A = z0 / sqrt2 diag(w, 1/w), E = z1 / sqrt2 diag(w, -1/w),
    // w = e^{i phi / 4}, z0^2 = e^{-i phi / 2} + ct, z1^2 = e^{-i phi / 2} - ct
    // (principal roots).
    const cplx w = std::exp(I * (0.25 * phi));
    const cplx h2 = std::exp(-I * (0.5 * phi));
    const cplx z0 = std::sqrt(h2 + ct) * is2, z1 = std::sqrt(h2 - ct) * is2;
    const cplx A[4] = {z0 * w, 0, 0, z0 / w}, E[4] = {z1 * w, 0, 0, -z1 / w};
    // -i st (X X + Y Y) / 2 = (f X) (x) (g X) + (f Y) (x) (g Y) with
    // f = sqrt|st| (1 - i) / 2 and g = f sign(st).
    const cplx f = std::sqrt(std::abs(st)) * cplx(0.5, -0.5);
    const cplx g = st < 0 ? -f : f;
    term(A, 1.0, A, 1.0);
    term(X, f, X, g);
    term(Y, f, Y, g);
    term(E, 1.0, E, 1.0);
  }
  return t;
}

}  // namespace host
}  // namespace qsg
