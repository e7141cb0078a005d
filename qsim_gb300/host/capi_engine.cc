// C ABI of the host engine: circuits, workload generators, fusion plans,
// plan runs and CUDA-graph capture.  Declared in include/qsim_gb300.h.

#include <algorithm>
#include <cstring>
#include <new>

#include "capi_types.h"
#include "engine.h"
#include "learned.h"
#include "internal.h"
#include "runner.h"

using namespace qsg;
using namespace qsg::host;


struct qsg_plan {
  PlanRuntime rt;
};

namespace qsg {
void set_error_msg(const char* msg);
}

namespace qsg {
namespace host {

bool fuse_options_from(const qsg_fuse_options* o, FuseOptions* out) {
  FuseOptions fo;
  if (o) {
    fo.max_fused_size = o->max_fused_size;
    fo.seeds = o->seeds ? o->seeds : fo.seeds;
    fo.tensor_path = o->tensor_path != 0;
    fo.tc_min_k = o->tc_min_k ? o->tc_min_k : fo.tc_min_k;
    fo.tc_pair_bits = o->tc_pair_bits;
    fo.cost = qsg::cost_model_from_handle(o->cost_model);
  }
  *out = fo;
  return fo.max_fused_size >= 1 && fo.max_fused_size <= 6;
}

}  // namespace host
}  // namespace qsg

namespace {

int invalid(const char* msg) {
  qsg::set_error_msg(msg);
  return QSG_ERR_INVALID;
}

std::vector<cplx> to_cplx(const double* m, unsigned k) {
  const size_t d = size_t(1) << k;
  std::vector<cplx> out(d * d);
  for (size_t i = 0; i < d * d; ++i) out[i] = cplx(m[2 * i], m[2 * i + 1]);
  return out;
}

bool distinct_lt(const unsigned* qs, unsigned k, unsigned n) {
  for (unsigned i = 0; i < k; ++i) {
    if (qs[i] >= n) return false;
    for (unsigned j = 0; j < i; ++j)
      if (qs[i] == qs[j]) return false;
  }
  return true;
}

template <typename F>
int make_circuit(F&& f, qsg_circuit** out) {
  if (!out) return invalid("null output");
  *out = nullptr;
  auto* c = new (std::nothrow) qsg_circuit();
  if (!c) return QSG_ERR_OOM;
  f(c->c);
  *out = c;
  return QSG_OK;
}

}  // namespace

extern "C" {

int qsg_circuit_create(unsigned num_qubits, qsg_circuit** out) {
  if (num_qubits > 63) return invalid("too many qubits");
  return make_circuit([&](Circuit& c) { c.num_qubits = num_qubits; }, out);
}

int qsg_circuit_destroy(qsg_circuit* c) {
  delete c;
  return QSG_OK;
}

int qsg_circuit_info(const qsg_circuit* c, unsigned* num_qubits,
                     uint64_t* num_ops) {
  if (!c) return invalid("null circuit");
  if (num_qubits) *num_qubits = c->c.num_qubits;
  if (num_ops) *num_ops = c->c.ops.size();
  return QSG_OK;
}

int qsg_circuit_add_gate(qsg_circuit* c, unsigned time, const unsigned* qs,
                         unsigned k, const double* matrix) {
  if (!c || !matrix || (k && !qs)) return invalid("null argument");
  if (k > 6) return invalid("gates act on at most 6 qubits");
  if (!distinct_lt(qs, k, c->c.num_qubits)) return invalid("bad qubits");
  c->c.ops.push_back(
      make_gate(time, std::vector<unsigned>(qs, qs + k), to_cplx(matrix, k)));
  return QSG_OK;
}

int qsg_circuit_add_controlled_gate(qsg_circuit* c, unsigned time,
                                    const unsigned* qs, unsigned k,
                                    const unsigned* cqs, unsigned nc,
                                    uint64_t cvals, const double* matrix) {
  if (!c || !matrix || (k && !qs) || (nc && !cqs))
    return invalid("null argument");
  if (k > 6) return invalid("gates act on at most 6 qubits");
  std::vector<unsigned> all(qs, qs + k);
  all.insert(all.end(), cqs, cqs + nc);
  if (!distinct_lt(all.data(), all.size(), c->c.num_qubits))
    return invalid("bad qubits");
  Op op = make_gate(time, std::vector<unsigned>(qs, qs + k), to_cplx(matrix, k));
  // Sort controls with their values (lib/gate.h:93-146).
  std::vector<std::pair<unsigned, unsigned>> cp;
  for (unsigned i = 0; i < nc; ++i) cp.push_back({cqs[i], unsigned((cvals >> i) & 1)});
  std::sort(cp.begin(), cp.end());
  op.kind = nc ? OpKind::kControlled : OpKind::kGate;
  op.cvals = 0;
  for (unsigned i = 0; i < nc; ++i) {
    op.cqs.push_back(cp[i].first);
    op.cvals |= uint64_t(cp[i].second) << i;
  }
  c->c.ops.push_back(std::move(op));
  return QSG_OK;
}

int qsg_circuit_add_measurement(qsg_circuit* c, unsigned time,
                                const unsigned* qs, unsigned k) {
  if (!c || (k && !qs)) return invalid("null argument");
  if (!distinct_lt(qs, k, c->c.num_qubits)) return invalid("bad qubits");
  Op op;
  op.kind = OpKind::kMeasure;
  op.time = time;
  op.qs.assign(qs, qs + k);
  std::sort(op.qs.begin(), op.qs.end());
  c->c.ops.push_back(std::move(op));
  return QSG_OK;
}

int qsg_circuit_add_named_gate(qsg_circuit* c, unsigned time, const char* name,
                               const unsigned* qs, unsigned nq,
                               const double* params, unsigned np) {
  if (!c || !name) return invalid("null argument");
  if (!distinct_lt(qs, nq, c->c.num_qubits)) return invalid("bad qubits");
  Op op;
  if (!named_gate(name, time, std::vector<unsigned>(qs, qs + nq),
                  std::vector<double>(params, params + np), &op))
    return invalid("unknown gate or wrong arity");
  c->c.ops.push_back(std::move(op));
  return QSG_OK;
}

int qsg_circuit_parse(const char* text, unsigned maxtime, qsg_circuit** out) {
  if (!text || !out) return invalid("null argument");
  *out = nullptr;
  auto* c = new qsg_circuit();
  std::string err;
  if (!parse_qsim_text(text, maxtime, &c->c, &err)) {
    delete c;
    return invalid(err.c_str());
  }
  *out = c;
  return QSG_OK;
}

int qsg_circuit_grid(unsigned rows, unsigned cols, unsigned extra,
                     unsigned cycles, uint64_t seed, qsg_circuit** out) {
  if (rows * cols + extra > 63 || extra > cols) return invalid("bad grid");
  return make_circuit(
      [&](Circuit& c) { c = grid_random_circuit(rows, cols, extra, cycles, seed); },
      out);
}

int qsg_circuit_chain(unsigned n, unsigned cycles, uint64_t seed,
                      qsg_circuit** out) {
  if (n == 0 || n > 63) return invalid("bad qubit count");
  return make_circuit(
      [&](Circuit& c) { c = chain_random_circuit(n, cycles, seed); }, out);
}

int qsg_circuit_layered_u3(unsigned n, unsigned layers,
                           unsigned num_controlled, uint64_t seed,
                           qsg_circuit** out) {
  if (n < 3 || n > 63) return invalid("bad qubit count");
  return make_circuit(
      [&](Circuit& c) {
        c = layered_u3_circuit(n, layers, num_controlled, seed);
      },
      out);
}

int qsg_circuit_get_op(const qsg_circuit* c, uint64_t i, int* kind,
                       unsigned* time, unsigned* k, unsigned* qs, unsigned* nc,
                       unsigned* cqs, uint64_t* cvals, double* matrix) {
  if (!c || i >= c->c.ops.size()) return invalid("op index out of range");
  const Op& op = c->c.ops[i];
  if (kind) *kind = int(op.kind);
  if (time) *time = op.time;
  if (k) *k = op.qs.size();
  if (qs) std::copy(op.qs.begin(), op.qs.end(), qs);
  if (nc) *nc = op.cqs.size();
  if (cqs) std::copy(op.cqs.begin(), op.cqs.end(), cqs);
  if (cvals) *cvals = op.cvals;
  if (matrix) {
    for (size_t j = 0; j < op.m.size(); ++j) {
      matrix[2 * j] = op.m[j].real();
      matrix[2 * j + 1] = op.m[j].imag();
    }
  }
  return QSG_OK;
}

int qsg_circuit_get_schmidt(const qsg_circuit* c, uint64_t i,
                            unsigned* num_terms, double* terms) {
  if (!c || !num_terms || i >= c->c.ops.size())
    return invalid("op index out of range");
  const Op& op = c->c.ops[i];
  *num_terms = unsigned(op.schmidt.size() / 8);
  if (terms) {
    for (size_t j = 0; j < op.schmidt.size(); ++j) {
      terms[2 * j] = op.schmidt[j].real();
      terms[2 * j + 1] = op.schmidt[j].imag();
    }
  }
  return QSG_OK;
}

int qsg_circuit_set_schmidt(qsg_circuit* c, uint64_t i, unsigned num_terms,
                            const double* terms) {
  if (!c || i >= c->c.ops.size() || (num_terms && !terms))
    return invalid("op index out of range");
  Op& op = c->c.ops[i];
  if (op.kind != OpKind::kGate || op.qs.size() != 2 || num_terms > 4)
    return invalid("Schmidt terms need a two-qubit gate and at most 4 terms");
  // The terms must rebuild the gate: sum_t A_t (x) B_t, bit 0 <-> qs[0].
  double err = 0, scale = 0;
  for (unsigned r = 0; r < 4; ++r) {
    for (unsigned col = 0; col < 4; ++col) {
      cplx v = 0;
      for (unsigned t = 0; t < num_terms; ++t) {
        const double* a = terms + 16 * t;
        const double* b = a + 8;
        const unsigned ia = 2 * ((r & 1) * 2 + (col & 1));
        const unsigned ib = 2 * ((r >> 1) * 2 + (col >> 1));
        v += cplx(a[ia], a[ia + 1]) * cplx(b[ib], b[ib + 1]);
      }
      err = std::max(err, std::abs(v - op.m[r * 4 + col]));
      scale = std::max(scale, std::abs(op.m[r * 4 + col]));
    }
  }
  if (err > 1e-6 * std::max(1.0, scale))
    return invalid("Schmidt terms do not rebuild the gate");
  op.schmidt.assign(size_t(8) * num_terms, 0.0);
  for (size_t j = 0; j < op.schmidt.size(); ++j)
    op.schmidt[j] = cplx(terms[2 * j], terms[2 * j + 1]);
  return QSG_OK;
}

int qsg_pauli_sum(unsigned n, unsigned count, unsigned max_weight,
                  uint64_t seed, unsigned* weights, unsigned* qubits,
                  char* letters, double* coeffs) {
  if (!weights || !qubits || !letters || !coeffs) return invalid("null");
  if (n == 0 || max_weight == 0 || max_weight > 6) return invalid("bad sizes");
  auto terms = random_pauli_sum(n, count, max_weight, seed);
  for (unsigned i = 0; i < count; ++i) {
    weights[i] = terms[i].qs.size();
    for (unsigned j = 0; j < max_weight; ++j) {
      qubits[i * max_weight + j] = j < weights[i] ? terms[i].qs[j] : 0;
      letters[i * max_weight + j] = j < weights[i] ? terms[i].letters[j] : 'I';
    }
    coeffs[i] = terms[i].coeff;
  }
  return QSG_OK;
}

int qsg_plan_create(const qsg_circuit* c, const qsg_fuse_options* o,
                    qsg_plan** out) {
  if (!c || !out) return invalid("null argument");
  *out = nullptr;
  FuseOptions fo;
  if (!fuse_options_from(o, &fo))
    return invalid("max_fused_size must be 1..6");
  auto* p = new qsg_plan();
  p->rt.plan = fuse(c->c, fo);
  *out = p;
  return QSG_OK;
}

int qsg_plan_create_unfused(const qsg_circuit* c, qsg_plan** out) {
  if (!c || !out) return invalid("null argument");
  auto* p = new qsg_plan();
  p->rt.plan = unfused(c->c);
  *out = p;
  return QSG_OK;
}

int qsg_plan_destroy(qsg_plan* p) {
  delete p;
  return QSG_OK;
}

int qsg_plan_info(const qsg_plan* p, uint64_t* num_ops, unsigned* max_k,
                  uint64_t* num_tensor_ops) {
  if (!p) return invalid("null plan");
  if (num_ops) *num_ops = p->rt.plan.ops.size();
  if (max_k) *max_k = p->rt.plan.max_k();
  if (num_tensor_ops) {
    uint64_t t = 0;
    for (const auto& op : p->rt.plan.ops) t += op.path == Path::kTensor;
    *num_tensor_ops = t;
  }
  return QSG_OK;
}

int qsg_plan_tc_pairs(const qsg_plan* p, uint64_t* num_pairs,
                      unsigned char* pair_next) {
  if (!p) return invalid("null plan");
  uint64_t t = 0;
  const auto& ops = p->rt.plan.ops;
  for (size_t i = 0; i < ops.size(); ++i) {
    t += ops[i].tc_pair_next;
    if (pair_next) pair_next[i] = ops[i].tc_pair_next ? 1 : 0;
  }
  if (num_pairs) *num_pairs = t;
  return QSG_OK;
}

int qsg_plan_get_op(const qsg_plan* p, uint64_t i, int* kind, unsigned* k,
                    unsigned* qs, unsigned* nc, unsigned* cqs,
                    uint64_t* cvals, int* path, uint64_t* num_members,
                    double* matrix) {
  if (!p || i >= p->rt.plan.ops.size()) return invalid("op index out of range");
  const PlanOp& op = p->rt.plan.ops[i];
  if (kind) *kind = int(op.kind);
  if (k) *k = op.qs.size();
  if (qs) std::copy(op.qs.begin(), op.qs.end(), qs);
  if (nc) *nc = op.cqs.size();
  if (cqs) std::copy(op.cqs.begin(), op.cqs.end(), cqs);
  if (cvals) *cvals = op.cvals;
  if (path) *path = int(op.path);
  if (num_members) *num_members = op.members.size();
  if (matrix) {
    for (size_t j = 0; j < op.m.size(); ++j) {
      matrix[2 * j] = op.m[j].real();
      matrix[2 * j + 1] = op.m[j].imag();
    }
  }
  return QSG_OK;
}

int qsg_plan_run(qsg_ctx* ctx, qsg_plan* p, float* state, unsigned seed,
                 uint64_t* mbits, uint64_t mbits_cap, uint64_t* num_meas) {
  if (!ctx || !p || !state) return invalid("null argument");
  std::vector<uint64_t> bits;
  int rc = p->rt.run(ctx, state, seed, &bits);
  if (num_meas) *num_meas = bits.size();
  if (mbits)
    std::copy(bits.begin(), bits.begin() + std::min<size_t>(bits.size(), mbits_cap),
              mbits);
  return rc;
}

int qsg_unitary_run_plan(qsg_ctx* ctx, qsg_plan* p, float* u, unsigned n) {
  if (!ctx || !p || !u) return invalid("null argument");
  PlanRuntime& rt = p->rt;
  if (rt.plan.num_qubits != n || n > 20)
    return invalid("qsg_unitary_run_plan: plan and unitary sizes differ");
  // The unitary is a 2n-qubit state whose gates act on qubits < n (the
  // reference's row-wise application, lib/unitary_calculator_basic.h).
  int rc = rt.upload(ctx);
  if (rc) return rc;
  rc = rt.prepare_tc();
  if (rc) return rc;
  for (size_t i = 0; i < rt.plan.ops.size(); ++i) {
    const PlanOp& op = rt.plan.ops[i];
    if (op.kind == OpKind::kMeasure)
      return invalid("qsg_unitary_run_plan: plans with measurements");
    if (op.kind == OpKind::kGate && op.path == Path::kTensor &&
        op.tc_pair_next) {
      // Two blocks in one pass (their tile fits the n low qubits' union,
      // the same on the 2n-qubit view).
      rc = apply_gate_tc2_carry(ctx, u, 2 * n, op.qs.data(), rt.tc_operands(i),
                                rt.plan.ops[i + 1].qs.data(),
                                rt.tc_operands(i + 1), nullptr, 0, nullptr);
      ++i;
    } else if (op.kind == OpKind::kGate && op.path == Path::kTensor) {
      rc = apply_gate_tc(ctx, u, 2 * n, op.qs.data(), op.qs.size(),
                         op.m32.data(), rt.tc_operands(i));
    } else {
      const float* dm = (rt.dmat && rt.dmat_off[i] != size_t(-1))
                            ? rt.dmat + rt.dmat_off[i]
                            : nullptr;
      rc = apply_gate_ex(ctx, u, 2 * n, op.qs.data(), op.qs.size(),
                         op.cqs.data(), op.cqs.size(), op.cvals,
                         op.m32.data(), dm);
    }
    if (rc) return rc;
  }
  return QSG_OK;
}

int qsg_plan_capture(qsg_ctx* ctx, qsg_plan* p, float* state) {
  if (!ctx || !p || !state) return invalid("null argument");
  return p->rt.capture(ctx, state);
}

int qsg_plan_profile(qsg_ctx* ctx, qsg_plan* p, float* state, float* op_ms,
                     uint64_t cap) {
  if (!ctx || !p || !state || !op_ms) return invalid("null argument");
  std::vector<float> ms;
  int rc = p->rt.profile(ctx, state, &ms);
  std::copy(ms.begin(), ms.begin() + std::min<size_t>(ms.size(), cap), op_ms);
  return rc;
}

int qsg_plan_replay(qsg_ctx* ctx, qsg_plan* p) {
  if (!ctx || !p) return invalid("null argument");
  return p->rt.replay(ctx);
}

}  // extern "C"
