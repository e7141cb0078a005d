// Unitary calculator on the GPU (lib/unitaryspace_basic.h,
// lib/unitary_calculator_basic.h).
//
// The reference stores entry (i, j) of an n-qubit unitary at complex index
// i * 2^n + j and applies a gate by mixing the entries of every row over the
// column bits at its qubits (UnitaryCalculatorBasic::ApplyGateH, :126-184).
// That is a 2n-qubit state vector whose gates act on qubits < n, so the
// state-vector tile kernels run it unchanged; only the identity needs a
// kernel of its own.

#include <algorithm>

#include "common.cuh"
#include "internal.h"

namespace qsg {

namespace {

constexpr unsigned kMaxUnitaryQubits = kMaxQubits / 2;  // 2n <= 40

// Sets entries (i, i) to 1 (the buffer is zero).
__global__ void unitary_diag_kernel(float2* u, uint64_t dim) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < dim;
       i += uint64_t(gridDim.x) * blockDim.x)
    u[i * dim + i] = make_float2(1.f, 0.f);
}

bool unitary_qubits_ok(const unsigned* qs, unsigned k, unsigned n) {
  return valid_qubits(qs, k, n);
}

}  // namespace

}  // namespace qsg

using namespace qsg;

extern "C" {

uint64_t qsg_unitary_min_size(unsigned num_qubits) {
  return min_size(2 * num_qubits);
}

int qsg_unitary_create(qsg_ctx* ctx, unsigned num_qubits, float** out) {
  QSG_CHECK_ARG(ctx && out, "qsg_unitary_create: null argument");
  QSG_CHECK_ARG(num_qubits <= kMaxUnitaryQubits,
                "qsg_unitary_create: at most %u qubits", kMaxUnitaryQubits);
  return qsg_state_create(ctx, 2 * num_qubits, out);
}

int qsg_unitary_free(qsg_ctx* ctx, float* u) { return qsg_state_free(ctx, u); }

int qsg_unitary_set_all_zeros(qsg_ctx* ctx, float* u, unsigned n) {
  QSG_CHECK_ARG(ctx && u && n <= kMaxUnitaryQubits,
                "qsg_unitary_set_all_zeros: bad argument");
  return qsg_set_all_zeros(ctx, u, 2 * n);
}

int qsg_unitary_set_identity(qsg_ctx* ctx, float* u, unsigned n) {
  QSG_CHECK_ARG(ctx && u && n <= kMaxUnitaryQubits,
                "qsg_unitary_set_identity: bad argument");
  int rc = qsg_set_all_zeros(ctx, u, 2 * n);
  if (rc) return rc;
  const uint64_t dim = uint64_t{1} << n;
  const unsigned grid =
      unsigned(std::min<uint64_t>((dim + 255) / 256, uint64_t(ctx->num_sms) * 4));
  unitary_diag_kernel<<<grid, 256, 0, ctx->stream>>>(
      reinterpret_cast<float2*>(u), dim);
  QSG_LAUNCHED(ctx);
  return QSG_OK;
}

int qsg_unitary_get_entry(qsg_ctx* ctx, const float* u, unsigned n,
                          uint64_t i, uint64_t j, float* re_im) {
  QSG_CHECK_ARG(ctx && u && re_im && n <= kMaxUnitaryQubits,
                "qsg_unitary_get_entry: bad argument");
  QSG_CHECK_ARG((i >> n) == 0 && (j >> n) == 0,
                "qsg_unitary_get_entry: index out of range");
  return qsg_get_ampl(ctx, u, 2 * n, (i << n) | j, re_im);
}

int qsg_unitary_set_entry(qsg_ctx* ctx, float* u, unsigned n, uint64_t i,
                          uint64_t j, float re, float im) {
  QSG_CHECK_ARG(ctx && u && n <= kMaxUnitaryQubits,
                "qsg_unitary_set_entry: bad argument");
  QSG_CHECK_ARG((i >> n) == 0 && (j >> n) == 0,
                "qsg_unitary_set_entry: index out of range");
  return qsg_set_ampl(ctx, u, 2 * n, (i << n) | j, re, im);
}

int qsg_unitary_apply_gate(qsg_ctx* ctx, float* u, unsigned n,
                           const unsigned* qs, unsigned k,
                           const float* matrix) {
  QSG_CHECK_ARG(ctx && u && matrix && n <= kMaxUnitaryQubits,
                "qsg_unitary_apply_gate: bad argument");
  QSG_CHECK_ARG(unitary_qubits_ok(qs, k, n),
                "qsg_unitary_apply_gate: qubits must be sorted, distinct, < %u",
                n);
  return qsg_apply_gate(ctx, u, 2 * n, qs, k, matrix);
}

int qsg_unitary_apply_controlled_gate(qsg_ctx* ctx, float* u, unsigned n,
                                      const unsigned* qs, unsigned k,
                                      const unsigned* cqs, unsigned c,
                                      uint64_t cvals, const float* matrix) {
  QSG_CHECK_ARG(ctx && u && matrix && n <= kMaxUnitaryQubits,
                "qsg_unitary_apply_controlled_gate: bad argument");
  QSG_CHECK_ARG(unitary_qubits_ok(qs, k, n) && unitary_qubits_ok(cqs, c, n),
                "qsg_unitary_apply_controlled_gate: qubits must be < %u", n);
  return qsg_apply_controlled_gate(ctx, u, 2 * n, qs, k, cqs, c, cvals,
                                   matrix);
}

}  // extern "C"
