// Internal entry points shared between the CUDA translation units and the
// host engine (plain C++, no CUDA types).
#pragma once

#include <cstdint>

#include "qsim_gb300.h"

namespace qsg {

// Applies a (controlled) gate.  `dev_matrix`, when not null, is a device copy
// of the row-major interleaved matrix that replaces the upload of
// `host_matrix` (used by captured plans for k = 6, whose matrix does not fit
// in kernel parameters).
int apply_gate_ex(qsg_ctx* ctx, float* state, unsigned n, const unsigned* qs,
                  unsigned k, const unsigned* cqs, unsigned c, uint64_t cvals,
                  const float* host_matrix, const float* dev_matrix);

// One-time set-up of the tile kernel used for a k-qubit gate (pair: qubit 0
// is not a target; mode 0 apply, 1 expectation).  Must precede capture.
int apply_gate_prepare(unsigned k, bool pair, int mode);

// True if the k-qubit matrix (row-major interleaved complex) has one
// nonzero per row, at column r ^ xm for one xm (Pauli strings, diagonal
// gates and their products); then d[2r], d[2r+1] = M[r][r ^ xm].
bool monomial_xor(unsigned k, const float* m, uint32_t* xm, float* d);
// <s|M|s> of such a matrix in one read pass (expect.cu).
int expectation_monomial(qsg_ctx* ctx, const float* state, unsigned n,
                         const unsigned* qs, unsigned k, uint32_t xm,
                         const float* d, double* out_re_im);

// Device allocation helpers for host-side objects.
int dev_alloc(qsg_ctx* ctx, size_t bytes, void** out);
int dev_free(qsg_ctx* ctx, void* p);
int dev_upload(qsg_ctx* ctx, void* dst, const void* src, size_t bytes);
void* ctx_stream(qsg_ctx* ctx);
int ctx_device(qsg_ctx* ctx);

}  // namespace qsg
