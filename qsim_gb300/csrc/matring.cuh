// Device-side copies of gate matrices too large for kernel parameters
// (k >= 5), and the final FP64 reduction of per-block partial sums.
#pragma once

#include "common.cuh"

namespace qsg {

// Copies `nfloats` floats of `host_matrix` to a slot of a device ring buffer
// through a pinned staging slot; the copy is ordered on the context stream
// before any later launch.  `*dev` stays valid until 64 further uploads.
int matring_upload(qsg_ctx* ctx, const float* host_matrix, size_t nfloats,
                   const float** dev);

// Sums `count` double2 partials (device) in a fixed order and returns the
// total to the host (synchronises the stream).
int reduce_partials_d2(qsg_ctx* ctx, const double2* partial, uint64_t count,
                       double* out_re_im);

// <psi| M |psi> of a k <= 6-qubit operator on the tensor cores (n >= 12;
// tc_gate.cu).  *overflow: an amplitude was too large for the split (the
// result is then not valid; use the CUDA-core path).
int expectation_tc(qsg_ctx* ctx, const float* state, unsigned n,
                   const unsigned* qs, unsigned k, const float* m32,
                   double* out_re_im, bool* overflow);

// Releases the ring buffers of a context.
void matring_release(qsg_ctx* ctx);
// Releases the tensor-core operand ring of a context (tc_gate.cu).
void tcring_release(qsg_ctx* ctx);

}  // namespace qsg
