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

// Releases the ring buffers of a context.
void matring_release(qsg_ctx* ctx);
// Releases the tensor-core operand ring of a context (tc_gate.cu).
void tcring_release(qsg_ctx* ctx);

}  // namespace qsg
