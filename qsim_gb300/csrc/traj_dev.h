// Device-side description of one quantum channel, shared by the trajectory
// kernels (traj.cu) and the host trajectory engine (plain C++).
#pragma once

#include <cstdint>

#include "qsim_gb300.h"

namespace qsg {

// Largest channel handled by the device-side Kraus choice: at most two
// qubits and sixteen Kraus operators.  Every non-unitary channel of the
// reference's Cirq channel set (lib/channels_cirq.h) is a one-qubit channel
// whose K^dagger K matrices are diagonal, which is the form used here.
constexpr unsigned kTrajMaxChannelQubits = 2;
constexpr unsigned kTrajMaxKops = 16;

struct TrajChannelDev {
  int nq;                 // channel qubits (1 or 2)
  unsigned q[2];          // sorted ascending
  int nkops;
  int unitary[kTrajMaxKops];
  double prob[kTrajMaxKops];     // lower bounds (exact for unitary ones)
  // Diagonal of K^dagger K in the channel-qubit basis (index bit j <-> q[j]),
  // stored with the values the reference's single-precision kd_k holds.
  float kd[kTrajMaxKops][4];
  // K on the channel qubits: row-major interleaved complex, 2^nq x 2^nq.
  float mat[kTrajMaxKops][32];
};

// Device work of the trajectory engine (traj.cu).
//
// Channel statistics: one read pass that sums |psi_i|^2 by the values of up
// to two qubits (nq = 0 gives the norm).  Writes `*nparts` partial sums of
// four doubles each into `partial` (room for traj_max_parts(ctx) * 4).
unsigned traj_max_parts(qsg_ctx* ctx);
int traj_channel_stats(qsg_ctx* ctx, const float* state, unsigned n,
                       unsigned nq, const unsigned* q, double* partial,
                       unsigned* nparts);
// Kraus-operator choice on the device for a channel whose lower-bound pass
// failed: `cp0` is the sum of the lower bounds, `r` the trajectory's draw.
// Writes the chosen index (or 0xffffffff when none is chosen) to
// `choice_out` and the chosen operator times 1/sqrt(norm) to `mat_out`.  With
// `ch` null it writes the normalisation factor 1/sqrt(norm) as a 0-qubit
// matrix.
int traj_choose(qsg_ctx* ctx, const double* partial, unsigned nparts,
                const TrajChannelDev* ch, double cp0, double r,
                uint32_t* choice_out, float* mat_out);
// Applies the nq-qubit matrix held in device memory (nq = 0: a scalar).
int traj_apply(qsg_ctx* ctx, float* state, unsigned n, unsigned nq,
               const unsigned* q, const float* mat_dev);

// Rescales `state` by sqrt(norm_before / norm_after), the norms given as
// traj_channel_stats partials (nq = 0) of the state before and after a
// unitary sequence of launches.
int norm_restore(qsg_ctx* ctx, float* state, unsigned n, const double* before,
                 unsigned nb, const double* after, unsigned na);

}  // namespace qsg
