// Trajectory kernels: channel statistics, device-side Kraus-operator choice
// and application of the chosen operator from device memory.
//
// The reference samples a non-unitary channel whose lower-bound test failed
// by normalising the state and computing <psi|K^dagger K|psi> for each
// non-unitary Kraus operator (lib/qtrajectory.h:331-380): a Norm pass, a
// Multiply pass and one ExpectationValue pass per operator, each followed by
// a host synchronisation.  Here one read pass sums |psi_i|^2 by the values
// of the channel qubits; the norm and every operator's probability follow
// from those sums because K^dagger K is diagonal on the channel qubits.  The
// choice is made on the device by one small kernel, which also folds the
// normalisation into the chosen operator, so a trajectory never waits for
// the host.

#include <cmath>

#include "common.cuh"
#include "traj_dev.h"

namespace qsg {

constexpr int kTrajThreads = 256;
constexpr int kTrajUnroll = 4;

__device__ __forceinline__ unsigned traj_bin(uint64_t i, unsigned nq,
                                             unsigned q0, unsigned q1) {
  unsigned b = 0;
  if (nq > 0) b = unsigned(i >> q0) & 1u;
  if (nq > 1) b |= (unsigned(i >> q1) & 1u) << 1;
  return b;
}

// partial[4 * block + b] = sum of |psi_i|^2 over the block's amplitudes whose
// channel-qubit value is b.  FP32 over kTrajUnroll units per thread, FP64
// beyond.
__global__ void __launch_bounds__(kTrajThreads)
    traj_stats_kernel(const float4* __restrict__ s, uint64_t units,
                      unsigned nq, unsigned q0, unsigned q1,
                      double* __restrict__ partial) {
  double acc[4] = {0, 0, 0, 0};
  const uint64_t tile = uint64_t(kTrajThreads) * kTrajUnroll;
  for (uint64_t b0 = blockIdx.x * tile; b0 < units;
       b0 += uint64_t(gridDim.x) * tile) {
    float f[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int j = 0; j < kTrajUnroll; ++j) {
      const uint64_t i = b0 + j * kTrajThreads + threadIdx.x;
      if (i < units) {
        const float4 x = s[i];
        const float p0 = x.x * x.x + x.y * x.y;
        const float p1 = x.z * x.z + x.w * x.w;
        const unsigned c0 = traj_bin(2 * i, nq, q0, q1);
        const unsigned c1 = traj_bin(2 * i + 1, nq, q0, q1);
#pragma unroll
        for (unsigned b = 0; b < 4; ++b) {
          f[b] += (c0 == b ? p0 : 0.f) + (c1 == b ? p1 : 0.f);
        }
      }
    }
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[b] += f[b];
  }
  __shared__ double red[kTrajThreads / 32][4];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    double v = acc[b];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp][b] = v;
  }
  __syncthreads();
  if (threadIdx.x < 4) {
    double v = 0;
    for (int w = 0; w < kTrajThreads / 32; ++w) v += red[w][threadIdx.x];
    partial[4 * blockIdx.x + threadIdx.x] = v;
  }
}

// Sums the partials, then (thread 0) restates the second sampling loop of
// lib/qtrajectory.h:351-380 with probabilities from the channel sums.
__global__ void __launch_bounds__(kTrajThreads)
    traj_choose_kernel(const double* __restrict__ partial, unsigned nparts,
                       const TrajChannelDev* __restrict__ ch, double cp0,
                       double r, uint32_t* __restrict__ choice_out,
                       float* __restrict__ mat_out) {
  double acc[4] = {0, 0, 0, 0};
  for (unsigned i = threadIdx.x; i < nparts; i += kTrajThreads) {
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[b] += partial[4 * i + b];
  }
  __shared__ double red[kTrajThreads / 32][4];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    double v = acc[b];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp][b] = v;
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  double bins[4] = {0, 0, 0, 0};
  for (int w = 0; w < kTrajThreads / 32; ++w)
    for (int b = 0; b < 4; ++b) bins[b] += red[w][b];
  const double norm = bins[0] + bins[1] + bins[2] + bins[3];
  // The reference multiplies the state by fp_type(1 / sqrt(norm)).
  const float a = float(1.0 / sqrt(norm));
  if (ch == nullptr) {
    mat_out[0] = a;
    mat_out[1] = 0.f;
    return;
  }
  const unsigned d = 1u << ch->nq;
  double cp = cp0, max_prob = 0;
  int max_index = 0, chosen = -1;
  for (int i = 0; i < ch->nkops; ++i) {
    if (ch->unitary[i]) continue;
    double ev = 0;
    for (unsigned b = 0; b < d; ++b) ev += double(ch->kd[i][b]) * bins[b];
    const double prob = ev / norm;
    if (prob > max_prob) {
      max_prob = prob;
      max_index = i;
    }
    cp += prob - ch->prob[i];
    if (r < cp || i == ch->nkops - 1) {
      chosen = r < cp ? i : max_index;
      break;
    }
  }
  *choice_out = chosen < 0 ? 0xffffffffu : uint32_t(chosen);
  const unsigned nf = 2 * d * d;
  for (unsigned j = 0; j < nf; ++j) {
    float v;
    if (chosen < 0) {
      // Nothing chosen: only the normalisation is applied.
      const unsigned row = (j / 2) / d, col = (j / 2) % d;
      v = (j % 2 == 0 && row == col) ? a : 0.f;
    } else {
      v = ch->mat[chosen][j] * a;
    }
    mat_out[j] = v;
  }
}

// Applies an nq-qubit (nq <= 2) matrix read from device memory; one group of
// 2^nq amplitudes per thread and iteration.
__global__ void __launch_bounds__(kTrajThreads)
    traj_apply_kernel(float2* __restrict__ s, uint64_t groups, unsigned nq,
                      unsigned q0, unsigned q1,
                      const float* __restrict__ mat) {
  __shared__ float2 m[16];
  if (threadIdx.x < 16) {
    const unsigned d = 1u << nq;
    m[threadIdx.x] = threadIdx.x < d * d
                         ? make_float2(mat[2 * threadIdx.x], mat[2 * threadIdx.x + 1])
                         : make_float2(0.f, 0.f);
  }
  __syncthreads();
  for (uint64_t g = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
       g < groups; g += uint64_t(gridDim.x) * blockDim.x) {
    if (nq == 0) {
      const float2 v = s[g];
      s[g] = make_float2(m[0].x * v.x - m[0].y * v.y,
                         m[0].x * v.y + m[0].y * v.x);
    } else if (nq == 1) {
      const uint64_t lo = g & ((uint64_t{1} << q0) - 1);
      const uint64_t i0 = ((g - lo) << 1) | lo;
      const uint64_t i1 = i0 | (uint64_t{1} << q0);
      const float2 v0 = s[i0], v1 = s[i1];
      float2 w[2];
#pragma unroll
      for (int r = 0; r < 2; ++r) {
        const float2 a = m[2 * r], b = m[2 * r + 1];
        w[r] = make_float2(a.x * v0.x - a.y * v0.y + b.x * v1.x - b.y * v1.y,
                           a.x * v0.y + a.y * v0.x + b.x * v1.y + b.y * v1.x);
      }
      s[i0] = w[0];
      s[i1] = w[1];
    } else {
      uint64_t i = g;
      i = ((i >> q0) << (q0 + 1)) | (i & ((uint64_t{1} << q0) - 1));
      i = ((i >> q1) << (q1 + 1)) | (i & ((uint64_t{1} << q1) - 1));
      const uint64_t idx[4] = {i, i | (uint64_t{1} << q0),
                               i | (uint64_t{1} << q1),
                               i | (uint64_t{1} << q0) | (uint64_t{1} << q1)};
      float2 v[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) v[c] = s[idx[c]];
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        float re = 0.f, im = 0.f;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const float2 a = m[4 * r + c];
          re += a.x * v[c].x - a.y * v[c].y;
          im += a.x * v[c].y + a.y * v[c].x;
        }
        s[idx[r]] = make_float2(re, im);
      }
    }
  }
}

// Rescales the state by sqrt(norm_before / norm_after), both given as the
// partial sums of traj_stats_kernel (4 doubles per block); every block sums
// the partials itself.
__global__ void __launch_bounds__(kTrajThreads)
    norm_restore_kernel(float4* __restrict__ s, uint64_t units,
                        const double* __restrict__ before, unsigned nb,
                        const double* __restrict__ after, unsigned na) {
  __shared__ double red[2][kTrajThreads / 32];
  double b = 0, a = 0;
  for (unsigned i = threadIdx.x; i < 4 * nb; i += kTrajThreads) b += before[i];
  for (unsigned i = threadIdx.x; i < 4 * na; i += kTrajThreads) a += after[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    b += __shfl_xor_sync(0xffffffffu, b, o);
    a += __shfl_xor_sync(0xffffffffu, a, o);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    red[0][warp] = b;
    red[1][warp] = a;
  }
  __syncthreads();
  b = 0;
  a = 0;
  for (int w = 0; w < kTrajThreads / 32; ++w) {
    b += red[0][w];
    a += red[1][w];
  }
  const float f = a > 0 ? float(sqrt(b / a)) : 1.f;
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < units;
       i += uint64_t(gridDim.x) * blockDim.x) {
    float4 x = s[i];
    s[i] = make_float4(x.x * f, x.y * f, x.z * f, x.w * f);
  }
}

// ---------------------------------------------------------------------------

static unsigned traj_grid(qsg_ctx* ctx, uint64_t work, uint64_t per_block) {
  uint64_t g = (work + per_block - 1) / per_block;
  const uint64_t cap = uint64_t(ctx->num_sms) * 4;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return unsigned(g);
}

unsigned traj_max_parts(qsg_ctx* ctx) { return unsigned(ctx->num_sms) * 4; }

int traj_channel_stats(qsg_ctx* ctx, const float* state, unsigned n,
                       unsigned nq, const unsigned* q, double* partial,
                       unsigned* nparts) {
  QSG_CHECK_ARG(n >= 1 && nq <= kTrajMaxChannelQubits,
                "channel statistics: bad sizes (n=%u, nq=%u)", n, nq);
  const uint64_t units = uint64_t{1} << (n - 1);
  const unsigned grid =
      traj_grid(ctx, units, uint64_t(kTrajThreads) * kTrajUnroll);
  traj_stats_kernel<<<grid, kTrajThreads, 0, ctx->stream>>>(
      reinterpret_cast<const float4*>(state), units, nq, nq > 0 ? q[0] : 0,
      nq > 1 ? q[1] : 0, partial);
  QSG_LAUNCHED(ctx);
  *nparts = grid;
  return QSG_OK;
}

int traj_choose(qsg_ctx* ctx, const double* partial, unsigned nparts,
                const TrajChannelDev* ch, double cp0, double r,
                uint32_t* choice_out, float* mat_out) {
  traj_choose_kernel<<<1, kTrajThreads, 0, ctx->stream>>>(
      partial, nparts, ch, cp0, r, choice_out, mat_out);
  QSG_LAUNCHED(ctx);
  return QSG_OK;
}

int traj_apply(qsg_ctx* ctx, float* state, unsigned n, unsigned nq,
               const unsigned* q, const float* mat_dev) {
  QSG_CHECK_ARG(n >= nq && n >= 1 && nq <= kTrajMaxChannelQubits,
                "trajectory apply: bad sizes (n=%u, nq=%u)", n, nq);
  const uint64_t groups = uint64_t{1} << (n - nq);
  const unsigned grid = traj_grid(ctx, groups, uint64_t(kTrajThreads) * 8);
  traj_apply_kernel<<<grid, kTrajThreads, 0, ctx->stream>>>(
      reinterpret_cast<float2*>(state), groups, nq, nq > 0 ? q[0] : 0,
      nq > 1 ? q[1] : 0, mat_dev);
  QSG_LAUNCHED(ctx);
  return QSG_OK;
}

int norm_restore(qsg_ctx* ctx, float* state, unsigned n, const double* before,
                 unsigned nb, const double* after, unsigned na) {
  QSG_CHECK_ARG(n >= 1, "norm restore: n >= 1");
  const uint64_t units = uint64_t{1} << (n - 1);
  const unsigned grid = traj_grid(ctx, units, uint64_t(kTrajThreads) * 8);
  norm_restore_kernel<<<grid, kTrajThreads, 0, ctx->stream>>>(
      reinterpret_cast<float4*>(state), units, before, nb, after, na);
  QSG_LAUNCHED(ctx);
  return QSG_OK;
}

}  // namespace qsg
