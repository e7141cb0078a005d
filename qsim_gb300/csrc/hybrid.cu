// Device helpers of the hybrid simulator (host/hybrid.cc).
//
// A part's batch state holds 2^bits path blocks of 2^n amplitudes (block b =
// path b).  hybrid_broadcast copies block 0 into every other block (the
// checkpointed state every path starts from); hybrid_collect adds, per
// bitstring, sum_b s0[i0 + b 2^n0] * s1[i1 + b 2^n1] to an FP64 accumulator
// (the reference's per-path results[i] += a0 * a1, lib/hybrid.h:423-433).

#include <algorithm>

#include "common.cuh"
#include "internal.h"

namespace qsg {

namespace {

constexpr int kThreads = 256;

// Amplitudes [2^n, 2^(n+bits)) <- amplitude (i mod 2^n); 16-byte units
// when a block holds at least two amplitudes.
__global__ void __launch_bounds__(kThreads)
    broadcast_units_kernel(float4* s, uint64_t block_units, uint64_t total) {
  for (uint64_t u = block_units + blockIdx.x * uint64_t(kThreads) + threadIdx.x;
       u < total; u += uint64_t(gridDim.x) * kThreads)
    s[u] = s[u & (block_units - 1)];
}

__global__ void __launch_bounds__(kThreads)
    broadcast_amps_kernel(float2* s, uint64_t block, uint64_t total) {
  for (uint64_t i = block + blockIdx.x * uint64_t(kThreads) + threadIdx.x;
       i < total; i += uint64_t(gridDim.x) * kThreads)
    s[i] = s[i & (block - 1)];
}

// One warp per bitstring, lanes over path blocks: FP32 products, FP64 sums.
__global__ void __launch_bounds__(kThreads)
    collect_kernel(const float2* __restrict__ s0, unsigned n0,
                   const float2* __restrict__ s1, unsigned n1, uint64_t blocks,
                   const uint64_t* __restrict__ idx, uint64_t m,
                   double2* __restrict__ acc) {
  const unsigned lane = threadIdx.x & 31;
  const uint64_t warps = uint64_t(gridDim.x) * (kThreads / 32);
  for (uint64_t w = (blockIdx.x * uint64_t(kThreads) + threadIdx.x) / 32;
       w < m; w += warps) {
    const uint64_t i0 = idx[2 * w], i1 = idx[2 * w + 1];
    double re = 0, im = 0;
    uint64_t b = lane;
    // Four blocks per lane and step, loads first: the gathers are scattered
    // 8-byte reads, so more of them in flight hide more latency.
    for (; b + 96 < blocks; b += 128) {
      float2 a[4], c[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        a[j] = s0[i0 + ((b + 32 * j) << n0)];
        c[j] = s1[i1 + ((b + 32 * j) << n1)];
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        re += double(a[j].x * c[j].x - a[j].y * c[j].y);
        im += double(a[j].x * c[j].y + a[j].y * c[j].x);
      }
    }
    for (; b < blocks; b += 32) {
      const float2 a = s0[i0 + (b << n0)];
      const float2 c = s1[i1 + (b << n1)];
      re += double(a.x * c.x - a.y * c.y);
      im += double(a.x * c.y + a.y * c.x);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      re += __shfl_down_sync(0xffffffffu, re, o);
      im += __shfl_down_sync(0xffffffffu, im, o);
    }
    if (lane == 0) {
      double2 v = acc[w];
      v.x += re;
      v.y += im;
      acc[w] = v;
    }
  }
}

unsigned grid_for(qsg_ctx* ctx, uint64_t items) {
  const uint64_t g = (items + kThreads - 1) / kThreads;
  return unsigned(std::max<uint64_t>(
      1, std::min<uint64_t>(g, uint64_t(ctx->num_sms) * 8)));
}

}  // namespace

int hybrid_broadcast(qsg_ctx* ctx, float* state, unsigned n, unsigned bits) {
  if (bits == 0) return QSG_OK;
  const uint64_t block = uint64_t{1} << n, total = block << bits;
  if (n >= 1) {
    broadcast_units_kernel<<<grid_for(ctx, (total - block) / 2), kThreads, 0,
                             ctx->stream>>>(reinterpret_cast<float4*>(state),
                                            block / 2, total / 2);
  } else {
    broadcast_amps_kernel<<<grid_for(ctx, total - block), kThreads, 0,
                            ctx->stream>>>(reinterpret_cast<float2*>(state),
                                           block, total);
  }
  QSG_LAUNCHED(ctx);
  return QSG_OK;
}

int hybrid_collect(qsg_ctx* ctx, const float* s0, unsigned n0, const float* s1,
                   unsigned n1, unsigned bits, const uint64_t* idx, uint64_t m,
                   double* acc) {
  if (m == 0) return QSG_OK;
  collect_kernel<<<grid_for(ctx, m * 32), kThreads, 0, ctx->stream>>>(
      reinterpret_cast<const float2*>(s0), n0,
      reinterpret_cast<const float2*>(s1), n1, uint64_t{1} << bits, idx, m,
      reinterpret_cast<double2*>(acc));
  QSG_LAUNCHED(ctx);
  return QSG_OK;
}

}  // namespace qsg
