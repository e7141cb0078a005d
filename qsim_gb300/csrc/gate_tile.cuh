// Tile geometry and the shared-memory tile kernel that applies a fused
// k-qubit matrix (k <= 6), a controlled matrix, or computes <s|M|s>.
//
// Replaces the reference kernels ApplyGateH/L_Kernel,
// ApplyControlledGateH/LH/L_Kernel and ExpectationValueH/L_Kernel
// (lib/simulator_cuda_kernels.h:30-693) with one design:
//
//  * A tile is 2^b consecutive amplitudes (a "run", >= 512 B) times the 2^h
//    combinations of the targets that lie above bit b.  Tile index bit j < b
//    is state bit j; tile bit b+i is the i-th high target.  Every group of
//    2^k amplitudes that the gate mixes lies inside one tile.
//  * A CTA streams its tiles HBM -> registers -> shared memory with 128-bit
//    coalesced loads, computes on shared memory, and streams the tile back.
//  * Shared memory is addressed in 16-byte units (two amplitudes).  A per-gate
//    XOR swizzle of unit bits 0..2 makes the 128-bit accesses of the compute
//    phase bank-conflict free whatever the target positions are.
//  * When qubit 0 is not a target ("pair" mode) one work item holds two
//    groups that differ in bit 0, so each 16-byte unit feeds both.  When
//    qubit 0 is a target, a unit holds members (2p, 2p+1) of one group.
//  * For k <= 4 the matrix sits in kernel-parameter (constant) space and is
//    read with compile-time offsets, so FFMAs take it as a constant operand.
//    For k = 5, 6 it is staged column-major in shared memory and 2^(k-4)
//    threads split the rows of one work item.
#pragma once

#include "common.cuh"

namespace qsg {

constexpr int kTileThreads = 128;

struct TileGeom {
  uint64_t num_tiles;
  uint64_t cvals_high;       // high control values at their bit positions
  uint64_t cmask_low;        // controls below bit b (tile bits == state bits)
  uint64_t cvals_low;
  uint64_t run_off[64];      // amplitude offset of run r (high-target bits)
  uint32_t ins_pos[kMaxQubits];  // ascending bit positions >= b that the
                                 // outer tile index skips (high targets and
                                 // high controls)
  uint32_t n_ins;
  uint32_t b;                // run bits
  uint32_t tb;               // tile bits
  uint32_t h;                // high targets
  uint32_t items;            // work items per tile
  uint32_t item_skip[8];     // ascending tile positions skipped by the item
  uint32_t n_item_skip;      // index ({0} U target tile positions)
  uint32_t moff[64];         // tile offset (amplitudes) of member m
  uint32_t sw_src[3];        // unit-bit XOR swizzle: unit bit sw_dst[i] ^=
  uint32_t sw_dst[3];        // unit bit sw_src[i]
  uint32_t n_sw;
};

template <int K>
struct GateArgs {
  TileGeom g;
  // k <= 4: row-major interleaved complex matrix in parameter space.
  float m[K <= 4 ? 2 * (1 << (2 * K)) : 2];
  // k >= 5: device copy of the row-major matrix.
  const float2* mat;
};

template <int K, bool PAIR>
struct TileShape {
  static constexpr int D = 1 << K;
  static constexpr int S = K >= 5 ? (1 << (K - 4)) : 1;  // row split
  static constexpr int R = D / S;                         // rows per thread
  static constexpr int ITEMS = kTileThreads / S;
  static constexpr int LOG_ITEMS = K >= 5 ? 11 - K : 7;
  static constexpr int TB = LOG_ITEMS + K + (PAIR ? 1 : 0);  // full tile
  static constexpr int UNITS = 1 << (TB - 1);
  static constexpr int LPT = UNITS / kTileThreads;  // 16-B units per thread
  static constexpr int MAT_FLOAT2 = K >= 5 ? D * D : 0;
  static constexpr size_t SMEM = size_t(UNITS) * 16 + size_t(MAT_FLOAT2) * 8;
};

__device__ __forceinline__ uint64_t expand_outer(uint64_t t,
                                                 const TileGeom& g) {
  uint64_t x = t << g.b;
  for (uint32_t i = 0; i < g.n_ins; ++i) {
    uint32_t p = g.ins_pos[i];
    uint64_t lo = x & ((uint64_t{1} << p) - 1);
    x = lo | ((x ^ lo) << 1);
  }
  return x | g.cvals_high;
}

__device__ __forceinline__ uint32_t expand_item(uint32_t w,
                                                const TileGeom& g) {
  uint32_t e = w;
  for (uint32_t i = 0; i < g.n_item_skip; ++i) {
    uint32_t p = g.item_skip[i];
    uint32_t lo = e & ((1u << p) - 1);
    e = lo | ((e ^ lo) << 1);
  }
  return e;
}

__device__ __forceinline__ uint32_t swz(uint32_t u, const TileGeom& g) {
  uint32_t x = 0;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    if (i < (int)g.n_sw) x |= ((u >> g.sw_src[i]) & 1u) << g.sw_dst[i];
  }
  return u ^ x;
}

template <int LPT>
__device__ __forceinline__ void tile_load(const float4* __restrict__ st,
                                          float4* tile, uint64_t base,
                                          const TileGeom& g) {
  const uint32_t nunits = 1u << (g.tb - 1);
  const uint32_t rl = g.b - 1;
  const uint32_t pmask = (1u << rl) - 1;
  float4 buf[LPT];
#pragma unroll
  for (int j = 0; j < LPT; ++j) {
    uint32_t u = threadIdx.x + j * kTileThreads;
    if (u < nunits) {
      uint64_t a = ((base + g.run_off[u >> rl]) >> 1) + (u & pmask);
      buf[j] = st[a];
    }
  }
#pragma unroll
  for (int j = 0; j < LPT; ++j) {
    uint32_t u = threadIdx.x + j * kTileThreads;
    if (u < nunits) tile[swz(u, g)] = buf[j];
  }
}

template <int LPT>
__device__ __forceinline__ void tile_store(float4* __restrict__ st,
                                           const float4* tile, uint64_t base,
                                           const TileGeom& g) {
  const uint32_t nunits = 1u << (g.tb - 1);
  const uint32_t rl = g.b - 1;
  const uint32_t pmask = (1u << rl) - 1;
#pragma unroll
  for (int j = 0; j < LPT; ++j) {
    uint32_t u = threadIdx.x + j * kTileThreads;
    if (u < nunits) {
      uint64_t a = ((base + g.run_off[u >> rl]) >> 1) + (u & pmask);
      st[a] = tile[swz(u, g)];
    }
  }
}

// Matrix element (row, col) as float2.
template <int K>
struct MatAccess {
  static constexpr int D = 1 << K;
  const GateArgs<K>& a;
  const float2* smat;  // column-major copy for K >= 5
  __device__ __forceinline__ float2 operator()(int row, int col) const {
    if constexpr (K <= 4) {
      return make_float2(a.m[2 * (row * D + col)], a.m[2 * (row * D + col) + 1]);
    } else {
      return smat[col * D + row];
    }
  }
};

__device__ __forceinline__ void cmac(float& ar, float& ai, float2 m, float vr,
                                     float vi) {
  ar = fmaf(m.x, vr, ar);
  ar = fmaf(-m.y, vi, ar);
  ai = fmaf(m.x, vi, ai);
  ai = fmaf(m.y, vr, ai);
}

// MODE 0: apply, MODE 1: expectation value.
template <int K, bool PAIR, int MODE>
__global__ void __launch_bounds__(kTileThreads, K <= 3 ? 4 : (K == 4 ? 3 : 2))
    gate_tile_kernel(float4* __restrict__ st,
                     const __grid_constant__ GateArgs<K> a,
                     double2* __restrict__ partial) {
  using SH = TileShape<K, PAIR>;
  constexpr int D = SH::D;
  constexpr int R = SH::R;
  constexpr int ITEMS = SH::ITEMS;
  constexpr int NACC = PAIR ? 4 : 2;

  extern __shared__ float4 smem[];
  const TileGeom& g = a.g;
  float4* tile = smem;
  float2* smat = reinterpret_cast<float2*>(smem + SH::UNITS);

  if constexpr (K >= 5) {
    // Column-major copy: smat[c * D + r] = M[r][c].
    for (int i = threadIdx.x; i < D * D; i += kTileThreads) {
      int r = i / D, c = i % D;
      smat[c * D + r] = a.mat[i];
    }
    __syncthreads();
  }
  MatAccess<K> M{a, smat};

  const uint32_t tid = threadIdx.x;
  const int rb = SH::S == 1 ? 0 : int(tid / ITEMS);
  const uint32_t item = tid % ITEMS;
  const bool active = item < g.items;
  const uint32_t e = expand_item(item, g);
  const uint32_t swe = swz(e >> 1, g) ^ (e >> 1);
  const bool ok0 = (e & g.cmask_low) == g.cvals_low;
  const bool ok1 = ((e | 1u) & g.cmask_low) == g.cvals_low;

  double er = 0, ei = 0;

  for (uint64_t t = blockIdx.x; t < g.num_tiles; t += gridDim.x) {
    const uint64_t base = expand_outer(t, g);
    tile_load<SH::LPT>(st, tile, base, g);
    __syncthreads();

    float acc[R][NACC];
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
      for (int j = 0; j < NACC; ++j) acc[r][j] = 0.f;

    if (active) {
      if constexpr (PAIR) {
#pragma unroll(K >= 5 ? 2 : D)
        for (int c = 0; c < D; ++c) {
          const float4 v = tile[((e | g.moff[c]) >> 1) ^ swe];
#pragma unroll
          for (int r = 0; r < R; ++r) {
            const float2 m = M(rb * R + r, c);
            cmac(acc[r][0], acc[r][1], m, v.x, v.y);
            cmac(acc[r][2], acc[r][3], m, v.z, v.w);
          }
        }
      } else {
#pragma unroll(K >= 5 ? 2 : D / 2)
        for (int p = 0; p < D / 2; ++p) {
          const float4 v = tile[((e | g.moff[2 * p]) >> 1) ^ swe];
#pragma unroll
          for (int r = 0; r < R; ++r) {
            const float2 m0 = M(rb * R + r, 2 * p);
            const float2 m1 = M(rb * R + r, 2 * p + 1);
            cmac(acc[r][0], acc[r][1], m0, v.x, v.y);
            cmac(acc[r][0], acc[r][1], m1, v.z, v.w);
          }
        }
      }
    }

    if constexpr (MODE == 1) {
      if (active) {
        if constexpr (PAIR) {
#pragma unroll
          for (int r = 0; r < R; ++r) {
            const float4 v = tile[((e | g.moff[rb * R + r]) >> 1) ^ swe];
            er += double(v.x) * acc[r][0] + double(v.y) * acc[r][1];
            ei += double(v.x) * acc[r][1] - double(v.y) * acc[r][0];
            er += double(v.z) * acc[r][2] + double(v.w) * acc[r][3];
            ei += double(v.z) * acc[r][3] - double(v.w) * acc[r][2];
          }
        } else {
#pragma unroll
          for (int r = 0; r < R; r += 2) {
            const float4 v = tile[((e | g.moff[rb * R + r]) >> 1) ^ swe];
            er += double(v.x) * acc[r][0] + double(v.y) * acc[r][1];
            ei += double(v.x) * acc[r][1] - double(v.y) * acc[r][0];
            er += double(v.z) * acc[r + 1][0] + double(v.w) * acc[r + 1][1];
            ei += double(v.z) * acc[r + 1][1] - double(v.w) * acc[r + 1][0];
          }
        }
      }
      __syncthreads();
    } else {
      __syncthreads();
      if (active) {
        if constexpr (PAIR) {
#pragma unroll
          for (int r = 0; r < R; ++r) {
            float4* p = &tile[((e | g.moff[rb * R + r]) >> 1) ^ swe];
            if (ok0 && ok1) {
              *p = make_float4(acc[r][0], acc[r][1], acc[r][2], acc[r][3]);
            } else if (ok0) {
              *reinterpret_cast<float2*>(&p->x) =
                  make_float2(acc[r][0], acc[r][1]);
            } else if (ok1) {
              *reinterpret_cast<float2*>(&p->z) =
                  make_float2(acc[r][2], acc[r][3]);
            }
          }
        } else {
          if (ok0) {
#pragma unroll
            for (int r = 0; r < R; r += 2) {
              tile[((e | g.moff[rb * R + r]) >> 1) ^ swe] = make_float4(
                  acc[r][0], acc[r][1], acc[r + 1][0], acc[r + 1][1]);
            }
          }
        }
      }
      __syncthreads();
      tile_store<SH::LPT>(st, tile, base, g);
      __syncthreads();
    }
  }

  if constexpr (MODE == 1) {
    // Block reduction of (er, ei) in FP64, fixed order.
    __shared__ double red[2][kTileThreads / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      er += __shfl_down_sync(0xffffffffu, er, o);
      ei += __shfl_down_sync(0xffffffffu, ei, o);
    }
    const int w = threadIdx.x / 32, l = threadIdx.x % 32;
    if (l == 0) {
      red[0][w] = er;
      red[1][w] = ei;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double sr = 0, si = 0;
      for (int i = 0; i < kTileThreads / 32; ++i) {
        sr += red[0][i];
        si += red[1][i];
      }
      partial[blockIdx.x] = make_double2(sr, si);
    }
  }
}

}  // namespace qsg
