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
//  * A persistent CTA walks its tiles with a two-stage cp.async pipeline:
//    16-byte copies land directly in (swizzled) shared memory while the
//    previous tile is being computed; results go from registers straight
//    back to HBM with 128-bit stores.
//  * Shared memory is addressed in 16-byte units (two amplitudes).  A per-gate
//    XOR swizzle of unit bits 0..2 makes the 128-bit accesses of the compute
//    phase bank-conflict free whatever the target positions are.
//  * When qubit 0 is not a target ("pair" mode) one work item holds two
//    groups that differ in bit 0, so each 16-byte unit feeds both.  When
//    qubit 0 is a target, a unit holds members (2p, 2p+1) of one group.
//  * For k <= 3 the matrix sits in kernel-parameter (constant) space and is
//    read with compile-time offsets, so FFMAs take it as a constant operand.
//    For k >= 4 it is staged column-major in shared memory (broadcast
//    128-bit reads of two rows) and 2^(k-3) threads split the rows of one
//    work item (8 rows each), which keeps the code small and the register
//    count low enough for five or more CTAs per SM.  (Measured slower for
//    k = 4 on GB300: packed two-lane FMAs, fma.rn.f32x2, which issue to one
//    of the two FMA sub-pipes only; and the matrix as constant-bank
//    operands with a fully unrolled code path per row block, which
//    overflows the instruction cache.)
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

// Host: builds the tile geometry of a (controlled) gate with 2^log_items
// work items per tile; `pair` when qubit 0 is not a target.  False on
// inconsistent input.  Defined in gate.cu.
bool plan_tile(unsigned n, const unsigned* qs, unsigned k,
               const unsigned* cqs, unsigned c, uint64_t cvals, bool pair,
               int log_items, TileGeom& g);

template <int K>
struct GateArgs {
  TileGeom g;
  // k <= 5: row-major interleaved complex matrix in parameter space.
  float m[K <= 5 ? 2 * (1 << (2 * K)) : 2];
  // k == 6: device copy of the row-major matrix (32 KiB exceeds the
  // kernel-parameter limit).
  const float2* mat;
};

template <int K, bool PAIR>
struct TileShape {
  static constexpr int D = 1 << K;
  static constexpr int LOG_S = K >= 4 ? K - 3 : 0;
  static constexpr int S = 1 << LOG_S;                    // row split
  static constexpr int R = D / S;                         // rows per thread
  static constexpr int ITEMS = kTileThreads / S;
  static constexpr int LOG_ITEMS = 7 - LOG_S;
  static constexpr bool SMEM_MAT = K >= 4;
  static constexpr int TB = LOG_ITEMS + K + (PAIR ? 1 : 0);  // full tile
  static constexpr int UNITS = 1 << (TB - 1);
  static constexpr int LPT = UNITS / kTileThreads;  // 16-B units per thread
  static constexpr int MAT_FLOAT2 = SMEM_MAT ? D * D : 0;
  static constexpr int STAGES = 2;
  static constexpr size_t SMEM =
      size_t(STAGES) * UNITS * 16 + size_t(MAT_FLOAT2) * 8;
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

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const uint32_t sa = static_cast<uint32_t>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa),
               "l"(gmem)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Issues the 16-byte copies of tile `t` into `tile` (one commit group).
template <int LPT>
__device__ __forceinline__ void tile_load_async(const float4* __restrict__ st,
                                                float4* tile, uint64_t t,
                                                const TileGeom& g) {
  if (t < g.num_tiles) {
    const uint64_t base = expand_outer(t, g);
    const uint32_t nunits = 1u << (g.tb - 1);
    const uint32_t rl = g.b - 1;
    const uint32_t pmask = (1u << rl) - 1;
#pragma unroll
    for (int j = 0; j < LPT; ++j) {
      const uint32_t u = threadIdx.x + j * kTileThreads;
      if (u < nunits) {
        const uint64_t a = ((base + g.run_off[u >> rl]) >> 1) + (u & pmask);
        cp_async16(&tile[swz(u, g)], &st[a]);
      }
    }
  }
  cp_async_commit();
}

// Global float4 index of tile unit u (u = logical, unswizzled unit index).
__device__ __forceinline__ uint64_t unit_addr(uint64_t base, uint32_t u,
                                              const TileGeom& g) {
  const uint32_t rl = g.b - 1;
  return ((base + g.run_off[u >> rl]) >> 1) + (u & ((1u << rl) - 1));
}

// Matrix element (row, col) as float2 (k <= 3: parameter space).
template <int K>
struct MatAccess {
  static constexpr int D = 1 << K;
  const GateArgs<K>& a;
  __device__ __forceinline__ float2 operator()(int row, int col) const {
    return make_float2(a.m[2 * (row * D + col)], a.m[2 * (row * D + col) + 1]);
  }
};

// Matrix held in registers (k <= 2), loaded from memory once per gate.
template <int K>
struct RegMat {
  static constexpr int D = 1 << K;
  float2 m[D * D];
  __device__ __forceinline__ explicit RegMat(const float* src) {
#pragma unroll
    for (int i = 0; i < D * D; ++i) m[i] = make_float2(src[2 * i], src[2 * i + 1]);
  }
  __device__ __forceinline__ float2 operator()(int row, int col) const {
    return m[row * D + col];
  }
};

// Placeholder accessor for gates whose matrix is read from shared memory.
struct NoMat {
  __device__ __forceinline__ float2 operator()(int, int) const {
    return make_float2(0.f, 0.f);
  }
};

__device__ __forceinline__ void cmac(float& ar, float& ai, float2 m, float vr,
                                     float vi) {
  ar = fmaf(m.x, vr, ar);
  ar = fmaf(-m.y, vi, ar);
  ai = fmaf(m.x, vi, ai);
  ai = fmaf(m.y, vr, ai);
}

// One CTA's share of a gate pass: tiles t0, t0 + step, ... of geometry g,
// pipelined through STAGES shared-memory tile buffers (cp.async).  MODE 0
// applies the matrix, MODE 1 accumulates <s|M|s> into (er, ei), MODE 2 (a
// Hermitian M, k <= 3: one thread holds every row) accumulates it as
// sum_r M_rr |v_r|^2 + 2 Re conj(v_r) sum_(c > r) M_rc v_c, half the
// products, with ei = 0.  SMAT: the
// matrix is read column-major from `smat` (2^k x 2^k float2, staged by the
// caller); otherwise from the accessor M.  PRE: the tile-invariant parts of
// every load and store address are computed once per pass and kept in
// registers (the address arithmetic otherwise shares the issue slots with
// the FFMAs; k = 4 is issue-bound).  Used by the tile kernel below
// (grid-stride over tiles) and by the packed-batch kernel (one CTA walks all
// tiles of a trajectory's gate).
template <int K, bool PAIR, int MODE, bool SMAT, int STAGES, bool PRE = false,
          class MA>
__device__ __forceinline__ void tile_pass(float4* __restrict__ st,
                                          const TileGeom& g, const MA& M,
                                          const float2* smat, float4* tile,
                                          uint64_t t0, uint64_t step,
                                          double& er, double& ei) {
  using SH = TileShape<K, PAIR>;
  constexpr int D = SH::D;
  constexpr int R = SH::R;
  constexpr int ITEMS = SH::ITEMS;
  constexpr int NACC = PAIR ? 4 : 2;

  const uint32_t tid = threadIdx.x;
  const int rb = SH::S == 1 ? 0 : int(tid / ITEMS);
  const uint32_t item = tid % ITEMS;
  const bool active = item < g.items;
  const uint32_t e = expand_item(item, g);
  const uint32_t swe = swz(e >> 1, g) ^ (e >> 1);
  const bool ok0 = (e & g.cmask_low) == g.cvals_low;
  const bool ok1 = ((e | 1u) & g.cmask_low) == g.cvals_low;

  // With PRE: per load unit j its swizzled shared-memory index and its
  // offset from the tile's base unit, per output row r its offset; a tile's
  // base and the run offsets are both even, so (base + run_off) / 2 =
  // base / 2 + run_off / 2.
  uint32_t ld_s[PRE ? SH::LPT : 1];
  uint64_t ld_g[PRE ? SH::LPT : 1];
  uint64_t st_g[PRE ? R : 1];
  uint32_t ld_ok = 0;
  if constexpr (PRE) {
    const uint32_t rl = g.b - 1, pmask = (1u << rl) - 1;
    const uint32_t nunits = 1u << (g.tb - 1);
#pragma unroll
    for (int j = 0; j < SH::LPT; ++j) {
      const uint32_t u = threadIdx.x + j * kTileThreads;
      ld_s[j] = swz(u, g);
      ld_g[j] = u < nunits ? (g.run_off[u >> rl] >> 1) + (u & pmask) : 0;
      ld_ok |= uint32_t(u < nunits) << j;
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const uint32_t u = (e | g.moff[rb * R + r]) >> 1;
      st_g[r] = (g.run_off[u >> rl] >> 1) + (u & pmask);
    }
  }
  auto load_tile = [&](float4* buf, uint64_t tt) {
    if constexpr (PRE) {
      if (tt < g.num_tiles) {
        const uint64_t b2 = expand_outer(tt, g) >> 1;
#pragma unroll
        for (int j = 0; j < SH::LPT; ++j)
          if ((ld_ok >> j) & 1) cp_async16(&buf[ld_s[j]], &st[b2 + ld_g[j]]);
      }
      cp_async_commit();
    } else {
      tile_load_async<SH::LPT>(st, buf, tt, g);
    }
  };
  // Global unit index of output row r of this thread's item (u: its
  // tile unit).
  auto out_addr = [&](uint64_t base, int r, uint32_t u) -> uint64_t {
    if constexpr (PRE) {
      return (base >> 1) + st_g[r];
    } else {
      return unit_addr(base, u, g);
    }
  };

  // MODE 1: this thread's sum over its tiles, FP32 with Kahan compensation
  // (s - c), added to (er, ei) in FP64 once at the end: an FP64 add per
  // tile costs GB300's narrow FP64 pipe as much as the pass's loads.
  float ksr = 0.f, kcr = 0.f, ksi = 0.f, kci = 0.f;

  // Pipeline: tiles t0 .. t0 + (STAGES-1) step are in flight on entry.
  uint64_t t = t0;
#pragma unroll
  for (int q = 0; q < STAGES; ++q) load_tile(tile + q * SH::UNITS, t + q * step);

  for (int stage = 0; t < g.num_tiles; t += step) {
    float4* cur = tile + stage * SH::UNITS;
    cp_async_wait<STAGES - 1>();
    __syncthreads();
    const uint64_t base = expand_outer(t, g);

    float acc[R][NACC];
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
      for (int j = 0; j < NACC; ++j) acc[r][j] = 0.f;

    if (active) {
      if constexpr (SMAT) {
        // Rows rb*R .. rb*R+R-1 of column c are contiguous in smat.  Columns
        // unrolled by 4 for k = 4 (3 % faster than 2 on GB300), by 2 above.
        const float4* mbase = reinterpret_cast<const float4*>(smat + rb * R);
        if constexpr (PAIR) {
#pragma unroll (K == 4 ? 4 : 2)
          for (int c = 0; c < D; ++c) {
            const float4 v = cur[((e | g.moff[c]) >> 1) ^ swe];
            const float4* mc = mbase + c * (D / 2);
#pragma unroll
            for (int r2 = 0; r2 < R / 2; ++r2) {
              const float4 mm = mc[r2];
              const float2 m0 = make_float2(mm.x, mm.y);
              const float2 m1 = make_float2(mm.z, mm.w);
              cmac(acc[2 * r2][0], acc[2 * r2][1], m0, v.x, v.y);
              cmac(acc[2 * r2][2], acc[2 * r2][3], m0, v.z, v.w);
              cmac(acc[2 * r2 + 1][0], acc[2 * r2 + 1][1], m1, v.x, v.y);
              cmac(acc[2 * r2 + 1][2], acc[2 * r2 + 1][3], m1, v.z, v.w);
            }
          }
        } else {
#pragma unroll (K == 4 ? 4 : 2)
          for (int p = 0; p < D / 2; ++p) {
            const float4 v = cur[((e | g.moff[2 * p]) >> 1) ^ swe];
            const float4* mc0 = mbase + (2 * p) * (D / 2);
            const float4* mc1 = mbase + (2 * p + 1) * (D / 2);
#pragma unroll
            for (int r2 = 0; r2 < R / 2; ++r2) {
              const float4 a0 = mc0[r2], a1 = mc1[r2];
              cmac(acc[2 * r2][0], acc[2 * r2][1], make_float2(a0.x, a0.y), v.x, v.y);
              cmac(acc[2 * r2][0], acc[2 * r2][1], make_float2(a1.x, a1.y), v.z, v.w);
              cmac(acc[2 * r2 + 1][0], acc[2 * r2 + 1][1], make_float2(a0.z, a0.w), v.x, v.y);
              cmac(acc[2 * r2 + 1][0], acc[2 * r2 + 1][1], make_float2(a1.z, a1.w), v.z, v.w);
            }
          }
        }
      } else if constexpr (PAIR) {
#pragma unroll
        for (int c = 0; c < D; ++c) {
          if (MODE == 2 && c == 0) continue;
          const float4 v = cur[((e | g.moff[c]) >> 1) ^ swe];
#pragma unroll
          for (int r = 0; r < R; ++r) {
            if (MODE == 2 && r >= c) continue;
            const float2 m = M(r, c);
            cmac(acc[r][0], acc[r][1], m, v.x, v.y);
            cmac(acc[r][2], acc[r][3], m, v.z, v.w);
          }
        }
      } else {
#pragma unroll
        for (int p = 0; p < D / 2; ++p) {
          const float4 v = cur[((e | g.moff[2 * p]) >> 1) ^ swe];
#pragma unroll
          for (int r = 0; r < R; ++r) {
            if (MODE != 2 || r < 2 * p) {
              const float2 m0 = M(r, 2 * p);
              cmac(acc[r][0], acc[r][1], m0, v.x, v.y);
            }
            if (MODE != 2 || r < 2 * p + 1) {
              const float2 m1 = M(r, 2 * p + 1);
              cmac(acc[r][0], acc[r][1], m1, v.z, v.w);
            }
          }
        }
      }
    }

    if constexpr (MODE == 2) {
      // Hermitian: diagonal |v_r|^2 terms plus twice the real part of
      // conj(v_r) times the upper-triangle sums.
      if (active) {
        float fr = 0.f;
        if constexpr (PAIR) {
#pragma unroll
          for (int r = 0; r < R; ++r) {
            const float4 v = cur[((e | g.moff[r]) >> 1) ^ swe];
            const float d = M(r, r).x;
            const float n2 = fmaf(v.x, v.x, fmaf(v.y, v.y, fmaf(v.z, v.z, v.w * v.w)));
            const float o = fmaf(v.x, acc[r][0], fmaf(v.y, acc[r][1],
                            fmaf(v.z, acc[r][2], v.w * acc[r][3])));
            fr = fmaf(d, n2, fmaf(2.f, o, fr));
          }
        } else {
#pragma unroll
          for (int r = 0; r < R; r += 2) {
            const float4 v = cur[((e | g.moff[r]) >> 1) ^ swe];
            const float d0 = M(r, r).x, d1 = M(r + 1, r + 1).x;
            const float o = fmaf(v.x, acc[r][0], fmaf(v.y, acc[r][1],
                            fmaf(v.z, acc[r + 1][0], v.w * acc[r + 1][1])));
            fr = fmaf(d0, fmaf(v.x, v.x, v.y * v.y),
                      fmaf(d1, fmaf(v.z, v.z, v.w * v.w), fmaf(2.f, o, fr)));
          }
        }
        const float yr = fr - kcr, tr = ksr + yr;
        kcr = (tr - ksr) - yr;
        ksr = tr;
      }
    } else if constexpr (MODE == 1) {
      // v^dagger (M v) over this item's rows: FP32 products and item sum,
      // compensated FP32 accumulation across tiles, FP64 across threads.
      if (active) {
        float fr = 0.f, fi = 0.f;
        if constexpr (PAIR) {
#pragma unroll
          for (int r = 0; r < R; ++r) {
            const float4 v = cur[((e | g.moff[rb * R + r]) >> 1) ^ swe];
            fr += fmaf(v.x, acc[r][0], v.y * acc[r][1]) +
                  fmaf(v.z, acc[r][2], v.w * acc[r][3]);
            fi += fmaf(v.x, acc[r][1], -v.y * acc[r][0]) +
                  fmaf(v.z, acc[r][3], -v.w * acc[r][2]);
          }
        } else {
#pragma unroll
          for (int r = 0; r < R; r += 2) {
            const float4 v = cur[((e | g.moff[rb * R + r]) >> 1) ^ swe];
            fr += fmaf(v.x, acc[r][0], v.y * acc[r][1]) +
                  fmaf(v.z, acc[r + 1][0], v.w * acc[r + 1][1]);
            fi += fmaf(v.x, acc[r][1], -v.y * acc[r][0]) +
                  fmaf(v.z, acc[r + 1][1], -v.w * acc[r + 1][0]);
          }
        }
        const float yr = fr - kcr, tr = ksr + yr;
        kcr = (tr - ksr) - yr;
        ksr = tr;
        const float yi = fi - kci, ti = ksi + yi;
        kci = (ti - ksi) - yi;
        ksi = ti;
      }
    } else if (active) {
      // Controlled rows keep their input where the control test fails, so
      // those units are left untouched in HBM.
      if constexpr (PAIR) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const uint32_t u = (e | g.moff[rb * R + r]) >> 1;
          float4* gp = st + out_addr(base, r, u);
          if (ok0 && ok1) {
            *gp = make_float4(acc[r][0], acc[r][1], acc[r][2], acc[r][3]);
          } else if (ok0) {
            *reinterpret_cast<float2*>(&gp->x) =
                make_float2(acc[r][0], acc[r][1]);
          } else if (ok1) {
            *reinterpret_cast<float2*>(&gp->z) =
                make_float2(acc[r][2], acc[r][3]);
          }
        }
      } else if (ok0) {
#pragma unroll
        for (int r = 0; r < R; r += 2) {
          const uint32_t u = (e | g.moff[rb * R + r]) >> 1;
          st[out_addr(base, r, u)] = make_float4(
              acc[r][0], acc[r][1], acc[r + 1][0], acc[r + 1][1]);
        }
      }
    }
    // Every thread is done reading `cur`: refill it with the tile STAGES
    // steps ahead.
    __syncthreads();
    load_tile(cur, t + uint64_t(STAGES) * step);
    stage = stage + 1 == STAGES ? 0 : stage + 1;
  }
  cp_async_wait<0>();
  if constexpr (MODE >= 1) {
    er += double(ksr) - double(kcr);
    ei += double(ksi) - double(kci);
  }
}

// MODE 0: apply, MODE 1: expectation value, MODE 2: expectation value of a
// Hermitian matrix (k <= 3).
// k = 4 keeps its addresses in registers (PRE) at four CTAs per SM: 15 %
// faster than five CTAs without (3.40 against 4.1 ms per 30-qubit pass).
template <int K, bool PAIR, int MODE>
__global__ void __launch_bounds__(kTileThreads, K <= 4 ? 4 : 5)
    gate_tile_kernel(float4* __restrict__ st,
                     const __grid_constant__ GateArgs<K> a,
                     double2* __restrict__ partial) {
  using SH = TileShape<K, PAIR>;
  constexpr int D = SH::D;
  extern __shared__ float4 smem[];
  float2* smat = reinterpret_cast<float2*>(smem + SH::STAGES * SH::UNITS);
  if constexpr (SH::SMEM_MAT) {
    // Column-major copy: smat[c * D + r] = M[r][c].
    for (int i = threadIdx.x; i < D * D; i += kTileThreads) {
      const int r = i / D, c = i % D;
      if constexpr (K <= 5) {
        smat[c * D + r] = make_float2(a.m[2 * i], a.m[2 * i + 1]);
      } else {
        smat[c * D + r] = a.mat[i];
      }
    }
    __syncthreads();
  }
  double er = 0, ei = 0;
  tile_pass<K, PAIR, MODE, SH::SMEM_MAT, SH::STAGES, K == 4>(
      st, a.g, MatAccess<K>{a}, smat, smem, blockIdx.x, gridDim.x, er, ei);

  if constexpr (MODE >= 1) {
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
