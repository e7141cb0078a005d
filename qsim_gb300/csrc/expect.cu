// ExpectationValue of monomial operators in one read pass.
//
// The reference evaluates <psi|M|psi> with the dense 2^k x 2^k matrix
// (ExpectationValueH/L_Kernel, lib/simulator_cuda_kernels.h:482-693), also
// for the Pauli strings that lib/expect.h:105-151 fuses into <= 6-qubit
// gates.  A Pauli string (and any product of Pauli and diagonal gates) has
// one nonzero per row, at column r ^ xm: M psi at index i is d[r(i)] times
// psi at i ^ X, where r(i) are the bits of i on the target qubits and X is
// xm spread onto them.  So
//
//   <psi|M|psi> = sum_i conj(psi_i) d[r(i)] psi_(i ^ X),
//
// a bandwidth-bound pass (for Pauli strings d[r] is a constant times the sign
// (-1)^popcount(i & zmask), one AND and one popcount per amplitude; other
// monomials look d up by the target bits of i): each thread reads a 16-byte
// unit (two amplitudes)
// and, when X flips qubits above qubit 0, its partner unit, and adds both
// units' terms, so every amplitude is read once (8 N bytes).  Products are
// FP32; partial sums FP32 over a thread's units of one step, compensated
// (Kahan) FP32 across steps, FP64 across threads.

#include <algorithm>
#include <cstring>

#include "common.cuh"
#include "internal.h"
#include "matring.cuh"

namespace qsg {

namespace {

constexpr int kEvThreads = 256;
constexpr int kEvUnroll = 4;

struct MonoArgs {
  float2 d[64];        // d[r] = M[r][r ^ xm]
  float2 c0;           // SIGNED form: d[r] = c0 (-1)^popcount(r & zm)
  uint64_t zmask;      // SIGNED form: zm spread onto the state bits
  uint32_t qpos[6];    // target qubits (bit j of r <-> qpos[j])
  uint32_t k;
  uint32_t x0;         // bit 0 of X (qubit 0 flipped)
  uint64_t ux;         // X >> 1: partner unit offset (0: the unit itself)
  uint32_t ub;         // lowest set bit of ux (when ux != 0)
  // Table form in mono_fast_kernel: rows of amplitude offsets 2 j
  // kEvThreads (rj), of offset 1 (r1) and of 2 ux (rx).
  uint32_t rj[4];
  uint32_t r1, rx;
};

__device__ __forceinline__ uint32_t row_of(uint64_t i, const MonoArgs& a) {
  uint32_t r = 0;
#pragma unroll
  for (int j = 0; j < 6; ++j)
    if (j < int(a.k)) r |= uint32_t((i >> a.qpos[j]) & 1) << j;
  return r;
}

// conj(p) * d * q, FP32.
__device__ __forceinline__ void term(float& er, float& ei, float2 p, float2 d,
                                     float2 q) {
  const float tr = d.x * q.x - d.y * q.y;
  const float ti = d.x * q.y + d.y * q.x;
  er = fmaf(p.x, tr, fmaf(p.y, ti, er));
  ei = fmaf(p.x, ti, fmaf(-p.y, tr, ei));
}

// d for amplitude index i: the table entry of i's target bits, or for a
// Pauli-type operator (SIGNED) c0 with the sign of popcount(i & zmask).
template <bool SIGNED>
__device__ __forceinline__ float2 dval(uint64_t i, const MonoArgs& a) {
  if constexpr (SIGNED) {
    const bool neg = (__popcll(i & a.zmask) & 1) != 0;
    return neg ? make_float2(-a.c0.x, -a.c0.y) : a.c0;
  } else {
    return a.d[row_of(i, a)];
  }
}

template <bool SIGNED>
__global__ void __launch_bounds__(kEvThreads)
    mono_ev_kernel(const float4* __restrict__ s, uint64_t work,
                   const __grid_constant__ MonoArgs a,
                   double2* __restrict__ partial) {
  // FP32 sums per step, accumulated across steps in FP32 with Kahan
  // compensation (s - c) and converted to FP64 once: an FP64 add per step
  // would load GB300's narrow FP64 pipe.
  float sr = 0.f, cr = 0.f, si = 0.f, ci = 0.f;
  const uint64_t tile = uint64_t(kEvThreads) * kEvUnroll;
  for (uint64_t b0 = blockIdx.x * tile; b0 < work;
       b0 += uint64_t(gridDim.x) * tile) {
    float4 x[kEvUnroll], y[kEvUnroll];
    uint64_t u[kEvUnroll];
#pragma unroll
    for (int j = 0; j < kEvUnroll; ++j) {
      const uint64_t w = b0 + j * kEvThreads + threadIdx.x;
      // Work item w -> unit u with bit ub of u clear (ux != 0), or u = w.
      uint64_t uu = w;
      if (a.ux) {
        const uint64_t lo = w & ((uint64_t{1} << a.ub) - 1);
        uu = lo | ((w ^ lo) << 1);
      }
      u[j] = uu;
      x[j] = w < work ? s[uu] : make_float4(0.f, 0.f, 0.f, 0.f);
      if (a.ux)
        y[j] = w < work ? s[uu ^ a.ux] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    float fr = 0.f, fi = 0.f;
#pragma unroll
    for (int j = 0; j < kEvUnroll; ++j) {
      const uint64_t w = b0 + j * kEvThreads + threadIdx.x;
      if (w >= work) continue;
      const uint64_t i0 = 2 * u[j];
      const float2 p0 = make_float2(x[j].x, x[j].y);
      const float2 p1 = make_float2(x[j].z, x[j].w);
      if (a.ux == 0) {
        // Partner of amplitude i0 + t is i0 + (t ^ x0), in the same unit.
        const float2 q0 = a.x0 ? p1 : p0, q1 = a.x0 ? p0 : p1;
        term(fr, fi, p0, dval<SIGNED>(i0, a), q0);
        term(fr, fi, p1, dval<SIGNED>(i0 + 1, a), q1);
      } else {
        const uint64_t k0 = 2 * (u[j] ^ a.ux);
        const float2 r0 = make_float2(y[j].x, y[j].y);
        const float2 r1 = make_float2(y[j].z, y[j].w);
        const float2 q0 = a.x0 ? r1 : r0, q1 = a.x0 ? r0 : r1;
        const float2 v0 = a.x0 ? p1 : p0, v1 = a.x0 ? p0 : p1;
        term(fr, fi, p0, dval<SIGNED>(i0, a), q0);
        term(fr, fi, p1, dval<SIGNED>(i0 + 1, a), q1);
        term(fr, fi, r0, dval<SIGNED>(k0, a), v0);
        term(fr, fi, r1, dval<SIGNED>(k0 + 1, a), v1);
      }
    }
    const float yr = fr - cr, tr = sr + yr;
    cr = (tr - sr) - yr;
    sr = tr;
    const float yi = fi - ci, ti = si + yi;
    ci = (ti - si) - yi;
    si = ti;
  }
  double ar = double(sr) - double(cr), ai = double(si) - double(ci);
  __shared__ double red[2][kEvThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ar += __shfl_down_sync(0xffffffffu, ar, o);
    ai += __shfl_down_sync(0xffffffffu, ai, o);
  }
  if (threadIdx.x % 32 == 0) {
    red[0][threadIdx.x / 32] = ar;
    red[1][threadIdx.x / 32] = ai;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double sr = 0, si = 0;
    for (int i = 0; i < kEvThreads / 32; ++i) {
      sr += red[0][i];
      si += red[1][i];
    }
    partial[blockIdx.x] = make_double2(sr, si);
  }
}

// Monomial operators over whole tiles of work, one thread deriving its
// kEvUnroll units per step from one base unit u0 (unit j is u0 + j
// kEvThreads, bits 8..9 of u0 clear).  The per-amplitude form above spends
// its issue on 64-bit index and sign arithmetic (the integer pipe 79 %
// busy, DRAM 57 %, at 27 qubits).  SIGNED (Pauli-type, d[r] = c0
// (-1)^popcount(r & zm)): S = sum_i (-1)^par(i) conj(psi_i) psi_(i ^ X),
// par(i) the parity of i & zmask, and c0 S per block; par(2 (u0 + j
// kEvThreads)) = par(2 u0) ^ par(2 j kEvThreads), the unit's second
// amplitude adds bit 0 of zmask, the partner unit u ^ ux adds par(2 ux).
// Table form: the row r(i) of amplitude i (its target bits) is r(2 u0)
// | rj[j] for unit j, | r1 for the unit's second amplitude, ^ rx for the
// partner unit; d[r] from shared memory.  FORM 0: no partner unit (X on
// qubit 0 at most).  FORM 1: the partner is far (a set bit of ux at or
// above bit 10, `ub` the highest): work items are the units with bit ub
// clear, each with its partner, every amplitude once.  FORM 2: the partner
// is near (ux < 1024, inside the same tile of 1024 units): every unit takes
// its own two terms and reads its partner, which the tile's other threads
// read too (a cache hit, DRAM still reads each byte once).
template <int FORM, bool X0, bool SIGNED>
__global__ void __launch_bounds__(kEvThreads)
    mono_fast_kernel(const float4* __restrict__ s, uint64_t work,
                     const __grid_constant__ MonoArgs a,
                     double2* __restrict__ partial) {
  constexpr uint64_t kTile = uint64_t(kEvThreads) * kEvUnroll;
  static_assert(kTile == 1024, "unit offsets j kEvThreads use bits 8..9");
  static_assert(kEvUnroll == 4, "rj holds four rows");
  const uint32_t tid = threadIdx.x;
  __shared__ float2 dtab[SIGNED ? 1 : 64];
  if constexpr (!SIGNED) {
    if (tid < 64) dtab[tid] = a.d[tid];
    __syncthreads();
  }
  // Per unit offset j: its parity (SIGNED) or its table-row bits; par0
  // below is likewise the base unit's parity or table row.
  uint32_t pj[kEvUnroll];
#pragma unroll
  for (int j = 0; j < kEvUnroll; ++j)
    pj[j] = SIGNED ? __popcll((uint64_t(2 * j) * kEvThreads) & a.zmask) & 1u
                   : a.rj[j];
  // Signs as floats: bit 0 of zmask (second amplitude of a unit), the
  // partner unit's parity.
  const float f_z0 = (a.zmask & 1) ? -1.f : 1.f;
  const float f_px = (__popcll((2 * a.ux) & a.zmask) & 1) ? -1.f : 1.f;
  float sr = 0.f, cr = 0.f, si = 0.f, ci = 0.f;
  auto acc = [](float& er, float& ei, float sg, float2 p, float2 q) {
    const float tr = fmaf(p.x, q.x, p.y * q.y);
    const float ti = fmaf(p.x, q.y, -p.y * q.x);
    er = fmaf(sg, tr, er);
    ei = fmaf(sg, ti, ei);
  };
  // conj(p) d q.
  auto acc_d = [](float& er, float& ei, float2 d, float2 p, float2 q) {
    const float qr = fmaf(d.x, q.x, -d.y * q.y);
    const float qi = fmaf(d.x, q.y, d.y * q.x);
    er = fmaf(p.x, qr, fmaf(p.y, qi, er));
    ei = fmaf(p.x, qi, fmaf(-p.y, qr, ei));
  };
  for (uint64_t b0 = blockIdx.x * kTile; b0 < work;
       b0 += uint64_t(gridDim.x) * kTile) {
    const uint64_t w = b0 + tid;
    uint64_t u0 = w;
    if constexpr (FORM == 1) {
      const uint64_t lo = w & ((uint64_t{1} << a.ub) - 1);
      u0 = lo | ((w ^ lo) << 1);
    }
    const uint32_t par0 =
        SIGNED ? __popcll((2 * u0) & a.zmask) & 1u : row_of(2 * u0, a);
    const float4* sp = s + u0;
    const uint64_t v0 = u0 ^ a.ux;
    float4 x[kEvUnroll], y[kEvUnroll];
#pragma unroll
    for (int j = 0; j < kEvUnroll; ++j) {
      x[j] = sp[j * kEvThreads];
      if constexpr (FORM != 0) y[j] = s[v0 ^ (uint64_t(j) * kEvThreads)];
    }
    float fr = 0.f, fi = 0.f;
#pragma unroll
    for (int j = 0; j < kEvUnroll; ++j) {
      const float2 p0 = make_float2(x[j].x, x[j].y);
      const float2 p1 = make_float2(x[j].z, x[j].w);
      if constexpr (!SIGNED) {
        const uint32_t ra = par0 | pj[j], rb = ra | a.r1;
        if constexpr (FORM == 0) {
          acc_d(fr, fi, dtab[ra], p0, X0 ? p1 : p0);
          acc_d(fr, fi, dtab[rb], p1, X0 ? p0 : p1);
        } else {
          const float2 r0 = make_float2(y[j].x, y[j].y);
          const float2 r1 = make_float2(y[j].z, y[j].w);
          acc_d(fr, fi, dtab[ra], p0, X0 ? r1 : r0);
          acc_d(fr, fi, dtab[rb], p1, X0 ? r0 : r1);
          if constexpr (FORM == 1) {
            const uint32_t rc = ra ^ a.rx, rd = rc | a.r1;
            acc_d(fr, fi, dtab[rc], r0, X0 ? p1 : p0);
            acc_d(fr, fi, dtab[rd], r1, X0 ? p0 : p1);
          }
        }
        continue;
      }
      const float sa = __int_as_float(0x3f800000u | ((par0 ^ pj[j]) << 31));
      const float sb = sa * f_z0;
      if constexpr (FORM == 0) {
        acc(fr, fi, sa, p0, X0 ? p1 : p0);
        acc(fr, fi, sb, p1, X0 ? p0 : p1);
      } else {
        const float2 r0 = make_float2(y[j].x, y[j].y);
        const float2 r1 = make_float2(y[j].z, y[j].w);
        acc(fr, fi, sa, p0, X0 ? r1 : r0);
        acc(fr, fi, sb, p1, X0 ? r0 : r1);
        if constexpr (FORM == 1) {
          const float sc = sa * f_px, sd = sc * f_z0;
          acc(fr, fi, sc, r0, X0 ? p1 : p0);
          acc(fr, fi, sd, r1, X0 ? p0 : p1);
        }
      }
    }
    const float yr = fr - cr, tr = sr + yr;
    cr = (tr - sr) - yr;
    sr = tr;
    const float yi = fi - ci, ti = si + yi;
    ci = (ti - si) - yi;
    si = ti;
  }
  double ar = double(sr) - double(cr), ai = double(si) - double(ci);
  __shared__ double red[2][kEvThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ar += __shfl_down_sync(0xffffffffu, ar, o);
    ai += __shfl_down_sync(0xffffffffu, ai, o);
  }
  if (tid % 32 == 0) {
    red[0][tid / 32] = ar;
    red[1][tid / 32] = ai;
  }
  __syncthreads();
  if (tid == 0) {
    double sr2 = 0, si2 = 0;
    for (int i = 0; i < kEvThreads / 32; ++i) {
      sr2 += red[0][i];
      si2 += red[1][i];
    }
    const double c0r = SIGNED ? a.c0.x : 1.0, c0i = SIGNED ? a.c0.y : 0.0;
    partial[blockIdx.x] =
        make_double2(c0r * sr2 - c0i * si2, c0r * si2 + c0i * sr2);
  }
}

}  // namespace

bool monomial_xor(unsigned k, const float* m, uint32_t* xm, float* d) {
  const unsigned dim = 1u << k;
  for (unsigned r = 0; r < dim; ++r) {
    int col = -1;
    for (unsigned c = 0; c < dim; ++c) {
      const float re = m[2 * (r * dim + c)], im = m[2 * (r * dim + c) + 1];
      if (re != 0.f || im != 0.f) {
        if (col >= 0) return false;
        col = int(c);
      }
    }
    // An all-zero row fits any pattern: take the one row 0 fixed.
    const uint32_t x = col < 0 ? (r == 0 ? 0u : *xm) : uint32_t(col) ^ r;
    if (r == 0) *xm = x;
    else if (x != *xm) return false;
    d[2 * r] = col < 0 ? 0.f : m[2 * (r * dim + col)];
    d[2 * r + 1] = col < 0 ? 0.f : m[2 * (r * dim + col) + 1];
  }
  return true;
}

int expectation_monomial(qsg_ctx* ctx, const float* state, unsigned n,
                         const unsigned* qs, unsigned k, uint32_t xm,
                         const float* d, double* out_re_im) {
  QSG_CHECK_ARG(k >= 1 && k <= 6 && n >= 1, "monomial EV: bad sizes");
  MonoArgs a;
  std::memset(&a, 0, sizeof(a));
  a.k = k;
  uint64_t X = 0;
  for (unsigned j = 0; j < k; ++j) {
    a.qpos[j] = qs[j];
    if ((xm >> j) & 1) X |= uint64_t{1} << qs[j];
  }
  for (unsigned r = 0; r < (1u << k); ++r)
    a.d[r] = make_float2(d[2 * r], d[2 * r + 1]);
  // Pauli-type phases: d[r] = d[0] (-1)^popcount(r & zm), zm read off the
  // single-bit rows.
  bool signed_form = d[0] != 0.f || d[1] != 0.f;
  uint32_t zm = 0;
  for (unsigned j = 0; signed_form && j < k; ++j) {
    const float* dj = d + 2 * (1u << j);
    if (dj[0] == -d[0] && dj[1] == -d[1]) zm |= 1u << j;
    else if (!(dj[0] == d[0] && dj[1] == d[1])) signed_form = false;
  }
  for (unsigned r = 0; signed_form && r < (1u << k); ++r) {
    const float sgn = (__builtin_popcount(r & zm) & 1) ? -1.f : 1.f;
    if (d[2 * r] != sgn * d[0] || d[2 * r + 1] != sgn * d[1])
      signed_form = false;
  }
  a.c0 = make_float2(d[0], d[1]);
  for (unsigned j = 0; j < k; ++j)
    if ((zm >> j) & 1) a.zmask |= uint64_t{1} << qs[j];
  a.x0 = uint32_t(X & 1);
  a.ux = X >> 1;
  a.ub = a.ux ? unsigned(__builtin_ctzll(a.ux)) : 0;
  const uint64_t units = n == 0 ? 1 : (uint64_t{1} << (n - 1));
  uint64_t work = a.ux ? units / 2 : units;
  const uint64_t per_block = uint64_t(kEvThreads) * kEvUnroll;
  // Whole tiles of work take mono_fast_kernel: FORM 0 without a partner
  // unit, 2 with a near one (ux < one tile), 1 with a far one (paired on
  // the highest bit of ux).
  int form = -1;
  {
    const uint64_t wf = a.ux == 0 || a.ux < per_block ? units : units / 2;
    if (wf % per_block == 0) {
      form = a.ux == 0 ? 0 : a.ux < per_block ? 2 : 1;
      work = wf;
      if (form == 1) a.ub = 63u - unsigned(__builtin_clzll(a.ux));
    }
  }
  auto row = [&](uint64_t i) {
    uint32_t r = 0;
    for (unsigned j = 0; j < k; ++j) r |= uint32_t((i >> qs[j]) & 1) << j;
    return r;
  };
  for (int j = 0; j < kEvUnroll; ++j)
    a.rj[j] = row(uint64_t(2 * j) * kEvThreads);
  a.r1 = row(1);
  a.rx = row(2 * a.ux);
  uint64_t grid = (work + per_block - 1) / per_block;
  grid = std::min<uint64_t>(grid, uint64_t(ctx->num_sms) * 8);
  if (grid < 1) grid = 1;
  void* p = nullptr;
  int rc = get_scratch(ctx, (grid + 1) * sizeof(double2), &p);
  if (rc) return rc;
  double2* partial = static_cast<double2*>(p);
  const float4* sv = reinterpret_cast<const float4*>(state);
  const unsigned gb = unsigned(grid);
#define QSG_MONO(F, X, S)                                                   \
  mono_fast_kernel<F, X, S><<<gb, kEvThreads, 0, ctx->stream>>>(sv, work, a, \
                                                               partial)
  switch (form < 0 ? -1 : 4 * form + 2 * (a.x0 ? 1 : 0) + (signed_form ? 1 : 0)) {
    case 0: QSG_MONO(0, false, false); break;
    case 1: QSG_MONO(0, false, true); break;
    case 2: QSG_MONO(0, true, false); break;
    case 3: QSG_MONO(0, true, true); break;
    case 4: QSG_MONO(1, false, false); break;
    case 5: QSG_MONO(1, false, true); break;
    case 6: QSG_MONO(1, true, false); break;
    case 7: QSG_MONO(1, true, true); break;
    case 8: QSG_MONO(2, false, false); break;
    case 9: QSG_MONO(2, false, true); break;
    case 10: QSG_MONO(2, true, false); break;
    case 11: QSG_MONO(2, true, true); break;
    default:
      if (signed_form)
        mono_ev_kernel<true><<<gb, kEvThreads, 0, ctx->stream>>>(sv, work, a, partial);
      else
        mono_ev_kernel<false><<<gb, kEvThreads, 0, ctx->stream>>>(sv, work, a, partial);
  }
#undef QSG_MONO
  QSG_LAUNCHED(ctx);
  return reduce_partials_d2(ctx, partial, grid, out_re_im);
}

}  // namespace qsg
