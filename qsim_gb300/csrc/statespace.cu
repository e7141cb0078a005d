// State-space kernels: initialisation, elementwise ops, FP64 reductions,
// chunked CDF scans for Sample / Measure, and Collapse.
//
// Replaces StateSpaceCUDA (lib/statespace_cuda.h:109-373) and its kernels
// (lib/statespace_cuda_kernels.h:181-351).  The reference samples with a
// single thread scanning all 2^n amplitudes (SampleKernel, :301-326); here
// the state is cut into chunks of 2^13 amplitudes, chunk sums are scanned on
// the device, and one CTA per chunk that holds samples resolves them with a
// block-wide scan and binary searches.  Products and short partial sums are
// FP32 (GB300 issues FP64 at a small fraction of the FP32 rate), every
// longer sum is FP64, and every partition is fixed, so results are
// deterministic for a given n and GPU.

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <random>
#include <vector>

#include "common.cuh"
#include "matring.cuh"

namespace qsg {

constexpr int kRedThreads = 256;
constexpr unsigned kChunkBits = 13;              // amplitudes per chunk 2^13
constexpr int kScanThreads = 256;
constexpr int kAmpsPerScanThread = 32;           // 256 * 32 = 8192

inline unsigned chunk_bits(unsigned n) { return n < kChunkBits ? n : kChunkBits; }
inline uint64_t num_chunks(unsigned n) { return uint64_t{1} << (n - chunk_bits(n)); }

// ---------------------------------------------------------------------------
// Elementwise kernels (grid-stride over float4 units = two amplitudes).

__global__ void fill_zero_kernel(float4* s, uint64_t units) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < units;
       i += uint64_t(gridDim.x) * blockDim.x)
    s[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

__global__ void set_one_kernel(float* s) { s[0] = 1.f; s[1] = 0.f; }

__global__ void uniform_kernel(float4* s, uint64_t units, uint64_t namps,
                               float v) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < units;
       i += uint64_t(gridDim.x) * blockDim.x) {
    float a0 = 2 * i < namps ? v : 0.f;
    float a1 = 2 * i + 1 < namps ? v : 0.f;
    s[i] = make_float4(a0, 0.f, a1, 0.f);
  }
}

__global__ void bulk_set_kernel(float2* s, uint64_t namps, uint64_t mask,
                                uint64_t bits, float re, float im,
                                bool exclude) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < namps;
       i += uint64_t(gridDim.x) * blockDim.x) {
    bool set = ((i & mask) == bits) ^ exclude;
    if (set) s[i] = make_float2(re, im);
  }
}

__global__ void add_kernel(const float4* __restrict__ a, float4* __restrict__ b,
                           uint64_t units) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < units;
       i += uint64_t(gridDim.x) * blockDim.x) {
    float4 x = a[i], y = b[i];
    b[i] = make_float4(x.x + y.x, x.y + y.y, x.z + y.z, x.w + y.w);
  }
}

__global__ void multiply_kernel(float4* s, uint64_t units, float a) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < units;
       i += uint64_t(gridDim.x) * blockDim.x) {
    float4 x = s[i];
    s[i] = make_float4(x.x * a, x.y * a, x.z * a, x.w * a);
  }
}

__global__ void collapse_kernel(float4* s, uint64_t units, uint64_t mask,
                                uint64_t bits, float renorm) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < units;
       i += uint64_t(gridDim.x) * blockDim.x) {
    float4 x = s[i];
    bool k0 = ((2 * i) & mask) == bits;
    bool k1 = ((2 * i + 1) & mask) == bits;
    s[i] = make_float4(k0 ? x.x * renorm : 0.f, k0 ? x.y * renorm : 0.f,
                       k1 ? x.z * renorm : 0.f, k1 ? x.w * renorm : 0.f);
  }
}

// ---------------------------------------------------------------------------
// Reductions.  OP 0: sum |s1|^2 (masked), 1: Re<s1|s2>, 2: <s1|s2>.
// GB300's FP64 rate is a small fraction of its FP32 rate, so products and
// short partial sums (8 float4 units = 16 amplitudes per thread) are FP32,
// as the reference's CUDA kernels form products in FP32; every partial is
// then accumulated in FP64 (lib/statespace_cuda_kernels.h:31-177 uses FP64
// accumulation).

constexpr int kRedUnroll = 8;

template <int OP>
__global__ void __launch_bounds__(kRedThreads)
    reduce_kernel(const float4* __restrict__ s1, const float4* __restrict__ s2,
                  uint64_t units, uint64_t mask, uint64_t bits,
                  double2* __restrict__ partial) {
  double ar = 0, ai = 0;
  const uint64_t tile = uint64_t(kRedThreads) * kRedUnroll;
  for (uint64_t b0 = blockIdx.x * tile; b0 < units;
       b0 += uint64_t(gridDim.x) * tile) {
    float4 x[kRedUnroll], y[kRedUnroll];
#pragma unroll
    for (int j = 0; j < kRedUnroll; ++j) {
      const uint64_t i = b0 + j * kRedThreads + threadIdx.x;
      x[j] = i < units ? s1[i] : make_float4(0.f, 0.f, 0.f, 0.f);
      if constexpr (OP != 0)
        y[j] = i < units ? s2[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    float fr = 0.f, fi = 0.f;
#pragma unroll
    for (int j = 0; j < kRedUnroll; ++j) {
      const uint64_t i = b0 + j * kRedThreads + threadIdx.x;
      if constexpr (OP == 0) {
        float p0 = fmaf(x[j].x, x[j].x, x[j].y * x[j].y);
        float p1 = fmaf(x[j].z, x[j].z, x[j].w * x[j].w);
        if (mask != 0) {
          if (((2 * i) & mask) != bits) p0 = 0.f;
          if (((2 * i + 1) & mask) != bits) p1 = 0.f;
        }
        fr += p0 + p1;
      } else {
        fr += fmaf(x[j].x, y[j].x, x[j].y * y[j].y) +
              fmaf(x[j].z, y[j].z, x[j].w * y[j].w);
        if constexpr (OP == 2) {
          fi += fmaf(x[j].x, y[j].y, -x[j].y * y[j].x) +
                fmaf(x[j].z, y[j].w, -x[j].w * y[j].z);
        }
      }
    }
    ar += double(fr);
    if constexpr (OP == 2) ai += double(fi);
  }
  __shared__ double red[2][kRedThreads / 32];
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
    for (int i = 0; i < kRedThreads / 32; ++i) {
      sr += red[0][i];
      si += red[1][i];
    }
    partial[blockIdx.x] = make_double2(sr, si);
  }
}

__global__ void __launch_bounds__(1024)
    final_reduce_kernel(const double2* __restrict__ partial, uint64_t count,
                        double2* __restrict__ out) {
  double ar = 0, ai = 0;
  for (uint64_t i = threadIdx.x; i < count; i += blockDim.x) {
    ar += partial[i].x;
    ai += partial[i].y;
  }
  __shared__ double red[2][32];
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
    for (unsigned i = 0; i < blockDim.x / 32; ++i) {
      sr += red[0][i];
      si += red[1][i];
    }
    *out = make_double2(sr, si);
  }
}

// ---------------------------------------------------------------------------
// Chunk scans.  A chunk is 2^cb consecutive amplitudes (cb <= 13).
//
// chunk_sum_kernel: coalesced float4 loads, FP32 products and per-thread
// partial sums, FP64 block total.
//
// ChunkCdf (used by the sample, measure and find kernels): the chunk's
// probabilities are staged in shared memory (FP32, padded so a thread's
// 32-element segment is conflict-free); thread t owns segment
// [t*32, t*32+32) and its FP32 running sum; the segment totals are scanned
// in FP64.  The CDF at element i of segment t is
//   base + seg_prefix[t] + (double)(running FP32 sum up to i).
// A position is found by a binary search over segment prefixes followed by a
// sequential walk of at most 32 elements.

constexpr int kSeg = kAmpsPerScanThread;                   // 32
constexpr int kChunkAmps = kScanThreads * kSeg;             // 8192
constexpr int kPadAmps = kChunkAmps + kChunkAmps / 32;      // padded floats

__device__ __forceinline__ int pad_idx(int i) { return i + (i >> 5); }

__global__ void __launch_bounds__(kScanThreads)
    chunk_sum_kernel(const float2* __restrict__ s, uint32_t cb,
                     uint64_t nchunks, double* __restrict__ out) {
  __shared__ double red[kScanThreads / 32];
  // 16-byte units (two amplitudes), all of a thread's units of a chunk in
  // flight at once (16 for a full 2^13-amplitude chunk).
  constexpr int kU = kChunkAmps / 2 / kScanThreads;
  const uint32_t units = cb == 0 ? 1 : (1u << (cb - 1));
  for (uint64_t m = blockIdx.x; m < nchunks; m += gridDim.x) {
    float f = 0.f;
    if (cb == 0) {
      if (threadIdx.x == 0) {
        const float2 a = s[m];
        f = fmaf(a.x, a.x, a.y * a.y);
      }
    } else {
      const float4* c = reinterpret_cast<const float4*>(s + (m << cb));
      float4 v[kU];
#pragma unroll
      for (int j = 0; j < kU; ++j) {
        const uint32_t i = threadIdx.x + j * kScanThreads;
        v[j] = i < units ? c[i] : make_float4(0.f, 0.f, 0.f, 0.f);
      }
#pragma unroll
      for (int j = 0; j < kU; ++j)
        f += fmaf(v[j].x, v[j].x, v[j].y * v[j].y) +
             fmaf(v[j].z, v[j].z, v[j].w * v[j].w);
    }
    double d = f;
    for (int o = 16; o > 0; o >>= 1) d += __shfl_down_sync(0xffffffffu, d, o);
    if (threadIdx.x % 32 == 0) red[threadIdx.x / 32] = d;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0;
      for (int i = 0; i < kScanThreads / 32; ++i) t += red[i];
      out[m] = t;
    }
    __syncthreads();
  }
}

struct ChunkCdf {
  float* p;          // padded FP32 probabilities
  double* seg;       // [kScanThreads + 1] exclusive segment prefixes
  uint32_t camps;
};

// Loads chunk c and builds the segment prefixes.  All threads must call it.
__device__ void chunk_cdf_build(const float2* __restrict__ s, uint32_t cb,
                                uint64_t c, float* p, double* seg) {
  const uint32_t camps = 1u << cb;
  const float2* ch = s + (c << cb);
  for (uint32_t i = threadIdx.x; i < camps; i += kScanThreads) {
    float2 a = ch[i];
    p[pad_idx(i)] = fmaf(a.x, a.x, a.y * a.y);
  }
  __syncthreads();
  float f = 0.f;
  const uint32_t beg = threadIdx.x * kSeg;
  for (int j = 0; j < kSeg; ++j) {
    uint32_t i = beg + j;
    if (i < camps) f += p[pad_idx(i)];
  }
  // Block exclusive scan of the segment totals in FP64.
  __shared__ double wsum[kScanThreads / 32];
  double x = f;
  const int lane = threadIdx.x % 32, w = threadIdx.x / 32;
  for (int o = 1; o < 32; o <<= 1) {
    double y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  double xe = __shfl_up_sync(0xffffffffu, x, 1);
  if (lane == 0) xe = 0.0;
  if (lane == 31) wsum[w] = x;
  __syncthreads();
  if (threadIdx.x == 0) {
    double acc = 0;
    for (int i = 0; i < kScanThreads / 32; ++i) {
      double v = wsum[i];
      wsum[i] = acc;
      acc += v;
    }
  }
  __syncthreads();
  seg[threadIdx.x] = wsum[w] + xe;
  if (threadIdx.x == kScanThreads - 1) seg[kScanThreads] = wsum[w] + xe + f;
  __syncthreads();
}

// First i in the chunk with x < base + CDF(i); camps-1 if none.  `strict`
// false uses x <= CDF (the reference's `while (r > partial_norms[m])`).
__device__ uint32_t chunk_cdf_find(const float* p, const double* seg,
                                   uint32_t camps, double base, double x) {
  uint32_t nseg = (camps + kSeg - 1) / kSeg;
  // first segment t with x < base + seg[t+1]
  uint32_t lo = 0, hi = nseg;
  while (lo < hi) {
    uint32_t mid = (lo + hi) / 2;
    if (x < base + seg[mid + 1]) hi = mid; else lo = mid + 1;
  }
  if (lo >= nseg) return camps - 1;
  const double b = base + seg[lo];
  float f = 0.f;
  const uint32_t beg = lo * kSeg;
  for (int j = 0; j < kSeg; ++j) {
    uint32_t i = beg + j;
    if (i >= camps) break;
    f += p[pad_idx(i)];
    if (x < b + double(f)) return i;
  }
  uint32_t last = beg + kSeg - 1;
  return last < camps ? last : camps - 1;
}

// Inclusive prefix over chunk totals (one CTA, fixed order):
// incl[m] = sum_{j<=m} sums[j].
__global__ void __launch_bounds__(1024)
    chunk_prefix_kernel(const double* __restrict__ sums, uint64_t nchunks,
                        double* __restrict__ incl) {
  __shared__ double ws[32];
  const uint64_t per = (nchunks + blockDim.x - 1) / blockDim.x;
  const uint64_t beg = threadIdx.x * per;
  // Loads in batches of 8 independent reads; the sum keeps index order.
  double s = 0;
  for (uint64_t j0 = 0; j0 < per; j0 += 8) {
    double v[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const uint64_t i = beg + j0 + q;
      v[q] = (j0 + q < per && i < nchunks) ? sums[i] : 0.0;
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) s += v[q];
  }
  double x = s;
  const int lane = threadIdx.x % 32, w = threadIdx.x / 32;
  for (int o = 1; o < 32; o <<= 1) {
    double y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  double xe = __shfl_up_sync(0xffffffffu, x, 1);
  if (lane == 0) xe = 0.0;
  if (lane == 31) ws[w] = x;
  __syncthreads();
  if (threadIdx.x == 0) {
    double acc = 0;
    for (unsigned i = 0; i < blockDim.x / 32; ++i) {
      double v = ws[i];
      ws[i] = acc;
      acc += v;
    }
  }
  __syncthreads();
  double run = ws[w] + xe;
  for (uint64_t j0 = 0; j0 < per; j0 += 8) {
    double v[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const uint64_t i = beg + j0 + q;
      v[q] = (j0 + q < per && i < nchunks) ? sums[i] : 0.0;
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const uint64_t i = beg + j0 + q;
      if (j0 + q < per && i < nchunks) {
        run += v[q];
        incl[i] = run;
      }
    }
  }
}

// Two-level prefix for many chunks: the one-CTA kernel above reads every
// chunk sum twice from one SM (33 us of a 230 us Sample at 27 qubits).
// Level 1: the sum of each block of kPrefixBlock chunk sums (fixed-order
// tree); level 2: a one-block scan of the block sums (chunk_prefix_kernel
// beyond 1024 blocks); level 3: each
// block's inclusive scan plus the inclusive sum of the blocks before it.
// Every order is fixed, so the result does not vary between runs.
constexpr int kPrefixBlock = 256;

__global__ void __launch_bounds__(kPrefixBlock)
    prefix_block_sums_kernel(const double* __restrict__ sums, uint64_t nchunks,
                             double* __restrict__ block_tot) {
  __shared__ double ws[kPrefixBlock / 32];
  const uint64_t i = blockIdx.x * uint64_t(kPrefixBlock) + threadIdx.x;
  double v = i < nchunks ? sums[i] : 0.0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x % 32, w = threadIdx.x / 32;
  if (lane == 0) ws[w] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int k = 0; k < kPrefixBlock / 32; ++k) t += ws[k];
    block_tot[blockIdx.x] = t;
  }
}

// Any block size that is a multiple of 32 up to 1024; block_incl null: no
// offset (a one-block scan of the block sums).
__global__ void __launch_bounds__(1024)
    prefix_block_apply_kernel(const double* __restrict__ sums,
                              uint64_t nchunks,
                              const double* __restrict__ block_incl,
                              double* __restrict__ incl) {
  __shared__ double ws[32];
  const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  double x = i < nchunks ? sums[i] : 0.0;
  const int lane = threadIdx.x % 32, w = threadIdx.x / 32;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const double y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[w] = x;
  __syncthreads();
  if (threadIdx.x == 0) {
    double acc = (blockIdx.x == 0 || !block_incl) ? 0.0 : block_incl[blockIdx.x - 1];
    for (int k = 0; k < int(blockDim.x / 32); ++k) {
      const double t = ws[k];
      ws[k] = acc;
      acc += t;
    }
  }
  __syncthreads();
  if (i < nchunks) incl[i] = ws[w] + x;
}

// r[j] = u[j] * total, total = incl[nchunks-1].
__global__ void scale_uniforms_kernel(const double* __restrict__ u,
                                      uint64_t m, const double* __restrict__ incl,
                                      uint64_t nchunks, double* __restrict__ r) {
  const double total = incl[nchunks - 1];
  for (uint64_t j = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; j < m;
       j += uint64_t(gridDim.x) * blockDim.x)
    r[j] = u[j] * total;
}

// First j in [0, m) with r[j] >= x (r sorted ascending).
__device__ __forceinline__ uint64_t lower_bound_d(const double* r, uint64_t m,
                                                  double x) {
  uint64_t lo = 0, hi = m;
  while (lo < hi) {
    uint64_t mid = (lo + hi) / 2;
    if (r[mid] < x) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// Sample j belongs to chunk c iff incl[c-1] <= r[j] < incl[c], i.e. c is
// the first chunk with r[j] < incl[c] (nchunks if none: the sample gets
// 2^n - 1, lib/statespace_basic.h:222-224).  One thread per sample.
__global__ void sample_locate_kernel(const double* __restrict__ incl,
                                     uint64_t nchunks,
                                     const double* __restrict__ r, uint64_t m,
                                     uint32_t* __restrict__ chunk_of) {
  for (uint64_t j = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; j < m;
       j += uint64_t(gridDim.x) * blockDim.x) {
    const double x = r[j];
    uint64_t lo = 0, hi = nchunks;
    while (lo < hi) {
      const uint64_t mid = (lo + hi) / 2;
      if (x < incl[mid]) hi = mid; else lo = mid + 1;
    }
    chunk_of[j] = uint32_t(lo);
  }
}

// One CTA per sample; the CTA of the first sample of each chunk's run (the
// samples are sorted, so a chunk's samples are consecutive) builds that
// chunk's CDF and resolves the whole run: inside the chunk a sample's index
// is the first k with r[j] < incl[c-1] + CDF(k).  Only chunks that hold
// samples are read.
__global__ void __launch_bounds__(kScanThreads)
    sample_resolve_kernel(const float2* __restrict__ s, uint32_t cb,
                          uint64_t nchunks, const double* __restrict__ incl,
                          const double* __restrict__ r, uint64_t m,
                          const uint32_t* __restrict__ chunk_of,
                          uint64_t last_index, uint64_t* __restrict__ out) {
  __shared__ float p[kPadAmps];
  __shared__ double seg[kScanThreads + 1];
  for (uint64_t j = blockIdx.x; j < m; j += gridDim.x) {
    const uint32_t c = chunk_of[j];
    if (j > 0 && chunk_of[j - 1] == c) continue;  // uniform across the block
    // End of the run: first j' > j with chunk_of[j'] != c.
    uint64_t lo = j + 1, hi = m;
    while (lo < hi) {
      const uint64_t mid = (lo + hi) / 2;
      if (chunk_of[mid] == c) lo = mid + 1; else hi = mid;
    }
    const uint64_t end = lo;
    if (c >= nchunks) {
      for (uint64_t t = j + threadIdx.x; t < end; t += blockDim.x)
        out[t] = last_index;
      continue;
    }
    chunk_cdf_build(s, cb, c, p, seg);
    const double base = c == 0 ? 0.0 : incl[c - 1];
    for (uint64_t t = j + threadIdx.x; t < end; t += blockDim.x)
      out[t] = (uint64_t(c) << cb) + chunk_cdf_find(p, seg, 1u << cb, base, r[t]);
    __syncthreads();
  }
}

// FindMeasuredBits: first k of chunk c with r < in-chunk CDF(k) (last index
// of the chunk if none); masked.
__global__ void __launch_bounds__(kScanThreads)
    find_in_chunk_kernel(const float2* __restrict__ s, uint32_t cb, uint64_t c,
                         double r, uint64_t mask, uint64_t* __restrict__ out) {
  __shared__ float p[kPadAmps];
  __shared__ double seg[kScanThreads + 1];
  chunk_cdf_build(s, cb, c, p, seg);
  if (threadIdx.x == 0)
    *out = ((c << cb) + chunk_cdf_find(p, seg, 1u << cb, 0.0, r)) & mask;
}

// Measure on the device: r = u * total; chunk c = first with r <= incl[c]
// (the reference's `while (r > partial_norms[m]) ++m`), r -= incl[c-1], then
// the in-chunk search of FindMeasuredBits.
__global__ void __launch_bounds__(kScanThreads)
    measure_kernel(const float2* __restrict__ s, uint32_t cb, uint64_t nchunks,
                   const double* __restrict__ incl, double u, uint64_t mask,
                   uint64_t* __restrict__ out) {
  __shared__ float p[kPadAmps];
  __shared__ double seg[kScanThreads + 1];
  __shared__ uint64_t sc;
  __shared__ double sr;
  if (threadIdx.x == 0) {
    double total = incl[nchunks - 1];
    double r = u * total;
    uint64_t lo = 0, hi = nchunks - 1;  // first c with r <= incl[c]
    while (lo < hi) {
      uint64_t mid = (lo + hi) / 2;
      if (r > incl[mid]) lo = mid + 1; else hi = mid;
    }
    sc = lo;
    sr = lo > 0 ? r - incl[lo - 1] : r;
  }
  __syncthreads();
  const uint64_t c = sc;
  chunk_cdf_build(s, cb, c, p, seg);
  if (threadIdx.x == 0)
    *out = ((c << cb) + chunk_cdf_find(p, seg, 1u << cb, 0.0, sr)) & mask;
}

// ---------------------------------------------------------------------------
// Host helpers.

static unsigned grid_for(qsg_ctx* ctx, uint64_t work, int threads) {
  uint64_t g = (work + threads - 1) / threads;
  uint64_t cap = uint64_t(ctx->num_sms) * 8;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (unsigned)g;
}

static inline uint64_t units_of(unsigned n) {
  return n == 0 ? 1 : (uint64_t{1} << (n - 1));
}

int reduce_partials_d2(qsg_ctx* ctx, const double2* partial, uint64_t count,
                       double* out_re_im) {
  double2* dres = const_cast<double2*>(partial) + count;  // scratch tail
  final_reduce_kernel<<<1, 1024, 0, ctx->stream>>>(partial, count, dres);
  QSG_LAUNCHED(ctx);
  void* h = nullptr;
  int rc = get_hscratch(ctx, sizeof(double2), &h);
  if (rc) return rc;
  QSG_CUDA(cudaMemcpyAsync(h, dres, sizeof(double2), cudaMemcpyDeviceToHost,
                           ctx->stream));
  QSG_CUDA(cudaStreamSynchronize(ctx->stream));
  std::memcpy(out_re_im, h, sizeof(double2));
  return QSG_OK;
}

template <int OP>
static int reduce(qsg_ctx* ctx, const float* s1, const float* s2, unsigned n,
                  uint64_t mask, uint64_t bits, double* out) {
  const uint64_t units = units_of(n);
  const unsigned grid = grid_for(ctx, units, kRedThreads * kRedUnroll);
  void* p = nullptr;
  int rc = get_scratch(ctx, (grid + 1) * sizeof(double2), &p);
  if (rc) return rc;
  double2* partial = static_cast<double2*>(p);
  reduce_kernel<OP><<<grid, kRedThreads, 0, ctx->stream>>>(
      reinterpret_cast<const float4*>(s1), reinterpret_cast<const float4*>(s2),
      units, mask, bits, partial);
  QSG_LAUNCHED(ctx);
  return reduce_partials_d2(ctx, partial, grid, out);
}

// Chunk sums + inclusive prefix into scratch: returns pointers.
static int chunk_prefix(qsg_ctx* ctx, const float* s, unsigned n,
                        size_t extra_bytes, double** sums, double** incl,
                        void** extra) {
  const uint64_t nc = num_chunks(n);
  // Chunk counts above this take the two-level prefix.
  constexpr uint64_t kOneCtaPrefixMax = 4096;
  const uint64_t nb = nc > kOneCtaPrefixMax ? (nc + kPrefixBlock - 1) / kPrefixBlock : 0;
  void* p = nullptr;
  size_t bytes = (2 * nc + 2 * nb) * sizeof(double) + extra_bytes + 256;
  int rc = get_scratch(ctx, bytes, &p);
  if (rc) return rc;
  *sums = static_cast<double*>(p);
  *incl = *sums + nc;
  double* block_tot = *incl + nc;
  double* block_incl = block_tot + nb;
  if (extra) *extra = reinterpret_cast<char*>(block_incl + nb);
  const unsigned grid = (unsigned)std::min<uint64_t>(nc, 65535ull * 16);
  chunk_sum_kernel<<<grid, kScanThreads, 0, ctx->stream>>>(
      reinterpret_cast<const float2*>(s), chunk_bits(n), nc, *sums);
  QSG_LAUNCHED(ctx);
  if (nb == 0) {
    chunk_prefix_kernel<<<1, 1024, 0, ctx->stream>>>(*sums, nc, *incl);
    QSG_LAUNCHED(ctx);
    return QSG_OK;
  }
  prefix_block_sums_kernel<<<(unsigned)nb, kPrefixBlock, 0, ctx->stream>>>(
      *sums, nc, block_tot);
  QSG_LAUNCHED(ctx);
  if (nb <= 1024) {
    // One block, one block sum per thread.
    const unsigned t = unsigned((nb + 31) / 32 * 32);
    prefix_block_apply_kernel<<<1, t, 0, ctx->stream>>>(block_tot, nb, nullptr,
                                                        block_incl);
  } else {
    chunk_prefix_kernel<<<1, 1024, 0, ctx->stream>>>(block_tot, nb, block_incl);
  }
  QSG_LAUNCHED(ctx);
  prefix_block_apply_kernel<<<(unsigned)nb, kPrefixBlock, 0, ctx->stream>>>(
      *sums, nc, block_incl, *incl);  // blockDim = kPrefixBlock per block
  QSG_LAUNCHED(ctx);
  return QSG_OK;
}

void matring_release(qsg_ctx* ctx) {
  for (int i = 0; i < qsg_ctx::kRingSlots; ++i) {
    if (ctx->ring_ev[i]) cudaEventDestroy(ctx->ring_ev[i]);
    ctx->ring_ev[i] = nullptr;
  }
  if (ctx->ring_dev) cudaFree(ctx->ring_dev);
  if (ctx->ring_host) cudaFreeHost(ctx->ring_host);
  ctx->ring_dev = nullptr;
  ctx->ring_host = nullptr;
}

int matring_upload(qsg_ctx* ctx, const float* host_matrix, size_t nfloats,
                   const float** dev) {
  if (nfloats > qsg_ctx::kRingSlotFloats) {
    set_error("matrix too large for the upload ring");
    return QSG_ERR_INVALID;
  }
  if (!ctx->ring_dev) {
    const size_t bytes =
        qsg_ctx::kRingSlots * qsg_ctx::kRingSlotFloats * sizeof(float);
    QSG_CUDA(cudaMalloc(&ctx->ring_dev, bytes));
    QSG_CUDA(cudaMallocHost(&ctx->ring_host, bytes));
    for (int i = 0; i < qsg_ctx::kRingSlots; ++i) {
      QSG_CUDA(cudaEventCreateWithFlags(&ctx->ring_ev[i],
                                        cudaEventDisableTiming));
    }
  }
  const int slot = ctx->ring_next;
  ctx->ring_next = (slot + 1) % qsg_ctx::kRingSlots;
  if (ctx->ring_used[slot]) QSG_CUDA(cudaEventSynchronize(ctx->ring_ev[slot]));
  float* h = ctx->ring_host + slot * qsg_ctx::kRingSlotFloats;
  float* d = ctx->ring_dev + slot * qsg_ctx::kRingSlotFloats;
  std::memcpy(h, host_matrix, nfloats * sizeof(float));
  QSG_CUDA(cudaMemcpyAsync(d, h, nfloats * sizeof(float),
                           cudaMemcpyHostToDevice, ctx->stream));
  QSG_CUDA(cudaEventRecord(ctx->ring_ev[slot], ctx->stream));
  ctx->ring_used[slot] = true;
  *dev = d;
  return QSG_OK;
}

// libstdc++'s std::generate_canonical<double, 53>(std::mt19937&) and
// uniform_real_distribution<double>(0, 1): two 32-bit draws
// (lo + hi * 2^32) / 2^64, clamped below 1.
static double canonical_u01(std::mt19937& g) {
  std::uniform_real_distribution<double> d(0.0, 1.0);
  return d(g);
}

}  // namespace qsg

using namespace qsg;

extern "C" {

int qsg_internal_to_normal(qsg_ctx* ctx, float* state, unsigned n) {
  QSG_CHECK_ARG(ctx && state && n <= kMaxQubits, "bad argument");
  return QSG_OK;
}

int qsg_normal_to_internal(qsg_ctx* ctx, float* state, unsigned n) {
  QSG_CHECK_ARG(ctx && state && n <= kMaxQubits, "bad argument");
  return QSG_OK;
}

int qsg_set_all_zeros(qsg_ctx* ctx, float* state, unsigned n) {
  QSG_CHECK_ARG(ctx && state && n <= kMaxQubits, "qsg_set_all_zeros: bad arg");
  const uint64_t units = min_size(n) / 4;
  fill_zero_kernel<<<grid_for(ctx, units, 256), 256, 0, ctx->stream>>>(
      reinterpret_cast<float4*>(state), units);
  QSG_LAUNCHED(ctx);
  return QSG_OK;
}

int qsg_set_state_zero(qsg_ctx* ctx, float* state, unsigned n) {
  int rc = qsg_set_all_zeros(ctx, state, n);
  if (rc) return rc;
  set_one_kernel<<<1, 1, 0, ctx->stream>>>(state);
  QSG_LAUNCHED(ctx);
  return QSG_OK;
}

int qsg_set_state_uniform(qsg_ctx* ctx, float* state, unsigned n) {
  QSG_CHECK_ARG(ctx && state && n <= kMaxQubits, "qsg_set_state_uniform");
  const uint64_t units = min_size(n) / 4;
  const float v = float(1.0 / std::sqrt(double(uint64_t{1} << n)));
  uniform_kernel<<<grid_for(ctx, units, 256), 256, 0, ctx->stream>>>(
      reinterpret_cast<float4*>(state), units, uint64_t{1} << n, v);
  QSG_LAUNCHED(ctx);
  return QSG_OK;
}

int qsg_get_ampl(qsg_ctx* ctx, const float* state, unsigned n, uint64_t i,
                 float* re_im) {
  QSG_CHECK_ARG(ctx && state && re_im, "qsg_get_ampl: null argument");
  QSG_CHECK_ARG(n <= kMaxQubits && i < (uint64_t{1} << n),
                "qsg_get_ampl: index out of range");
  void* h = nullptr;
  int rc = get_hscratch(ctx, 8, &h);
  if (rc) return rc;
  QSG_CUDA(cudaMemcpyAsync(h, state + 2 * i, 8, cudaMemcpyDeviceToHost,
                           ctx->stream));
  QSG_CUDA(cudaStreamSynchronize(ctx->stream));
  std::memcpy(re_im, h, 8);
  return QSG_OK;
}

int qsg_set_ampl(qsg_ctx* ctx, float* state, unsigned n, uint64_t i, float re,
                 float im) {
  QSG_CHECK_ARG(ctx && state, "qsg_set_ampl: null argument");
  QSG_CHECK_ARG(n <= kMaxQubits && i < (uint64_t{1} << n),
                "qsg_set_ampl: index out of range");
  float v[2] = {re, im};
  // Pageable source: the runtime stages it before returning.
  QSG_CUDA(cudaMemcpyAsync(state + 2 * i, v, 8, cudaMemcpyHostToDevice,
                           ctx->stream));
  QSG_CUDA(cudaStreamSynchronize(ctx->stream));
  return QSG_OK;
}

int qsg_bulk_set_ampl(qsg_ctx* ctx, float* state, unsigned n, uint64_t mask,
                      uint64_t bits, float re, float im, int exclude) {
  QSG_CHECK_ARG(ctx && state && n <= kMaxQubits, "qsg_bulk_set_ampl");
  const uint64_t namps = uint64_t{1} << n;
  bulk_set_kernel<<<grid_for(ctx, namps, 256), 256, 0, ctx->stream>>>(
      reinterpret_cast<float2*>(state), namps, mask, bits, re, im,
      exclude != 0);
  QSG_LAUNCHED(ctx);
  return QSG_OK;
}

int qsg_add(qsg_ctx* ctx, const float* src, float* dest, unsigned n) {
  QSG_CHECK_ARG(ctx && src && dest && n <= kMaxQubits, "qsg_add");
  const uint64_t units = units_of(n);
  add_kernel<<<grid_for(ctx, units, 256), 256, 0, ctx->stream>>>(
      reinterpret_cast<const float4*>(src), reinterpret_cast<float4*>(dest),
      units);
  QSG_LAUNCHED(ctx);
  return QSG_OK;
}

int qsg_multiply(qsg_ctx* ctx, float a, float* state, unsigned n) {
  QSG_CHECK_ARG(ctx && state && n <= kMaxQubits, "qsg_multiply");
  const uint64_t units = units_of(n);
  multiply_kernel<<<grid_for(ctx, units, 256), 256, 0, ctx->stream>>>(
      reinterpret_cast<float4*>(state), units, a);
  QSG_LAUNCHED(ctx);
  return QSG_OK;
}

int qsg_inner_product(qsg_ctx* ctx, const float* s1, const float* s2,
                      unsigned n, double* out_re_im) {
  QSG_CHECK_ARG(ctx && s1 && s2 && out_re_im && n <= kMaxQubits,
                "qsg_inner_product");
  return reduce<2>(ctx, s1, s2, n, 0, 0, out_re_im);
}

int qsg_real_inner_product(qsg_ctx* ctx, const float* s1, const float* s2,
                           unsigned n, double* out) {
  QSG_CHECK_ARG(ctx && s1 && s2 && out && n <= kMaxQubits,
                "qsg_real_inner_product");
  double r[2];
  int rc = reduce<1>(ctx, s1, s2, n, 0, 0, r);
  *out = r[0];
  return rc;
}

int qsg_norm(qsg_ctx* ctx, const float* state, unsigned n, double* out) {
  QSG_CHECK_ARG(ctx && state && out && n <= kMaxQubits, "qsg_norm");
  double r[2];
  int rc = reduce<0>(ctx, state, nullptr, n, 0, 0, r);
  *out = r[0];
  return rc;
}

// ---------------------------------------------------------------------------
// Allocation-free Norm.  Same kernels and partition as qsg_norm, but the
// per-block partial sums and the result live in a fixed file-scope device
// array instead of the context's scratch (which the context grows with
// cudaMalloc, and whose pinned result slot comes from cudaMallocHost, on
// first use).  Every slot is written before it is read, so nothing in the
// array has to start at zero.

constexpr unsigned kNormNoAllocPartials = 4096;  // 64 KiB of double2
static __device__ __align__(256) double2
    g_norm_noalloc_scratch[kNormNoAllocPartials + 1];

constexpr int kNoAllocMaxDevices = 64;
static std::mutex g_norm_noalloc_mu;
static double2* g_norm_noalloc_ptr[kNoAllocMaxDevices] = {};

// Device address of the array for `device`, looked up once per device with
// that device current (qsg_norm_noalloc makes it current first).
static int norm_noalloc_scratch(int device, double2** out) {
  std::lock_guard<std::mutex> lock(g_norm_noalloc_mu);
  if (device < 0 || device >= kNoAllocMaxDevices) {
    set_error("qsg_norm_noalloc: device %d out of range", device);
    return QSG_ERR_INVALID;
  }
  if (g_norm_noalloc_ptr[device] == nullptr) {
    // The caller has made `device` current.
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_norm_noalloc_scratch);
    if (e != cudaSuccess)
      return cuda_status(e, "cudaGetSymbolAddress(norm scratch)");
    g_norm_noalloc_ptr[device] = static_cast<double2*>(p);
  }
  *out = g_norm_noalloc_ptr[device];
  return QSG_OK;
}

int qsg_norm_noalloc(qsg_ctx* ctx, const float* state, unsigned n,
                     double* out) {
  QSG_CHECK_ARG(ctx && state && out, "qsg_norm_noalloc: null argument");
  QSG_CHECK_ARG(n <= kMaxQubits, "qsg_norm_noalloc: %u qubits (maximum %u)",
                n, kMaxQubits);
  const uint64_t units = units_of(n);
  const unsigned grid = grid_for(ctx, units, kRedThreads * kRedUnroll);
  QSG_CHECK_ARG(grid <= kNormNoAllocPartials,
                "qsg_norm_noalloc: %u partial sums needed, the fixed scratch "
                "holds %u", grid, kNormNoAllocPartials);
  // The context's device is current for the whole call (the symbol lookup,
  // the launches on ctx->stream and the copy); the caller's device comes
  // back on every return path.
  int caller_device = -1;
  QSG_CUDA(cudaGetDevice(&caller_device));
  if (caller_device != ctx->device) QSG_CUDA(cudaSetDevice(ctx->device));
  struct Restore {
    int dev, ctx_dev;
    ~Restore() {
      if (dev != ctx_dev) cudaSetDevice(dev);
    }
  } restore{caller_device, ctx->device};
  double2* scratch = nullptr;
  int rc = norm_noalloc_scratch(ctx->device, &scratch);
  if (rc) return rc;
  reduce_kernel<0><<<grid, kRedThreads, 0, ctx->stream>>>(
      reinterpret_cast<const float4*>(state), nullptr, units, 0, 0, scratch);
  QSG_LAUNCHED(ctx);
  double2* result = scratch + kNormNoAllocPartials;
  final_reduce_kernel<<<1, 1024, 0, ctx->stream>>>(scratch, grid, result);
  QSG_LAUNCHED(ctx);
  double2 r = make_double2(0.0, 0.0);
  QSG_CUDA(cudaMemcpyAsync(&r, result, sizeof(double2),
                           cudaMemcpyDeviceToHost, ctx->stream));
  QSG_CUDA(cudaStreamSynchronize(ctx->stream));
  *out = r.x;
  return QSG_OK;
}

uint64_t qsg_num_chunks(unsigned n) { return num_chunks(n); }

int qsg_partial_norms(qsg_ctx* ctx, const float* state, unsigned n,
                      double* out) {
  QSG_CHECK_ARG(ctx && state && out && n <= kMaxQubits, "qsg_partial_norms");
  double *sums, *incl;
  int rc = chunk_prefix(ctx, state, n, 0, &sums, &incl, nullptr);
  if (rc) return rc;
  QSG_CUDA(cudaMemcpyAsync(out, sums, num_chunks(n) * sizeof(double),
                           cudaMemcpyDeviceToHost, ctx->stream));
  QSG_CUDA(cudaStreamSynchronize(ctx->stream));
  return QSG_OK;
}

int qsg_find_measured_bits(qsg_ctx* ctx, const float* state, unsigned n,
                           uint64_t m, double r, uint64_t mask,
                           uint64_t* out) {
  QSG_CHECK_ARG(ctx && state && out && n <= kMaxQubits,
                "qsg_find_measured_bits");
  QSG_CHECK_ARG(m < num_chunks(n), "qsg_find_measured_bits: chunk %llu out "
                "of range", (unsigned long long)m);
  void* p = nullptr;
  int rc = get_scratch(ctx, 64, &p);
  if (rc) return rc;
  uint64_t* d = static_cast<uint64_t*>(p);
  find_in_chunk_kernel<<<1, kScanThreads, 0, ctx->stream>>>(
      reinterpret_cast<const float2*>(state), chunk_bits(n), m, r, mask, d);
  QSG_LAUNCHED(ctx);
  void* h = nullptr;
  rc = get_hscratch(ctx, 8, &h);
  if (rc) return rc;
  QSG_CUDA(cudaMemcpyAsync(h, d, 8, cudaMemcpyDeviceToHost, ctx->stream));
  QSG_CUDA(cudaStreamSynchronize(ctx->stream));
  std::memcpy(out, h, 8);
  return QSG_OK;
}

// Samples for sorted values `vals`: uniforms in [0,1) scaled on the device
// by the CDF total (scaled), or thresholds on the running sum of |s|^2.
static int sample_impl(qsg_ctx* ctx, const float* state, unsigned n,
                       uint64_t num_samples, const double* vals, bool scaled,
                       uint64_t* out_bitstrings) {
  const double* sorted_u = vals;
  const uint64_t nc = num_chunks(n);
  const uint32_t cb = chunk_bits(n);
  const size_t ubytes = num_samples * sizeof(double);
  double *sums, *incl;
  void* extra = nullptr;
  int rc = chunk_prefix(ctx, state, n,
                        2 * ubytes + num_samples * 8 + num_samples * 4 + 64,
                        &sums, &incl, &extra);
  if (rc) return rc;
  double* du = static_cast<double*>(extra);
  double* dr = du + num_samples;
  uint64_t* dout = reinterpret_cast<uint64_t*>(dr + num_samples);
  uint32_t* dchunk = reinterpret_cast<uint32_t*>(dout + num_samples);
  if (scaled) {
    QSG_CUDA(cudaMemcpyAsync(du, sorted_u, ubytes, cudaMemcpyHostToDevice,
                             ctx->stream));
    scale_uniforms_kernel<<<grid_for(ctx, num_samples, 256), 256, 0,
                            ctx->stream>>>(du, num_samples, incl, nc, dr);
    QSG_LAUNCHED(ctx);
  } else {
    QSG_CUDA(cudaMemcpyAsync(dr, sorted_u, ubytes, cudaMemcpyHostToDevice,
                             ctx->stream));
  }
  sample_locate_kernel<<<grid_for(ctx, num_samples, 256), 256, 0,
                         ctx->stream>>>(incl, nc, dr, num_samples, dchunk);
  QSG_LAUNCHED(ctx);
  const unsigned grid = (unsigned)std::min<uint64_t>(num_samples, 1u << 20);
  sample_resolve_kernel<<<grid, kScanThreads, 0, ctx->stream>>>(
      reinterpret_cast<const float2*>(state), cb, nc, incl, dr, num_samples,
      dchunk, (uint64_t{1} << n) - 1, dout);
  QSG_LAUNCHED(ctx);
  QSG_CUDA(cudaMemcpyAsync(out_bitstrings, dout, num_samples * 8,
                           cudaMemcpyDeviceToHost, ctx->stream));
  QSG_CUDA(cudaStreamSynchronize(ctx->stream));
  return QSG_OK;
}

int qsg_sample_sorted(qsg_ctx* ctx, const float* state, unsigned n,
                      uint64_t num_samples, const double* sorted_u,
                      uint64_t* out_bitstrings) {
  QSG_CHECK_ARG(ctx && state && n <= kMaxQubits, "qsg_sample_sorted");
  if (num_samples == 0) return QSG_OK;
  QSG_CHECK_ARG(sorted_u && out_bitstrings, "qsg_sample_sorted: null");
  return sample_impl(ctx, state, n, num_samples, sorted_u, true,
                     out_bitstrings);
}

int qsg_sample_thresholds(qsg_ctx* ctx, const float* state, unsigned n,
                          uint64_t num_samples, const double* sorted_r,
                          uint64_t* out_bitstrings) {
  QSG_CHECK_ARG(ctx && state && n <= kMaxQubits, "qsg_sample_thresholds");
  if (num_samples == 0) return QSG_OK;
  QSG_CHECK_ARG(sorted_r && out_bitstrings, "qsg_sample_thresholds: null");
  return sample_impl(ctx, state, n, num_samples, sorted_r, false,
                     out_bitstrings);
}

int qsg_sample(qsg_ctx* ctx, const float* state, unsigned n,
               uint64_t num_samples, unsigned seed, uint64_t* out_bitstrings) {
  QSG_CHECK_ARG(ctx && state && n <= kMaxQubits, "qsg_sample");
  if (num_samples == 0) return QSG_OK;
  std::vector<double> u(num_samples);
  std::mt19937 g(seed);
  for (auto& x : u) x = canonical_u01(g);
  std::sort(u.begin(), u.end());
  return qsg_sample_sorted(ctx, state, n, num_samples, u.data(),
                           out_bitstrings);
}

int qsg_collapse(qsg_ctx* ctx, float* state, unsigned n, uint64_t mask,
                 uint64_t bits) {
  QSG_CHECK_ARG(ctx && state && n <= kMaxQubits, "qsg_collapse");
  double r[2];
  int rc = reduce<0>(ctx, state, nullptr, n, mask, bits, r);
  if (rc) return rc;
  if (mask == 0) {
    // The reference's masked reduce degenerates to the plain norm.
  }
  const float renorm = float(1.0 / std::sqrt(r[0]));
  const uint64_t units = units_of(n);
  collapse_kernel<<<grid_for(ctx, units, 256), 256, 0, ctx->stream>>>(
      reinterpret_cast<float4*>(state), units, mask, bits, renorm);
  QSG_LAUNCHED(ctx);
  return QSG_OK;
}

int qsg_measure(qsg_ctx* ctx, float* state, unsigned n, uint64_t mask,
                double u, int collapse, uint64_t* out_bits) {
  QSG_CHECK_ARG(ctx && state && out_bits && n <= kMaxQubits, "qsg_measure");
  QSG_CHECK_ARG(u >= 0.0 && u < 1.0, "qsg_measure: u must be in [0,1)");
  double *sums, *incl;
  void* extra = nullptr;
  int rc = chunk_prefix(ctx, state, n, 64, &sums, &incl, &extra);
  if (rc) return rc;
  uint64_t* d = static_cast<uint64_t*>(extra);
  measure_kernel<<<1, kScanThreads, 0, ctx->stream>>>(
      reinterpret_cast<const float2*>(state), chunk_bits(n), num_chunks(n),
      incl, u, mask, d);
  QSG_LAUNCHED(ctx);
  void* h = nullptr;
  rc = get_hscratch(ctx, 8, &h);
  if (rc) return rc;
  QSG_CUDA(cudaMemcpyAsync(h, d, 8, cudaMemcpyDeviceToHost, ctx->stream));
  QSG_CUDA(cudaStreamSynchronize(ctx->stream));
  std::memcpy(out_bits, h, 8);
  if (collapse) return qsg_collapse(ctx, state, n, mask, *out_bits);
  return QSG_OK;
}

}  // extern "C"
