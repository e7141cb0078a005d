// Persistent kernel for packed trajectory batches (see batch_dev.h).
//
// Each CTA (128 threads) takes the next trajectory from a global queue
// (items are sorted largest first on the host), runs its whole program on
// the state it owns (the item's own buffer or the CTA's slot), and takes the
// next one; one launch serves the batch.  Inside a trajectory:
//
//  * GATE: the fused k-qubit matrix (k <= 4), optionally controlled, applied
//    by the same shared-memory tile pass as the single-gate kernel
//    (tile_pass in gate_tile.cuh, geometry planned on the host), walking
//    every tile of the state with a cp.async pipeline whose depth fills a
//    32 KiB tile budget (2 to 8 tiles in flight).  Matrices of k <= 2 sit in
//    registers, larger ones column-major in shared memory.
//  * CHANNEL: the device-side Kraus choice of lib/qtrajectory.h:331-380: one
//    read pass sums |psi_i|^2 by the values of the channel qubits (FP32 over
//    a thread's amplitudes of one step, FP64 across steps and threads); the
//    norm and every <K^dagger K> follow (K^dagger K is diagonal), one thread
//    restates the reference's second sampling loop, and the chosen operator
//    times (float)(1/sqrt(norm)) is applied with a tile pass.
//  * NORMALIZE: norm pass, then the state times (float)(1/sqrt(norm)).
//
// CTAs never wait on one another: the only inter-CTA communication is the
// atomic queue counter.

#include <cmath>
#include <cstring>
#include <map>
#include <tuple>
#include <vector>

#include "batch_dev.h"
#include "common.cuh"
#include "gate_tile.cuh"

namespace qsg {

namespace {

constexpr int kBatchThreads = kTileThreads;  // 128

// One entry of the geometry table.
struct BatchGeom {
  TileGeom g;
  uint32_t k;
  uint32_t pair;
};

struct BatchShared {
  BatchGeom geom;                   // geometry of the current op
  float2 smat[16 * 16];             // column-major matrix (k >= 3)
  float2 cmat[16];                  // chosen channel operator (scaled)
  double red[kBatchThreads / 32][4];
  double bins[4];
  float scale;
  int chosen;
  uint32_t item;
};

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Sums |psi_i|^2 by the values of up to two qubits into sm.bins (FP64).
__device__ void cta_bins(const float4* __restrict__ s4, uint64_t units,
                         unsigned nq, unsigned q0, unsigned q1,
                         BatchShared& sm) {
  double acc[4] = {0, 0, 0, 0};
  constexpr int U = 8;
  const uint64_t stride = uint64_t(U) * blockDim.x;
  for (uint64_t i0 = threadIdx.x; i0 < units; i0 += stride) {
    float4 x[U];
#pragma unroll
    for (int j = 0; j < U; ++j) {
      const uint64_t i = i0 + uint64_t(j) * blockDim.x;
      x[j] = i < units ? s4[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    float f[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int j = 0; j < U; ++j) {
      const uint64_t i = i0 + uint64_t(j) * blockDim.x;
      const float p0 = x[j].x * x[j].x + x[j].y * x[j].y;
      const float p1 = x[j].z * x[j].z + x[j].w * x[j].w;
      unsigned c0 = 0, c1 = 0;
      if (nq > 0) {
        c0 = unsigned((2 * i) >> q0) & 1u;
        c1 = unsigned((2 * i + 1) >> q0) & 1u;
      }
      if (nq > 1) {
        c0 |= (unsigned((2 * i) >> q1) & 1u) << 1;
        c1 |= (unsigned((2 * i + 1) >> q1) & 1u) << 1;
      }
#pragma unroll
      for (unsigned b = 0; b < 4; ++b)
        f[b] += (c0 == b ? p0 : 0.f) + (c1 == b ? p1 : 0.f);
    }
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[b] += f[b];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    double v = acc[b];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) sm.red[warp][b] = v;
  }
  __syncthreads();
  if (threadIdx.x < 4) {
    double v = 0;
    for (unsigned w = 0; w < blockDim.x / 32; ++w) v += sm.red[w][threadIdx.x];
    sm.bins[threadIdx.x] = v;
  }
  __syncthreads();
}

// The second sampling loop of lib/qtrajectory.h:351-380 with probabilities
// from the channel sums (one thread).  Writes the chosen operator times
// (float)(1/sqrt(norm)) into sm.cmat (or only sm.scale when none is chosen).
__device__ void choose(const TrajChannelDev* ch, double cp0, double r,
                       BatchShared& sm) {
  const double norm = sm.bins[0] + sm.bins[1] + sm.bins[2] + sm.bins[3];
  const float a = float(1.0 / sqrt(norm));
  sm.scale = a;
  const unsigned d = 1u << ch->nq;
  double cp = cp0, max_prob = 0;
  int max_index = 0, chosen = -1;
  for (int i = 0; i < ch->nkops; ++i) {
    if (ch->unitary[i]) continue;
    double ev = 0;
    for (unsigned b = 0; b < d; ++b) ev += double(ch->kd[i][b]) * sm.bins[b];
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
  sm.chosen = chosen;
  if (chosen >= 0) {
    for (unsigned j = 0; j < d * d; ++j)
      sm.cmat[j] = make_float2(ch->mat[chosen][2 * j] * a,
                               ch->mat[chosen][2 * j + 1] * a);
  }
}

__device__ void cta_scale(float4* __restrict__ s4, uint64_t units, float a) {
  for (uint64_t i = threadIdx.x; i < units; i += blockDim.x) {
    const float4 x = s4[i];
    s4[i] = make_float4(x.x * a, x.y * a, x.z * a, x.w * a);
  }
}

// Pipeline depth of the tile pass: as many tiles as fit the tile budget
// BUDGET (bytes of tile buffers per CTA), 2..8.
template <int K, bool PAIR, int BUDGET>
struct BatchStages {
  static constexpr int kTile = TileShape<K, PAIR>::UNITS * 16;
  static constexpr int kFit = BUDGET / kTile;
  static constexpr int value = kFit > 8 ? 8 : (kFit < 2 ? 2 : kFit);
};

// One gate pass over every tile of the state.  `mat` points at the
// row-major interleaved matrix (global or shared memory); k >= 3 matrices
// were staged column-major into sm.smat by the caller.
template <int K, bool PAIR, int BUDGET>
__device__ __forceinline__ void batch_gate_pass(float4* st, BatchShared& sm,
                                             float4* tiles, const float* mat) {
  static_assert(TileShape<K, PAIR>::UNITS * 16 * BatchStages<K, PAIR, BUDGET>::value <=
                    BUDGET,
                "tile budget");
  double er = 0, ei = 0;
  if constexpr (K >= 3) {
    tile_pass<K, PAIR, 0, 1, BatchStages<K, PAIR, BUDGET>::value>(
        st, sm.geom.g, NoMat{}, sm.smat, tiles, 0, 1, er, ei);
  } else {
    const RegMat<K> m(mat);
    tile_pass<K, PAIR, 0, 0, BatchStages<K, PAIR, BUDGET>::value>(
        st, sm.geom.g, m, nullptr, tiles, 0, 1, er, ei);
  }
}

// Copies geometry entry `gi` into shared memory and, for k >= 3, the matrix
// column-major into sm.smat; then runs the pass.
template <int BUDGET>
__device__ void batch_gate(float4* st, BatchShared& sm, float4* tiles,
                           const BatchGeom* __restrict__ geoms, uint32_t gi,
                           const float* mat) {
  const uint32_t* src = reinterpret_cast<const uint32_t*>(geoms + gi);
  uint32_t* dst = reinterpret_cast<uint32_t*>(&sm.geom);
  for (uint32_t i = threadIdx.x; i < sizeof(BatchGeom) / 4; i += blockDim.x)
    dst[i] = src[i];
  __syncthreads();
  const uint32_t k = sm.geom.k;
  const bool pair = sm.geom.pair != 0;
  if (k >= 3) {
    const uint32_t d = 1u << k;
    for (uint32_t i = threadIdx.x; i < d * d; i += blockDim.x) {
      const uint32_t r = i / d, c = i % d;
      sm.smat[c * d + r] = make_float2(mat[2 * i], mat[2 * i + 1]);
    }
    __syncthreads();
  }
  switch (k * 2 + (pair ? 1 : 0)) {
    case 2: batch_gate_pass<1, false, BUDGET>(st, sm, tiles, mat); break;
    case 3: batch_gate_pass<1, true, BUDGET>(st, sm, tiles, mat); break;
    case 4: batch_gate_pass<2, false, BUDGET>(st, sm, tiles, mat); break;
    case 5: batch_gate_pass<2, true, BUDGET>(st, sm, tiles, mat); break;
    case 6: batch_gate_pass<3, false, BUDGET>(st, sm, tiles, mat); break;
    case 7: batch_gate_pass<3, true, BUDGET>(st, sm, tiles, mat); break;
    case 8: batch_gate_pass<4, false, BUDGET>(st, sm, tiles, mat); break;
    case 9: batch_gate_pass<4, true, BUDGET>(st, sm, tiles, mat); break;
    default: break;
  }
}

template <int BUDGET>
__global__ void __launch_bounds__(kBatchThreads, BUDGET <= 32768 ? 4 : 2)
    batch_traj_kernel(const BatchLaunch l, const BatchItemDev* __restrict__ items,
                      uint32_t num_items, const BatchOp* __restrict__ ops,
                      uint32_t* __restrict__ log,
                      unsigned long long* __restrict__ times,
                      uint32_t* __restrict__ counter, int* __restrict__ error) {
  __shared__ BatchShared sm;
  extern __shared__ float4 tiles[];
  const BatchGeom* geoms = static_cast<const BatchGeom*>(l.geoms);
  float* const slot = l.slots ? l.slots + blockIdx.x * l.slot_floats : nullptr;
  for (;;) {
    if (threadIdx.x == 0) sm.item = atomicAdd(counter, 1u);
    __syncthreads();
    const uint32_t it = sm.item;
    __syncthreads();
    if (it >= num_items) break;
    const BatchItemDev item = items[it];
    unsigned long long t0 = 0;
    if (threadIdx.x == 0) t0 = global_ns();
    float* const st = item.state ? item.state : slot;
    float4* const s4 = reinterpret_cast<float4*>(st);
    const unsigned n = item.n;
    const uint64_t units = uint64_t{1} << (n - 1);
    uint32_t log_slot = item.log_begin;
    for (uint32_t oi = 0; oi < item.num_ops; ++oi) {
      const BatchOp& op = ops[item.op_begin + oi];
      if (op.kind == kBatchSetZero) {
        for (uint64_t i = threadIdx.x; i < units; i += blockDim.x)
          s4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (threadIdx.x == 0) st[0] = 1.f;
      } else if (op.kind == kBatchGate) {
        batch_gate<BUDGET>(s4, sm, tiles, geoms, op.geom, op.mat);
      } else if (op.kind == kBatchChannel) {
        const TrajChannelDev* ch = op.ch;
        const unsigned nq = unsigned(ch->nq);
        cta_bins(s4, units, nq, ch->q[0], nq > 1 ? ch->q[1] : 0, sm);
        if (threadIdx.x == 0) {
          choose(ch, op.cp0, op.r, sm);
          log[log_slot] = sm.chosen < 0 ? 0xffffffffu : uint32_t(sm.chosen);
        }
        ++log_slot;
        __syncthreads();
        if (sm.chosen < 0) {
          cta_scale(s4, units, sm.scale);
        } else {
          batch_gate<BUDGET>(s4, sm, tiles, geoms, op.geom,
                     reinterpret_cast<const float*>(sm.cmat));
        }
      } else if (op.kind == kBatchNormalize) {
        cta_bins(s4, units, 0, 0, 0, sm);
        const double norm = sm.bins[0] + sm.bins[1] + sm.bins[2] + sm.bins[3];
        cta_scale(s4, units, float(1.0 / sqrt(norm)));
      } else if (threadIdx.x == 0) {
        atomicExch(error, 2);
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      times[2 * uint64_t(it)] = t0;
      times[2 * uint64_t(it) + 1] = global_ns();
    }
  }
}

}  // namespace

int batch_plan_geometries(const BatchItemDev* items, size_t num_items,
                          BatchOp* ops, std::vector<unsigned char>* table) {
  using Key = std::tuple<uint32_t, uint64_t, uint64_t, uint64_t>;
  std::map<Key, uint32_t> index;
  std::vector<BatchGeom> entries;
  for (size_t i = 0; i < num_items; ++i) {
    const BatchItemDev& it = items[i];
    for (uint32_t j = 0; j < it.num_ops; ++j) {
      BatchOp& op = ops[it.op_begin + j];
      if (op.kind != kBatchGate && op.kind != kBatchChannel) continue;
      const uint64_t cmask = op.kind == kBatchGate ? op.cmask : 0;
      const uint64_t cvals = op.kind == kBatchGate ? op.cvals : 0;
      const Key key{it.n, op.tmask, cmask, cvals};
      auto f = index.find(key);
      if (f != index.end()) {
        op.geom = f->second;
        continue;
      }
      unsigned qs[64], cqs[64], k = 0, c = 0;
      uint64_t cv = 0;
      for (unsigned q = 0; q < 64; ++q) {
        if ((op.tmask >> q) & 1) qs[k++] = q;
        if ((cmask >> q) & 1) {
          if ((cvals >> q) & 1) cv |= uint64_t{1} << c;
          cqs[c++] = q;
        }
      }
      if (k < 1 || k > kBatchMaxK || c > kBatchMaxControls ||
          k + c > it.n || (op.tmask & cmask) != 0 ||
          (it.n < 64 && ((op.tmask | cmask) >> it.n) != 0)) {
        set_error("packed batch: bad gate qubits");
        return QSG_ERR_INVALID;
      }
      BatchGeom e;
      std::memset(&e, 0, sizeof(e));
      e.k = k;
      e.pair = qs[0] != 0;
      const int log_items = k >= 4 ? 7 - int(k - 3) : 7;
      if (!plan_tile(it.n, qs, k, cqs, c, cv, e.pair != 0, log_items, e.g)) {
        set_error("packed batch: tile planning failed (n=%u, k=%u)", it.n, k);
        return QSG_ERR_INVALID;
      }
      const uint32_t id = uint32_t(entries.size());
      entries.push_back(e);
      index.emplace(key, id);
      op.geom = id;
    }
  }
  if (entries.empty()) entries.emplace_back();
  table->resize(entries.size() * sizeof(BatchGeom));
  std::memcpy(table->data(), entries.data(), table->size());
  return QSG_OK;
}

template <int BUDGET>
static int batch_setup() {
  static int done = 0;
  if (!done) {
    QSG_CUDA(cudaFuncSetAttribute(batch_traj_kernel<BUDGET>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  BUDGET));
    done = 1;
  }
  return QSG_OK;
}

template <int BUDGET>
static int launch_budget(cudaStream_t s, const BatchLaunch& l,
                         const BatchItemDev* items, uint32_t num_items,
                         const BatchOp* ops, uint32_t* log,
                         unsigned long long* times, uint32_t* counter,
                         int* error) {
  int rc = batch_setup<BUDGET>();
  if (rc) return rc;
  batch_traj_kernel<BUDGET><<<l.ctas, l.threads, BUDGET, s>>>(
      l, items, num_items, ops, log, times, counter, error);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_status(e, "packed batch launch");
  return QSG_OK;
}

int batch_launch(void* stream, const BatchLaunch& l, const BatchItemDev* items,
                 uint32_t num_items, const BatchOp* ops, uint32_t* log,
                 unsigned long long* times, uint32_t* counter, int* error) {
  if (l.threads != unsigned(kBatchThreads) || l.ctas == 0 || !l.geoms) {
    set_error("packed batch: bad launch shape");
    return QSG_ERR_INVALID;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  switch (l.tile_kib) {
    case 32: return launch_budget<32768>(s, l, items, num_items, ops, log, times, counter, error);
    case 64: return launch_budget<65536>(s, l, items, num_items, ops, log, times, counter, error);
    case 96: return launch_budget<98304>(s, l, items, num_items, ops, log, times, counter, error);
    default: break;
  }
  set_error("packed batch: tile budget must be 32, 64 or 96 KiB");
  return QSG_ERR_INVALID;
}

int batch_max_ctas_per_sm(unsigned threads, unsigned tile_kib, int* out) {
  int rc = QSG_OK;
  const void* f = nullptr;
  switch (tile_kib) {
    case 32: rc = batch_setup<32768>(); f = (const void*)batch_traj_kernel<32768>; break;
    case 64: rc = batch_setup<65536>(); f = (const void*)batch_traj_kernel<65536>; break;
    case 96: rc = batch_setup<98304>(); f = (const void*)batch_traj_kernel<98304>; break;
    default:
      set_error("packed batch: tile budget must be 32, 64 or 96 KiB");
      return QSG_ERR_INVALID;
  }
  if (rc) return rc;
  QSG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      out, f, int(threads), size_t(tile_kib) * 1024));
  return QSG_OK;
}

}  // namespace qsg
