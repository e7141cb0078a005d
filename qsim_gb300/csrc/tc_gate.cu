// Tensor-core (tcgen05) application of fused gates, k <= 6 target qubits.
//
// The reference applies every fused gate on CUDA cores
// (ApplyGateH/L_Kernel, lib/simulator_cuda_kernels.h:30-202); for k >= 5 a
// pass there is bound by FP32 issue.  Here a gate is a real GEMM on the
// 5th-generation tensor cores:
//
//   * A gate on fewer than 6 qubits is padded to 6 targets with the identity
//     on the lowest free qubits, so one kernel shape serves k <= 6.
//   * Real form: out = A_real * in with A_real the 128 x 128 matrix
//     [[Mr, -Mi], [Mi, Mr]] interleaved by (member, re/im), and `in` the
//     tile's 64 groups x 128 real components.  One CTA tile = 64 groups x 64
//     members = 4096 amplitudes; D (128 x 64 FP32) lives in tensor memory.
//   * Split TF32: A = A_hi + A_lo and B = B_hi + B_lo with every part
//     pre-rounded to TF32; D = A_hi B_hi + A_hi B_lo + A_lo B_hi (3 x 16
//     MMAs of M=128, N=64, K=8), FP32 accumulation.  The dropped A_lo B_lo
//     term and the rounding of the lo parts leave ~2^-21 relative error per
//     product, the FP32 level of the CUDA-core path.
//   * Operands sit in shared memory in the canonical no-swizzle K-major
//     layout (8-row x 16-byte core matrices; LBO = 128 B between core
//     matrices along K, SBO = 4 KiB between 8-row blocks).  The gate's two
//     parts (128 KiB) are copied once per CTA; amplitudes arrive with 8-byte
//     cp.async straight into their (group, member) slots, double buffered.
//   * One thread issues the MMAs and commits them to an mbarrier; every wait
//     is bounded and sets an error flag instead of hanging.  The epilogue
//     reads D with tcgen05.ld, pairs re/im lanes with a shuffle and stores
//     amplitudes to HBM.

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace qsg {

namespace tc {

constexpr int kThreads = 128;
constexpr int kK = 6;                  // targets per tensor-core gate
constexpr int kD = 1 << kK;            // members per group (64)
constexpr int kReal = 2 * kD;          // real dimension (128) = M = K
constexpr int kGroups = 64;            // N
constexpr int kTileBits = 12;          // 64 groups x 64 members
constexpr int kTileAmps = 1 << kTileBits;
constexpr uint32_t kABytes = kReal * kReal * 4;        // 64 KiB per part
constexpr uint32_t kBBytes = kGroups * kReal * 4;      // 32 KiB per buffer
constexpr uint32_t kLBO = 128;                          // K-adjacent cores
constexpr uint32_t kSBOA = (kReal / 4) * 128;           // 4 KiB
constexpr uint32_t kSBOB = (kReal / 4) * 128;           // 4 KiB
constexpr uint32_t kTmemCols = 128;   // D uses 64; headroom
constexpr long long kWaitCycles = 4000000000LL;         // ~2 s at 2 GHz

// Shared-memory map (bytes).
constexpr uint32_t kOffAhi = 0;
constexpr uint32_t kOffAlo = kOffAhi + kABytes;
constexpr uint32_t kOffB0 = kOffAlo + kABytes;
constexpr uint32_t kOffB1 = kOffB0 + kBBytes;
constexpr uint32_t kOffBlo = kOffB1 + kBBytes;
constexpr uint32_t kOffTabLoadS = kOffBlo + kBBytes;     // 32 x u32
constexpr uint32_t kOffTabLoadG = kOffTabLoadS + 128;    // 32 x u64
constexpr uint32_t kOffTabGroup = kOffTabLoadG + 256;    // 64 x u64
constexpr uint32_t kOffBar = kOffTabGroup + 512;         // mbarrier
constexpr uint32_t kOffTmem = kOffBar + 16;              // tmem address
constexpr uint32_t kSmemBytes = kOffTmem + 16;

static_assert(kSmemBytes <= 232448, "shared memory budget");

// Byte offset of real element (row, k) in a K-major no-swizzle operand with
// rows of `kReal` K-elements.
__host__ __device__ constexpr uint32_t kmajor_off(uint32_t row, uint32_t k,
                                                  uint32_t sbo) {
  return (row / 8) * sbo + (k / 4) * kLBO + (row % 8) * 16 + (k % 4) * 4;
}

// Tile geometry of a 6-target gate on n >= 12 qubits.
struct TcGeom {
  uint64_t num_tiles;
  uint64_t bitpos_state[kTileBits];  // state bit of tile bit j
  uint32_t ins_pos[kMaxQubits];      // state bits skipped by the tile index
  uint32_t n_ins;
  uint32_t b;                        // run bits
  uint32_t tile_is_target[kTileBits];
  uint32_t target_slot[kTileBits];   // member bit of a target tile bit
  uint32_t group_slot[kTileBits];    // group bit of a non-target tile bit
};

struct TcArgs {
  TcGeom g;
  const uint4* operands;  // A_hi | A_lo smem images (kABytes each)
  int* error;             // set on a timed-out wait
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t make_desc(uint32_t saddr, uint32_t lbo,
                                              uint32_t sbo) {
  uint64_t d = 0;
  d |= uint64_t((saddr >> 4) & 0x3FFF);
  d |= uint64_t((lbo >> 4) & 0x3FFF) << 16;
  d |= uint64_t((sbo >> 4) & 0x3FFF) << 32;
  d |= uint64_t(1) << 46;  // descriptor version for tcgen05
  // base offset 0, relative LBO mode, no swizzle (bits 61-63 = 0)
  return d;
}

// Instruction descriptor: D = F32, A = B = TF32, both K-major, N = 64,
// M = 128.
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) |
                            (uint32_t(kGroups >> 3) << 17) |
                            (uint32_t(kReal >> 4) << 24);

__device__ __forceinline__ void cp_async8(uint32_t saddr, const void* g) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(saddr),
               "l"(g)
               : "memory");
}
__device__ __forceinline__ void cp_async16(uint32_t saddr, const void* g) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(saddr),
               "l"(g)
               : "memory");
}
__device__ __forceinline__ void cp_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

__device__ __forceinline__ float tf32_round(float x) {
  // Round to nearest (ties away) at mantissa bit 13: the result is exactly
  // representable in TF32, so the MMA reads it unchanged.
  uint32_t u = __float_as_uint(x);
  u = (u + 0x1000u) & 0xFFFFE000u;
  return __uint_as_float(u);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)),
               "r"(count)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n"
      " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a, uint64_t b,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          d_tmem),
      "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 "
      "[%0];\n" ::"r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, "
      "[%32];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]),
        "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]),
        "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
        "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
        "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
}

__device__ __forceinline__ void tmem_wait_ld() {
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
}
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

// Tile index e (12 bits) -> state offset: OR of the state bits of e's bits.
__device__ __forceinline__ uint64_t tile_goff(uint32_t e, const TcGeom& g) {
  uint64_t o = 0;
#pragma unroll
  for (int j = 0; j < kTileBits; ++j)
    if ((e >> j) & 1) o |= uint64_t{1} << g.bitpos_state[j];
  return o;
}

// Tile index e -> byte offset of its 8-byte amplitude in a B buffer.
__device__ __forceinline__ uint32_t tile_soff(uint32_t e, const TcGeom& g) {
  uint32_t n = 0, m = 0;
#pragma unroll
  for (int j = 0; j < kTileBits; ++j) {
    const uint32_t bit = (e >> j) & 1;
    if (g.tile_is_target[j]) m |= bit << g.target_slot[j];
    else n |= bit << g.group_slot[j];
  }
  return kmajor_off(n, 2 * m, kSBOB);
}

__device__ __forceinline__ uint64_t expand_outer_tc(uint64_t t,
                                                    const TcGeom& g) {
  uint64_t x = t << g.b;
  for (uint32_t i = 0; i < g.n_ins; ++i) {
    const uint32_t p = g.ins_pos[i];
    const uint64_t lo = x & ((uint64_t{1} << p) - 1);
    x = lo | ((x ^ lo) << 1);
  }
  return x;
}

__global__ void __launch_bounds__(kThreads, 1)
    tc_gate_kernel(float2* __restrict__ st, const __grid_constant__ TcArgs a) {
  extern __shared__ __align__(1024) unsigned char smem[];
  const TcGeom& g = a.g;
  const uint32_t tid = threadIdx.x;
  const uint32_t warp = tid / 32, lane = tid % 32;
  uint32_t* tab_ls = reinterpret_cast<uint32_t*>(smem + kOffTabLoadS);
  uint64_t* tab_lg = reinterpret_cast<uint64_t*>(smem + kOffTabLoadG);
  uint64_t* tab_grp = reinterpret_cast<uint64_t*>(smem + kOffTabGroup);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + kOffBar);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + kOffTmem);
  const uint32_t sbase = smem_u32(smem);

  // Gate operands: one copy per CTA.
  for (uint32_t i = tid; i < 2 * kABytes / 16; i += kThreads)
    cp_async16(sbase + kOffAhi + 16 * i, a.operands + i);
  cp_commit();

  // Address tables.  Tile index e = lo7 | (j << 7): offsets are bitwise
  // linear in e, so per-thread bases OR per-j table entries.
  if (tid < 32) {
    tab_ls[tid] = tile_soff(tid << 7, g);
    tab_lg[tid] = tile_goff(tid << 7, g);
  }
  if (tid < kGroups) {
    uint32_t e = 0, gi = tid;
    for (int j = 0; j < kTileBits; ++j) {
      if (!g.tile_is_target[j]) {
        e |= (gi & 1) << j;
        gi >>= 1;
      }
    }
    tab_grp[tid] = tile_goff(e, g);
  }
  if (tid == 0) {
    mbar_init(bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 0) {
    asm volatile(
        "tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
            smem_u32(tmem_slot)),
        "r"(kTmemCols)
        : "memory");
    asm volatile(
        "tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::
            : "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  const uint32_t my_ls = tile_soff(tid, g);
  const uint64_t my_lg = tile_goff(tid, g);

  // Epilogue role: TMEM lane = 32*warp + lane = output row 2r + part.
  const uint32_t row = 32 * warp + lane;
  const uint32_t r_member = row / 2;
  uint64_t member_goff = 0;
  {
    uint32_t e = 0, mi = r_member;
    for (int j = 0; j < kTileBits; ++j) {
      if (g.tile_is_target[j]) {
        e |= ((mi >> g.target_slot[j]) & 1) << j;
      }
    }
    member_goff = tile_goff(e, g);
  }

  auto issue_loads = [&](uint64_t t, uint32_t boff) {
    if (t < g.num_tiles) {
      const uint64_t base = expand_outer_tc(t, g);
      const float2* gp = st + (base | my_lg);
#pragma unroll 8
      for (int j = 0; j < kTileAmps / kThreads; ++j) {
        cp_async8(sbase + boff + (my_ls | tab_ls[j]), gp + tab_lg[j]);
      }
    }
    cp_commit();
  };

  uint64_t t = blockIdx.x;
  issue_loads(t, kOffB0);
  issue_loads(t + gridDim.x, kOffB1);
  cp_wait<2>();  // the operand group is complete
  uint32_t phase = 0;
  bool failed = false;

  for (int stage = 0; t < g.num_tiles; t += gridDim.x, stage ^= 1) {
    const uint32_t boff = stage ? kOffB1 : kOffB0;
    cp_wait<1>();
    __syncthreads();
    // Split the tile: hi (in place) and lo parts, both TF32-exact.
    {
      float4* hb = reinterpret_cast<float4*>(smem + boff);
      float4* lb = reinterpret_cast<float4*>(smem + kOffBlo);
      for (uint32_t i = tid; i < kBBytes / 16; i += kThreads) {
        float4 x = hb[i], h, l;
        h.x = tf32_round(x.x); l.x = tf32_round(x.x - h.x);
        h.y = tf32_round(x.y); l.y = tf32_round(x.y - h.y);
        h.z = tf32_round(x.z); l.z = tf32_round(x.z - h.z);
        h.w = tf32_round(x.w); l.w = tf32_round(x.w - h.w);
        hb[i] = h;
        lb[i] = l;
      }
    }
    fence_async_smem();
    __syncthreads();

    if (tid == 0) {
      tc_fence_after();
      const uint32_t ahi = sbase + kOffAhi, alo = sbase + kOffAlo;
      const uint32_t bhi = sbase + boff, blo = sbase + kOffBlo;
      uint32_t acc = 0;
#pragma unroll 1
      for (int kk = 0; kk < kReal / 8; ++kk) {
        const uint32_t ko = kk * 2 * kLBO;  // two core matrices per K=8
        mma_tf32(tmem, make_desc(ahi + ko, kLBO, kSBOA),
                 make_desc(bhi + ko, kLBO, kSBOB), acc);
        acc = 1;
        mma_tf32(tmem, make_desc(ahi + ko, kLBO, kSBOA),
                 make_desc(blo + ko, kLBO, kSBOB), 1);
        mma_tf32(tmem, make_desc(alo + ko, kLBO, kSBOA),
                 make_desc(bhi + ko, kLBO, kSBOB), 1);
      }
      mma_commit(bar);
    }
    // Bounded wait for the MMAs of this tile.
    {
      const long long t0 = clock64();
      while (!mbar_try_wait(bar, phase)) {
        if (clock64() - t0 > kWaitCycles) {
          failed = true;
          break;
        }
      }
      phase ^= 1;
    }
    if (__syncthreads_or(failed)) {
      if (tid == 0) atomicExch(a.error, 1);
      failed = true;
      break;
    }
    tc_fence_after();

    // Epilogue: row `row` of D holds output component (r_member, row & 1)
    // of the 64 groups.  Even lanes store groups 0..31, odd lanes 32..63.
    const uint64_t base = expand_outer_tc(t, g);
    uint32_t v0[32], v1[32];
    const uint32_t taddr = tmem + ((32 * warp) << 16);
    tmem_ld32(taddr, v0);
    tmem_ld32(taddr + 32, v1);
    tmem_wait_ld();
    const bool odd = lane & 1;
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      // Even lane sends its value of columns 32..63, odd lane of 0..31.
      const uint32_t send = odd ? v0[j] : v1[j];
      const uint32_t recv = __shfl_xor_sync(0xffffffffu, send, 1);
      const uint32_t mine = odd ? v1[j] : v0[j];
      const float re = __uint_as_float(odd ? recv : mine);
      const float im = __uint_as_float(odd ? mine : recv);
      const uint32_t grp = odd ? 32 + j : j;
      st[base | member_goff | tab_grp[grp]] = make_float2(re, im);
    }
    tc_fence_before();
    __syncthreads();
    issue_loads(t + 2 * uint64_t(gridDim.x), boff);
  }
  cp_wait<0>();
  if (failed) {
    // Give the MMAs of the abandoned tile one more bounded wait before the
    // tensor memory they write is released.
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, phase ^ 1) && clock64() - t0 < kWaitCycles) {
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(
                     tmem),
                 "r"(kTmemCols)
                 : "memory");
  }
}

// Pads (qs, m32) to 6 targets with the identity on the lowest free qubits.
static void pad_to_6(unsigned n, const unsigned* qs, unsigned k,
                     const float* m32, unsigned* qs6, std::vector<float>& m6) {
  std::vector<unsigned> all(qs, qs + k);
  for (unsigned q = 0; all.size() < 6 && q < n; ++q)
    if (std::find(all.begin(), all.end(), q) == all.end()) all.push_back(q);
  std::sort(all.begin(), all.end());
  // pos[j]: bit of original target j inside the 6-bit index.
  unsigned pos[6];
  uint32_t tmask = 0;
  for (unsigned j = 0; j < k; ++j) {
    pos[j] = unsigned(std::find(all.begin(), all.end(), qs[j]) - all.begin());
    tmask |= 1u << pos[j];
  }
  auto sub = [&](unsigned i) {
    unsigned r = 0;
    for (unsigned j = 0; j < k; ++j) r |= ((i >> pos[j]) & 1) << j;
    return r;
  };
  const unsigned d = 1u << k;
  m6.assign(2 * kD * kD, 0.f);
  for (unsigned r = 0; r < kD; ++r)
    for (unsigned c = 0; c < kD; ++c) {
      if ((r & ~tmask) != (c & ~tmask)) continue;
      const unsigned rs = sub(r), cs = sub(c);
      m6[2 * (r * kD + c)] = m32[2 * (rs * d + cs)];
      m6[2 * (r * kD + c) + 1] = m32[2 * (rs * d + cs) + 1];
    }
  for (unsigned j = 0; j < 6; ++j) qs6[j] = all[j];
}

static float tf32_host(float x) {
  uint32_t u;
  std::memcpy(&u, &x, 4);
  u = (u + 0x1000u) & 0xFFFFE000u;
  float r;
  std::memcpy(&r, &u, 4);
  return r;
}

// A_real images (hi, lo) in the K-major no-swizzle shared-memory layout.
static void build_a_images(const float* m6, unsigned char* out) {
  float* hi = reinterpret_cast<float*>(out);
  float* lo = reinterpret_cast<float*>(out + kABytes);
  for (uint32_t r = 0; r < kD; ++r)
    for (uint32_t c = 0; c < kD; ++c) {
      const float mr = m6[2 * (r * kD + c)], mi = m6[2 * (r * kD + c) + 1];
      const float v[2][2] = {{mr, -mi}, {mi, mr}};
      for (uint32_t pr = 0; pr < 2; ++pr)
        for (uint32_t pc = 0; pc < 2; ++pc) {
          const float x = v[pr][pc];
          const float h = tf32_host(x);
          const float l = tf32_host(x - h);
          const uint32_t off = kmajor_off(2 * r + pr, 2 * c + pc, kSBOA) / 4;
          hi[off] = h;
          lo[off] = l;
        }
    }
}

static bool plan_tc(unsigned n, const unsigned* qs6, TcGeom& g) {
  std::memset(&g, 0, sizeof(g));
  if (n < kTileBits) return false;
  const unsigned tb = kTileBits;
  unsigned h = 0, b = tb;
  for (h = 0; h <= kK; ++h) {
    b = tb - h;
    unsigned cnt = 0;
    for (unsigned j = 0; j < kK; ++j) cnt += qs6[j] >= b;
    if (cnt == h) break;
  }
  if (h > kK) return false;
  g.b = b;
  // Tile bit j < b is state bit j; tile bit b + i is the i-th high target.
  for (unsigned j = 0; j < b; ++j) g.bitpos_state[j] = j;
  for (unsigned i = 0; i < h; ++i) g.bitpos_state[b + i] = qs6[kK - h + i];
  unsigned tslot = 0, gslot = 0;
  for (unsigned j = 0; j < tb; ++j) {
    const unsigned sb = g.bitpos_state[j];
    bool is_t = std::find(qs6, qs6 + kK, sb) != qs6 + kK;
    g.tile_is_target[j] = is_t;
    if (is_t) {
      // member bit = index of this target in the sorted target list
      g.target_slot[j] = unsigned(std::find(qs6, qs6 + kK, sb) - qs6);
      ++tslot;
    } else {
      g.group_slot[j] = gslot++;
    }
  }
  if (tslot != kK || gslot != 6) return false;
  std::vector<unsigned> ins(qs6 + kK - h, qs6 + kK);
  std::sort(ins.begin(), ins.end());
  g.n_ins = ins.size();
  for (size_t i = 0; i < ins.size(); ++i) g.ins_pos[i] = ins[i];
  g.num_tiles = uint64_t{1} << (n - tb);
  return true;
}

}  // namespace tc

size_t tc_operand_bytes(unsigned) { return 2 * size_t(tc::kABytes); }

void tc_build_operands(unsigned k, const float* m32, void* host_out) {
  // The plan stores matrices already padded to 6 targets (k == 6).
  (void)k;
  tc::build_a_images(m32, static_cast<unsigned char*>(host_out));
}

// Pads a gate to 6 targets for the tensor-core path (plan construction).
void tc_pad_gate(unsigned n, const unsigned* qs, unsigned k, const float* m32,
                 unsigned* qs6, float* m6_out) {
  std::vector<float> m6;
  tc::pad_to_6(n, qs, k, m32, qs6, m6);
  std::memcpy(m6_out, m6.data(), m6.size() * sizeof(float));
}

static int* g_tc_err = nullptr;

int apply_gate_tc(qsg_ctx* ctx, float* state, unsigned n, const unsigned* qs,
                  unsigned k, const float* m32, const void* operands) {
  using namespace tc;
  if (k != kK) {
    set_error("tensor-core gates are planned with 6 targets (got %u)", k);
    return QSG_ERR_INVALID;
  }
  TcArgs a;
  if (!plan_tc(n, qs, a.g)) {
    set_error("tensor-core path needs n >= %d qubits (n = %u)", kTileBits, n);
    return QSG_ERR_UNSUPPORTED;
  }
  if (!operands) {
    set_error("tensor-core gate without device operands");
    return QSG_ERR_INVALID;
  }
  a.operands = static_cast<const uint4*>(operands);
  if (!g_tc_err) {
    QSG_CUDA(cudaMalloc(&g_tc_err, sizeof(int)));
    QSG_CUDA(cudaMemset(g_tc_err, 0, sizeof(int)));
  }
  a.error = g_tc_err;
  static bool attr = false;
  if (!attr) {
    QSG_CUDA(cudaFuncSetAttribute(tc_gate_kernel,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  int(kSmemBytes)));
    attr = true;
  }
  const uint64_t grid = std::min<uint64_t>(a.g.num_tiles, ctx->num_sms);
  tc_gate_kernel<<<unsigned(grid), kThreads, kSmemBytes, ctx->stream>>>(
      reinterpret_cast<float2*>(state), a);
  QSG_LAUNCHED(ctx);
  (void)m32;
  return QSG_OK;
}

// Reads and clears the tensor-core kernels' error flag (1 = a bounded wait
// gave up).
int tc_check_error(qsg_ctx* ctx, int* out) {
  *out = 0;
  if (!g_tc_err) return QSG_OK;
  QSG_CUDA(cudaStreamSynchronize(ctx->stream));
  QSG_CUDA(cudaMemcpy(out, g_tc_err, sizeof(int), cudaMemcpyDeviceToHost));
  QSG_CUDA(cudaMemset(g_tc_err, 0, sizeof(int)));
  return QSG_OK;
}

void set_error_msg(const char* msg) { set_error("%s", msg); }

}  // namespace qsg

using namespace qsg;

extern "C" {

int qsg_apply_gate_tc(qsg_ctx* ctx, float* state, unsigned n,
                      const unsigned* qs, unsigned k, const float* matrix) {
  QSG_CHECK_ARG(ctx && state && matrix, "qsg_apply_gate_tc: null argument");
  if (k > 6) {
    set_error("gates on %u qubits are not supported (maximum 6)", k);
    return QSG_ERR_UNSUPPORTED;
  }
  QSG_CHECK_ARG(valid_qubits(qs, k, n), "qsg_apply_gate_tc: bad qubits");
  if (n < unsigned(tc::kTileBits)) {
    set_error("tensor-core path needs n >= %d qubits", tc::kTileBits);
    return QSG_ERR_UNSUPPORTED;
  }
  unsigned qs6[6];
  std::vector<float> m6(2 * tc::kD * tc::kD);
  tc_pad_gate(n, qs, k, matrix, qs6, m6.data());
  // Operands for a single call: synchronous upload into a context-owned
  // buffer (the stream is drained first, so the previous call's operands
  // are no longer read).
  static thread_local std::vector<unsigned char> host;
  host.resize(tc_operand_bytes(6));
  tc_build_operands(6, m6.data(), host.data());
  void* dev = nullptr;
  int rc = get_tc_operand_slot(ctx, host.size(), &dev);
  if (rc) return rc;
  QSG_CUDA(cudaStreamSynchronize(ctx->stream));
  QSG_CUDA(cudaMemcpy(dev, host.data(), host.size(), cudaMemcpyHostToDevice));
  return apply_gate_tc(ctx, state, n, qs6, 6, m6.data(), dev);
}

int qsg_tc_error(qsg_ctx* ctx, int* out) {
  QSG_CHECK_ARG(ctx && out, "qsg_tc_error: null argument");
  return tc_check_error(ctx, out);
}

}  // extern "C"
