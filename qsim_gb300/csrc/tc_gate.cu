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
//     members = 4096 amplitudes (32 KiB).
//   * Split FP16 with a power-of-two scale: the tile is multiplied by
//     sigma = 2^min(floor(n/2), 14), which brings the typical amplitude of a
//     normalised state (2^(-n/2)) near 1, so that both parts of its split
//     are normal FP16 numbers; amplitudes must satisfy |psi_i| <= 4 (any
//     state of norm <= 4), the FP16 maximum being 65504.  A = A_hi + A_lo and
//     B = B_hi + B_lo with every part an FP16 number, and
//     D = A_hi B_hi + A_hi B_lo + A_lo B_hi (3 x 8 MMAs of M=128, N=64,
//     K=16), FP32 accumulation, D / sigma in the epilogue.  FP16 keeps the
//     11-bit significand of TF32 and runs at twice its tensor rate; the
//     dropped A_lo B_lo term and the rounding of the lo parts leave ~2^-21
//     relative error per product, the FP32 level of the CUDA-core path.
//   * Tensor memory holds the gate (A_hi, A_lo: 2 x 64 columns of FP16
//     pairs, loaded once per CTA) and four 64-column accumulators, so the
//     MMAs of tile i run while the epilogue drains tiles i-1..i-3.
//   * Shared memory: two raw tile buffers fed by 16-byte cp.async in tile
//     order, and four operand buffers (B_hi, B_lo: 16 KiB each) in the
//     canonical no-swizzle K-major layout (8-row x 16-byte core matrices;
//     LBO = 128 B along K, SBO = 2 KiB between 8-row blocks), written by a
//     split pass with conflict-free 128-bit stores.
//   * One thread issues the MMAs and commits them to an mbarrier; every wait
//     is bounded by a clock budget and sets an error flag instead of hanging.
//     The epilogue reads D with tcgen05.ld, pairs re/im lanes with a shuffle,
//     stages the tile in its own operand buffer and stores it with coalesced
//     128-bit writes.
//
// All tile addressing is bitwise linear: a tile index e (12 bits) maps each
// of its bits to one state bit, one group bit or one member bit, so every
// offset is an OR of a per-thread part and a per-iteration table entry.

#include <algorithm>
#include <functional>
#include <cmath>
#include <cstring>
#include <vector>

#include <cuda_fp16.h>

#include "common.cuh"
#include "internal.h"
#include "matring.cuh"

namespace qsg {

namespace tc {

// Warp roles: 8 producer warps (split raw tiles into operands, refill raw
// buffers), 8 epilogue warps (drain tensor memory, stage, store; two per TMEM
// lane quadrant) and one MMA warp (its lane 0 issues every tcgen05.mma).
constexpr int kProdWarps = 8, kEpiWarps = 8;
constexpr int kProdThreads = 32 * kProdWarps;            // 256
constexpr int kEpiThreads = 32 * kEpiWarps;              // 256
constexpr int kThreads = kProdThreads + kEpiThreads + 32;  // 544
constexpr int kRoleBits = 8;                              // log2(256)
constexpr int kK = 6;                  // targets per tensor-core gate
constexpr int kD = 1 << kK;            // members per group (64)
constexpr int kReal = 2 * kD;          // real dimension (128) = M = K
constexpr int kGroups = 64;            // N
constexpr int kTileBits = 12;          // 64 groups x 64 members
constexpr int kTileAmps = 1 << kTileBits;
// Operands in memory: the padded 64 x 64 complex FP32 gate, row-major
// interleaved; the kernel converts it to the FP16 A images itself.
constexpr uint32_t kOperandBytes = kD * kD * 8;          // 32 KiB
constexpr uint32_t kTileBytes = kTileAmps * 8;           // 32 KiB
constexpr uint32_t kLBO = 128;                           // K-adjacent cores
constexpr uint32_t kSBOB = (kReal / 8) * 128;            // 2 KiB
constexpr uint32_t kTmemCols = 512;
constexpr uint32_t kTmemAhi = 0, kTmemAlo = 64, kTmemD = 128;  // columns
constexpr long long kWaitCycles = 4000000000LL;          // ~2 s at 2 GHz
// Two raw stages measured 1 % faster per 30-qubit circuit than three (and
// four with three operand buffers 3 % slower), four operand buffers.
constexpr int kRawStages = 2;
constexpr int kNB = 4;                 // operand buffers = accumulators
constexpr int kUnitsPerRole = kTileAmps / 2 / kProdThreads;  // 8 (= epilogue)
constexpr int kSplitPerRole = kTileAmps / 4 / kProdThreads;  // 4 quads

// Shared-memory map (bytes).
constexpr uint32_t kOffRaw = 0;                                  // 2 x 32 KiB
constexpr uint32_t kOffOp = kOffRaw + kRawStages * kTileBytes;    // 4 x 32 KiB
constexpr uint32_t kBImgBytes = kGroups * kReal * 2;              // 16 KiB
constexpr uint32_t kOpBytes = 2 * kBImgBytes;                     // hi | lo
// The epilogue stages its output tile in the operand buffer of that tile
// (its MMAs have completed when the accumulator is full).
constexpr uint32_t kOffTabG = kOffOp + kNB * kOpBytes;  // 8 x u64 unit goff
constexpr uint32_t kOffTabSplitE = kOffTabG + 64;       // 4 x u32 raw index
constexpr uint32_t kOffTabSplitO = kOffTabSplitE + 16;  // 4 x u32 op offset
constexpr uint32_t kOffTabGrpE = kOffTabSplitO + 16;    // 64 x u32 group e
constexpr uint32_t kOffTabRd = kOffTabGrpE + 256;       // 8 x u32 stage read
constexpr uint32_t kOffTabWr = kOffTabRd + 32;          // 8 x u32 raw write
constexpr uint32_t kNumBars = 4 * kNB + 2;  // + gate ready, + never arrived
constexpr uint32_t kOffBar = kOffTabWr + 32;            // mbarriers
constexpr uint32_t kOffFlag = kOffBar + 8 * kNumBars;   // failure flag
constexpr uint32_t kOffNorm = kOffFlag + 16;             // 16 x f64 + carry
constexpr uint32_t kOffTmem = kOffNorm + 16 * 8 + 16;
constexpr uint32_t kSmemBytes = kOffTmem + 16;

static_assert(kSmemBytes <= 232448, "shared memory budget");

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
  // XOR swizzles of tile indices, X(e) = XOR_i bit(e, src[i]) * msk[i]
  // with src >= 4 and msk < 16, so that the accesses of a half-warp fall on
  // distinct banks.  `out`: epilogue staging (8-byte writes by member x
  // group-bit-4 lanes, 16-byte linear reads).  `raw`: raw tile buffer
  // (16-byte cp.async writes, 8-byte split reads by group-bits-0..2 x
  // member-bit-2 lanes); it never touches bit 0.
  uint32_t out_src[8], out_msk[8], out_n;
  uint32_t raw_src[8], raw_msk[8], raw_n;
};

struct TcArgs {
  TcGeom g;
  // The padded 6-qubit gate, 64 x 64 complex FP32, row-major interleaved.
  const float2* operands;
  float scale;      // sigma: tile values are split as FP16 after * sigma
  float inv_scale;  // 1 / sigma, applied to D (both powers of two)
  int* error;       // set on a timed-out wait
  // Norm carry of unitary plans (null: off).  prev: the previous tensor-core
  // pass's per-CTA (sum |input|^2, sum |output|^2), prev_count CTAs; this
  // pass scales its input by sqrt(sum in / sum out) of that pass, undoing
  // the norm its FP32 accumulation lost, and writes its own sums to out.
  const double* prev;
  uint32_t prev_count;
  double* out;
  // Clock budget of every bounded wait (kWaitCycles in normal launches).
  long long wait_cycles;
  // Failure-detection test hook (0 in normal launches): the MMA thread
  // first waits on a barrier that no thread ever arrives at, so its bounded
  // wait runs out before any MMA is issued and every role takes the error
  // exit (the state is left as it was).
  int stall;
  // Expectation-value launches: per-CTA sum of conj(psi_i) (M psi)_i, and
  // a flag set when an amplitude times sigma left the FP16 range (the
  // result is then not used).
  double2* ev_partial;
  int* ev_overflow;
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

// Instruction descriptor of kind::f16: D = F32 (bits 4-5 = 1), A = B =
// F16 (bits 7-9, 10-12 = 0), both K-major, N = 64 (bits 17-22 = N / 8),
// M = 128 (bits 24-28 = M / 16); A is read from tensor memory.
constexpr uint32_t kIdesc = (1u << 4) | (uint32_t(kGroups >> 3) << 17) |
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

// FP16 pair (lo = first value in the low half) of two floats, round to
// nearest.
__device__ __forceinline__ uint32_t pack_half2(float a, float b) {
  const __half2 h = __floats2half2_rn(a, b);
  return *reinterpret_cast<const uint32_t*>(&h);
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

// D[tmem] (+)= A[tmem] * B[smem descriptor].
__device__ __forceinline__ void mma_f16_ts(uint32_t d_tmem, uint32_t a_tmem,
                                           uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n}\n" ::"r"(
          d_tmem),
      "r"(a_tmem), "l"(b), "r"(kIdesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void tmem_st32(uint32_t taddr,
                                          const uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], "
      "{%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,"
      "%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};\n" ::"r"(
          taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]),
      "r"(r[6]), "r"(r[7]), "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]),
      "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15]), "r"(r[16]), "r"(r[17]),
      "r"(r[18]), "r"(r[19]), "r"(r[20]), "r"(r[21]), "r"(r[22]), "r"(r[23]),
      "r"(r[24]), "r"(r[25]), "r"(r[26]), "r"(r[27]), "r"(r[28]), "r"(r[29]),
      "r"(r[30]), "r"(r[31])
      : "memory");
}

__device__ __forceinline__ void tmem_wait_st() {
  asm volatile("tcgen05.wait::st.sync.aligned;\n" ::: "memory");
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

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]),
        "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]),
        "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
        "=r"(r[15])
      : "r"(taddr));
}

// 16 lanes x 32 columns: thread t gets, for x < 4, words 4x, 4x+1 of lane
// t / 4 and words 4x+2, 4x+3 of lane t / 4 + 8, at columns 8x + 2 (t % 4)
// and 8x + 2 (t % 4) + 1.
__device__ __forceinline__ void tmem_ld16x256_x4(uint32_t taddr,
                                                 uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.16x256b.x4.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]),
        "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]),
        "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
        "=r"(r[15])
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
__host__ __device__ __forceinline__ uint64_t tile_goff(uint32_t e, const TcGeom& g) {
  uint64_t o = 0;
#pragma unroll
  for (int j = 0; j < kTileBits; ++j)
    if ((e >> j) & 1) o |= uint64_t{1} << g.bitpos_state[j];
  return o;
}

// Group n (6 bits) and member m (6 bits) -> tile index e.
__host__ __device__ __forceinline__ uint32_t tile_e(uint32_t n, uint32_t m,
                                           const TcGeom& g) {
  uint32_t e = 0;
#pragma unroll
  for (int j = 0; j < kTileBits; ++j) {
    const uint32_t bit = g.tile_is_target[j] ? (m >> g.target_slot[j]) & 1
                                             : (n >> g.group_slot[j]) & 1;
    e |= bit << j;
  }
  return e;
}

// Split-pass work item idx (10 bits) = (n bits 0-2 | quad q << 3 |
// n bits 3-5 << 7): the 16-byte operand row chunk (8 FP16 K-elements) of
// group n, members 4q .. 4q+3.  Lanes 0..7 of a warp cover the 8 rows of one
// core matrix, so the 128-bit operand stores are conflict free.
__host__ __device__ __forceinline__ uint32_t split_n(uint32_t idx) {
  return (idx & 7) | ((idx >> 7) << 3);
}
__host__ __device__ __forceinline__ uint32_t split_q(uint32_t idx) {
  return (idx >> 3) & 15;
}
__host__ __device__ __forceinline__ uint32_t op_off(uint32_t n, uint32_t q) {
  return (n / 8) * kSBOB + q * kLBO + (n % 8) * 16;
}

// N: the most entries a swizzle can have (4 for one access pattern; one
// solved for two patterns at once can have up to 8).
template <int N = 8>
__host__ __device__ __forceinline__ uint32_t swz_x(uint32_t e, const uint32_t* src,
                                          const uint32_t* msk, uint32_t n) {
  uint32_t x = 0;
#pragma unroll
  for (int i = 0; i < N; ++i)
    if (i < int(n) && ((e >> src[i]) & 1u)) x ^= msk[i];
  return x;
}
// s(e) = e ^ X(e); for disjoint a, b: s(a | b) = s(a) ^ s(b).
template <int N = 8>
__host__ __device__ __forceinline__ uint32_t swz_out(uint32_t e, const TcGeom& g) {
  return e ^ swz_x<N>(e, g.out_src, g.out_msk, g.out_n);
}
template <int N = 8>
__host__ __device__ __forceinline__ uint32_t swz_raw(uint32_t e, const TcGeom& g) {
  return e ^ swz_x<N>(e, g.raw_src, g.raw_msk, g.raw_n);
}

__host__ __device__ __forceinline__ uint64_t expand_outer_tc(uint64_t t,
                                                    const TcGeom& g) {
  uint64_t x = t << g.b;
  for (uint32_t i = 0; i < g.n_ins; ++i) {
    const uint32_t p = g.ins_pos[i];
    const uint64_t lo = x & ((uint64_t{1} << p) - 1);
    x = lo | ((x ^ lo) << 1);
  }
  return x;
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(bar))
               : "memory");
}

// Named barrier over `count` threads; returns true if any of them passed
// true (bar.red.or).
__device__ __forceinline__ bool bar_or(int id, int count, bool v) {
  uint32_t out;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n"
      " bar.red.or.pred q, %2, %3, p;\n selp.u32 %0, 1, 0, q;\n}\n"
      : "=r"(out)
      : "r"(uint32_t(v)), "r"(id), "r"(count)
      : "memory");
  return out != 0;
}

__device__ __forceinline__ void bar_sync(int id, int count) {
  asm volatile("bar.sync %0, %1;\n" ::"r"(id), "r"(count) : "memory");
}

// Bounded wait on an mbarrier phase; false if the clock budget ran out or
// another role already failed.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity,
                                          volatile int* flag,
                                          long long budget) {
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity)) {
    if (*flag) return false;
    if (clock64() - t0 > budget) {
      *flag = 1;
      return false;
    }
  }
  return true;
}

// EV = false: apply the gate (read and write the state).  EV = true:
// <psi| M |psi> (ExpectationValue): the state is only read; the epilogue
// multiplies each output amplitude (M psi)_i by conj(psi_i), psi_i taken
// back from the tile's FP16 hi + lo operand images, and nothing is stored.
template <bool EV>
__global__ void __launch_bounds__(kThreads, 1)
    tc_gate_kernel(float2* __restrict__ st, const __grid_constant__ TcArgs a) {
  extern __shared__ __align__(1024) unsigned char smem[];
  const TcGeom& g = a.g;
  const uint32_t tid = threadIdx.x;
  const uint32_t warp = tid / 32, lane = tid % 32;
  uint64_t* tab_g = reinterpret_cast<uint64_t*>(smem + kOffTabG);
  uint32_t* tab_se = reinterpret_cast<uint32_t*>(smem + kOffTabSplitE);
  uint32_t* tab_so = reinterpret_cast<uint32_t*>(smem + kOffTabSplitO);
  uint32_t* tab_ge = reinterpret_cast<uint32_t*>(smem + kOffTabGrpE);
  uint32_t* tab_rd = reinterpret_cast<uint32_t*>(smem + kOffTabRd);
  uint32_t* tab_wr = reinterpret_cast<uint32_t*>(smem + kOffTabWr);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + kOffBar);
  uint64_t* op_full = bars + 0;         // [kNB] producers -> MMA
  uint64_t* op_free = bars + kNB;       // [kNB] epilogue (staging read) -> producers
  uint64_t* acc_full = bars + 2 * kNB;  // [kNB] MMA commit -> epilogue
  uint64_t* acc_free = bars + 3 * kNB;  // [kNB] epilogue -> MMA
  uint64_t* gate_ready = bars + 4 * kNB;  // epilogue (gate in TMEM) -> MMA
  uint64_t* never = bars + 4 * kNB + 1;   // no thread arrives (test hook)
  volatile int* flag = reinterpret_cast<volatile int*>(smem + kOffFlag);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + kOffTmem);
  const uint32_t sbase = smem_u32(smem);

  // ---- set-up ------------------------------------------------------------
  // Unit u = rtid + 256 j (rtid: thread index inside a role, j < 8) of a
  // tile is tile index e = 2u: bits 1..8 from rtid, bits 9..11 from j.
  if (tid < kUnitsPerRole) {
    tab_g[tid] = tile_goff(uint32_t(tid) << (kRoleBits + 1), g);
    tab_rd[tid] = swz_out<4>(uint32_t(tid) << (kRoleBits + 1), g);
    tab_wr[tid] = swz_raw<4>(uint32_t(tid) << (kRoleBits + 1), g);
  }
  if (tid < kSplitPerRole) {
    // Split item idx = rtid + 256 j: j supplies idx bits 8, 9 (n bits 4, 5).
    const uint32_t idx = tid << kRoleBits;
    tab_se[tid] = swz_raw<4>(tile_e(split_n(idx), 4 * split_q(idx), g), g);
    tab_so[tid] = op_off(split_n(idx), split_q(idx));
  }
  if (tid < kGroups) tab_ge[tid] = swz_out<4>(tile_e(tid, 0, g), g);
  if (tid == 0) {
    // Accumulators and operand buffers are released by each epilogue warp
    // (eight arrivals), the rest by one thread.
    for (uint32_t i = 0; i < kNumBars; ++i) {
      const bool per_warp = (i >= kNB && i < 2 * kNB) || (i >= 3 * kNB && i < 4 * kNB);
      mbar_init(&bars[i], per_warp ? kEpiWarps : 1);
    }
    *flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  const uint32_t mma_warp = kProdWarps + kEpiWarps;
  if (warp == mma_warp) {
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
  // Tile counters fit 32 bits: at most 2^(40 - 12) tiles.
  const uint64_t step = gridDim.x;
  const uint64_t t0 = blockIdx.x;
  const uint32_t T =
      t0 < g.num_tiles ? uint32_t((g.num_tiles - t0 + step - 1) / step) : 0;

  if (warp < kProdWarps) {
    // ======================== producers ==================================
    const uint32_t rt = tid;
    const uint64_t my_g = tile_goff(rt << 1, g);
    const uint32_t my_wr = swz_raw<4>(rt << 1, g);
    const uint32_t my_se = swz_raw<4>(tile_e(split_n(rt), 4 * split_q(rt), g), g);
    const uint32_t my_so = op_off(split_n(rt), split_q(rt));
    // Swizzled tile offsets of member bits 0 and 1 (members 4q + 1, + 2).
    uint32_t e_m1 = 0, e_m2 = 0;
    for (int j = 0; j < kTileBits; ++j) {
      if (g.tile_is_target[j] && g.target_slot[j] == 0) e_m1 = 1u << j;
      if (g.tile_is_target[j] && g.target_slot[j] == 1) e_m2 = 1u << j;
    }
    e_m1 = swz_raw<4>(e_m1, g);
    e_m2 = swz_raw<4>(e_m2, g);
    // Norm carry: the previous pass's (sum in, sum out), reduced by each
    // producer warp in the same order (identical results in every warp).
    float carry = 1.f;
    if (a.prev) {
      double pin = 0, pout = 0;
      for (uint32_t i = lane; i < a.prev_count; i += 32) {
        pin += a.prev[2 * i];
        pout += a.prev[2 * i + 1];
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        pin += __shfl_xor_sync(0xffffffffu, pin, o);
        pout += __shfl_xor_sync(0xffffffffu, pout, o);
      }
      if (pout > 0) carry = float(sqrt(pin / pout));
    }
    const float sc = a.scale * carry;
    // sum |input|^2 over this thread's items (unscaled): FP32 per tile,
    // Kahan-compensated FP32 across tiles (FP64 issue is scarce on GB300).
    float sin_s = 0.f, sin_c = 0.f;
    bool ovf = false;  // EV: an amplitude times sigma beyond FP16's range
    auto issue_loads = [&](uint32_t i, int stage) {
      if (i < T) {
        const float4* gp = reinterpret_cast<const float4*>(
            st + (expand_outer_tc(t0 + uint64_t(i) * step, g) | my_g));
        const uint32_t sdst = sbase + kOffRaw + stage * kTileBytes;
#pragma unroll
        for (int j = 0; j < kUnitsPerRole; ++j)
          cp_async16(sdst + 8 * (my_wr ^ tab_wr[j]), gp + (tab_g[j] >> 1));
      }
      cp_commit();
    };
    for (int q = 0; q < kRawStages; ++q) issue_loads(q, q);
    for (uint32_t i = 0; i < T; ++i) {
      const int rs = i % kRawStages;
      const int s = i % kNB;
      cp_wait<kRawStages - 1>();
      // Operand buffer s is free once the epilogue read tile i-kNB out of it
      // (the ((i-kNB)/kNB)-th completion of op_free[s]).
      bool bad = false;
      if (i >= kNB) bad = !mbar_wait(&op_free[s], ((i - kNB) / kNB) & 1, flag,
                                     a.wait_cycles);
      if (bar_or(1, kProdThreads, bad)) break;
      // Split the raw tile into FP16 hi / lo operand rows (K-major): four
      // members (8 K-elements, one 16-byte core-matrix row) per item.
      const float2* raw = reinterpret_cast<const float2*>(smem + kOffRaw + rs * kTileBytes);
      const uint32_t obuf = kOffOp + s * kOpBytes;
      float tile_in = 0.f;
      // All raw reads of the tile first, then the splits and the operand
      // stores: the stores go to another buffer, but the compiler cannot
      // move a later shared-memory load above an earlier store, so
      // interleaving them would expose one load latency per quad.
      float2 xv[kSplitPerRole][4];
      uint32_t tso[kSplitPerRole];
#pragma unroll
      for (int j = 0; j < kSplitPerRole; ++j) {
        const uint32_t e0 = my_se ^ tab_se[j];
        tso[j] = tab_so[j];
        if (e_m1 == 1) {
          // Members 4q, 4q+1 (and 4q+2, 4q+3) are 16-byte units.
          const float4* raw4 = reinterpret_cast<const float4*>(raw);
          const float4 p0 = raw4[e0 >> 1], p1 = raw4[(e0 ^ e_m2) >> 1];
          xv[j][0] = make_float2(p0.x, p0.y);
          xv[j][1] = make_float2(p0.z, p0.w);
          xv[j][2] = make_float2(p1.x, p1.y);
          xv[j][3] = make_float2(p1.z, p1.w);
        } else {
          xv[j][0] = raw[e0];
          xv[j][1] = raw[e0 ^ e_m1];
          xv[j][2] = raw[e0 ^ e_m2];
          xv[j][3] = raw[e0 ^ e_m1 ^ e_m2];
        }
      }
#pragma unroll
      for (int j = 0; j < kSplitPerRole; ++j) {
        const float2 x0 = xv[j][0], x1 = xv[j][1], x2 = xv[j][2], x3 = xv[j][3];
        float x[8];
        if (a.out) {
          tile_in = fmaf(x0.x, x0.x, fmaf(x0.y, x0.y, tile_in));
          tile_in = fmaf(x1.x, x1.x, fmaf(x1.y, x1.y, tile_in));
          tile_in = fmaf(x2.x, x2.x, fmaf(x2.y, x2.y, tile_in));
          tile_in = fmaf(x3.x, x3.x, fmaf(x3.y, x3.y, tile_in));
        }
        x[0] = x0.x * sc; x[1] = x0.y * sc; x[2] = x1.x * sc; x[3] = x1.y * sc;
        x[4] = x2.x * sc; x[5] = x2.y * sc; x[6] = x3.x * sc; x[7] = x3.y * sc;
        uint4 h, l;
        uint32_t* hp = &h.x;
        uint32_t* lp = &l.x;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const __half2 hh = __floats2half2_rn(x[2 * c], x[2 * c + 1]);
          const float2 hf = __half22float2(hh);
          hp[c] = *reinterpret_cast<const uint32_t*>(&hh);
          lp[c] = pack_half2(x[2 * c] - hf.x, x[2 * c + 1] - hf.y);
          if constexpr (EV)
            ovf |= fmaxf(fabsf(x[2 * c]), fabsf(x[2 * c + 1])) > 65504.f;
        }
        const uint32_t o = my_so | tso[j];
        *reinterpret_cast<uint4*>(smem + obuf + o) = h;
        *reinterpret_cast<uint4*>(smem + obuf + kBImgBytes + o) = l;
      }
      if (a.out) {
        const float y = tile_in - sin_c;
        const float t2 = sin_s + y;
        sin_c = (t2 - sin_s) - y;
        sin_s = t2;
      }
      fence_async_smem();
      bar_sync(1, kProdThreads);
      if (rt == 0) mbar_arrive(&op_full[s]);
      issue_loads(i + kRawStages, rs);  // raw[rs] is consumed
    }
    cp_wait<0>();
    if constexpr (EV) {
      if (__any_sync(0xffffffffu, ovf) && lane == 0) atomicOr(a.ev_overflow, 1);
    }
    if (a.out) {
      // The input this pass applies the gate to is carry * input.
      double sum_in = (double(sin_s) - double(sin_c)) * double(carry) *
                      double(carry);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
        sum_in += __shfl_xor_sync(0xffffffffu, sum_in, o);
      if (lane == 0)
        reinterpret_cast<double*>(smem + kOffNorm)[warp] = sum_in;
    }
  } else if (warp < kProdWarps + kEpiWarps) {
    // ======================== epilogue ===================================
    const uint32_t et = tid - kProdThreads;
    const uint32_t ew = warp - kProdWarps;
    const uint32_t quad = warp % 4, chalf = ew / 4;  // TMEM lane quadrant
    const uint32_t lane_base = (32 * quad) << 16;
    const uint32_t row = 32 * quad + lane;
    // Gate into tensor memory: rows of this quadrant, columns of this half
    // (A_hi and A_lo, 64 columns of FP16 pairs each).  Row 16a + 8p + b is
    // the real (p = 0) or imaginary (p = 1) part of member 8a + b, so that a
    // 16x256b load gives one thread both parts of an output amplitude; word
    // w holds columns 2w, 2w + 1 of that row of [[Mr, -Mi], [Mi, Mr]]
    // interleaved by (member, re/im), i.e. (Mr, -Mi) or (Mi, Mr) of M[r][w],
    // split into FP16 hi and lo parts.
    {
      const uint32_t member = 8 * (row >> 4) + (row & 7);
      const float2* mrow = a.operands + size_t(member) * kD + 32 * chalf;
      const bool im_row = (row >> 3) & 1;
      uint32_t hw[32], lw[32];
#pragma unroll
      for (int q = 0; q < 32; ++q) {
        const float2 m = mrow[q];
        const float x0 = im_row ? m.y : m.x;
        const float x1 = im_row ? m.x : -m.y;
        const __half2 h = __floats2half2_rn(x0, x1);
        const float2 hf = __half22float2(h);
        hw[q] = *reinterpret_cast<const uint32_t*>(&h);
        lw[q] = pack_half2(x0 - hf.x, x1 - hf.y);
      }
      tmem_st32(tmem + lane_base + kTmemAhi + 32 * chalf, hw);
      tmem_st32(tmem + lane_base + kTmemAlo + 32 * chalf, lw);
      tmem_wait_st();
      tc_fence_before();
      bar_sync(2, kEpiThreads);
      if (et == 0) mbar_arrive(gate_ready);  // gate loaded: MMAs may start
    }
    const uint64_t my_g = tile_goff(et << 1, g);
    const uint32_t my_rd = swz_out<4>(et << 1, g);
    // Drain (16x256b loads of lane halves h = 0, 1 of this quadrant): this
    // thread holds member 8 (2 quad + h) + lane / 4 of groups
    // 32 chalf + 2 (lane % 4) + 8x + {0, 1}, x < 4; my_me[h] is the staging
    // slot of its first group, tab_ge[8x + e] the offset of the others.
    const uint32_t col0 = 32 * chalf + 2 * (lane & 3);
    uint32_t my_me[2];
#pragma unroll
    for (int h = 0; h < 2; ++h)
      my_me[h] = swz_out<4>(tile_e(col0, 8 * (2 * quad + h) + lane / 4, g), g);
    const float inv = a.inv_scale;
    // sum |output|^2 over this thread's outputs: FP32 per tile, Kahan FP32
    // across tiles.
    float sout_s = 0.f, sout_c = 0.f;
    // EV: this thread's sum of conj(psi) (M psi), FP32 per tile, FP64
    // across tiles; my_xo[h] is the operand-image byte offset of its
    // amplitude (member 8 (2 quad + h) + lane / 4, group col0): group bit 0
    // adds 16 bytes, group bits 3, 4 add 2 KiB each step.
    double ev_re = 0, ev_im = 0;
    uint32_t my_xo[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const uint32_t m = 8 * (2 * quad + h) + lane / 4;
      my_xo[h] = op_off(col0, m >> 2) + (m & 3) * 4;
    }
    for (uint32_t i = 0; i < T; ++i) {
      const int s = i % kNB;
      const bool bad =
          !mbar_wait(&acc_full[s], (i / kNB) & 1, flag, a.wait_cycles);
      if (bar_or(2, kEpiThreads, bad)) break;
      tc_fence_after();
      uint32_t v[32];
      const uint32_t taddr = tmem + lane_base + kTmemD + 64 * s + 32 * chalf;
      tmem_ld16x256_x4(taddr, v);
      tmem_ld16x256_x4(taddr + (16u << 16), v + 16);
      tmem_wait_ld();
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&acc_free[s]);  // this warp's part drained
      if constexpr (EV) {
        const unsigned char* ob = smem + kOffOp + s * kOpBytes;
        float pr = 0.f, pi = 0.f;
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
          for (int x = 0; x < 4; ++x)
#pragma unroll
            for (int e = 0; e < 2; ++e) {
              const float yr = __uint_as_float(v[16 * h + 4 * x + e]) * inv;
              const float yi = __uint_as_float(v[16 * h + 4 * x + 2 + e]) * inv;
              const uint32_t o = my_xo[h] + 16u * e + kSBOB * uint32_t(x);
              const float2 ph = __half22float2(
                  *reinterpret_cast<const __half2*>(ob + o));
              const float2 pl = __half22float2(
                  *reinterpret_cast<const __half2*>(ob + kBImgBytes + o));
              const float xr = (ph.x + pl.x) * inv, xi = (ph.y + pl.y) * inv;
              pr = fmaf(xr, yr, fmaf(xi, yi, pr));
              pi = fmaf(xr, yi, fmaf(-xi, yr, pi));
            }
        ev_re += double(pr);
        ev_im += double(pi);
        // This warp has read its part of the operand images.
        __syncwarp();
        if (lane == 0) mbar_arrive(&op_free[s]);
        continue;
      }
      float2* stage = reinterpret_cast<float2*>(smem + kOffOp + s * kOpBytes);
      float fo = 0.f;
#pragma unroll
      for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int x = 0; x < 4; ++x)
#pragma unroll
          for (int e = 0; e < 2; ++e) {
            const float re = __uint_as_float(v[16 * h + 4 * x + e]) * inv;
            const float im = __uint_as_float(v[16 * h + 4 * x + 2 + e]) * inv;
            stage[my_me[h] ^ tab_ge[8 * x + e]] = make_float2(re, im);
            fo = fmaf(re, re, fmaf(im, im, fo));
          }
      {
        const float y = fo - sout_c;
        const float t2 = sout_s + y;
        sout_c = (t2 - sout_s) - y;
        sout_s = t2;
      }
      bar_sync(2, kEpiThreads);
      const uint64_t base = expand_outer_tc(t0 + uint64_t(i) * step, g);
      float4* gp = reinterpret_cast<float4*>(st + (base | my_g));
      const float4* so = reinterpret_cast<const float4*>(stage);
#pragma unroll
      for (int j = 0; j < kUnitsPerRole; ++j) {
        const uint32_t sidx = my_rd ^ tab_rd[j];
        float4 w = so[sidx >> 1];
        if (sidx & 1) w = make_float4(w.z, w.w, w.x, w.y);
        gp[tab_g[j] >> 1] = w;
      }
      // This warp has read its part of the staging: one of the eight
      // arrivals that free operand buffer s.
      __syncwarp();
      if (lane == 0) mbar_arrive(&op_free[s]);
    }
    if constexpr (EV) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        ev_re += __shfl_xor_sync(0xffffffffu, ev_re, o);
        ev_im += __shfl_xor_sync(0xffffffffu, ev_im, o);
      }
      if (lane == 0) {
        reinterpret_cast<double*>(smem + kOffNorm)[ew] = ev_re;
        reinterpret_cast<double*>(smem + kOffNorm)[kEpiWarps + ew] = ev_im;
      }
    }
    if (!EV && a.out) {
      double sum_out = double(sout_s) - double(sout_c);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
        sum_out += __shfl_xor_sync(0xffffffffu, sum_out, o);
      if (lane == 0)
        reinterpret_cast<double*>(smem + kOffNorm)[kProdWarps + ew] = sum_out;
    }
  } else if (lane == 0) {
    // ======================== MMA issuer =================================
    // Test hook: a wait that nothing ends; it gives up after the budget and
    // sets the flag, and the loop below then issues nothing.
    const bool stalled = a.stall && !mbar_wait(never, 0, flag, a.wait_cycles);
    for (uint32_t i = 0; !stalled && i < T; ++i) {
      const int s = i % kNB;
      if (!mbar_wait(&op_full[s], (i / kNB) & 1, flag, a.wait_cycles)) break;
      // The gate must be in tensor memory before the first MMA, and
      // accumulator s is free once the epilogue drained tile i-kNB (the
      // ((i-kNB)/kNB)-th completion of acc_free[s]).
      if (i == 0) {
        if (!mbar_wait(gate_ready, 0, flag, a.wait_cycles)) break;
      } else if (i >= kNB) {
        if (!mbar_wait(&acc_free[s], ((i - kNB) / kNB) & 1, flag,
                       a.wait_cycles))
          break;
      }
      tc_fence_after();
      const uint32_t obuf = kOffOp + s * kOpBytes;
      const uint32_t d = tmem + kTmemD + 64 * s;
      const uint64_t dhi = make_desc(sbase + obuf, kLBO, kSBOB);
      const uint64_t dlo = make_desc(sbase + obuf + kBImgBytes, kLBO, kSBOB);
      // K = 16 FP16 elements per MMA: two core matrices along K (256 B) and
      // eight tensor-memory columns of A.
#pragma unroll
      for (int kk = 0; kk < kReal / 16; ++kk) {
        const uint64_t ko = uint64_t(kk) * (2 * kLBO >> 4);
        mma_f16_ts(d, tmem + kTmemAhi + 8 * kk, dhi + ko, kk > 0);
        mma_f16_ts(d, tmem + kTmemAhi + 8 * kk, dlo + ko, 1);
        mma_f16_ts(d, tmem + kTmemAlo + 8 * kk, dhi + ko, 1);
      }
      mma_commit(&acc_full[s]);
    }
  }

  // ---- tear-down -----------------------------------------------------------
  __syncthreads();
  if (EV && tid == 0) {
    const double* nsum = reinterpret_cast<const double*>(smem + kOffNorm);
    double sr = 0, si = 0;
    for (int w = 0; w < kEpiWarps; ++w) {
      sr += nsum[w];
      si += nsum[kEpiWarps + w];
    }
    a.ev_partial[blockIdx.x] = make_double2(sr, si);
  }
  if (!EV && a.out && tid == 0) {
    const double* nsum = reinterpret_cast<const double*>(smem + kOffNorm);
    double si = 0, so = 0;
    for (int w = 0; w < kProdWarps; ++w) si += nsum[w];
    for (int w = 0; w < kEpiWarps; ++w) so += nsum[kProdWarps + w];
    a.out[2 * blockIdx.x] = si;
    a.out[2 * blockIdx.x + 1] = so;
  }
  if (warp == mma_warp) {
    if (*flag) {
      if (lane == 0) atomicExch(a.error, 1);
      // The MMAs of an abandoned tile get one more bounded wait before
      // their tensor memory is released.
      const long long c0 = clock64();
      while (clock64() - c0 < a.wait_cycles / 4) {
      }
    }
    __syncwarp();
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

// XOR swizzle (src, msk, n) for which each set of four tile bits in
// `sets` maps its 16 index combinations onto 16 distinct values modulo 16
// (distinct banks for a half-warp of 8-byte accesses, or a quarter-warp of
// 16-byte ones when bit 0 is not among them and masks keep bit 0 clear):
// a tile bit v < 4 contributes the unit vector e_v, a bit v >= 4 the mask
// chosen for it, and each set's four vectors must be linearly independent
// over GF(2).  Depth-first search over the masks of the high bits; false if
// none exists.
static bool solve_swizzle(const std::vector<std::vector<unsigned>>& sets,
                          unsigned allowed, uint32_t* src, uint32_t* msk,
                          uint32_t* n) {
  std::vector<unsigned> high;
  for (const auto& v : sets)
    for (unsigned b : v)
      if (b >= 4 && std::find(high.begin(), high.end(), b) == high.end())
        high.push_back(b);
  if (high.size() > 8) return false;
  std::vector<uint32_t> m(high.size(), 0);
  auto vec = [&](unsigned b, size_t assigned, bool* known) -> uint32_t {
    if (b < 4) {
      *known = true;
      return 1u << b;
    }
    const size_t i = size_t(std::find(high.begin(), high.end(), b) - high.begin());
    *known = i < assigned;
    return *known ? m[i] : 0;
  };
  // Independence of the known vectors of every set (rank by elimination).
  auto ok = [&](size_t assigned) {
    for (const auto& v : sets) {
      uint32_t basis[4] = {0, 0, 0, 0};
      for (unsigned b : v) {
        bool known;
        uint32_t x = vec(b, assigned, &known);
        if (!known) continue;
        for (int bit = 3; bit >= 0; --bit) {
          if (!((x >> bit) & 1)) continue;
          if (!basis[bit]) {
            basis[bit] = x;
            break;
          }
          x ^= basis[bit];
        }
        if (!x) return false;
      }
    }
    return true;
  };
  std::function<bool(size_t)> dfs = [&](size_t i) {
    if (i == high.size()) return true;
    for (uint32_t c = 1; c < 16; ++c) {
      if (c & ~allowed) continue;
      m[i] = c;
      if (ok(i + 1) && dfs(i + 1)) return true;
    }
    return false;
  };
  if (!ok(0) || !dfs(0)) return false;
  *n = unsigned(high.size());
  for (size_t i = 0; i < high.size(); ++i) {
    src[i] = high[i];
    msk[i] = m[i];
  }
  return true;
}

// Member / group roles of the tile bits: tord[m] is the tile bit of member
// bit m, gord[k] the tile bit of group bit k (together all 12 tile bits,
// the tile's bit -> state-bit map already set), and the swizzles of the raw
// buffer (unless `raw` is false: a gate whose operand does not come from a
// raw tile) and the epilogue staging for those roles.
static bool tc_roles_ordered(TcGeom& g, const unsigned* tord,
                             const unsigned* gord, bool raw = true) {
  unsigned seen = 0;
  for (unsigned j = 0; j < unsigned(kTileBits); ++j) {
    g.tile_is_target[j] = 0;
    g.target_slot[j] = 0;
    g.group_slot[j] = 0;
  }
  for (unsigned m = 0; m < unsigned(kK); ++m) {
    if (tord[m] >= unsigned(kTileBits) || gord[m] >= unsigned(kTileBits))
      return false;
    g.tile_is_target[tord[m]] = 1;
    g.target_slot[tord[m]] = m;
    g.group_slot[gord[m]] = m;
    seen |= (1u << tord[m]) | (1u << gord[m]);
  }
  if (seen != (1u << kTileBits) - 1) return false;
  for (unsigned m = 0; m < unsigned(kK); ++m)
    if (g.tile_is_target[gord[m]]) return false;
  const unsigned* tpos = tord;
  const unsigned* gpos = gord;
  // Epilogue writes: half-warp lanes vary member bits 0, 1 (lane / 4) and
  // group bits 1, 2 (lane % 4).
  if (!solve_swizzle({{tpos[0], tpos[1], gpos[1], gpos[2]}}, 0xF, g.out_src,
                     g.out_msk, &g.out_n))
    return false;
  // Split reads: lanes vary group bits 0..2 and (half-warp) member bit 2;
  // 16-byte units keep bit 0 in place.  With member bit 0 on tile bit 0
  // (qubit 0) members 4q, 4q+1 are one 16-byte unit read by one LDS.128,
  // and the quarter-warp lanes (group bits 0..2) must hit distinct units
  // (bits 1..3 of the swizzled index).
  g.raw_n = 0;
  if (!raw) return true;
  if (tpos[0] == 0) {
    if (!solve_swizzle({{0, gpos[0], gpos[1], gpos[2]}}, 0xE, g.raw_src,
                       g.raw_msk, &g.raw_n))
      return false;
  } else if (!solve_swizzle({{gpos[0], gpos[1], gpos[2], tpos[2]}}, 0xE,
                            g.raw_src, g.raw_msk, &g.raw_n)) {
    return false;
  }
  return true;
}

// Roles for a gate with sorted targets qs6: member bit m is the tile bit of
// qs6[m], group bits follow the tile bits in order.
static bool tc_roles(TcGeom& g, const unsigned* qs6) {
  unsigned tord[kK], gord[kK], nt = 0, ng = 0;
  for (unsigned m = 0; m < unsigned(kK); ++m) {
    tord[m] = unsigned(kTileBits);
    for (unsigned j = 0; j < unsigned(kTileBits); ++j)
      if (g.bitpos_state[j] == qs6[m]) tord[m] = j;
    if (tord[m] == unsigned(kTileBits)) return false;
    ++nt;
  }
  for (unsigned j = 0; j < unsigned(kTileBits); ++j) {
    if (std::find(tord, tord + kK, j) != tord + kK) continue;
    if (ng == unsigned(kK)) return false;
    gord[ng++] = j;
  }
  if (nt != unsigned(kK) || ng != unsigned(kK)) return false;
  return tc_roles_ordered(g, tord, gord);
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
  if (!tc_roles(g, qs6)) return false;
  std::vector<unsigned> ins(qs6 + kK - h, qs6 + kK);
  std::sort(ins.begin(), ins.end());
  g.n_ins = ins.size();
  for (size_t i = 0; i < ins.size(); ++i) g.ins_pos[i] = ins[i];
  g.num_tiles = uint64_t{1} << (n - tb);
  return true;
}


// ===========================================================================
// Two gates per pass.  Gates A and B (6 targets each, padded) whose targets
// fit one 12-bit tile that starts at qubit 0 are applied in one read and
// one write of the state.  The producers split the raw tile for A; the
// epilogue drains A's accumulator (values still scaled by sigma) and writes
// them, split into FP16 hi / lo, straight into B's operand buffer; the MMA
// thread multiplies that by B; the epilogue drains B's accumulator, stages
// and stores the tile.  Both gates share the tile's bit -> state-bit map;
// each has its own member / group roles of the tile bits (geometries ga,
// gb), chosen so that a warp's 4-byte operand writes in A's drain fall on
// 32 distinct banks: the five tile bits a warp's lanes vary (A's member
// bits 0..2, A's group bits 1, 2) are B's member bits 0, 1 and group bits
// 0..2.  The gates' members are therefore numbered in that order, not by
// qubit (pa, pb map member bits to the sorted targets of the matrices).
// The MMA thread and the epilogue walk one job list, A(0), A(1), B(0),
// A(2), B(1), ..., A(T-1), B(T-2), B(T-1), so that a tile's B job finds its
// operand ready while the next tile's A job keeps the tensor cores busy;
// job k uses accumulator k % kNAcc2.  A operands live in kNA2 buffers
// (freed by the MMAs' completion), B operands in kNBB2 buffers that also
// stage B's result.  Numerically a pass is two one-gate passes without the
// FP32 round trip through HBM.
constexpr int kNA2 = 3;                  // A operand buffers
constexpr int kNBB2 = 2;                 // B operand / staging buffers
constexpr int kNAcc2 = 4;                // accumulators (64 columns each)
constexpr uint32_t kTmemGateB = 128;     // columns of gate B (A at 0)
constexpr uint32_t kTmemD2 = 256;        // first accumulator column
constexpr uint32_t kOffOpA2 = kOffRaw + kRawStages * kTileBytes;
constexpr uint32_t kOffOpB2 = kOffOpA2 + kNA2 * kOpBytes;
constexpr uint32_t kOffTabG2 = kOffOpB2 + kNBB2 * kOpBytes;  // 8 x u64
constexpr uint32_t kOffTabSE2 = kOffTabG2 + 64;              // 4 x u32
constexpr uint32_t kOffTabSO2 = kOffTabSE2 + 16;             // 4 x u32
constexpr uint32_t kOffTabGE2 = kOffTabSO2 + 16;             // 64 x u32 (B stage)
constexpr uint32_t kOffTabOB2 = kOffTabGE2 + 256;            // 64 x u32 (B operand)
constexpr uint32_t kOffTabRd2 = kOffTabOB2 + 256;            // 8 x u32 (B)
constexpr uint32_t kOffTabWr2 = kOffTabRd2 + 32;             // 8 x u32 (A raw)
constexpr uint32_t kNumBars2 = 2 * kNA2 + kNBB2 + 2 * kNAcc2 + 1;
constexpr uint32_t kOffBar2 = kOffTabWr2 + 32;
constexpr uint32_t kOffFlag2 = kOffBar2 + 8 * kNumBars2;
constexpr uint32_t kOffNorm2 = kOffFlag2 + 16;               // 16 x f64
constexpr uint32_t kOffTmem2 = kOffNorm2 + 16 * 8 + 16;
constexpr uint32_t kSmemBytes2 = kOffTmem2 + 16;
static_assert(kSmemBytes2 <= 232448, "shared memory budget (two gates)");
static_assert(kTmemD2 + kNAcc2 * 64 <= kTmemCols, "tensor memory budget");
static_assert(kOffBar2 % 8 == 0 && kOffNorm2 % 8 == 0, "alignment");

struct Tc2Args {
  TcGeom ga, gb;          // the same tile bits; A's and B's member roles
  const float2* opa;      // padded 64 x 64 complex FP32 gates, members in
  const float2* opb;      // sorted-qubit order
  // Member bit j of a gate's kernel numbering is member bit pa[j] (pb[j])
  // of its matrix.
  uint32_t pa[kK], pb[kK];
  float scale, inv_scale;
  int* error;
  const double* prev;     // norm carry, as TcArgs
  uint32_t prev_count;
  double* out;
  long long wait_cycles;
};

// Job k of a CTA with T tiles: its tile index i and whether it is gate B.
__device__ __forceinline__ void tc2_job(uint32_t k, uint32_t T, uint32_t* i,
                                        bool* is_b) {
  if (k == 0) {
    *i = 0;
    *is_b = false;
  } else if (k == 2 * T - 1) {
    *i = T - 1;
    *is_b = true;
  } else if (k & 1) {
    *i = (k + 1) / 2;
    *is_b = false;
  } else {
    *i = k / 2 - 1;
    *is_b = true;
  }
}

__host__ __device__ __forceinline__ uint32_t bit_perm(uint32_t m,
                                                      const uint32_t* p) {
  uint32_t r = 0;
#pragma unroll
  for (int j = 0; j < kK; ++j) r |= ((m >> j) & 1u) << p[j];
  return r;
}

// Byte offset, inside a B operand image, of the FP16 (re, im) pair of tile
// index e under gb's roles: member m of group n sits in row n, K chunk
// m / 4, at (m % 4) * 4 bytes.  Every tile bit adds a distinct power of two.
__host__ __device__ __forceinline__ uint32_t opb_off(uint32_t e,
                                                     const TcGeom& g) {
  uint32_t o = 0;
#pragma unroll
  for (int j = 0; j < kTileBits; ++j) {
    if (!((e >> j) & 1)) continue;
    if (g.tile_is_target[j]) {
      const uint32_t m = g.target_slot[j];
      o |= m < 2 ? (4u << m) : (kLBO << (m - 2));
    } else {
      const uint32_t k = g.group_slot[j];
      o |= k < 3 ? (16u << k) : (kSBOB << (k - 3));
    }
  }
  return o;
}

__global__ void __launch_bounds__(kThreads, 1)
    tc_gate2_kernel(float2* __restrict__ st,
                    const __grid_constant__ Tc2Args a) {
  extern __shared__ __align__(1024) unsigned char smem[];
  const TcGeom& ga = a.ga;
  const TcGeom& gb = a.gb;
  const uint32_t tid = threadIdx.x;
  const uint32_t warp = tid / 32, lane = tid % 32;
  uint64_t* tab_g = reinterpret_cast<uint64_t*>(smem + kOffTabG2);
  uint32_t* tab_se = reinterpret_cast<uint32_t*>(smem + kOffTabSE2);
  uint32_t* tab_so = reinterpret_cast<uint32_t*>(smem + kOffTabSO2);
  uint32_t* tab_ge = reinterpret_cast<uint32_t*>(smem + kOffTabGE2);
  uint32_t* tab_ob = reinterpret_cast<uint32_t*>(smem + kOffTabOB2);
  uint32_t* tab_rd = reinterpret_cast<uint32_t*>(smem + kOffTabRd2);
  uint32_t* tab_wr = reinterpret_cast<uint32_t*>(smem + kOffTabWr2);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + kOffBar2);
  uint64_t* opa_full = bars;                        // [kNA2] producers -> MMA
  uint64_t* opa_free = bars + kNA2;                 // [kNA2] MMA commit -> producers
  uint64_t* opb_full = bars + 2 * kNA2;             // [kNBB2] epilogue -> MMA
  uint64_t* acc_full = opb_full + kNBB2;            // [kNAcc2] MMA -> epilogue
  uint64_t* acc_free = acc_full + kNAcc2;           // [kNAcc2] epilogue -> MMA
  uint64_t* gate_ready = acc_free + kNAcc2;         // epilogue -> MMA
  volatile int* flag = reinterpret_cast<volatile int*>(smem + kOffFlag2);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + kOffTmem2);
  const uint32_t sbase = smem_u32(smem);

  // ---- set-up ------------------------------------------------------------
  if (tid < kUnitsPerRole) {
    tab_g[tid] = tile_goff(uint32_t(tid) << (kRoleBits + 1), ga);
    tab_rd[tid] = swz_out<4>(uint32_t(tid) << (kRoleBits + 1), gb);
    tab_wr[tid] = swz_raw<4>(uint32_t(tid) << (kRoleBits + 1), ga);
  }
  if (tid < kSplitPerRole) {
    const uint32_t idx = tid << kRoleBits;
    tab_se[tid] = swz_raw<4>(tile_e(split_n(idx), 4 * split_q(idx), ga), ga);
    tab_so[tid] = op_off(split_n(idx), split_q(idx));
  }
  if (tid < kGroups) {
    tab_ge[tid] = swz_out<4>(tile_e(tid, 0, gb), gb);
    tab_ob[tid] = opb_off(tile_e(tid, 0, ga), gb);
  }
  if (tid == 0) {
    // B operands and accumulators are released by each epilogue warp
    // (eight arrivals), the rest by one thread.
    for (uint32_t i = 0; i < kNumBars2; ++i) {
      const uint64_t* b = &bars[i];
      const bool per_warp = (b >= opb_full && b < opb_full + kNBB2) ||
                            (b >= acc_free && b < acc_free + kNAcc2);
      mbar_init(&bars[i], per_warp ? kEpiWarps : 1);
    }
    *flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  const uint32_t mma_warp = kProdWarps + kEpiWarps;
  if (warp == mma_warp) {
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
  // Tile and job counters fit 32 bits: at most 2^(40 - 12) tiles.
  const uint64_t step = gridDim.x;
  const uint64_t t0 = blockIdx.x;
  const uint32_t T =
      t0 < ga.num_tiles ? uint32_t((ga.num_tiles - t0 + step - 1) / step) : 0;
  const uint32_t jobs = 2 * T;

  if (warp < kProdWarps) {
    // ======================== producers (A splits) =======================
    const uint32_t rt = tid;
    const uint64_t my_g = tile_goff(rt << 1, ga);
    const uint32_t my_wr = swz_raw<4>(rt << 1, ga);
    const uint32_t my_se =
        swz_raw<4>(tile_e(split_n(rt), 4 * split_q(rt), ga), ga);
    const uint32_t my_so = op_off(split_n(rt), split_q(rt));
    uint32_t e_m1 = 0, e_m2 = 0;
    for (int j = 0; j < kTileBits; ++j) {
      if (ga.tile_is_target[j] && ga.target_slot[j] == 0) e_m1 = 1u << j;
      if (ga.tile_is_target[j] && ga.target_slot[j] == 1) e_m2 = 1u << j;
    }
    e_m1 = swz_raw<4>(e_m1, ga);
    e_m2 = swz_raw<4>(e_m2, ga);
    float carry = 1.f;
    if (a.prev) {
      double pin = 0, pout = 0;
      for (uint32_t i = lane; i < a.prev_count; i += 32) {
        pin += a.prev[2 * i];
        pout += a.prev[2 * i + 1];
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        pin += __shfl_xor_sync(0xffffffffu, pin, o);
        pout += __shfl_xor_sync(0xffffffffu, pout, o);
      }
      if (pout > 0) carry = float(sqrt(pin / pout));
    }
    const float sc = a.scale * carry;
    float sin_s = 0.f, sin_c = 0.f;
    auto issue_loads = [&](uint32_t i) {
      if (i < T) {
        const float4* gp = reinterpret_cast<const float4*>(
            st + (expand_outer_tc(t0 + uint64_t(i) * step, ga) | my_g));
        const uint32_t sdst = sbase + kOffRaw + (i % kRawStages) * kTileBytes;
#pragma unroll
        for (int j = 0; j < kUnitsPerRole; ++j)
          cp_async16(sdst + 8 * (my_wr ^ tab_wr[j]), gp + (tab_g[j] >> 1));
      }
      cp_commit();
    };
    for (int q = 0; q < kRawStages; ++q) issue_loads(q);
    for (uint32_t i = 0; i < T; ++i) {
      const int ba = int(i % kNA2);
      cp_wait<kRawStages - 1>();
      bool bad = false;
      if (i >= kNA2)
        bad = !mbar_wait(&opa_free[ba], uint32_t((i - kNA2) / kNA2) & 1, flag,
                         a.wait_cycles);
      if (bar_or(1, kProdThreads, bad)) break;
      const float2* raw = reinterpret_cast<const float2*>(
          smem + kOffRaw + (i % kRawStages) * kTileBytes);
      const uint32_t obuf = kOffOpA2 + ba * kOpBytes;
      float2 xv[kSplitPerRole][4];
#pragma unroll
      for (int j = 0; j < kSplitPerRole; ++j) {
        const uint32_t e0 = my_se ^ tab_se[j];
        if (e_m1 == 1) {
          const float4* raw4 = reinterpret_cast<const float4*>(raw);
          const float4 p0 = raw4[e0 >> 1], p1 = raw4[(e0 ^ e_m2) >> 1];
          xv[j][0] = make_float2(p0.x, p0.y);
          xv[j][1] = make_float2(p0.z, p0.w);
          xv[j][2] = make_float2(p1.x, p1.y);
          xv[j][3] = make_float2(p1.z, p1.w);
        } else {
          xv[j][0] = raw[e0];
          xv[j][1] = raw[e0 ^ e_m1];
          xv[j][2] = raw[e0 ^ e_m2];
          xv[j][3] = raw[e0 ^ e_m1 ^ e_m2];
        }
      }
      float tile_in = 0.f;
#pragma unroll
      for (int j = 0; j < kSplitPerRole; ++j) {
        const float2 x0 = xv[j][0], x1 = xv[j][1], x2 = xv[j][2], x3 = xv[j][3];
        if (a.out) {
          tile_in = fmaf(x0.x, x0.x, fmaf(x0.y, x0.y, tile_in));
          tile_in = fmaf(x1.x, x1.x, fmaf(x1.y, x1.y, tile_in));
          tile_in = fmaf(x2.x, x2.x, fmaf(x2.y, x2.y, tile_in));
          tile_in = fmaf(x3.x, x3.x, fmaf(x3.y, x3.y, tile_in));
        }
        float x[8];
        x[0] = x0.x * sc; x[1] = x0.y * sc; x[2] = x1.x * sc; x[3] = x1.y * sc;
        x[4] = x2.x * sc; x[5] = x2.y * sc; x[6] = x3.x * sc; x[7] = x3.y * sc;
        uint4 h, l;
        uint32_t* hp = &h.x;
        uint32_t* lp = &l.x;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const __half2 hh = __floats2half2_rn(x[2 * c], x[2 * c + 1]);
          const float2 hf = __half22float2(hh);
          hp[c] = *reinterpret_cast<const uint32_t*>(&hh);
          lp[c] = pack_half2(x[2 * c] - hf.x, x[2 * c + 1] - hf.y);
        }
        const uint32_t o = my_so | tab_so[j];
        *reinterpret_cast<uint4*>(smem + obuf + o) = h;
        *reinterpret_cast<uint4*>(smem + obuf + kBImgBytes + o) = l;
      }
      if (a.out) {
        const float y = tile_in - sin_c;
        const float t2 = sin_s + y;
        sin_c = (t2 - sin_s) - y;
        sin_s = t2;
      }
      fence_async_smem();
      bar_sync(1, kProdThreads);
      if (rt == 0) mbar_arrive(&opa_full[ba]);
      issue_loads(i + kRawStages);  // raw[i] is consumed
    }
    cp_wait<0>();
    if (a.out) {
      double sum_in = (double(sin_s) - double(sin_c)) * double(carry) *
                      double(carry);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
        sum_in += __shfl_xor_sync(0xffffffffu, sum_in, o);
      if (lane == 0)
        reinterpret_cast<double*>(smem + kOffNorm2)[warp] = sum_in;
    }
  } else if (warp < kProdWarps + kEpiWarps) {
    // ======================== epilogue ===================================
    const uint32_t et = tid - kProdThreads;
    const uint32_t ew = warp - kProdWarps;
    const uint32_t quad = warp % 4, chalf = ew / 4;
    const uint32_t lane_base = (32 * quad) << 16;
    const uint32_t row = 32 * quad + lane;
    // Both gates into tensor memory (A at column 0, B at kTmemGateB), rows
    // ordered as in the one-gate kernel, members in the kernel numbering.
#pragma unroll 1
    for (int gi = 0; gi < 2; ++gi) {
      const uint32_t* pm = gi ? a.pb : a.pa;
      const float2* mat = gi ? a.opb : a.opa;
      const uint32_t member = 8 * (row >> 4) + (row & 7);
      const float2* mrow = mat + size_t(bit_perm(member, pm)) * kD;
      const bool im_row = (row >> 3) & 1;
      uint32_t hw[32], lw[32];
#pragma unroll
      for (int q = 0; q < 32; ++q) {
        const float2 m = mrow[bit_perm(32 * chalf + q, pm)];
        const float x0 = im_row ? m.y : m.x;
        const float x1 = im_row ? m.x : -m.y;
        const __half2 h = __floats2half2_rn(x0, x1);
        const float2 hf = __half22float2(h);
        hw[q] = *reinterpret_cast<const uint32_t*>(&h);
        lw[q] = pack_half2(x0 - hf.x, x1 - hf.y);
      }
      const uint32_t base = gi ? kTmemGateB : 0;
      tmem_st32(tmem + lane_base + base + kTmemAhi + 32 * chalf, hw);
      tmem_st32(tmem + lane_base + base + kTmemAlo + 32 * chalf, lw);
    }
    tmem_wait_st();
    tc_fence_before();
    bar_sync(2, kEpiThreads);
    if (et == 0) mbar_arrive(gate_ready);
    const uint64_t my_g = tile_goff(et << 1, ga);
    const uint32_t my_rd = swz_out<4>(et << 1, gb);
    // This thread's amplitudes in a drain: member 8 (2 quad + h) + lane / 4
    // (A's numbering for A jobs, B's for B jobs) of groups
    // 32 chalf + 2 (lane % 4) + 8x + {0, 1}.
    const uint32_t col0 = 32 * chalf + 2 * (lane & 3);
    uint32_t my_ob[2], my_me[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const uint32_t m = 8 * (2 * quad + h) + lane / 4;
      my_ob[h] = opb_off(tile_e(col0, m, ga), gb);
      my_me[h] = swz_out<4>(tile_e(col0, m, gb), gb);
    }
    const float inv = a.inv_scale;
    float sout_s = 0.f, sout_c = 0.f;
    for (uint32_t k = 0; k < jobs; ++k) {
      uint32_t i;
      bool is_b;
      tc2_job(k, T, &i, &is_b);
      const int acc = int(k % kNAcc2);
      const int bb = int(i % kNBB2);
      const bool bad = !mbar_wait(&acc_full[acc], uint32_t(k / kNAcc2) & 1,
                                  flag, a.wait_cycles);
      if (bar_or(2, kEpiThreads, bad)) break;
      tc_fence_after();
      uint32_t v[32];
      const uint32_t taddr =
          tmem + lane_base + kTmemD2 + 64 * acc + 32 * chalf;
      tmem_ld16x256_x4(taddr, v);
      tmem_ld16x256_x4(taddr + (16u << 16), v + 16);
      tmem_wait_ld();
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&acc_free[acc]);  // this warp's part drained
      unsigned char* bufb = smem + kOffOpB2 + bb * kOpBytes;
      if (!is_b) {
        // A's result (scaled by sigma) as B's FP16 hi / lo operand.  The
        // buffer's previous tile, B(i - kNBB2), was stored by these threads
        // in an earlier job (the barrier that starts every job orders it).
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
          for (int x = 0; x < 4; ++x)
#pragma unroll
            for (int e = 0; e < 2; ++e) {
              const float re = __uint_as_float(v[16 * h + 4 * x + e]);
              const float im = __uint_as_float(v[16 * h + 4 * x + 2 + e]);
              const __half2 hh = __floats2half2_rn(re, im);
              const float2 hf = __half22float2(hh);
              const uint32_t o = my_ob[h] ^ tab_ob[8 * x + e];
              *reinterpret_cast<uint32_t*>(bufb + o) =
                  *reinterpret_cast<const uint32_t*>(&hh);
              *reinterpret_cast<uint32_t*>(bufb + kBImgBytes + o) =
                  pack_half2(re - hf.x, im - hf.y);
            }
        fence_async_smem();
        __syncwarp();
        if (lane == 0) mbar_arrive(&opb_full[bb]);  // one of eight arrivals
        continue;
      }
      // B's result: stage in B's buffer (its MMAs have completed), store.
      float2* stage = reinterpret_cast<float2*>(bufb);
      float fo = 0.f;
#pragma unroll
      for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int x = 0; x < 4; ++x)
#pragma unroll
          for (int e = 0; e < 2; ++e) {
            const float re = __uint_as_float(v[16 * h + 4 * x + e]) * inv;
            const float im = __uint_as_float(v[16 * h + 4 * x + 2 + e]) * inv;
            stage[my_me[h] ^ tab_ge[8 * x + e]] = make_float2(re, im);
            fo = fmaf(re, re, fmaf(im, im, fo));
          }
      {
        const float y = fo - sout_c;
        const float t2 = sout_s + y;
        sout_c = (t2 - sout_s) - y;
        sout_s = t2;
      }
      bar_sync(2, kEpiThreads);
      const uint64_t base = expand_outer_tc(t0 + uint64_t(i) * step, ga);
      float4* gp = reinterpret_cast<float4*>(st + (base | my_g));
      const float4* so = reinterpret_cast<const float4*>(stage);
#pragma unroll
      for (int j = 0; j < kUnitsPerRole; ++j) {
        const uint32_t sidx = my_rd ^ tab_rd[j];
        float4 w = so[sidx >> 1];
        if (sidx & 1) w = make_float4(w.z, w.w, w.x, w.y);
        gp[tab_g[j] >> 1] = w;
      }
      // The buffer takes B(i + kNBB2)'s operand in a later job, after the
      // barrier that starts every job.
    }
    if (a.out) {
      double sum_out = double(sout_s) - double(sout_c);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
        sum_out += __shfl_xor_sync(0xffffffffu, sum_out, o);
      if (lane == 0)
        reinterpret_cast<double*>(smem + kOffNorm2)[kProdWarps + ew] = sum_out;
    }
  } else if (lane == 0) {
    // ======================== MMA issuer =================================
    for (uint32_t k = 0; k < jobs; ++k) {
      uint32_t i;
      bool is_b;
      tc2_job(k, T, &i, &is_b);
      const int acc = int(k % kNAcc2);
      const int ba = int(i % kNA2), bb = int(i % kNBB2);
      const bool ok =
          is_b ? mbar_wait(&opb_full[bb], uint32_t(i / kNBB2) & 1, flag,
                           a.wait_cycles)
               : mbar_wait(&opa_full[ba], uint32_t(i / kNA2) & 1, flag,
                           a.wait_cycles);
      if (!ok) break;
      if (k == 0) {
        if (!mbar_wait(gate_ready, 0, flag, a.wait_cycles)) break;
      } else if (k >= kNAcc2) {
        if (!mbar_wait(&acc_free[acc], uint32_t((k - kNAcc2) / kNAcc2) & 1,
                       flag, a.wait_cycles))
          break;
      }
      tc_fence_after();
      const uint32_t obuf =
          is_b ? kOffOpB2 + bb * kOpBytes : kOffOpA2 + ba * kOpBytes;
      const uint32_t d = tmem + kTmemD2 + 64 * acc;
      const uint32_t gbase = tmem + (is_b ? kTmemGateB : 0);
      const uint64_t dhi = make_desc(sbase + obuf, kLBO, kSBOB);
      const uint64_t dlo = make_desc(sbase + obuf + kBImgBytes, kLBO, kSBOB);
#pragma unroll
      for (int kk = 0; kk < kReal / 16; ++kk) {
        const uint64_t ko = uint64_t(kk) * (2 * kLBO >> 4);
        mma_f16_ts(d, gbase + kTmemAhi + 8 * kk, dhi + ko, kk > 0);
        mma_f16_ts(d, gbase + kTmemAhi + 8 * kk, dlo + ko, 1);
        mma_f16_ts(d, gbase + kTmemAlo + 8 * kk, dhi + ko, 1);
      }
      mma_commit(&acc_full[acc]);
      // The A operand buffer is free once these MMAs have read it.
      if (!is_b) mma_commit(&opa_free[ba]);
    }
  }

  // ---- tear-down -----------------------------------------------------------
  __syncthreads();
  if (a.out && tid == 0) {
    const double* nsum = reinterpret_cast<const double*>(smem + kOffNorm2);
    double si = 0, so = 0;
    for (int w = 0; w < kProdWarps; ++w) si += nsum[w];
    for (int w = 0; w < kEpiWarps; ++w) so += nsum[kProdWarps + w];
    a.out[2 * blockIdx.x] = si;
    a.out[2 * blockIdx.x + 1] = so;
  }
  if (warp == mma_warp) {
    if (*flag) {
      if (lane == 0) atomicExch(a.error, 1);
      const long long c0 = clock64();
      while (clock64() - c0 < a.wait_cycles / 4) {
      }
    }
    __syncwarp();
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(
                     tmem),
                 "r"(kTmemCols)
                 : "memory");
  }
}

// Geometry of a pair.  The 12 tile bits are the union `u` of the two gates'
// (padded) targets, completed with the lowest other qubits; both geometries
// share the tile-bit -> state-bit map.  Tile bits are of four kinds: a
// target of both gates (TT), of A only (TG), of B only (GT), of neither
// (GG); with s TT bits there are 6 - s TG, 6 - s GT and s GG bits.  Five
// tile bits L, a TT, 3 - a TG, 2 - a GT and a GG ones, become A's member
// bits 0..2 (TT, TG), A's group bits 1, 2 (GT, GG), B's member bits 0, 1
// (TT, GT) and B's group bits 0..2 (TG, GG): then the lanes of a warp in
// A's drain (A member bits 0..2, A group bits 1, 2) write B's operand at 32
// distinct banks (B member bits 0, 1 and group bits 0..2 are the bank).
// Identical target sets (s = 6) admit no such L; false then.  pa[j] (pb[j])
// is the sorted-target index of the qubit of member bit j.
static bool plan_tc2(unsigned n, const unsigned* qa6, const unsigned* qb6,
                     TcGeom& ga, TcGeom& gb, uint32_t* pa, uint32_t* pb) {
  std::vector<unsigned> u(qa6, qa6 + kK);
  for (unsigned j = 0; j < kK; ++j)
    if (std::find(u.begin(), u.end(), qb6[j]) == u.end()) u.push_back(qb6[j]);
  if (u.size() > kTileBits || n < kTileBits) return false;
  for (unsigned q = 0; u.size() < kTileBits && q < n; ++q)
    if (std::find(u.begin(), u.end(), q) == u.end()) u.push_back(q);
  std::sort(u.begin(), u.end());
  // Run bits: tile bits j < b are state bits j; the h = 12 - b highest
  // members of u are the tile's high bits.
  unsigned h = 0, b = kTileBits;
  for (h = 0; h <= kTileBits; ++h) {
    b = kTileBits - h;
    unsigned cnt = 0;
    for (unsigned q : u) cnt += q >= b;
    if (cnt == h) break;
  }
  // Tile bit 0 must be state bit 0: the kernel moves amplitudes in pairs of
  // neighbours (16-byte units).
  if (h > kTileBits || b < 1) return false;
  uint64_t bitpos[kTileBits];
  for (unsigned j = 0; j < b; ++j) bitpos[j] = j;
  for (unsigned i = 0; i < h; ++i) bitpos[b + i] = u[kTileBits - h + i];
  auto in = [](const unsigned* q6, uint64_t sb) {
    return std::find(q6, q6 + kK, unsigned(sb)) != q6 + kK;
  };
  std::vector<unsigned> tt, tg, gt, gg;
  for (unsigned j = 0; j < unsigned(kTileBits); ++j) {
    const bool ia = in(qa6, bitpos[j]), ib = in(qb6, bitpos[j]);
    (ia ? (ib ? tt : tg) : (ib ? gt : gg)).push_back(j);
  }
  const int s = int(tt.size());
  // a TT bits in L; prefer the choice that puts tile bit 0 (qubit 0, if a
  // target of A) on A's member bit 0, for the producers' 16-byte reads.
  // (tt and tg list tile bits in ascending order: tile bit 0, when one of
  // them holds it, is their first element and is picked for any quota >= 1.)
  int na = -1;
  for (int a = std::max(0, s - 3); a <= std::min(2, s); ++a) {
    if (3 - a > 6 - s || 2 - a > 6 - s) continue;
    const bool zero_in = (!tt.empty() && tt[0] == 0 && a >= 1) ||
                         (!tg.empty() && tg[0] == 0 && 3 - a >= 1);
    if (na < 0 || zero_in) na = a;
    if (zero_in) break;
  }
  if (na < 0) return false;
  std::vector<unsigned> l_tt(tt.begin(), tt.begin() + na);
  std::vector<unsigned> l_tg(tg.begin(), tg.begin() + (3 - na));
  std::vector<unsigned> l_gt(gt.begin(), gt.begin() + (2 - na));
  std::vector<unsigned> l_gg(gg.begin(), gg.begin() + na);
  auto rest = [](const std::vector<unsigned>& all,
                 std::vector<unsigned> pick) {
    std::vector<unsigned> r;
    for (unsigned j : all)
      if (std::find(pick.begin(), pick.end(), j) == pick.end()) r.push_back(j);
    return r;
  };
  auto cat = [](std::vector<unsigned> x, const std::vector<unsigned>& y) {
    x.insert(x.end(), y.begin(), y.end());
    return x;
  };
  // A: member bits 0..2 = L's TT + TG bits (tile bit 0 first when there),
  // 3..5 the other A targets; group bit 0 an A group outside L, 1, 2 = L's
  // GT + GG bits, 3..5 the rest.
  std::vector<unsigned> at = cat(l_tt, l_tg);
  std::sort(at.begin(), at.end());
  std::vector<unsigned> a_targets = cat(tt, tg);
  std::sort(a_targets.begin(), a_targets.end());
  std::vector<unsigned> tord_a = cat(at, rest(a_targets, at));
  std::vector<unsigned> ag = cat(l_gt, l_gg);
  std::sort(ag.begin(), ag.end());
  std::vector<unsigned> a_groups = cat(gt, gg);
  std::sort(a_groups.begin(), a_groups.end());
  std::vector<unsigned> ag_rest = rest(a_groups, ag);
  if (ag_rest.empty()) return false;
  std::vector<unsigned> gord_a = {ag_rest[0], ag[0], ag[1]};
  for (size_t i = 1; i < ag_rest.size(); ++i) gord_a.push_back(ag_rest[i]);
  // B: member bits 0, 1 = L's TT + GT bits, 2..5 the other B targets;
  // group bits 0..2 = L's TG + GG bits, 3..5 the rest.
  std::vector<unsigned> bt = cat(l_tt, l_gt);
  std::sort(bt.begin(), bt.end());
  std::vector<unsigned> b_targets = cat(tt, gt);
  std::sort(b_targets.begin(), b_targets.end());
  std::vector<unsigned> tord_b = cat(bt, rest(b_targets, bt));
  std::vector<unsigned> bg = cat(l_tg, l_gg);
  std::sort(bg.begin(), bg.end());
  std::vector<unsigned> b_groups = cat(tg, gg);
  std::sort(b_groups.begin(), b_groups.end());
  std::vector<unsigned> gord_b = cat(bg, rest(b_groups, bg));
  if (tord_a.size() != 6 || gord_a.size() != 6 || tord_b.size() != 6 ||
      gord_b.size() != 6)
    return false;
  for (int gi = 0; gi < 2; ++gi) {
    TcGeom& g = gi ? gb : ga;
    std::memset(&g, 0, sizeof(g));
    g.b = b;
    for (unsigned j = 0; j < unsigned(kTileBits); ++j) g.bitpos_state[j] = bitpos[j];
    // B's operand comes from A's drain, not from a raw tile.
    if (!tc_roles_ordered(g, (gi ? tord_b : tord_a).data(),
                          (gi ? gord_b : gord_a).data(), gi == 0))
      return false;
    g.n_ins = h;
    for (unsigned i = 0; i < h; ++i) g.ins_pos[i] = u[kTileBits - h + i];
    g.num_tiles = uint64_t{1} << (n - kTileBits);
  }
  for (unsigned m = 0; m < unsigned(kK); ++m) {
    pa[m] = unsigned(std::find(qa6, qa6 + kK, unsigned(bitpos[tord_a[m]])) - qa6);
    pb[m] = unsigned(std::find(qb6, qb6 + kK, unsigned(bitpos[tord_b[m]])) - qb6);
  }
  return true;
}

}  // namespace tc

size_t tc_operand_bytes(unsigned) { return size_t(tc::kOperandBytes); }

void tc_build_operands(unsigned k, const float* m32, void* host_out) {
  // The plan stores matrices already padded to 6 targets (k == 6); the
  // kernel converts them to its FP16 operand images.
  (void)k;
  std::memcpy(host_out, m32, tc::kOperandBytes);
}

// Pads a gate to 6 targets for the tensor-core path (plan construction).
void tc_pad_gate(unsigned n, const unsigned* qs, unsigned k, const float* m32,
                 unsigned* qs6, float* m6_out) {
  std::vector<float> m6;
  tc::pad_to_6(n, qs, k, m32, qs6, m6);
  std::memcpy(m6_out, m6.data(), m6.size() * sizeof(float));
}

// Applies a gate given as a host matrix on the tensor cores: pads it to six
// targets, builds its FP16 operands in a pinned staging slot of the
// context's ring and uploads them asynchronously; the slot is reused only
// after its copy has completed (event), and later copies into the same
// device slot are ordered after this launch on the stream.
int apply_gate_tc(qsg_ctx* ctx, float* state, unsigned n, const unsigned* qs,
                  unsigned k, const float* m32, const void* operands);

// Pinned staging slots and device slots of the context's operand ring.
static int tc_ring_init(qsg_ctx* ctx) {
  constexpr size_t kSlot = (tc::kOperandBytes + 1023) & ~size_t(1023);
  if (ctx->tc_ring_dev) return QSG_OK;
  void* d = nullptr;
  void* h = nullptr;
  QSG_CUDA(cudaMalloc(&d, kSlot * qsg_ctx::kTcRingSlots));
  QSG_CUDA(cudaMallocHost(&h, kSlot * qsg_ctx::kTcRingSlots));
  ctx->tc_ring_dev = static_cast<unsigned char*>(d);
  ctx->tc_ring_host = static_cast<unsigned char*>(h);
  for (int i = 0; i < qsg_ctx::kTcRingSlots; ++i)
    QSG_CUDA(cudaEventCreateWithFlags(&ctx->tc_ring_ev[i],
                                      cudaEventDisableTiming));
  return QSG_OK;
}

// Uploads a padded 6-qubit gate (m6, 64 x 64 complex FP32) through a pinned
// staging slot of the context's operand ring; *dev is its device copy.
static int tc_ring_upload(qsg_ctx* ctx, const std::vector<float>& m6,
                          const void** dev) {
  using namespace tc;
  constexpr size_t kSlot = (kOperandBytes + 1023) & ~size_t(1023);
  int rc = tc_ring_init(ctx);
  if (rc) return rc;
  const int slot = ctx->tc_ring_next;
  ctx->tc_ring_next = (slot + 1) % qsg_ctx::kTcRingSlots;
  if (ctx->tc_ring_used[slot])
    QSG_CUDA(cudaEventSynchronize(ctx->tc_ring_ev[slot]));
  unsigned char* h = ctx->tc_ring_host + slot * kSlot;
  unsigned char* d = ctx->tc_ring_dev + slot * kSlot;
  std::memcpy(h, m6.data(), kOperandBytes);
  QSG_CUDA(cudaMemcpyAsync(d, h, kOperandBytes, cudaMemcpyHostToDevice,
                           ctx->stream));
  QSG_CUDA(cudaEventRecord(ctx->tc_ring_ev[slot], ctx->stream));
  ctx->tc_ring_used[slot] = true;
  *dev = d;
  return QSG_OK;
}

int apply_gate_tc_host(qsg_ctx* ctx, float* state, unsigned n,
                       const unsigned* qs, unsigned k, const float* m32) {
  using namespace tc;
  constexpr size_t kSlot = (kOperandBytes + 1023) & ~size_t(1023);
  int rc = tc_ring_init(ctx);
  if (rc) return rc;
  unsigned qs6[6];
  std::vector<float> m6;
  pad_to_6(n, qs, k, m32, qs6, m6);
  const int slot = ctx->tc_ring_next;
  ctx->tc_ring_next = (slot + 1) % qsg_ctx::kTcRingSlots;
  if (ctx->tc_ring_used[slot])
    QSG_CUDA(cudaEventSynchronize(ctx->tc_ring_ev[slot]));
  unsigned char* h = ctx->tc_ring_host + slot * kSlot;
  unsigned char* d = ctx->tc_ring_dev + slot * kSlot;
  std::memcpy(h, m6.data(), kOperandBytes);
  QSG_CUDA(cudaMemcpyAsync(d, h, kOperandBytes, cudaMemcpyHostToDevice,
                           ctx->stream));
  QSG_CUDA(cudaEventRecord(ctx->tc_ring_ev[slot], ctx->stream));
  ctx->tc_ring_used[slot] = true;
  return apply_gate_tc(ctx, state, n, qs6, 6, m6.data(), d);
}

void tcring_release(qsg_ctx* ctx) {
  for (int i = 0; i < qsg_ctx::kTcRingSlots; ++i) {
    if (ctx->tc_ring_ev[i]) cudaEventDestroy(ctx->tc_ring_ev[i]);
    ctx->tc_ring_ev[i] = nullptr;
    ctx->tc_ring_used[i] = false;
  }
  if (ctx->tc_ring_dev) cudaFree(ctx->tc_ring_dev);
  if (ctx->tc_ring_host) cudaFreeHost(ctx->tc_ring_host);
  ctx->tc_ring_dev = nullptr;
  ctx->tc_ring_host = nullptr;
}

static int* g_tc_err = nullptr;
static int* g_tc_ovf = nullptr;  // EV overflow flag
// Wait budget and test stall of the next launches; changed only for the
// duration of qsg_tc_stall_test on the calling thread.
static thread_local long long g_tc_wait_cycles = tc::kWaitCycles;
static thread_local int g_tc_stall = 0;

// One-time set-up (error flag, shared-memory opt-in); must precede any
// graph capture that contains tensor-core launches.
int tc_setup() {
  if (!g_tc_err) {
    QSG_CUDA(cudaMalloc(&g_tc_err, sizeof(int)));
    QSG_CUDA(cudaMemset(g_tc_err, 0, sizeof(int)));
    QSG_CUDA(cudaMalloc(&g_tc_ovf, sizeof(int)));
    QSG_CUDA(cudaMemset(g_tc_ovf, 0, sizeof(int)));
    QSG_CUDA(cudaFuncSetAttribute(tc::tc_gate_kernel<false>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  int(tc::kSmemBytes)));
    QSG_CUDA(cudaFuncSetAttribute(tc::tc_gate_kernel<true>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  int(tc::kSmemBytes)));
    QSG_CUDA(cudaFuncSetAttribute(tc::tc_gate2_kernel,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  int(tc::kSmemBytes2)));
  }
  return QSG_OK;
}

unsigned tc_grid(qsg_ctx* ctx, unsigned n) {
  if (n < unsigned(tc::kTileBits)) return 0;
  const uint64_t tiles = uint64_t{1} << (n - tc::kTileBits);
  return unsigned(std::min<uint64_t>(tiles, uint64_t(ctx->num_sms)));
}

int apply_gate_tc_carry(qsg_ctx* ctx, float* state, unsigned n,
                        const unsigned* qs, unsigned k, const float* m32,
                        const void* operands, const double* prev,
                        unsigned prev_count, double* out);

int apply_gate_tc(qsg_ctx* ctx, float* state, unsigned n, const unsigned* qs,
                  unsigned k, const float* m32, const void* operands) {
  return apply_gate_tc_carry(ctx, state, n, qs, k, m32, operands, nullptr, 0,
                             nullptr);
}

int apply_gate_tc_carry(qsg_ctx* ctx, float* state, unsigned n,
                        const unsigned* qs, unsigned k, const float* m32,
                        const void* operands, const double* prev,
                        unsigned prev_count, double* out) {
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
  a.operands = static_cast<const float2*>(operands);
  // sigma = 2^min(floor(n/2), 14): amplitudes of a normalised state (about
  // 2^(-n/2)) land near 1, where the lo parts of the split are normal FP16
  // numbers (relative error ~2^-23), and |psi_i| <= 4 stays below the FP16
  // maximum.
  const int e = std::min(int(n / 2), 14);
  a.scale = std::ldexp(1.0f, e);
  a.inv_scale = std::ldexp(1.0f, -e);
  int rc0 = tc_setup();
  if (rc0) return rc0;
  a.error = g_tc_err;
  a.prev = prev;
  a.prev_count = prev ? prev_count : 0;
  a.out = out;
  a.wait_cycles = g_tc_wait_cycles;
  a.stall = g_tc_stall;
  const uint64_t grid = std::min<uint64_t>(a.g.num_tiles, ctx->num_sms);
  a.ev_partial = nullptr;
  tc_gate_kernel<false><<<unsigned(grid), kThreads, kSmemBytes, ctx->stream>>>(
      reinterpret_cast<float2*>(state), a);
  QSG_LAUNCHED(ctx);
  (void)m32;
  return QSG_OK;
}

// Two padded 6-qubit gates (sorted targets qa6, qb6; device operands opa,
// opb) in one pass; the second gate is applied after the first.
int apply_gate_tc2_carry(qsg_ctx* ctx, float* state, unsigned n,
                         const unsigned* qa6, const void* opa,
                         const unsigned* qb6, const void* opb,
                         const double* prev, unsigned prev_count,
                         double* out) {
  using namespace tc;
  Tc2Args a;
  if (!plan_tc2(n, qa6, qb6, a.ga, a.gb, a.pa, a.pb)) {
    set_error("two-gate tensor-core pass: targets do not fit one 12-qubit "
              "tile (n = %u)", n);
    return QSG_ERR_UNSUPPORTED;
  }
  if (!opa || !opb) {
    set_error("tensor-core gate without device operands");
    return QSG_ERR_INVALID;
  }
  a.opa = static_cast<const float2*>(opa);
  a.opb = static_cast<const float2*>(opb);
  const int e = std::min(int(n / 2), 14);
  a.scale = std::ldexp(1.0f, e);
  a.inv_scale = std::ldexp(1.0f, -e);
  int rc0 = tc_setup();
  if (rc0) return rc0;
  a.error = g_tc_err;
  a.prev = prev;
  a.prev_count = prev ? prev_count : 0;
  a.out = out;
  a.wait_cycles = g_tc_wait_cycles;
  const uint64_t grid = std::min<uint64_t>(a.ga.num_tiles, ctx->num_sms);
  tc_gate2_kernel<<<unsigned(grid), kThreads, kSmemBytes2, ctx->stream>>>(
      reinterpret_cast<float2*>(state), a);
  QSG_LAUNCHED(ctx);
  return QSG_OK;
}

// Run bits b of the two-gate tile of two padded 6-qubit gates (tile bits
// 0..b-1 are state bits 0..b-1, i.e. 2^b contiguous amplitudes per row of
// the tile), or -1 if the pair does not fit a two-gate pass.
int tc2_run_bits(unsigned n, const unsigned* qa6, const unsigned* qb6) {
  tc::TcGeom ga, gb;
  uint32_t pa[tc::kK], pb[tc::kK];
  if (!tc::plan_tc2(n, qa6, qb6, ga, gb, pa, pb)) return -1;
  return int(ga.b);
}

// Test entry of the two-gate pass: pads both host matrices to 6 targets,
// uploads them through the context's operand ring and launches.
int apply_gate_tc2_host(qsg_ctx* ctx, float* state, unsigned n,
                        const unsigned* qa, unsigned ka, const float* ma,
                        const unsigned* qb, unsigned kb, const float* mb) {
  using namespace tc;
  constexpr size_t kSlot = (kOperandBytes + 1023) & ~size_t(1023);
  unsigned qa6[6], qb6[6];
  std::vector<float> ma6, mb6;
  pad_to_6(n, qa, ka, ma, qa6, ma6);
  pad_to_6(n, qb, kb, mb, qb6, mb6);
  if (std::equal(qa6, qa6 + 6, qb6)) {
    // The same six qubits: one pass of the product B A (FP64 on the host).
    std::vector<float> prod(2 * kD * kD);
    for (unsigned r = 0; r < unsigned(kD); ++r)
      for (unsigned c = 0; c < unsigned(kD); ++c) {
        double re = 0, im = 0;
        for (unsigned j = 0; j < unsigned(kD); ++j) {
          const double br = mb6[2 * (r * kD + j)], bi = mb6[2 * (r * kD + j) + 1];
          const double ar = ma6[2 * (j * kD + c)], ai = ma6[2 * (j * kD + c) + 1];
          re += br * ar - bi * ai;
          im += br * ai + bi * ar;
        }
        prod[2 * (r * kD + c)] = float(re);
        prod[2 * (r * kD + c) + 1] = float(im);
      }
    return apply_gate_tc_host(ctx, state, n, qa6, 6, prod.data());
  }
  if (tc2_run_bits(n, qa6, qb6) < 1) {
    set_error("two-gate tensor-core pass: the padded targets of the two "
              "gates span 12 qubits without qubit 0 (no tile of them starts "
              "at qubit 0)");
    return QSG_ERR_UNSUPPORTED;
  }
  int rc = tc_ring_init(ctx);
  if (rc) return rc;
  unsigned char* dev[2];
  const std::vector<float>* src[2] = {&ma6, &mb6};
  for (int gi = 0; gi < 2; ++gi) {
    const int slot = ctx->tc_ring_next;
    ctx->tc_ring_next = (slot + 1) % qsg_ctx::kTcRingSlots;
    if (ctx->tc_ring_used[slot])
      QSG_CUDA(cudaEventSynchronize(ctx->tc_ring_ev[slot]));
    unsigned char* h = ctx->tc_ring_host + slot * kSlot;
    dev[gi] = ctx->tc_ring_dev + slot * kSlot;
    std::memcpy(h, src[gi]->data(), kOperandBytes);
    QSG_CUDA(cudaMemcpyAsync(dev[gi], h, kOperandBytes, cudaMemcpyHostToDevice,
                             ctx->stream));
    QSG_CUDA(cudaEventRecord(ctx->tc_ring_ev[slot], ctx->stream));
    ctx->tc_ring_used[slot] = true;
  }
  return apply_gate_tc2_carry(ctx, state, n, qa6, dev[0], qb6, dev[1],
                              nullptr, 0, nullptr);
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

// <psi| M |psi> of a k-qubit operator (k <= 6, padded to 6 targets with the
// identity, which leaves the value unchanged) on the tensor cores: one read
// of the state, per-CTA FP64 partials summed in a fixed order.
int expectation_tc(qsg_ctx* ctx, const float* state, unsigned n,
                   const unsigned* qs, unsigned k, const float* m32,
                   double* out_re_im, bool* overflow) {
  using namespace tc;
  *overflow = false;
  if (n < unsigned(kTileBits) || k > unsigned(kK)) {
    set_error("tensor-core expectation values need n >= %d, k <= 6",
              kTileBits);
    return QSG_ERR_UNSUPPORTED;
  }
  unsigned qs6[6];
  std::vector<float> m6;
  pad_to_6(n, qs, k, m32, qs6, m6);
  TcArgs a;
  std::memset(&a, 0, sizeof(a));
  if (!plan_tc(n, qs6, a.g)) {
    set_error("tensor-core path needs n >= %d qubits (n = %u)", kTileBits, n);
    return QSG_ERR_UNSUPPORTED;
  }
  const void* dev = nullptr;
  int rc = tc_ring_upload(ctx, m6, &dev);
  if (rc) return rc;
  rc = tc_setup();
  if (rc) return rc;
  a.operands = static_cast<const float2*>(dev);
  const int e = std::min(int(n / 2), 14);
  a.scale = std::ldexp(1.0f, e);
  a.inv_scale = std::ldexp(1.0f, -e);
  a.error = g_tc_err;
  a.wait_cycles = g_tc_wait_cycles;
  const uint64_t grid = std::min<uint64_t>(a.g.num_tiles, ctx->num_sms);
  void* p = nullptr;
  rc = get_scratch(ctx, (grid + 1) * sizeof(double2), &p);
  if (rc) return rc;
  a.ev_partial = static_cast<double2*>(p);
  a.ev_overflow = g_tc_ovf;
  QSG_CUDA(cudaMemsetAsync(g_tc_ovf, 0, sizeof(int), ctx->stream));
  tc_gate_kernel<true><<<unsigned(grid), kThreads, kSmemBytes, ctx->stream>>>(
      const_cast<float2*>(reinterpret_cast<const float2*>(state)), a);
  QSG_LAUNCHED(ctx);
  rc = reduce_partials_d2(ctx, a.ev_partial, grid, out_re_im);  // synchronises
  if (rc) return rc;
  int ovf = 0;
  QSG_CUDA(cudaMemcpy(&ovf, g_tc_ovf, sizeof(int), cudaMemcpyDeviceToHost));
  *overflow = ovf != 0;
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
  // Operands built on the host and uploaded through the context's ring
  // (asynchronous; the call does not wait for the stream).
  return apply_gate_tc_host(ctx, state, n, qs, k, matrix);
}

int qsg_apply_gate_tc2(qsg_ctx* ctx, float* state, unsigned n,
                       const unsigned* qa, unsigned ka, const float* ma,
                       const unsigned* qb, unsigned kb, const float* mb) {
  QSG_CHECK_ARG(ctx && state && ma && mb, "qsg_apply_gate_tc2: null argument");
  if (ka > 6 || kb > 6) {
    set_error("gates on more than 6 qubits are not supported");
    return QSG_ERR_UNSUPPORTED;
  }
  QSG_CHECK_ARG(valid_qubits(qa, ka, n) && valid_qubits(qb, kb, n),
                "qsg_apply_gate_tc2: bad qubits");
  if (n < unsigned(tc::kTileBits)) {
    set_error("tensor-core path needs n >= %d qubits", tc::kTileBits);
    return QSG_ERR_UNSUPPORTED;
  }
  return apply_gate_tc2_host(ctx, state, n, qa, ka, ma, qb, kb, mb);
}

int qsg_expectation_value_tc(qsg_ctx* ctx, const float* state, unsigned n,
                             const unsigned* qs, unsigned k,
                             const float* matrix, double* out_re_im) {
  QSG_CHECK_ARG(ctx && state && matrix && out_re_im,
                "qsg_expectation_value_tc: null argument");
  QSG_CHECK_ARG(k >= 1 && k <= 6 && valid_qubits(qs, k, n),
                "qsg_expectation_value_tc: bad qubits");
  bool overflow = false;
  const int rc = expectation_tc(ctx, state, n, qs, k, matrix, out_re_im,
                                &overflow);
  if (rc == QSG_OK && overflow) {
    set_error("qsg_expectation_value_tc: an amplitude exceeds the range of "
              "the tensor-core split (|psi_i| > 4)");
    return QSG_ERR_UNSUPPORTED;
  }
  return rc;
}

int qsg_tc_error(qsg_ctx* ctx, int* out) {
  QSG_CHECK_ARG(ctx && out, "qsg_tc_error: null argument");
  return tc_check_error(ctx, out);
}

int qsg_tc_stall_test(qsg_ctx* ctx, float* state, unsigned n,
                      long long wait_cycles) {
  QSG_CHECK_ARG(ctx && state, "qsg_tc_stall_test: null argument");
  QSG_CHECK_ARG(wait_cycles >= 1000 && wait_cycles <= tc::kWaitCycles,
                "qsg_tc_stall_test: wait budget %lld out of [1000, %lld]",
                wait_cycles, tc::kWaitCycles);
  QSG_CHECK_ARG(n >= unsigned(tc::kTileBits) && n <= 24,
                "qsg_tc_stall_test: %u qubits (12..24)", n);
  // The identity on qubits 0..5: had an MMA run, the state would not change.
  std::vector<float> eye(2 * 64 * 64, 0.f);
  for (int i = 0; i < 64; ++i) eye[2 * (i * 64 + i)] = 1.f;
  const unsigned qs[6] = {0, 1, 2, 3, 4, 5};
  int before = 0;
  int rc = tc_check_error(ctx, &before);   // clears an older flag
  if (rc) return rc;
  g_tc_wait_cycles = wait_cycles;
  g_tc_stall = 1;
  rc = apply_gate_tc_host(ctx, state, n, qs, 6, eye.data());
  g_tc_wait_cycles = tc::kWaitCycles;
  g_tc_stall = 0;
  if (rc) return rc;
  int err = 0;
  rc = tc_check_error(ctx, &err);
  if (rc) return rc;
  if (err) {
    set_error("tensor-core kernel: a bounded wait gave up (test stall)");
    return QSG_ERR_TIMEOUT;
  }
  return QSG_OK;
}

}  // extern "C"
