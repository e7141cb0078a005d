// Host planning and launch of the tile kernels for ApplyGate,
// ApplyControlledGate and ExpectationValue (lib/simulator_cuda.h:70-260).

#include <algorithm>
#include <cmath>
#include <atomic>
#include <cstring>
#include <vector>

#include "gate_tile.cuh"
#include "internal.h"
#include "matring.cuh"

namespace qsg {

// Builds the tile geometry of a (controlled) gate.  `pair` selects pair mode
// (qubit 0 is not a target).  Returns false on inconsistent input.
bool plan_tile(unsigned n, const unsigned* qs, unsigned k,
               const unsigned* cqs, unsigned c, uint64_t cvals, bool pair,
               int log_items, TileGeom& g) {
  std::memset(&g, 0, sizeof(g));
  unsigned tb = std::min<unsigned>(n, log_items + k + (pair ? 1 : 0));
  unsigned h = 0, b = tb;
  for (h = 0; h <= k; ++h) {
    b = tb - h;
    unsigned cnt = 0;
    for (unsigned j = 0; j < k; ++j) cnt += qs[j] >= b;
    if (cnt == h) break;
  }
  if (h > k || b < 1) return false;
  g.tb = tb;
  g.b = b;
  g.h = h;
  g.items = 1u << (tb - k - (pair ? 1 : 0));

  unsigned tpos[kMaxTargets];
  for (unsigned j = 0; j < k; ++j) {
    tpos[j] = qs[j] < b ? qs[j] : b + (j - (k - h));
  }
  std::vector<unsigned> ins;
  for (unsigned j = k - h; j < k; ++j) ins.push_back(qs[j]);
  unsigned chigh = 0;
  for (unsigned i = 0; i < c; ++i) {
    uint64_t bit = (cvals >> i) & 1;
    if (cqs[i] < b) {
      g.cmask_low |= uint64_t{1} << cqs[i];
      g.cvals_low |= bit << cqs[i];
    } else {
      g.cvals_high |= bit << cqs[i];
      ins.push_back(cqs[i]);
      ++chigh;
    }
  }
  std::sort(ins.begin(), ins.end());
  g.n_ins = ins.size();
  for (size_t i = 0; i < ins.size(); ++i) g.ins_pos[i] = ins[i];
  if (n < tb + chigh) return false;
  g.num_tiles = uint64_t{1} << (n - tb - chigh);

  for (unsigned r = 0; r < (1u << h); ++r) {
    uint64_t off = 0;
    for (unsigned i = 0; i < h; ++i) {
      if ((r >> i) & 1) off |= uint64_t{1} << qs[k - h + i];
    }
    g.run_off[r] = off;
  }

  std::vector<unsigned> skip{0};
  for (unsigned j = 0; j < k; ++j) {
    if (tpos[j] != 0) skip.push_back(tpos[j]);
  }
  std::sort(skip.begin(), skip.end());
  g.n_item_skip = skip.size();
  for (size_t i = 0; i < skip.size(); ++i) g.item_skip[i] = skip[i];

  for (unsigned m = 0; m < (1u << k); ++m) {
    uint32_t off = 0;
    for (unsigned j = 0; j < k; ++j) {
      if ((m >> j) & 1) off |= 1u << tpos[j];
    }
    g.moff[m] = off;
  }

  // Swizzle: the three lowest item-free tile positions f vary across the
  // 8 lanes of a 128-bit shared-memory phase.  Positions f <= 3 land on
  // distinct unit bits 0..2 by themselves; each f >= 4 is XORed onto a unit
  // bit 0..2 held by a target (those bits are not item-free).
  std::vector<unsigned> srcs, dsts;
  unsigned found = 0;
  for (unsigned p = 1; p < tb && found < 3; ++p) {
    if (std::find(skip.begin(), skip.end(), p) != skip.end()) continue;
    ++found;
    if (p >= 4) srcs.push_back(p - 1);
  }
  for (unsigned j = 0; j < k; ++j) {
    if (tpos[j] >= 1 && tpos[j] <= 3) dsts.push_back(tpos[j] - 1);
  }
  g.n_sw = std::min(srcs.size(), dsts.size());
  for (unsigned i = 0; i < g.n_sw; ++i) {
    g.sw_src[i] = srcs[i];
    g.sw_dst[i] = dsts[i];
  }
  return true;
}

// One-time set-up of a tile-kernel instantiation: the shared-memory opt-in
// (static shared memory adds to the dynamic size, so it is raised for every
// instantiation) and the occupancy that sizes the persistent grid.  Done
// before any graph capture by apply_gate_prepare.
template <int K, bool PAIR, int MODE>
static int tile_setup(int* occupancy) {
  // Host threads driving separate streams may race here; the set-up is
  // idempotent and the result is published once it is complete.
  static std::atomic<int> o{0};
  int cur = o.load(std::memory_order_acquire);
  if (cur == 0) {
    auto kern = gate_tile_kernel<K, PAIR, MODE>;
    const size_t smem = TileShape<K, PAIR>::SMEM;
    QSG_CUDA(cudaFuncSetAttribute(
        kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int v = 0;
    QSG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &v, kern, kTileThreads, smem));
    cur = v < 1 ? 1 : v;
    o.store(cur, std::memory_order_release);
  }
  *occupancy = cur;
  return QSG_OK;
}

template <int K, bool PAIR, int MODE>
static int launch_tile(qsg_ctx* ctx, float* state, unsigned n,
                       const unsigned* qs, const unsigned* cqs, unsigned c,
                       uint64_t cvals, const float* matrix,
                       const float* dev_matrix, double* out_re_im) {
  using SH = TileShape<K, PAIR>;
  GateArgs<K> a;
  if (!plan_tile(n, qs, K, cqs, c, cvals, PAIR, SH::LOG_ITEMS, a.g)) {
    set_error("tile planning failed (n=%u, k=%d)", n, K);
    return QSG_ERR_INVALID;
  }
  if constexpr (K <= 5) {
    std::memcpy(a.m, matrix, sizeof(a.m));
    a.mat = nullptr;
  } else if (dev_matrix) {
    a.mat = reinterpret_cast<const float2*>(dev_matrix);
  } else {
    const float* dm = nullptr;
    int rc = matring_upload(ctx, matrix, 2 * (1 << (2 * K)), &dm);
    if (rc) return rc;
    a.mat = reinterpret_cast<const float2*>(dm);
  }

  auto kern = gate_tile_kernel<K, PAIR, MODE>;
  const size_t smem = SH::SMEM;
  int o = 0;
  int rc0 = tile_setup<K, PAIR, MODE>(&o);
  if (rc0) return rc0;
  uint64_t grid = std::min<uint64_t>(a.g.num_tiles,
                                     uint64_t(ctx->num_sms) * uint64_t(o));
  if (grid < 1) grid = 1;

  double2* partial = nullptr;
  if (MODE >= 1) {
    void* p = nullptr;
    int rc = get_scratch(ctx, (grid + 1) * sizeof(double2), &p);
    if (rc) return rc;
    partial = static_cast<double2*>(p);
  }
  kern<<<(unsigned)grid, kTileThreads, smem, ctx->stream>>>(
      reinterpret_cast<float4*>(state), a, partial);
  QSG_LAUNCHED(ctx);

  if (MODE >= 1) {
    return reduce_partials_d2(ctx, partial, grid, out_re_im);
  }
  return QSG_OK;
}

template <int MODE>
static int dispatch(qsg_ctx* ctx, float* state, unsigned n,
                    const unsigned* qs, unsigned k, const unsigned* cqs,
                    unsigned c, uint64_t cvals, const float* matrix,
                    double* out, const float* dev_matrix = nullptr) {
  // A 0-qubit state is handled as a 1-qubit state whose amplitude 1 is the
  // zero padding of the buffer.
  unsigned ne = n == 0 ? 1 : n;
  bool pair = (k == 0) || qs[0] != 0;
#define QSG_CASE(KK)                                                         \
  case KK:                                                                   \
    if (pair)                                                                \
      return launch_tile<KK, true, MODE>(ctx, state, ne, qs, cqs, c, cvals,  \
                                         matrix, dev_matrix, out);           \
    if constexpr (KK > 0)                                                    \
      return launch_tile<KK, false, MODE>(ctx, state, ne, qs, cqs, c, cvals, \
                                          matrix, dev_matrix, out);          \
    break;
  switch (k) {
    QSG_CASE(0)
    QSG_CASE(1)
    QSG_CASE(2)
    QSG_CASE(3)
    QSG_CASE(4)
    QSG_CASE(5)
    QSG_CASE(6)
    default:
      break;
  }
#undef QSG_CASE
  set_error("gates on %u qubits are not supported (maximum 6)", k);
  return QSG_ERR_UNSUPPORTED;
}

// ExpectationValue of a Hermitian matrix on 1..3 qubits: the tile kernel's
// MODE 2 (the upper triangle of the matrix, half the products of MODE 1).
static int dispatch_hermitian_ev(qsg_ctx* ctx, const float* state, unsigned n,
                                 const unsigned* qs, unsigned k,
                                 const float* matrix, double* out) {
  float* s = const_cast<float*>(state);
  const bool pair = qs[0] != 0;
#define QSG_HCASE(KK)                                                          \
  case KK:                                                                     \
    return pair ? launch_tile<KK, true, 2>(ctx, s, n, qs, nullptr, 0, 0,        \
                                           matrix, nullptr, out)               \
                : launch_tile<KK, false, 2>(ctx, s, n, qs, nullptr, 0, 0,       \
                                            matrix, nullptr, out);
  switch (k) {
    QSG_HCASE(1)
    QSG_HCASE(2)
    QSG_HCASE(3)
    default:
      break;
  }
#undef QSG_HCASE
  set_error("Hermitian expectation values take 1..3 qubits (got %u)", k);
  return QSG_ERR_UNSUPPORTED;
}

// m == m^dagger exactly (FP32 entries).
static bool is_hermitian(const float* m, unsigned k) {
  const unsigned d = 1u << k;
  for (unsigned r = 0; r < d; ++r)
    for (unsigned c = r; c < d; ++c) {
      const float* a = m + 2 * (r * d + c);
      const float* b = m + 2 * (c * d + r);
      if (a[0] != b[0] || a[1] != -b[1]) return false;
    }
  return true;
}

int apply_gate_prepare(unsigned k, bool pair, int mode) {
  int o = 0;
#define QSG_PREP(KK)                                                   \
  case KK:                                                             \
    if (pair)                                                          \
      return mode ? tile_setup<KK, true, 1>(&o) : tile_setup<KK, true, 0>(&o); \
    if constexpr (KK > 0)                                              \
      return mode ? tile_setup<KK, false, 1>(&o)                       \
                  : tile_setup<KK, false, 0>(&o);                      \
    return QSG_OK;
  switch (k) {
    QSG_PREP(0)
    QSG_PREP(1)
    QSG_PREP(2)
    QSG_PREP(3)
    QSG_PREP(4)
    QSG_PREP(5)
    QSG_PREP(6)
    default:
      return QSG_ERR_UNSUPPORTED;
  }
#undef QSG_PREP
}

int apply_gate_ex(qsg_ctx* ctx, float* state, unsigned n, const unsigned* qs,
                  unsigned k, const unsigned* cqs, unsigned c, uint64_t cvals,
                  const float* host_matrix, const float* dev_matrix) {
  if (k > kMaxTargets) {
    set_error("gates on %u qubits are not supported (maximum 6)", k);
    return QSG_ERR_UNSUPPORTED;
  }
  uint64_t cv = c == 0 ? 0 : (c < 64 ? (cvals & ((uint64_t{1} << c) - 1)) : cvals);
  return dispatch<0>(ctx, state, n, qs, k, c ? cqs : nullptr, c, cv,
                     host_matrix, nullptr, dev_matrix);
}

}  // namespace qsg

using namespace qsg;

extern "C" {

int qsg_apply_gate(qsg_ctx* ctx, float* state, unsigned n, const unsigned* qs,
                   unsigned k, const float* matrix) {
  QSG_CHECK_ARG(ctx && state && matrix, "qsg_apply_gate: null argument");
  QSG_CHECK_ARG(n <= kMaxQubits, "qsg_apply_gate: too many qubits");
  if (k > kMaxTargets) {
    set_error("gates on %u qubits are not supported (maximum 6)", k);
    return QSG_ERR_UNSUPPORTED;
  }
  QSG_CHECK_ARG(valid_qubits(qs, k, n),
                "qsg_apply_gate: qubits must be sorted, distinct and < %u", n);
  return dispatch<0>(ctx, state, n, qs, k, nullptr, 0, 0, matrix, nullptr);
}

int qsg_apply_controlled_gate(qsg_ctx* ctx, float* state, unsigned n,
                              const unsigned* qs, unsigned k,
                              const unsigned* cqs, unsigned c, uint64_t cvals,
                              const float* matrix) {
  QSG_CHECK_ARG(ctx && state && matrix, "qsg_apply_controlled_gate: null");
  QSG_CHECK_ARG(n <= kMaxQubits, "qsg_apply_controlled_gate: too many qubits");
  if (k > kMaxTargets) {
    set_error("gates on %u qubits are not supported (maximum 6)", k);
    return QSG_ERR_UNSUPPORTED;
  }
  QSG_CHECK_ARG(valid_qubits(qs, k, n), "qsg_apply_controlled_gate: bad qs");
  QSG_CHECK_ARG(valid_qubits(cqs, c, n), "qsg_apply_controlled_gate: bad cqs");
  for (unsigned i = 0; i < c; ++i)
    for (unsigned j = 0; j < k; ++j)
      QSG_CHECK_ARG(cqs[i] != qs[j],
                    "qsg_apply_controlled_gate: qubit %u is both target and "
                    "control", qs[j]);
  if (c == 0) {
    return dispatch<0>(ctx, state, n, qs, k, nullptr, 0, 0, matrix, nullptr);
  }
  uint64_t cv = c < 64 ? (cvals & ((uint64_t{1} << c) - 1)) : cvals;
  return dispatch<0>(ctx, state, n, qs, k, cqs, c, cv, matrix, nullptr);
}

// Smallest dense ExpectationValue taken by the tensor cores.
constexpr unsigned kTcEvMinK = 4;

int qsg_expectation_value(qsg_ctx* ctx, const float* state, unsigned n,
                          const unsigned* qs, unsigned k, const float* matrix,
                          double* out_re_im) {
  QSG_CHECK_ARG(ctx && state && matrix && out_re_im,
                "qsg_expectation_value: null argument");
  QSG_CHECK_ARG(n <= kMaxQubits, "qsg_expectation_value: too many qubits");
  if (k == 0 || k > kMaxTargets) {
    set_error("expectation values need 1..6 qubits (got %u)", k);
    return QSG_ERR_UNSUPPORTED;
  }
  QSG_CHECK_ARG(valid_qubits(qs, k, n), "qsg_expectation_value: bad qs");
  // Pauli strings and other monomial operators: one read pass.
  uint32_t xm = 0;
  float d[2 * 64];
  if (monomial_xor(k, matrix, &xm, d))
    return expectation_monomial(ctx, state, n, qs, k, xm, d, out_re_im);
  // Dense operators of >= 4 qubits on the tensor cores: one read of the
  // state at any k (30 qubits, GB300: 2.5 ms against 3.2, 6.0 and 11.3 ms
  // on the CUDA cores for k = 4, 5, 6; k <= 3 stays on the CUDA cores).
  // A state with amplitudes too large for the split (|psi_i| > 4, e.g.
  // after Multiply) falls back to the CUDA cores.
  float mmax = 0.f;
  for (unsigned i = 0; i < 2u << (2 * k); ++i)
    mmax = std::max(mmax, std::fabs(matrix[i]));
  if (k >= kTcEvMinK && n >= 12 && mmax <= 4096.f) {
    bool overflow = false;
    const int rc = expectation_tc(ctx, state, n, qs, k, matrix, out_re_im,
                                  &overflow);
    if (rc != QSG_OK || !overflow) return rc;
  }
  // Hermitian operators of <= 3 qubits (observables): half the products.
  if (k <= 3 && is_hermitian(matrix, k))
    return dispatch_hermitian_ev(ctx, state, n, qs, k, matrix, out_re_im);
  return dispatch<1>(ctx, const_cast<float*>(state), n, qs, k, nullptr, 0, 0,
                     matrix, out_re_im);
}

}  // extern "C"
