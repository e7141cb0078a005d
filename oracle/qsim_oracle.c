/*
 * qsim_oracle.c — TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the reference's state-vector algorithms, used as the
 * parity checker by tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg.  Nothing in the engine links or calls this file.
 *
 * Every function cites the reference code it follows (paths within
 * quantumlib/qsim).  The state is interleaved complex (re, im) in double
 * (FP64 oracle, as SimulatorBasic<For, double>) or float (the FP32 port used
 * as the timed CPU baseline, multi-threaded with OpenMP like the reference's
 * ParallelFor, lib/parfor.h:44-100).
 *
 * Pinning: tests/test_oracle_golden.py checks these functions against
 * golden outputs of the reference itself (tests/golden/, made by
 * oracle/ref_driver.cc compiled against the reference headers).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* ---- bit helpers: lib/bits.h:29-81 (ExpandBits = pdep) ---------------- */
static uint64_t expand_bits(uint64_t bits, unsigned n, uint64_t mask) {
  uint64_t e = 0;
  unsigned k = 0;
  for (unsigned i = 0; i < n; ++i) {
    if ((mask >> i) & 1) {
      e |= ((bits >> k) & 1) << i;
      ++k;
    }
  }
  return e;
}

/* Group base index: insert zero bits at the target positions
 * (lib/simulator.h:39-67 FillIndices, ms[] masks). */
static uint64_t group_base(uint64_t i, const unsigned* qs, unsigned k) {
  for (unsigned j = 0; j < k; ++j) {
    uint64_t lo = i & ((UINT64_C(1) << qs[j]) - 1);
    i = lo | ((i ^ lo) << 1);
  }
  return i;
}

static void member_offsets(const unsigned* qs, unsigned k, uint64_t* xss) {
  for (unsigned m = 0; m < (1u << k); ++m) {
    uint64_t a = 0;
    for (unsigned j = 0; j < k; ++j)
      if ((m >> j) & 1) a |= UINT64_C(1) << qs[j];
    xss[m] = a;
  }
}

/* ---- FP64 gate application: lib/simulator_basic.h:172-232 ------------- */
void orc_apply_gate_f64(double* s, unsigned n, const unsigned* qs, unsigned k,
                        const double* m) {
  const unsigned D = 1u << k;
  uint64_t xss[64];
  member_offsets(qs, k, xss);
  const uint64_t groups = UINT64_C(1) << (n - k);
#pragma omp parallel for schedule(static)
  for (int64_t g = 0; g < (int64_t)groups; ++g) {
    uint64_t b = group_base((uint64_t)g, qs, k);
    double vr[64], vi[64];
    for (unsigned c = 0; c < D; ++c) {
      vr[c] = s[2 * (b + xss[c])];
      vi[c] = s[2 * (b + xss[c]) + 1];
    }
    for (unsigned r = 0; r < D; ++r) {
      double ar = 0, ai = 0;
      for (unsigned c = 0; c < D; ++c) {
        double mr = m[2 * (r * D + c)], mi = m[2 * (r * D + c) + 1];
        ar += mr * vr[c] - mi * vi[c];
        ai += mr * vi[c] + mi * vr[c];
      }
      s[2 * (b + xss[r])] = ar;
      s[2 * (b + xss[r]) + 1] = ai;
    }
  }
}

/* lib/simulator_basic.h:234-292 with GetMasks7 (lib/simulator.h:364-375):
 * cvals bit i <-> cqs[i]. */
void orc_apply_controlled_gate_f64(double* s, unsigned n, const unsigned* qs,
                                   unsigned k, const unsigned* cqs, unsigned c,
                                   uint64_t cvals, const double* m) {
  uint64_t cmask = 0;
  for (unsigned i = 0; i < c; ++i) cmask |= UINT64_C(1) << cqs[i];
  const uint64_t cvalsh = expand_bits(cvals, n, cmask);
  const unsigned D = 1u << k;
  uint64_t xss[64];
  member_offsets(qs, k, xss);
  const uint64_t groups = UINT64_C(1) << (n - k);
#pragma omp parallel for schedule(static)
  for (int64_t g = 0; g < (int64_t)groups; ++g) {
    uint64_t b = group_base((uint64_t)g, qs, k);
    if ((b & cmask) != cvalsh) continue;
    double vr[64], vi[64];
    for (unsigned cc = 0; cc < D; ++cc) {
      vr[cc] = s[2 * (b + xss[cc])];
      vi[cc] = s[2 * (b + xss[cc]) + 1];
    }
    for (unsigned r = 0; r < D; ++r) {
      double ar = 0, ai = 0;
      for (unsigned cc = 0; cc < D; ++cc) {
        double mr = m[2 * (r * D + cc)], mi = m[2 * (r * D + cc) + 1];
        ar += mr * vr[cc] - mi * vi[cc];
        ai += mr * vi[cc] + mi * vr[cc];
      }
      s[2 * (b + xss[r])] = ar;
      s[2 * (b + xss[r]) + 1] = ai;
    }
  }
}

/* lib/simulator_basic.h:294-343: sum over groups of v^dagger (M v). */
void orc_expectation_value_f64(const double* s, unsigned n, const unsigned* qs,
                               unsigned k, const double* m, double* out) {
  const unsigned D = 1u << k;
  uint64_t xss[64];
  member_offsets(qs, k, xss);
  const uint64_t groups = UINT64_C(1) << (n - k);
  double er = 0, ei = 0;
#pragma omp parallel for schedule(static) reduction(+ : er, ei)
  for (int64_t g = 0; g < (int64_t)groups; ++g) {
    uint64_t b = group_base((uint64_t)g, qs, k);
    double vr[64], vi[64];
    for (unsigned c = 0; c < D; ++c) {
      vr[c] = s[2 * (b + xss[c])];
      vi[c] = s[2 * (b + xss[c]) + 1];
    }
    for (unsigned r = 0; r < D; ++r) {
      double ar = 0, ai = 0;
      for (unsigned c = 0; c < D; ++c) {
        double mr = m[2 * (r * D + c)], mi = m[2 * (r * D + c) + 1];
        ar += mr * vr[c] - mi * vi[c];
        ai += mr * vi[c] + mi * vr[c];
      }
      er += vr[r] * ar + vi[r] * ai;
      ei += vr[r] * ai - vi[r] * ar;
    }
  }
  out[0] = er;
  out[1] = ei;
}

/* ---- FP32 port (timed CPU baseline), same loop structure -------------- */
void orc_apply_gate_f32(float* s, unsigned n, const unsigned* qs, unsigned k,
                        const float* m) {
  const unsigned D = 1u << k;
  uint64_t xss[64];
  member_offsets(qs, k, xss);
  const uint64_t groups = UINT64_C(1) << (n - k);
#pragma omp parallel for schedule(static)
  for (int64_t g = 0; g < (int64_t)groups; ++g) {
    uint64_t b = group_base((uint64_t)g, qs, k);
    float vr[64], vi[64];
    for (unsigned c = 0; c < D; ++c) {
      vr[c] = s[2 * (b + xss[c])];
      vi[c] = s[2 * (b + xss[c]) + 1];
    }
    for (unsigned r = 0; r < D; ++r) {
      float ar = 0, ai = 0;
      for (unsigned c = 0; c < D; ++c) {
        float mr = m[2 * (r * D + c)], mi = m[2 * (r * D + c) + 1];
        ar += mr * vr[c] - mi * vi[c];
        ai += mr * vi[c] + mi * vr[c];
      }
      s[2 * (b + xss[r])] = ar;
      s[2 * (b + xss[r]) + 1] = ai;
    }
  }
}

/* ---- lane-batched gate application ------------------------------------
 * The reference's SIMD simulators (lib/simulator_avx512.h,
 * lib/simulator_neon.h, lib/simulator_sse.h: ApplyGateH / ApplyGateL) hold
 * the same amplitude of several consecutive groups in one vector register
 * and multiply the gate matrix into 2^k such registers at once.  This is the
 * portable restatement of that scheme: LANES consecutive groups at a time,
 * the group amplitudes held as LANES-wide real and imaginary rows, and the
 * matrix-vector product written as loops over the lanes that the C
 * compiler vectorises (NEON on Arm, SSE/AVX on x86).  When the lowest
 * target qubit is >= log2(LANES) the LANES groups are LANES consecutive
 * amplitudes of every member (the reference's H case); otherwise their
 * indices are gathered (the reference permutes inside registers, its L
 * case).  The per-row sum runs over the columns in order, as in orc_apply_gate_f64.
 * FP64: the oracle's fast path for large states.  FP32: the timed CPU
 * baseline ("port").  Multi-threaded over group chunks like the
 * reference's ParallelFor (lib/parfor.h:44-100). */
#define ORC_LANES 16
#define ORC_LANE_BITS 4 /* log2(ORC_LANES) */

#define ORC_DEFINE_LANE_APPLY(T, NAME)                                        \
  static inline __attribute__((always_inline)) void NAME##_body(             \
      T* s, unsigned n, const unsigned* qs, const unsigned k, const T* m) {  \
    const unsigned D = 1u << k;                                              \
    uint64_t xss[64];                                                        \
    member_offsets(qs, k, xss);                                              \
    const uint64_t groups = UINT64_C(1) << (n - k);                          \
    const int contiguous = (k == 0) || qs[0] >= ORC_LANE_BITS;               \
    _Pragma("omp parallel for schedule(static)")                             \
    for (int64_t g0 = 0; g0 < (int64_t)groups; g0 += ORC_LANES) {            \
      uint64_t base[ORC_LANES];                                              \
      T vr[64][ORC_LANES], vi[64][ORC_LANES];                                \
      for (unsigned l = 0; l < ORC_LANES; ++l)                               \
        base[l] = group_base((uint64_t)g0 + l, qs, k);                       \
      if (contiguous) {                                                      \
        for (unsigned c = 0; c < D; ++c) {                                   \
          const T* p = s + 2 * (base[0] + xss[c]);                           \
          for (unsigned l = 0; l < ORC_LANES; ++l) {                         \
            vr[c][l] = p[2 * l];                                             \
            vi[c][l] = p[2 * l + 1];                                         \
          }                                                                  \
        }                                                                    \
      } else {                                                               \
        for (unsigned c = 0; c < D; ++c)                                     \
          for (unsigned l = 0; l < ORC_LANES; ++l) {                         \
            vr[c][l] = s[2 * (base[l] + xss[c])];                            \
            vi[c][l] = s[2 * (base[l] + xss[c]) + 1];                        \
          }                                                                  \
      }                                                                      \
      for (unsigned r = 0; r < D; ++r) {                                     \
        T ar[ORC_LANES], ai[ORC_LANES];                                      \
        for (unsigned l = 0; l < ORC_LANES; ++l) ar[l] = ai[l] = 0;          \
        for (unsigned c = 0; c < D; ++c) {                                   \
          const T mr = m[2 * (r * D + c)], mi = m[2 * (r * D + c) + 1];      \
          for (unsigned l = 0; l < ORC_LANES; ++l) {                         \
            ar[l] += mr * vr[c][l] - mi * vi[c][l];                          \
            ai[l] += mr * vi[c][l] + mi * vr[c][l];                          \
          }                                                                  \
        }                                                                    \
        if (contiguous) {                                                    \
          T* p = s + 2 * (base[0] + xss[r]);                                 \
          for (unsigned l = 0; l < ORC_LANES; ++l) {                         \
            p[2 * l] = ar[l];                                                \
            p[2 * l + 1] = ai[l];                                            \
          }                                                                  \
        } else {                                                             \
          for (unsigned l = 0; l < ORC_LANES; ++l) {                         \
            s[2 * (base[l] + xss[r])] = ar[l];                               \
            s[2 * (base[l] + xss[r]) + 1] = ai[l];                           \
          }                                                                  \
        }                                                                    \
      }                                                                      \
    }                                                                        \
  }

ORC_DEFINE_LANE_APPLY(double, lanes_f64)
ORC_DEFINE_LANE_APPLY(float, lanes_f32)

/* Dispatch on k so that every loop bound above is a compile-time constant.
 * States with fewer than ORC_LANES groups take the one-group loops. */
void orc_apply_gate_lanes_f64(double* s, unsigned n, const unsigned* qs,
                              unsigned k, const double* m) {
  if (k > 6 || n < k + ORC_LANE_BITS) {
    orc_apply_gate_f64(s, n, qs, k, m);
    return;
  }
  switch (k) {
    case 0: lanes_f64_body(s, n, qs, 0, m); break;
    case 1: lanes_f64_body(s, n, qs, 1, m); break;
    case 2: lanes_f64_body(s, n, qs, 2, m); break;
    case 3: lanes_f64_body(s, n, qs, 3, m); break;
    case 4: lanes_f64_body(s, n, qs, 4, m); break;
    case 5: lanes_f64_body(s, n, qs, 5, m); break;
    default: lanes_f64_body(s, n, qs, 6, m); break;
  }
}

void orc_apply_gate_f32(float* s, unsigned n, const unsigned* qs, unsigned k,
                        const float* m);

void orc_port_apply_gate_f32(float* s, unsigned n, const unsigned* qs,
                             unsigned k, const float* m) {
  if (k > 6 || n < k + ORC_LANE_BITS) {
    orc_apply_gate_f32(s, n, qs, k, m);
    return;
  }
  switch (k) {
    case 0: lanes_f32_body(s, n, qs, 0, m); break;
    case 1: lanes_f32_body(s, n, qs, 1, m); break;
    case 2: lanes_f32_body(s, n, qs, 2, m); break;
    case 3: lanes_f32_body(s, n, qs, 3, m); break;
    case 4: lanes_f32_body(s, n, qs, 4, m); break;
    case 5: lanes_f32_body(s, n, qs, 5, m); break;
    default: lanes_f32_body(s, n, qs, 6, m); break;
  }
}

/* ---- FP32-state reductions of the CPU port ----------------------------
 * StateSpace::Norm (lib/statespace_basic.h:144-160: FP32 products, double
 * sums), Multiply (:125-142) and the one-qubit diagonal ExpectationValue that
 * QuantumTrajectorySimulator needs for <psi|K^dagger K|psi>
 * (lib/qtrajectory.h:331-380), multi-threaded like the reference's
 * ParallelFor reductions. */
double orc_port_norm_f32(const float* s, unsigned n) {
  const int64_t N = (int64_t)1 << n;
  double acc = 0;
#pragma omp parallel for schedule(static) reduction(+ : acc)
  for (int64_t i = 0; i < N; ++i)
    acc += (double)(s[2 * i] * s[2 * i] + s[2 * i + 1] * s[2 * i + 1]);
  return acc;
}

void orc_port_scale_f32(float* s, unsigned n, float a) {
  const int64_t N = (int64_t)2 << n;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < N; ++i) s[i] *= a;
}

/* sum_i |s_i|^2 d[bit q of i] */
double orc_port_diag1_ev_f32(const float* s, unsigned n, unsigned q,
                             double d0, double d1) {
  const int64_t N = (int64_t)1 << n;
  double a0 = 0, a1 = 0;
#pragma omp parallel for schedule(static) reduction(+ : a0, a1)
  for (int64_t i = 0; i < N; ++i) {
    const double p =
        (double)(s[2 * i] * s[2 * i] + s[2 * i + 1] * s[2 * i + 1]);
    if ((i >> q) & 1)
      a1 += p;
    else
      a0 += p;
  }
  return d0 * a0 + d1 * a1;
}

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void orc_set_num_threads(int t) {
#ifdef _OPENMP
  if (t > 0) omp_set_num_threads(t);
#else
  (void)t;
#endif
}

/* ---- reductions: lib/statespace_basic.h:144-180, 270-286 -------------- */
double orc_norm_f64(const double* s, unsigned n) {
  const uint64_t N = UINT64_C(1) << n;
  double acc = 0;
  for (uint64_t i = 0; i < N; ++i) acc += s[2 * i] * s[2 * i] + s[2 * i + 1] * s[2 * i + 1];
  return acc;
}

void orc_inner_product_f64(const double* a, const double* b, unsigned n,
                           double* out) {
  const uint64_t N = UINT64_C(1) << n;
  double re = 0, im = 0;
  for (uint64_t i = 0; i < N; ++i) {
    re += a[2 * i] * b[2 * i] + a[2 * i + 1] * b[2 * i + 1];
    im += a[2 * i] * b[2 * i + 1] - a[2 * i + 1] * b[2 * i];
  }
  out[0] = re;
  out[1] = im;
}

/* ---- std::mt19937 (Matsumoto & Nishimura 1998; ISO C++ [rand.eng.mers])
 * and libstdc++ generate_canonical<double, 53> with a 32-bit engine
 * (two draws, (g1 + g2 * 2^32) / 2^64, clamped below 1). ----------------- */
typedef struct {
  uint32_t mt[624];
  int idx;
} orc_mt19937;

void orc_mt_seed(orc_mt19937* g, uint32_t seed) {
  g->mt[0] = seed;
  for (int i = 1; i < 624; ++i)
    g->mt[i] = 1812433253u * (g->mt[i - 1] ^ (g->mt[i - 1] >> 30)) + (uint32_t)i;
  g->idx = 624;
}

uint32_t orc_mt_next(orc_mt19937* g) {
  if (g->idx >= 624) {
    for (int i = 0; i < 624; ++i) {
      uint32_t y = (g->mt[i] & 0x80000000u) | (g->mt[(i + 1) % 624] & 0x7fffffffu);
      g->mt[i] = g->mt[(i + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    }
    g->idx = 0;
  }
  uint32_t y = g->mt[g->idx++];
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return y;
}

double orc_canonical(orc_mt19937* g) {
  double sum = (double)orc_mt_next(g);
  sum += (double)orc_mt_next(g) * 4294967296.0;
  double r = sum / 18446744073709551616.0;
  if (r >= 1.0) r = nextafter(1.0, 0.0);
  return r;
}

size_t orc_mt_size(void) { return sizeof(orc_mt19937); }

/* uniform_real_distribution<double>(0, max)(g) */
double orc_uniform(orc_mt19937* g, double max_value) {
  return orc_canonical(g) * (max_value - 0.0) + 0.0;
}

static int cmp_double(const void* a, const void* b) {
  double x = *(const double*)a, y = *(const double*)b;
  return (x > y) - (x < y);
}

static int cmp_float(const void* a, const void* b) {
  float x = *(const float*)a, y = *(const float*)b;
  return (x > y) - (x < y);
}

/* lib/util.h:67-85 GenerateRandomValues: m draws of
 * uniform_real_distribution<double>(0, max) from mt19937(seed), sorted. */
void orc_generate_random_values(uint64_t m, uint32_t seed, double max_value,
                                double* out) {
  orc_mt19937 g;
  orc_mt_seed(&g, seed);
  for (uint64_t i = 0; i < m; ++i) out[i] = orc_uniform(&g, max_value);
  qsort(out, m, sizeof(double), cmp_double);
}

/* GenerateRandomValues<float> (lib/util.h:67-85): m draws of libstdc++'s
 * uniform_real_distribution<float>(0, max) from mt19937(seed), i.e.
 * generate_canonical<float, 24> from one 32-bit draw, (float(g) / 2^32)
 * clamped below 1, times max in float; sorted. */
void orc_generate_random_values_f32(uint64_t m, uint32_t seed, float max_value,
                                    float* out) {
  orc_mt19937 g;
  orc_mt_seed(&g, seed);
  for (uint64_t i = 0; i < m; ++i) {
    float c = (float)orc_mt_next(&g) / 4294967296.0f;
    if (c >= 1.0f) c = nextafterf(1.0f, 0.0f);
    out[i] = c * (max_value - 0.0f) + 0.0f;
  }
  qsort(out, m, sizeof(float), cmp_float);
}

/* Sample against given sorted thresholds (FP64 CDF scan, as
 * orc_sample_f64 after its draws). */
void orc_sample_thresholds_f64(const double* s, unsigned n, uint64_t m,
                               const double* rs, uint64_t* out) {
  const uint64_t N = UINT64_C(1) << n;
  uint64_t j = 0;
  double csum = 0;
  for (uint64_t k = 0; k < N && j < m; ++k) {
    csum += s[2 * k] * s[2 * k] + s[2 * k + 1] * s[2 * k + 1];
    while (j < m && rs[j] < csum) out[j++] = k;
  }
  for (; j < m; ++j) out[j] = N - 1;
}

/* lib/statespace_basic.h:187-226 Sample: FP64 CDF scan. */
void orc_sample_f64(const double* s, unsigned n, uint64_t m, uint32_t seed,
                    uint64_t* out) {
  if (m == 0) return;
  const uint64_t N = UINT64_C(1) << n;
  double norm = 0;
  for (uint64_t k = 0; k < N; ++k) norm += s[2 * k] * s[2 * k] + s[2 * k + 1] * s[2 * k + 1];
  double* rs = (double*)malloc(m * sizeof(double));
  orc_generate_random_values(m, seed, norm, rs);
  uint64_t j = 0;
  double csum = 0;
  for (uint64_t k = 0; k < N && j < m; ++k) {
    csum += s[2 * k] * s[2 * k] + s[2 * k + 1] * s[2 * k + 1];
    while (j < m && rs[j] < csum) out[j++] = k;
  }
  for (; j < m; ++j) out[j] = N - 1;
  free(rs);
}

/* Index found by a CDF search for r over the whole state (the combined
 * effect of StateSpace::VirtualMeasure, lib/statespace.h:97-140, and
 * FindMeasuredBits, lib/statespace_basic.h:275-296). */
uint64_t orc_find_index_f64(const double* s, unsigned n, double r) {
  const uint64_t N = UINT64_C(1) << n;
  double csum = 0;
  for (uint64_t k = 0; k < N; ++k) {
    csum += s[2 * k] * s[2 * k] + s[2 * k + 1] * s[2 * k + 1];
    if (r < csum) return k;
  }
  return N - 1;
}

/* lib/statespace_basic.h:229-259 Collapse. */
void orc_collapse_f64(double* s, unsigned n, uint64_t mask, uint64_t bits) {
  const uint64_t N = UINT64_C(1) << n;
  double norm = 0;
  for (uint64_t i = 0; i < N; ++i)
    if ((i & mask) == bits) norm += s[2 * i] * s[2 * i] + s[2 * i + 1] * s[2 * i + 1];
  double renorm = 1.0 / sqrt(norm);
  for (uint64_t i = 0; i < N; ++i) {
    if ((i & mask) == bits) {
      s[2 * i] *= renorm;
      s[2 * i + 1] *= renorm;
    } else {
      s[2 * i] = 0;
      s[2 * i + 1] = 0;
    }
  }
}
