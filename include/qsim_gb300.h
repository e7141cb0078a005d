/*
 * qsim_gb300.h — C ABI of the GB300 state-vector engine.
 *
 * Every entry point is plain C: opaque context handle, raw device pointers
 * to complex64 state vectors, host pointers for matrices and results, and an
 * int status (QSG_OK == 0).  No entry point exits the process; the last
 * error message of the calling thread is available from qsg_last_error().
 *
 * State layout: amplitude i of an n-qubit state is the float pair
 * (state[2i], state[2i+1]) = (re, im), i.e. normal (interleaved) order.  A
 * state buffer holds qsg_min_size(n) floats; amplitudes past 2^n are padding
 * and are kept at zero.  Bit q of an amplitude index is qubit q.
 *
 * Gate matrices are row-major interleaved complex float arrays of
 * 2 * 4^k floats for k target qubits; row/column bit j corresponds to qs[j]
 * and qs is sorted ascending (the convention of the reference's
 * lib/matrix.h:26-33 and lib/simulator_basic.h:172-232).
 *
 * Work is issued on the context's CUDA stream.  Calls that return a value to
 * the host synchronise that stream; the others are asynchronous.
 *
 * Each declaration names the reference member it replaces (file:line within
 * quantumlib/qsim).
 */
#ifndef QSIM_GB300_H_
#define QSIM_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum {
  QSG_OK = 0,
  QSG_ERR_INVALID = 1,       /* bad argument (qubit index, size, null ptr) */
  QSG_ERR_OOM = 2,           /* device or pinned-host allocation failed    */
  QSG_ERR_CUDA = 3,          /* CUDA runtime error                         */
  QSG_ERR_UNSUPPORTED = 4,   /* e.g. more target qubits than supported     */
  QSG_ERR_SIZE_MISMATCH = 5, /* states with different qubit counts         */
  QSG_ERR_TIMEOUT = 6,       /* a bounded device-side wait gave up         */
};

typedef struct qsg_ctx qsg_ctx;

/* Message for the last failing call on this thread ("" if none). */
const char* qsg_last_error(void);
/* Library version string. */
const char* qsg_version(void);

/* ---- context ------------------------------------------------------------
 * Replaces the per-object device workspace of SimulatorCUDA
 * (lib/simulator_cuda.h:52-54, d_ws/h_ws) and StateSpaceCUDA's scratch
 * (lib/statespace_cuda.h:378-390).  `stream` may be NULL: the context then
 * creates its own non-blocking stream.  One context per host thread. */
int qsg_ctx_create(int device, void* stream, qsg_ctx** out);
int qsg_ctx_destroy(qsg_ctx* ctx);
int qsg_ctx_sync(qsg_ctx* ctx);     /* VectorSpaceCUDA::DeviceSync :162 */
int qsg_ctx_num_sms(qsg_ctx* ctx, int* out);
void* qsg_ctx_stream(qsg_ctx* ctx);

/* ---- vector space (lib/vectorspace_cuda.h) ----------------------------- */
/* StateSpaceCUDA::MinSize (lib/statespace_cuda.h:81-83), in floats. */
uint64_t qsg_min_size(unsigned num_qubits);
/* VectorSpaceCUDA::Create(n) (lib/vectorspace_cuda.h:87-96).  On OOM returns
 * QSG_ERR_OOM and *out = NULL (the reference returns Null()). */
int qsg_state_create(qsg_ctx* ctx, unsigned num_qubits, float** out);
/* VectorSpaceCUDA::Free / detail::free (lib/vectorspace_cuda.h:108-110). */
int qsg_state_free(qsg_ctx* ctx, float* state);
/* Copy overloads (lib/vectorspace_cuda.h:116-160); sizes are MinSize(n). */
int qsg_copy_d2d(qsg_ctx* ctx, float* dest, const float* src, unsigned n);
int qsg_copy_d2h(qsg_ctx* ctx, float* host_dest, const float* src, unsigned n);
int qsg_copy_h2d(qsg_ctx* ctx, float* dest, const float* host_src, unsigned n);
/* Copy(src, size, dest) (:152-160): copies min(size, MinSize(n)) floats. */
int qsg_copy_h2d_partial(qsg_ctx* ctx, float* dest, const float* host_src,
                         uint64_t size, unsigned n);

/* Page-locked host buffers for fast host<->device copies of whole states.
 * No counterpart in the reference (its copies use pageable host memory,
 * lib/vectorspace_cuda.h:116-160).  qsg_host_alloc uses cudaMallocHost.
 * qsg_host_alloc_near allocates it with the calling thread's memory policy
 * set, for the call, to prefer the host NUMA node nearest to `device`
 * (cudaDevAttrHostNumaId; preferred, not strict, so a full node falls back
 * to another one): on hosts with several CPU sockets a pinned buffer on the
 * far socket slows device<->host copies.  Where the device reports no host
 * NUMA node it is qsg_host_alloc.  qsg_host_free releases either. */
int qsg_host_alloc(size_t bytes, void** out);
int qsg_host_alloc_near(int device, size_t bytes, void** out);
/* The host NUMA node nearest to `device` (cudaDevAttrHostNumaId), -1 where
 * the device reports none. */
int qsg_host_numa_node(int device, int* out);
int qsg_host_free(void* p);

/* ---- state space (lib/statespace_cuda.h) ------------------------------- */
/* InternalToNormalOrder / NormalToInternalOrder (:85-107).  The internal
 * order of this engine is the normal order, so both only validate. */
int qsg_internal_to_normal(qsg_ctx* ctx, float* state, unsigned n);
int qsg_normal_to_internal(qsg_ctx* ctx, float* state, unsigned n);
int qsg_set_all_zeros(qsg_ctx* ctx, float* state, unsigned n);   /* :109 */
int qsg_set_state_uniform(qsg_ctx* ctx, float* state, unsigned n); /* :115 */
int qsg_set_state_zero(qsg_ctx* ctx, float* state, unsigned n);  /* :130 */
int qsg_get_ampl(qsg_ctx* ctx, const float* state, unsigned n, uint64_t i,
                 float* re_im);                                    /* :138 */
int qsg_set_ampl(qsg_ctx* ctx, float* state, unsigned n, uint64_t i,
                 float re, float im);                              /* :150 */
/* BulkSetAmpl (:168-187): state[i] = re+i*im where ((i & mask) == bits)
 * XOR exclude. */
int qsg_bulk_set_ampl(qsg_ctx* ctx, float* state, unsigned n, uint64_t mask,
                      uint64_t bits, float re, float im, int exclude);
/* Add (:190-205): dest += src. */
int qsg_add(qsg_ctx* ctx, const float* src, float* dest, unsigned n);
/* Multiply (:208-217): state *= a. */
int qsg_multiply(qsg_ctx* ctx, float a, float* state, unsigned n);
/* InnerProduct (:219-229): sum conj(s1[i]) * s2[i] in FP64 -> out[2]. */
int qsg_inner_product(qsg_ctx* ctx, const float* s1, const float* s2,
                      unsigned n, double* out_re_im);
/* RealInnerProduct (:231-237). */
int qsg_real_inner_product(qsg_ctx* ctx, const float* s1, const float* s2,
                           unsigned n, double* out);
/* Norm (:239-241): sum |s[i]|^2 in FP64. */
int qsg_norm(qsg_ctx* ctx, const float* state, unsigned n, double* out);
/* Norm that allocates nothing; no counterpart in the reference.  For callers
 * that cannot allocate memory once they are running: a host application that
 * has already reserved nearly all device memory for its own pool (so a
 * cudaMalloc would fail or evict its data), a real-time loop with a fixed
 * memory budget, or a program that installs its own device allocator and
 * forbids allocation behind its back.  qsg_norm may grow the context's
 * scratch (cudaMalloc) and pinned result slot (cudaMallocHost) on its first
 * use; this variant keeps its partial sums in a fixed 64 KiB device array
 * inside the library and returns the result through a plain device-to-host
 * copy followed by a synchronisation of the context stream, so it never
 * allocates.  Same result as qsg_norm (same kernels and partition).  Limits:
 * the reduction may need at most 4096 partial sums (8 per SM; any GPU with
 * up to 512 SMs) and larger requests fail with QSG_ERR_INVALID.  The first
 * call on a device looks up the array's device address (with that device
 * made current).  The call
 * makes the context's device current for its duration and restores the
 * caller's device afterwards.  There is one array per device: calls that
 * overlap in time on the same device (from several threads or streams) race
 * on it and must be serialised by the caller. */
int qsg_norm_noalloc(qsg_ctx* ctx, const float* state, unsigned n,
                     double* out);
/* PartialNorms (:331-355).  The state is cut into qsg_num_chunks(n) equal
 * chunks of consecutive amplitudes; out[m] = sum of |s[i]|^2 over chunk m.
 * `out` must hold qsg_num_chunks(n) doubles. */
uint64_t qsg_num_chunks(unsigned n);
int qsg_partial_norms(qsg_ctx* ctx, const float* state, unsigned n,
                      double* out);
/* FindMeasuredBits (:357-373): first index k of chunk m at which the running
 * sum of |s|^2 inside the chunk exceeds r, masked by `mask` (last index of
 * the chunk if none). */
int qsg_find_measured_bits(qsg_ctx* ctx, const float* state, unsigned n,
                           uint64_t m, double r, uint64_t mask,
                           uint64_t* out);
/* Sample (:243-312).  `sorted_u` holds num_samples uniforms in [0,1), sorted
 * ascending (the host-side mt19937 draws of GenerateRandomValues,
 * lib/util.h:67-85, divided by their max_value).  The device forms
 * r_j = u_j * Norm and returns, per j, the first index k whose inclusive
 * running sum of |s|^2 exceeds r_j (2^n - 1 if none, as
 * lib/statespace_basic.h:222-224). */
int qsg_sample_sorted(qsg_ctx* ctx, const float* state, unsigned n,
                      uint64_t num_samples, const double* sorted_u,
                      uint64_t* out_bitstrings);
/* Sample with absolute thresholds: `sorted_r` holds num_samples values on
 * the scale of the running sum of |s|^2 (the reference's rs of
 * GenerateRandomValues<DistrRealType>(num_samples, seed, norm), converted to
 * double), sorted ascending; per j the first index k whose inclusive running
 * sum exceeds r_j (2^n - 1 if none).  Serves Sample<DistrRealType> for
 * DistrRealType other than double (lib/statespace_cuda.h:243-312), whose
 * draws the caller makes with its own std::uniform_real_distribution. */
int qsg_sample_thresholds(qsg_ctx* ctx, const float* state, unsigned n,
                          uint64_t num_samples, const double* sorted_r,
                          uint64_t* out_bitstrings);
/* Sample with the reference's RNG convention: std::mt19937(seed) +
 * uniform_real_distribution<double>(0, norm), sorted (lib/util.h:67-85). */
int qsg_sample(qsg_ctx* ctx, const float* state, unsigned n,
               uint64_t num_samples, unsigned seed, uint64_t* out_bitstrings);
/* Collapse (:316-329): zero amplitudes with (i & mask) != bits and scale the
 * rest by (float)(1/sqrt(masked norm)). */
int qsg_collapse(qsg_ctx* ctx, float* state, unsigned n, uint64_t mask,
                 uint64_t bits);
/* VirtualMeasure + Collapse (lib/statespace.h:84-140) fused on the device:
 * r = u * Norm, the index k found as in FindMeasuredBits over the whole
 * state, bits = k & mask; when `collapse` is set the state is collapsed on
 * bits.  `u` is the uniform in [0,1) the caller's generator produced. */
int qsg_measure(qsg_ctx* ctx, float* state, unsigned n, uint64_t mask,
                double u, int collapse, uint64_t* out_bits);

/* ---- simulator (lib/simulator_cuda.h) ---------------------------------- */
/* ApplyGate (:70-125): in-place v <- M v on target qubits qs[0..k), k <= 6. */
int qsg_apply_gate(qsg_ctx* ctx, float* state, unsigned n,
                   const unsigned* qs, unsigned k, const float* matrix);
/* ApplyControlledGate (:135-207): apply M on qs where the control qubits
 * cqs[0..c) (sorted) take the values of cvals (bit i <-> cqs[i]); k <= 6. */
int qsg_apply_controlled_gate(qsg_ctx* ctx, float* state, unsigned n,
                              const unsigned* qs, unsigned k,
                              const unsigned* cqs, unsigned c, uint64_t cvals,
                              const float* matrix);
/* ExpectationValue (:216-260): <s| M_qs |s> in FP64 -> out_re_im[2].
 * One read of the state for every operator: monomial operators (one
 * nonzero per row: Pauli strings, diagonal and phased-permutation
 * operators) take a one-pass kernel; dense Hermitian operators of 1..3
 * qubits sum the diagonal and twice the real part of the upper triangle
 * (out_re_im[1] is then 0); other dense operators of 1..3 qubits take the
 * CUDA-core tile kernel and of 4..6 qubits the tensor cores (CUDA cores
 * when an amplitude exceeds the FP16 split's range). */
int qsg_expectation_value(qsg_ctx* ctx, const float* state, unsigned n,
                          const unsigned* qs, unsigned k, const float* matrix,
                          double* out_re_im);
/* ApplyGate on the tensor cores (tcgen05, split FP16 with a power-of-two
 * state scale, FP32 accumulation): k <= 6 targets, n >= 12; the gate is
 * padded to 6 targets with the identity on the lowest free qubits.  Every
 * amplitude must satisfy |psi_i| <= 4 (true for any state of norm <= 4).
 * No counterpart in the reference, which applies every gate on CUDA cores
 * (lib/simulator_cuda.h:333-380). */
int qsg_apply_gate_tc(qsg_ctx* ctx, float* state, unsigned n,
                      const unsigned* qs, unsigned k, const float* matrix);
/* Two gates (k <= 6 targets each, A first) in one tensor-core pass over the
 * state; n >= 12, |psi_i| <= 4.  Their targets, each padded to 6 as in
 * qsg_apply_gate_tc, must span fewer than 12 qubits or include qubit 0 (a
 * 12-qubit tile of them starts at qubit 0; QSG_ERR_UNSUPPORTED otherwise);
 * gates on the same six qubits run as one pass of their product.  The
 * result is that of two qsg_apply_gate_tc calls, with one read and one
 * write of the state instead of two.  No counterpart in the reference,
 * which applies fused gates one pass each (lib/simulator_cuda.h:333-380). */
int qsg_apply_gate_tc2(qsg_ctx* ctx, float* state, unsigned n,
                       const unsigned* qa, unsigned ka, const float* ma,
                       const unsigned* qb, unsigned kb, const float* mb);
/* ExpectationValue on the tensor cores: <s| M_qs |s> for k <= 6 targets
 * (padded to 6 with the identity), n >= 12, |s_i| <= 4; the state is read
 * once and each tile's (M s) is multiplied by conj(s) in the epilogue, FP64
 * partials.  qsg_expectation_value takes this path for dense operators
 * where it is faster; this entry forces it.  The reference computes
 * ExpectationValue on CUDA cores (lib/simulator_cuda.h:216-260). */
int qsg_expectation_value_tc(qsg_ctx* ctx, const float* state, unsigned n,
                             const unsigned* qs, unsigned k,
                             const float* matrix, double* out_re_im);
/* Reads and clears the tensor-core kernels' error flag: 1 if a bounded
 * device-side wait gave up (the kernel then skipped its remaining tiles). */
int qsg_tc_error(qsg_ctx* ctx, int* out);
/* Failure-detection test of the tensor-core kernel's bounded waits; no
 * counterpart in the reference (its CUDA errors exit the process,
 * lib/util_cuda.h:31-39).  Launches the kernel with the identity on qubits
 * 0..5 of an n-qubit state (12 <= n <= 24) and a wait budget of
 * `wait_cycles` SM clocks (1000 .. ~2 s), its MMA thread first waiting on a
 * barrier that no thread arrives at: that wait runs out before any MMA is
 * issued, every role takes the error exit (tensor memory freed, copies in
 * flight awaited) and the state is left unchanged.  Returns QSG_ERR_TIMEOUT
 * when the kernel reported the expired wait (the expected result), and
 * clears the flag, so later launches on the context run normally. */
int qsg_tc_stall_test(qsg_ctx* ctx, float* state, unsigned n,
                      long long wait_cycles);
/* SIMDRegisterSize (:265-267). */
unsigned qsg_simd_register_size(void);

/* ---- host random numbers ------------------------------------------------
 * std::mt19937 + uniform_real_distribution<double>, the generators of
 * lib/util.h:61-85 (RandomValue, GenerateRandomValues) and of
 * QuantumTrajectorySimulator (lib/qtrajectory.h:268-302). */
typedef struct qsg_rng qsg_rng;
qsg_rng* qsg_rng_create(unsigned seed);
void qsg_rng_destroy(qsg_rng* rng);
uint32_t qsg_rng_next_u32(qsg_rng* rng);
/* uniform_real_distribution<double>(0, max_value)(rng) */
double qsg_rng_uniform(qsg_rng* rng, double max_value);
/* GenerateRandomValues (lib/util.h:67-85) without the sentinel: `num` sorted
 * draws of uniform_real_distribution<double>(0, max_value) from
 * std::mt19937(seed). */
void qsg_generate_random_values(uint64_t num, unsigned seed, double max_value,
                                double* out);

/* ---- circuits ----------------------------------------------------------
 * The operation list of lib/circuit.h:20-31 with the operation kinds of
 * lib/operation.h:35-37 (matrix gate, controlled gate, measurement).
 * Matrices are interleaved complex double, row-major, 2 * 4^k values, bit j
 * of the row/column index <-> qs[j] as given (qubits are sorted on entry and
 * the matrix permuted to match, as CreateGate, lib/gate.h:266-290). */
typedef struct qsg_circuit qsg_circuit;
int qsg_circuit_create(unsigned num_qubits, qsg_circuit** out);
int qsg_circuit_destroy(qsg_circuit* c);
int qsg_circuit_info(const qsg_circuit* c, unsigned* num_qubits,
                     uint64_t* num_ops);
int qsg_circuit_add_gate(qsg_circuit* c, unsigned time, const unsigned* qs,
                         unsigned k, const double* matrix);
/* ControlledGate (lib/gate.h:37-70): cvals bit i <-> cqs[i] as given. */
int qsg_circuit_add_controlled_gate(qsg_circuit* c, unsigned time,
                                    const unsigned* qs, unsigned k,
                                    const unsigned* cqs, unsigned nc,
                                    uint64_t cvals, const double* matrix);
int qsg_circuit_add_measurement(qsg_circuit* c, unsigned time,
                                const unsigned* qs, unsigned k);
/* Gates of lib/gates_qsim.h by their text-format names (docs/input_format.md)
 * plus "u3" (theta, phi, lambda). */
int qsg_circuit_add_named_gate(qsg_circuit* c, unsigned time, const char* name,
                               const unsigned* qs, unsigned nq,
                               const double* params, unsigned np);
/* CircuitQsimParser::FromStream (lib/circuit_qsim_parser.h:52-153). */
int qsg_circuit_parse(const char* text, unsigned maxtime, qsg_circuit** out);
/* Seeded synthetic workloads: grid random circuits (rows x cols plus a
 * ragged last row of `extra` qubits), linear-chain random circuits, and
 * layered U3 + CZ/CNOT circuits with controlled U3 gates. */
int qsg_circuit_grid(unsigned rows, unsigned cols, unsigned extra,
                     unsigned cycles, uint64_t seed, qsg_circuit** out);
int qsg_circuit_chain(unsigned n, unsigned cycles, uint64_t seed,
                      qsg_circuit** out);
int qsg_circuit_layered_u3(unsigned n, unsigned layers,
                           unsigned num_controlled, uint64_t seed,
                           qsg_circuit** out);
/* Reads back op i (qs/cqs arrays must hold the op's counts; matrix 2*4^k). */
int qsg_circuit_get_op(const qsg_circuit* c, uint64_t i, int* kind,
                       unsigned* time, unsigned* k, unsigned* qs, unsigned* nc,
                       unsigned* cqs, uint64_t* cvals, double* matrix);
/* Random Pauli strings (weight 1..max_weight, coefficients U[-1,1]); row i of
 * qubits/letters has max_weight slots, the first weights[i] used. */
int qsg_pauli_sum(unsigned n, unsigned count, unsigned max_weight,
                  uint64_t seed, unsigned* weights, unsigned* qubits,
                  char* letters, double* coeffs);

/* ---- fusion plans and runs ---------------------------------------------
 * MultiQubitGateFuser::FuseGates (lib/fuser_mqubit.h:282-526) +
 * QSimRunner::Run (lib/run_qsim.h:225-289). */
typedef struct qsg_plan qsg_plan;
typedef struct qsg_fuse_options {
  unsigned max_fused_size;  /* 1..6 */
  unsigned seeds;           /* front gates tried per block (0: default) */
  int tensor_path;          /* route blocks of >= tc_min_k qubits to tcgen05 */
  unsigned tc_min_k;        /* 0: default 5 */
  const void* cost_model;   /* a qsg_mlp* (NULL: gate-count rule) */
  /* Two-gate tensor-core passes (qsg_apply_gate_tc2): consecutive
   * tensor-core blocks share one pass over the state when their 12-qubit
   * tile has at least this many run bits (low qubits 0..b-1 in the tile)
   * and a pass of that tile shape measured faster than two; the set of
   * pairs with the largest predicted saving is taken, and plans are
   * compared by passes (a pair at its measured cost).  0: one pass per
   * block.  No counterpart in the reference. */
  unsigned tc_pair_bits;
} qsg_fuse_options;
int qsg_plan_create(const qsg_circuit* c, const qsg_fuse_options* opts,
                    qsg_plan** out);
/* One plan op per circuit op (no fusion). */
int qsg_plan_create_unfused(const qsg_circuit* c, qsg_plan** out);
int qsg_plan_destroy(qsg_plan* p);
int qsg_plan_info(const qsg_plan* p, uint64_t* num_ops, unsigned* max_k,
                  uint64_t* num_tensor_ops);
/* Two-gate tensor-core passes of the plan (qsg_fuse_options.tc_pair_bits),
 * and per op whether it starts one (pair_next[i] = 1 for the first op of a
 * pair; may be NULL, else num_ops entries). */
int qsg_plan_tc_pairs(const qsg_plan* p, uint64_t* num_pairs,
                      unsigned char* pair_next);
int qsg_plan_get_op(const qsg_plan* p, uint64_t i, int* kind, unsigned* k,
                    unsigned* qs, unsigned* nc, unsigned* cqs,
                    uint64_t* cvals, int* path, uint64_t* num_members,
                    double* matrix);
/* Applies the plan to `state`; measurements draw from std::mt19937(seed)
 * and their masked bits are written to mbits (up to mbits_cap). */
int qsg_plan_run(qsg_ctx* ctx, qsg_plan* p, float* state, unsigned seed,
                 uint64_t* mbits, uint64_t mbits_cap, uint64_t* num_meas);
/* Records the plan applied to `state` as a CUDA graph (no measurements);
 * qsg_plan_replay launches it on the context stream. */
int qsg_plan_capture(qsg_ctx* ctx, qsg_plan* p, float* state);
int qsg_plan_replay(qsg_ctx* ctx, qsg_plan* p);
/* Applies the plan's gate ops with a CUDA event pair around each launch;
 * op_ms[i] = milliseconds of op i (measurement ops are skipped, 0). */
int qsg_plan_profile(qsg_ctx* ctx, qsg_plan* p, float* state, float* op_ms,
                     uint64_t cap);

/* ---- fused-plan cache ----------------------------------------------------
 * QSimRunner::Run (lib/run_qsim.h:225-289) fuses the circuit on every call,
 * after CircuitQsimParser::FromStream (lib/circuit_qsim_parser.h:52-153) for
 * a text circuit.  A cache keys the fused plan by the circuit's operations
 * (qsg_plan_cache_run) or by the text and maxtime (qsg_plan_cache_run_text)
 * together with the fusion options; keys are hashed and compared in full.  A
 * hit skips parsing and fusion.  A plan without measurements is captured as
 * a CUDA graph on its first run on a state and replayed on later runs on the
 * same state and context; plans with measurements run op by op with
 * measurements from std::mt19937(seed) (as qsg_plan_run).  *hit is 1 when
 * the plan came from the cache.  Beyond `capacity` plans (0: unbounded) the
 * least recently used is dropped.  Runs are asynchronous on the context
 * stream, like qsg_plan_run without measurements.  A cost model is keyed by
 * its handle: after training a model further, call qsg_plan_cache_clear. */
typedef struct qsg_plan_cache qsg_plan_cache;
int qsg_plan_cache_create(unsigned capacity, qsg_plan_cache** out);
int qsg_plan_cache_destroy(qsg_plan_cache* cache);
int qsg_plan_cache_clear(qsg_plan_cache* cache);
int qsg_plan_cache_stats(qsg_plan_cache* cache, uint64_t* hits,
                         uint64_t* misses, uint64_t* evictions,
                         uint64_t* captures, uint64_t* size);
int qsg_plan_cache_run(qsg_ctx* ctx, qsg_plan_cache* cache,
                       const qsg_circuit* circuit,
                       const qsg_fuse_options* opts, float* state,
                       unsigned seed, uint64_t* mbits, uint64_t mbits_cap,
                       uint64_t* num_meas, int* hit);
int qsg_plan_cache_run_text(qsg_ctx* ctx, qsg_plan_cache* cache,
                            const char* text, unsigned maxtime,
                            const qsg_fuse_options* opts, float* state,
                            unsigned seed, uint64_t* mbits,
                            uint64_t mbits_cap, uint64_t* num_meas, int* hit);

/* ---- learned fusion planner --------------------------------------------
 * No counterpart in the reference (its fuser, lib/fuser_mqubit.h:282-526,
 * fuses up to a fixed max_fused_size).  A perceptron with 16 inputs, two
 * hidden layers of 64 ReLU units and one output predicts the time of one
 * fused-gate launch from features of the block (qsg_block_features):
 * output = log(microseconds) - (n - 24) log 2.  It is trained on the device
 * (forward, backward and Adam kernels of this library) on launch times the
 * engine records with qsg_plan_profile.  Passed as
 * qsg_fuse_options.cost_model, it makes qsg_plan_create choose block
 * boundaries, block sizes up to max_fused_size and the path of each block
 * (tensor cores for blocks of >= tc_min_k qubits when tensor_path is set) by
 * the lowest predicted time per fused gate.  The plan changes only speed:
 * every plan applies the same circuit. */
#define QSG_MLP_INPUTS 16
typedef struct qsg_mlp qsg_mlp;
uint64_t qsg_mlp_num_params(void);
/* He-uniform weights from std::mt19937_64(seed), zero biases. */
int qsg_mlp_create(uint64_t seed, qsg_mlp** out);
int qsg_mlp_destroy(qsg_mlp* m);
/* Host copies of the qsg_mlp_num_params() parameters: W1[16][64], b1[64],
 * W2[64][64], b2[64], W3[64], b3. */
int qsg_mlp_get_params(const qsg_mlp* m, float* out);
int qsg_mlp_set_params(qsg_mlp* m, const float* in);
/* Host arrays x[n][16], y[n].  Gradient of the mean squared error over all
 * samples (grad: qsg_mlp_num_params() floats) and that error, on the device. */
int qsg_mlp_gradient(qsg_ctx* ctx, const qsg_mlp* m, const float* x,
                     const float* y, uint64_t n, float* grad, double* loss);
/* `steps` Adam steps (rate lr) on minibatches of `batch` samples from
 * per-epoch permutations drawn from std::mt19937_64(seed). */
int qsg_mlp_train(qsg_ctx* ctx, qsg_mlp* m, const float* x, const float* y,
                  uint64_t n, unsigned steps, unsigned batch, float lr,
                  uint64_t seed, double* final_loss);
int qsg_mlp_predict(qsg_ctx* ctx, const qsg_mlp* m, const float* x,
                    uint64_t n, float* out);
/* Features of one launch: sorted target qubits as launched (the padded six
 * for the tensor-core path, path = 1), control count. */
int qsg_block_features(unsigned n, const unsigned* qs, unsigned k,
                       unsigned ncontrols, int path, float* out);
/* Predicted microseconds of a launch (qubits before tensor-core padding). */
int qsg_mlp_cost_us(const qsg_mlp* m, unsigned n, const unsigned* qs,
                    unsigned k, unsigned ncontrols, int path, double* out);

/* ---- noisy circuits and quantum trajectories ---------------------------
 * Channels (lib/channel.h:31-125, lib/channels_cirq.h), MakeNoisy
 * (lib/circuit_noisy.h:33-64) and QuantumTrajectorySimulator::RunOnce /
 * RunBatch (lib/qtrajectory.h:80-236).  Trajectory `rep` draws from
 * std::mt19937(rep) exactly as the reference does, so every Kraus choice that
 * the lower probability bounds decide is the reference's; choices that need
 * the state are made on the device.  Per-op statistics: entry i is the Kraus
 * index chosen for op i (0 for a gate), the measured bits of a measurement,
 * or QSG_NO_STAT where the reference records nothing; the reference's
 * stat.samples are the entries that are not QSG_NO_STAT. */
#define QSG_NO_STAT (~(uint64_t)0)
enum {
  QSG_CHANNEL_DEPOLARIZING = 0,      /* lib/channels_cirq.h:127-199, p      */
  QSG_CHANNEL_AMPLITUDE_DAMPING = 1, /* :274-300, gamma                     */
  QSG_CHANNEL_PHASE_DAMPING = 2,     /* :313-345, gamma                     */
  QSG_CHANNEL_BIT_FLIP = 3,          /* :425-447, p                         */
  QSG_CHANNEL_PHASE_FLIP = 4,        /* :393-415, p                         */
  QSG_CHANNEL_RESET = 5,             /* :359-380                            */
  /* Depolarizing on k <= 3 qubits as the reference's multi-qubit factory
   * builds it (:147-189): the Pauli of index digit j acts on register qubit
   * j, not on the channel's j-th qubit (the same as kind 0 when the channel
   * acts on qubits 0..k-1).  For trajectories identical to the reference's
   * on circuits that use that factory. */
  QSG_CHANNEL_DEPOLARIZING_REGISTER = 6
};
typedef struct qsg_noisy qsg_noisy;
int qsg_noisy_create(unsigned num_qubits, qsg_noisy** out);
int qsg_noisy_destroy(qsg_noisy* h);
int qsg_noisy_info(const qsg_noisy* h, unsigned* num_qubits,
                   uint64_t* num_ops, uint64_t* num_channels);
/* Appends the circuit's ops unchanged (times kept). */
int qsg_noisy_append_circuit(qsg_noisy* h, const qsg_circuit* c);
int qsg_noisy_add_channel(qsg_noisy* h, int kind, unsigned time,
                          const unsigned* qs, unsigned nq, double p);
/* A general channel: Kraus operator k is the matrix
 * matrices[k * 2 * 4^nq ...] on qs (interleaved complex double, bit j <->
 * qs[j]) with lower-bound probability probs[k]; K^dagger K is computed. */
int qsg_noisy_add_kraus_channel(qsg_noisy* h, unsigned time,
                                const unsigned* qs, unsigned nq,
                                unsigned num_kops, const int* unitary,
                                const double* probs, const double* matrices);
/* MakeNoisy with a depolarizing(p_depol) channel after each op on each of
 * its qubits; with gamma > 0 an amplitude damping(gamma) channel on every
 * qubit after each cycle of `cycle_len` time steps of the clean circuit. */
int qsg_noisy_make(const qsg_circuit* c, double p_depol, double gamma,
                   unsigned cycle_len, qsg_noisy** out);
int qsg_noisy_get_op(const qsg_noisy* h, uint64_t i, int* is_channel,
                     unsigned* time, unsigned* nq, unsigned* qs,
                     unsigned* num_kops);

typedef struct qsg_traj qsg_traj;
typedef struct qsg_traj_options {
  unsigned max_fused_size;         /* 0: 4 */
  unsigned seeds;                  /* 0: default */
  int collect_kop_stat;            /* lib/qtrajectory.h:48-58 */
  int collect_mea_stat;
  int normalize_before_mea_gates;
  int tensor_path;                 /* fused blocks of >= tc_min_k qubits on
                                      the tensor cores (padded to 6 targets;
                                      every trajectory is normalised at the
                                      end) */
  unsigned tc_min_k;               /* 0: 5 */
} qsg_traj_options;
/* Fuses the noisy circuit once (each channel as its first Kraus operator).
 * QSG_ERR_UNSUPPORTED for a non-unitary channel on more than 2 qubits or
 * whose K^dagger K is not diagonal. */
int qsg_traj_create(const qsg_noisy* h, const qsg_traj_options* opts,
                    qsg_traj** out);
int qsg_traj_destroy(qsg_traj* t);
int qsg_traj_info(const qsg_traj* t, unsigned* num_qubits, uint64_t* num_ops,
                  uint64_t* num_fused_ops);
/* RunOnce: trajectory `rep` from |0..0> on `state` (synchronous); stats
 * receives num_ops entries (may be NULL). */
int qsg_traj_run(qsg_ctx* ctx, qsg_traj* t, float* state, uint64_t rep,
                 uint64_t* stats);
/* QuantumTrajectorySimulator::RunOnce (lib/qtrajectory.h) on the state as
 * given (the caller prepares it), as the reference's Python module runs
 * noisy circuits from an input state. */
int qsg_traj_run_from(qsg_ctx* ctx, qsg_traj* t, float* state, uint64_t rep,
                      uint64_t* stats);
/* RunBatch over items (runners[item_runner[i]], item_rep[i]) on concurrent
 * streams of `device` (one host thread, stream, state buffer and workspace
 * each).  stats (may be NULL): the items' entries concatenated in item
 * order; out_states (may be NULL, or hold NULLs): per item a device buffer
 * of qsg_min_size(n) floats for the final state; latency_ms: per-item device
 * time; wall_s: batch wall time; launches: kernels launched. */
typedef struct qsg_batch_options {
  unsigned num_streams;  /* 0: 8 */
  unsigned big_qubits;   /* circuits of >= big_qubits qubits run only on   */
  unsigned big_streams;  /* the first big_streams streams (0 / 0: no split) */
} qsg_batch_options;
int qsg_traj_run_batch(int device, qsg_traj* const* runners,
                       uint64_t num_runners, const uint32_t* item_runner,
                       const uint64_t* item_rep, uint64_t num_items,
                       const qsg_batch_options* opts, uint64_t* stats,
                       float* const* out_states, float* latency_ms,
                       double* wall_s, uint64_t* launches);

/* RunBatch as one persistent kernel over a packed batch: every trajectory is
 * compiled on the host cores into a short device program (Kraus choices the
 * lower bounds decide are made there; the others are made on the device),
 * the batch is uploaded once and a single launch runs it, each CTA taking
 * whole trajectories, largest circuits first.  Replaces the reference's
 * serial loop over repetitions (lib/qtrajectory.h:141-236).  Items whose
 * circuit has measurements, fused blocks of more than 4 targets, or more
 * than max_qubits qubits run on the stream path of qsg_traj_run_batch
 * afterwards.  Arguments as qsg_traj_run_batch; latency_ms is the item's
 * device time inside the kernel; `info` (may be NULL) receives counts and
 * timings. */
typedef struct qsg_packed_options {
  unsigned ctas_per_sm;   /* 0: 4 (fewer if the state slots do not fit)   */
  unsigned max_qubits;    /* 0: 30                                         */
  unsigned host_threads;  /* threads compiling programs, 0: all cores     */
  unsigned tile_kib;      /* tile buffers per CTA: 32, 64 or 96 (0: 32)    */
  int overlap;            /* nonzero: stream path runs while the kernel runs */
  qsg_batch_options streams;  /* stream path for the other items          */
} qsg_packed_options;
typedef struct qsg_packed_info {
  uint64_t packed_items, stream_items, ops;
  unsigned ctas, tile_kib;
  double build_s, upload_s, kernel_s, stream_s;
} qsg_packed_info;
int qsg_traj_run_packed(int device, qsg_traj* const* runners,
                        uint64_t num_runners, const uint32_t* item_runner,
                        const uint64_t* item_rep, uint64_t num_items,
                        const qsg_packed_options* opts, uint64_t* stats,
                        float* const* out_states, float* latency_ms,
                        double* wall_s, uint64_t* launches,
                        qsg_packed_info* info);

/* ---- unitary calculator (lib/unitaryspace_basic.h,
 * lib/unitary_calculator_basic.h) ----------------------------------------
 * A unitary of n qubits (n <= 20) is stored as the reference stores it:
 * entry (i, j) at complex index i * 2^n + j, interleaved (re, im).  The
 * reference's ApplyGate (unitary_calculator_basic.h:126-184) mixes the
 * entries of every row over the column bits at qs, so the unitary is a
 * 2n-qubit state and its gates are the state-vector gates on qubits < n:
 * the same GB300 kernels run it.  From the identity, entry (i, j) after
 * gates G1..Gm is (Gm ... G1)[j][i], as in the reference. */
/* UnitarySpaceBasic::MinSize (unitaryspace_basic.h:49-51), in floats (at
 * least 64). */
uint64_t qsg_unitary_min_size(unsigned num_qubits);
/* CreateUnitary (unitaryspace.h:41-47): device buffer of MinSize floats. */
int qsg_unitary_create(qsg_ctx* ctx, unsigned num_qubits, float** out);
int qsg_unitary_free(qsg_ctx* ctx, float* u);
/* SetIdentity / SetAllZeros (unitaryspace_basic.h:53-74). */
int qsg_unitary_set_identity(qsg_ctx* ctx, float* u, unsigned n);
int qsg_unitary_set_all_zeros(qsg_ctx* ctx, float* u, unsigned n);
/* GetEntry / SetEntry (unitaryspace_basic.h:76-96). */
int qsg_unitary_get_entry(qsg_ctx* ctx, const float* u, unsigned n,
                          uint64_t i, uint64_t j, float* re_im);
int qsg_unitary_set_entry(qsg_ctx* ctx, float* u, unsigned n, uint64_t i,
                          uint64_t j, float re, float im);
/* UnitaryCalculatorBasic::ApplyGate / ApplyControlledGate
 * (unitary_calculator_basic.h:51-117): qubits < n, k <= 6. */
int qsg_unitary_apply_gate(qsg_ctx* ctx, float* u, unsigned n,
                           const unsigned* qs, unsigned k,
                           const float* matrix);
int qsg_unitary_apply_controlled_gate(qsg_ctx* ctx, float* u, unsigned n,
                                      const unsigned* qs, unsigned k,
                                      const unsigned* cqs, unsigned c,
                                      uint64_t cvals, const float* matrix);
/* Applies every op of a fused plan (of an n-qubit circuit) to the unitary;
 * a plan's tensor-core blocks (circuits of >= 12 qubits) run on tcgen05.
 * No counterpart in the reference, which applies gates one by one.  Plans
 * with measurements are rejected. */
int qsg_unitary_run_plan(qsg_ctx* ctx, qsg_plan* p, float* u, unsigned n);

/* ---- hybrid Schrodinger-Feynman simulation (qsimh) ----------------------
 * QSimHRunner::Run (lib/run_qsimh.h:43-104) over HybridSimulator
 * (lib/hybrid.h): the qubits are cut into parts[q] = 0 or 1; two-qubit gates
 * across the cut are replaced by their operator Schmidt terms (named gates
 * id2, cz, cnot/cx, sw, is, fs, cp, as lib/gates_qsim.h); the amplitudes of
 * `bitstrings` (bit q = qubit q) are summed over the paths of the cut gates
 * with the first num_prefix_gatexs gates' terms fixed by `prefix` and the
 * rest summed, and ADDED to results (interleaved complex double, as the
 * reference adds to its results vector).  Only one- and two-qubit matrix
 * gates are allowed (QSG_ERR_UNSUPPORTED otherwise).  The paths of the
 * suffix gates (after the num_root_gatexs root gates) run as one batch on
 * the device: up to max_batch_bits path bits (0: as many as fit in 45 % of
 * free HBM), the others loop on the host like the root paths.  All paths
 * are summed whatever the split, so the split changes speed only. */
typedef struct qsg_hybrid_options {
  uint64_t prefix;
  unsigned num_prefix_gatexs;
  unsigned num_root_gatexs;
  unsigned max_fused_size;   /* 0: 4 */
  int tensor_path;           /* fused blocks of >= 5 qubits on tcgen05,
                                consecutive ones in two-gate passes where
                                their tile allows (tc_pair_bits 2) */
  unsigned max_batch_bits;   /* 0: by free memory */
} qsg_hybrid_options;
typedef struct qsg_hybrid_info {
  unsigned num_qubits0, num_qubits1;
  unsigned num_ops0, num_ops1;  /* per part, cut gates included */
  unsigned num_gatexs;          /* gates on the cut */
  unsigned prefix_bits, root_bits, suffix_bits;
  unsigned batch_bits;          /* suffix path bits run as one batch */
  uint64_t paths_run;
} qsg_hybrid_info;
/* HybridSimulator::SplitLattice: counts only (no GPU). */
int qsg_hybrid_split(const qsg_circuit* c, const unsigned* parts,
                     unsigned num_parts, qsg_hybrid_info* info);
int qsg_hybrid_run(qsg_ctx* ctx, const qsg_circuit* c, const unsigned* parts,
                   unsigned num_parts, const qsg_hybrid_options* opts,
                   const uint64_t* bitstrings, uint64_t num_bitstrings,
                   double* results, qsg_hybrid_info* info);
/* Operator Schmidt terms of circuit op i (two-qubit named gates): terms[16 t
 * .. 16 t + 7] = factor on the op's first (lower) qubit, then 8 values of the
 * factor on its second qubit, each a 2x2 row-major interleaved complex
 * matrix; *num_terms = 0 for other ops.  terms may be NULL. */
int qsg_circuit_get_schmidt(const qsg_circuit* c, uint64_t i,
                            unsigned* num_terms, double* terms);
/* Sets the operator Schmidt terms of two-qubit op i (same layout; the
 * terms must sum to the op's matrix), for gates other than the named ones,
 * e.g. the Cirq gate set of lib/gates_cirq.h, whose decompositions the
 * reference defines per gate.  At most 4 terms. */
int qsg_circuit_set_schmidt(qsg_circuit* c, uint64_t i, unsigned num_terms,
                            const double* terms);

/* ---- timing ------------------------------------------------------------ */
/* CUDA-event timing on the context stream: qsg_timer_start records an event,
 * qsg_timer_stop records a second one, synchronises and returns the elapsed
 * milliseconds. */
int qsg_timer_start(qsg_ctx* ctx);
int qsg_timer_stop(qsg_ctx* ctx, float* ms);
/* Number of kernels this library launched on the context so far. */
uint64_t qsg_ctx_launch_count(qsg_ctx* ctx);
/* Bytes the context currently holds in its on-demand reduction scratch
 * (device, cudaMalloc) and in its pinned result slot (host, cudaMallocHost);
 * both start at 0 and grow on first use.  No counterpart in the reference
 * (its StateSpaceCUDA allocates its scratch in the constructor,
 * lib/statespace_cuda.h:54-66); a diagnostic for callers with a memory
 * budget. */
int qsg_ctx_scratch_bytes(qsg_ctx* ctx, size_t* device_bytes,
                          size_t* pinned_bytes);

#ifdef __cplusplus
}  /* extern "C" */
#endif

#endif  /* QSIM_GB300_H_ */
