// Plan runtime: a fused plan plus the device resources that running or
// capturing it needs.
#pragma once

#include <cstddef>
#include <vector>

#include "engine.h"

namespace qsg {

// Tensor-core (tcgen05) application of a k = 5, 6 fused gate; `operands` are
// the device operands built by tc_build_operands.  Defined in tc_gate.cu.
int apply_gate_tc(qsg_ctx* ctx, float* state, unsigned n, const unsigned* qs,
                  unsigned k, const float* m32, const void* operands);
// The same with the norm carry of unitary plans: `prev` (null for the first
// tensor-core pass) holds the previous pass's per-CTA (sum |in|^2,
// sum |out|^2) from `prev_count` CTAs, whose ratio rescales this pass's
// input; this pass writes its own sums to `out` (tc_grid(n) pairs).
int apply_gate_tc_carry(qsg_ctx* ctx, float* state, unsigned n,
                        const unsigned* qs, unsigned k, const float* m32,
                        const void* operands, const double* prev,
                        unsigned prev_count, double* out);
// Two padded 6-qubit gates (sorted targets qa6 then qb6, device operands
// opa, opb) in one tensor-core pass, with the norm carry as above (sums of
// the first gate's input and the second gate's output).
int apply_gate_tc2_carry(qsg_ctx* ctx, float* state, unsigned n,
                         const unsigned* qa6, const void* opa,
                         const unsigned* qb6, const void* opb,
                         const double* prev, unsigned prev_count,
                         double* out);
// CTAs of a tensor-core pass on n qubits.
unsigned tc_grid(qsg_ctx* ctx, unsigned n);
// A gate given as a host matrix (k <= 6, n >= 12) on the tensor cores, its
// operands built per call and uploaded through the context's ring.
int apply_gate_tc_host(qsg_ctx* ctx, float* state, unsigned n,
                       const unsigned* qs, unsigned k, const float* m32);
// Size in bytes of the device operands of a k-qubit tensor-core gate, and
// their construction from the interleaved FP32 matrix.
size_t tc_operand_bytes(unsigned k);
void tc_build_operands(unsigned k, const float* m32, void* host_out);

void set_error_msg(const char* msg);
// Pads a gate to 6 targets (identity on the lowest free qubits) for the
// tensor-core path; m6_out holds 2 * 64 * 64 floats.
void tc_pad_gate(unsigned n, const unsigned* qs, unsigned k, const float* m32,
                 unsigned* qs6, float* m6_out);
int tc_check_error(qsg_ctx* ctx, int* out);
int tc_setup();

namespace host {

struct PlanRuntime {
  Plan plan;
  qsg_ctx* ctx = nullptr;
  float* dmat = nullptr;             // k = 6 matrices (CUDA-core path)
  std::vector<size_t> dmat_off;
  void* tc_buf = nullptr;            // tensor-core operands
  std::vector<size_t> tc_off;
  bool tc_ready = false;
  void* graph = nullptr;             // cudaGraph_t
  void* graph_exec = nullptr;        // cudaGraphExec_t
  float* captured_state = nullptr;
  int device = -1;                   // device of dmat / tc_buf / norm_buf
  // Tensor-core plans of unitary gates keep the norm: the tensor cores'
  // FP32 accumulation rounds toward zero and shrinks the norm by ~6e-7 per
  // pass, so each tensor-core pass rescales its input by the norm ratio the
  // previous one measured (only the last pass's loss remains).
  bool restore_norm = false;
  bool uploaded = false;
  double* norm_buf = nullptr;        // two sets of per-CTA norm sums

  PlanRuntime() = default;
  PlanRuntime(const PlanRuntime&) = delete;
  PlanRuntime& operator=(const PlanRuntime&) = delete;
  ~PlanRuntime();

  void release();
  int upload(qsg_ctx* ctx);
  int prepare_tc();
  const void* tc_operands(size_t i) const;
  // Launches op i, and op i + 1 with it when op i starts a two-gate
  // tensor-core pass (plan.ops[i].tc_pair_next).
  int launch_op(size_t i, float* state);
  // Every gate op in order (with the norm restoration); no measurements.
  int launch_all(float* state);
  // Runs every op; measurement bits are appended to `mbits`.
  int run(qsg_ctx* ctx, float* state, unsigned seed,
          std::vector<uint64_t>* mbits);
  int capture(qsg_ctx* ctx, float* state);
  // Runs the gate ops with a CUDA event around each; per-op milliseconds
  // (measurements are skipped and get 0; a two-gate tensor-core pass is
  // timed as its first op, the second gets 0).
  int profile(qsg_ctx* ctx, float* state, std::vector<float>* ms);
  int replay(qsg_ctx* ctx);
};

}  // namespace host
}  // namespace qsg
