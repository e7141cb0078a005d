// Plan execution.  Replaces the hot loop of QSimRunner::Run
// (lib/run_qsim.h:264-280 and :225-289) and the measurement dispatch of
// lib/gate_appl.h:94-139: every fused op is one launch on the context stream;
// a measurement draws one uniform from std::mt19937(seed) (RandomValue,
// lib/util.h:61-65) and runs VirtualMeasure + Collapse on the device.
//
// A plan without measurements can be captured once into a CUDA graph for a
// given state buffer and replayed; k = 6 matrices and tensor-core operands
// then live in a device buffer owned by the plan.

#include <cmath>
#include <cstring>
#include <random>

#include <cuda_runtime.h>

#include "engine.h"
#include "internal.h"
#include "runner.h"
#include "traj_dev.h"

namespace qsg {
namespace host {

PlanRuntime::~PlanRuntime() { release(); }

void PlanRuntime::release() {
  if (graph_exec) cudaGraphExecDestroy(static_cast<cudaGraphExec_t>(graph_exec));
  if (graph) cudaGraphDestroy(static_cast<cudaGraph_t>(graph));
  graph_exec = graph = nullptr;
  // Freed on the device that holds them, without the context: the context
  // may already be gone (cudaFree waits for the device).
  if ((dmat || tc_buf || norm_buf) && device >= 0) {
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(device);
    if (dmat) cudaFree(dmat);
    if (tc_buf) cudaFree(tc_buf);
    if (norm_buf) cudaFree(norm_buf);
    cudaSetDevice(cur);
  }
  norm_buf = nullptr;
  restore_norm = false;
  uploaded = false;
  dmat = nullptr;
  tc_buf = nullptr;
  dmat_off.clear();
  tc_off.clear();
  tc_ready = false;
}

int PlanRuntime::upload(qsg_ctx* c) {
  if (uploaded) return QSG_OK;
  ctx = c;
  device = ctx_device(c);
  bool tc = false, unitary = true;
  for (const auto& op : plan.ops) {
    if (op.kind == OpKind::kMeasure) unitary = false;
    if (op.kind == OpKind::kGate && op.path == Path::kTensor) tc = true;
  }
  if (tc && unitary) {
    // Known from the member gates (set at fusion), not recomputed here:
    // a 64 x 64 product check per block cost ~0.3 ms of host time per
    // tensor-core op on every run of a new plan.
    for (const auto& op : plan.ops)
      if (!op.unitary) {
        unitary = false;
        break;
      }
  }
  if (tc && unitary) {
    void* p = nullptr;
    int rc = dev_alloc(ctx, 2 * size_t(traj_max_parts(ctx)) * 4 * sizeof(double),
                       &p);
    if (rc) return rc;
    norm_buf = static_cast<double*>(p);
    restore_norm = true;
  }
  size_t total = 0;
  dmat_off.assign(plan.ops.size(), size_t(-1));
  for (size_t i = 0; i < plan.ops.size(); ++i) {
    const auto& op = plan.ops[i];
    if (op.kind == OpKind::kMeasure) continue;
    // k = 6 matrices of CUDA-core passes (tensor-core passes read their own
    // operands, prepare_tc).
    if (op.qs.size() >= 6 && op.path != Path::kTensor) {
      dmat_off[i] = total;
      total += op.m32.size();
    }
  }
  if (total == 0) {
    uploaded = true;
    return QSG_OK;
  }
  void* p = nullptr;
  int rc = dev_alloc(ctx, total * sizeof(float), &p);
  if (rc) return rc;
  dmat = static_cast<float*>(p);
  std::vector<float> host(total);
  for (size_t i = 0; i < plan.ops.size(); ++i) {
    if (dmat_off[i] == size_t(-1)) continue;
    std::memcpy(&host[dmat_off[i]], plan.ops[i].m32.data(),
                plan.ops[i].m32.size() * sizeof(float));
  }
  rc = dev_upload(ctx, dmat, host.data(), total * sizeof(float));
  if (rc == QSG_OK) uploaded = true;
  return rc;
}

int PlanRuntime::prepare_tc() {
  if (tc_ready) return QSG_OK;
  for (const auto& op : plan.ops) {
    if (op.kind == OpKind::kGate && op.path == Path::kTensor) {
      int rc = tc_setup();
      if (rc) return rc;
      break;
    }
  }
  size_t total = 0;
  tc_off.assign(plan.ops.size(), size_t(-1));
  for (size_t i = 0; i < plan.ops.size(); ++i) {
    const auto& op = plan.ops[i];
    if (op.kind == OpKind::kGate && op.path == Path::kTensor) {
      tc_off[i] = total;
      total += (tc_operand_bytes(op.qs.size()) + 1023) & ~size_t(1023);
    }
  }
  if (total > 0) {
    void* p = nullptr;
    int rc = dev_alloc(ctx, total, &p);
    if (rc) return rc;
    tc_buf = p;
    device = ctx_device(ctx);
    std::vector<unsigned char> host(total);
    for (size_t i = 0; i < plan.ops.size(); ++i) {
      if (tc_off[i] == size_t(-1)) continue;
      tc_build_operands(plan.ops[i].qs.size(), plan.ops[i].m32.data(),
                        host.data() + tc_off[i]);
    }
    rc = dev_upload(ctx, tc_buf, host.data(), total);
    if (rc) return rc;
  }
  tc_ready = true;
  return QSG_OK;
}

const void* PlanRuntime::tc_operands(size_t i) const {
  if (!tc_buf || tc_off[i] == size_t(-1)) return nullptr;
  return static_cast<const unsigned char*>(tc_buf) + tc_off[i];
}

int PlanRuntime::launch_op(size_t i, float* state) {
  const PlanOp& op = plan.ops[i];
  const unsigned n = plan.num_qubits;
  const float* dm = (dmat && dmat_off[i] != size_t(-1)) ? dmat + dmat_off[i]
                                                        : nullptr;
  if (op.kind == OpKind::kGate && op.path == Path::kTensor) {
    if (op.tc_pair_next)
      return apply_gate_tc2_carry(ctx, state, n, op.qs.data(), tc_operands(i),
                                  plan.ops[i + 1].qs.data(),
                                  tc_operands(i + 1), nullptr, 0, nullptr);
    return apply_gate_tc(ctx, state, n, op.qs.data(), op.qs.size(),
                         op.m32.data(), tc_operands(i));
  }
  return apply_gate_ex(ctx, state, n, op.qs.data(), op.qs.size(),
                       op.cqs.data(), op.cqs.size(), op.cvals, op.m32.data(),
                       dm);
}

int PlanRuntime::launch_all(float* state) {
  const unsigned n = plan.num_qubits;
  // Unitary tensor-core plans carry the norm from pass to pass: each
  // tensor-core pass writes its (sum in, sum out) partials into one half of
  // norm_buf and rescales its input by the previous pass's ratio, read from
  // the other half.
  const size_t half = size_t(traj_max_parts(ctx)) * 4;
  const double* prev = nullptr;
  unsigned prev_count = 0;
  int which = 0;
  for (size_t i = 0; i < plan.ops.size(); ++i) {
    const PlanOp& op = plan.ops[i];
    int rc;
    if (restore_norm && op.kind == OpKind::kGate && op.path == Path::kTensor) {
      double* out = norm_buf + which * half;
      if (op.tc_pair_next) {
        rc = apply_gate_tc2_carry(ctx, state, n, op.qs.data(), tc_operands(i),
                                  plan.ops[i + 1].qs.data(),
                                  tc_operands(i + 1), prev, prev_count, out);
      } else {
        rc = apply_gate_tc_carry(ctx, state, n, op.qs.data(), op.qs.size(),
                                 op.m32.data(), tc_operands(i), prev,
                                 prev_count, out);
      }
      prev = out;
      prev_count = tc_grid(ctx, n);
      which ^= 1;
    } else {
      rc = launch_op(i, state);
    }
    if (rc) return rc;
    if (op.tc_pair_next) ++i;
  }
  return QSG_OK;
}

int PlanRuntime::run(qsg_ctx* c, float* state, unsigned seed,
                     std::vector<uint64_t>* mbits) {
  ctx = c;
  int rc = upload(ctx);
  if (rc) return rc;
  rc = prepare_tc();
  if (rc) return rc;
  if (restore_norm) return launch_all(state);
  std::mt19937 rgen(seed);
  const unsigned n = plan.num_qubits;
  for (size_t i = 0; i < plan.ops.size(); ++i) {
    const PlanOp& op = plan.ops[i];
    if (op.kind == OpKind::kMeasure) {
      uint64_t mask = 0;
      for (unsigned q : op.qs) mask |= uint64_t{1} << q;
      std::uniform_real_distribution<double> d(0.0, 1.0);
      const double u = d(rgen);
      uint64_t bits = 0;
      rc = qsg_measure(ctx, state, n, mask, u, 1, &bits);
      if (rc) return rc;
      if (mbits) mbits->push_back(bits);
      continue;
    }
    rc = launch_op(i, state);
    if (rc) return rc;
    if (op.tc_pair_next) ++i;
  }
  return QSG_OK;
}

int PlanRuntime::capture(qsg_ctx* c, float* state) {
  ctx = c;
  for (const auto& op : plan.ops) {
    if (op.kind == OpKind::kMeasure) {
      set_error_msg("plans with measurements cannot be captured");
      return QSG_ERR_UNSUPPORTED;
    }
  }
  int rc = upload(ctx);
  if (rc) return rc;
  rc = prepare_tc();
  if (rc) return rc;
  // One-time kernel attribute and occupancy set-up happens before the graph
  // is recorded.
  for (const auto& op : plan.ops) {
    if (op.path == Path::kTensor) continue;
    const bool pair = op.qs.empty() || op.qs[0] != 0;
    rc = apply_gate_prepare(op.qs.size(), pair, 0);
    if (rc) return rc;
  }
  if (graph_exec) {
    cudaGraphExecDestroy(static_cast<cudaGraphExec_t>(graph_exec));
    cudaGraphDestroy(static_cast<cudaGraph_t>(graph));
    graph_exec = graph = nullptr;
  }
  cudaStream_t s = static_cast<cudaStream_t>(ctx_stream(ctx));
  if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) !=
      cudaSuccess) {
    set_error_msg("cudaStreamBeginCapture failed");
    return QSG_ERR_CUDA;
  }
  rc = launch_all(state);
  if (rc) {
    cudaGraph_t g = nullptr;
    cudaStreamEndCapture(s, &g);
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  cudaGraph_t g = nullptr;
  if (cudaStreamEndCapture(s, &g) != cudaSuccess) {
    set_error_msg("cudaStreamEndCapture failed");
    return QSG_ERR_CUDA;
  }
  cudaGraphExec_t ge = nullptr;
  if (cudaGraphInstantiate(&ge, g, 0) != cudaSuccess) {
    cudaGraphDestroy(g);
    set_error_msg("cudaGraphInstantiate failed");
    return QSG_ERR_CUDA;
  }
  graph = g;
  graph_exec = ge;
  captured_state = state;
  return QSG_OK;
}

int PlanRuntime::profile(qsg_ctx* c, float* state, std::vector<float>* ms) {
  ctx = c;
  int rc = upload(ctx);
  if (rc) return rc;
  rc = prepare_tc();
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(ctx_stream(ctx));
  const size_t nops = plan.ops.size();
  std::vector<cudaEvent_t> ev(nops + 1);
  for (auto& e : ev) cudaEventCreate(&e);
  cudaEventRecord(ev[0], s);
  for (size_t i = 0; i < nops; ++i) {
    if (plan.ops[i].kind != OpKind::kMeasure) {
      rc = launch_op(i, state);
      if (rc) break;
    }
    cudaEventRecord(ev[i + 1], s);
    if (plan.ops[i].tc_pair_next) {
      // The pair's time is op i's; op i + 1 gets 0.
      cudaEventRecord(ev[i + 2], s);
      ++i;
    }
  }
  cudaEventSynchronize(ev[nops]);
  ms->assign(nops, 0.f);
  for (size_t i = 0; rc == QSG_OK && i < nops; ++i)
    cudaEventElapsedTime(&(*ms)[i], ev[i], ev[i + 1]);
  for (auto& e : ev) cudaEventDestroy(e);
  return rc;
}

int PlanRuntime::replay(qsg_ctx* c) {
  if (!graph_exec) {
    set_error_msg("plan has no captured graph");
    return QSG_ERR_INVALID;
  }
  cudaStream_t s = static_cast<cudaStream_t>(ctx_stream(c));
  if (cudaGraphLaunch(static_cast<cudaGraphExec_t>(graph_exec), s) !=
      cudaSuccess) {
    set_error_msg("cudaGraphLaunch failed");
    return QSG_ERR_CUDA;
  }
  return QSG_OK;
}

}  // namespace host
}  // namespace qsg
