// Internal definitions shared by the CUDA translation units of the engine.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>

#include "qsim_gb300.h"

namespace qsg {

// Thread-local last error message (qsg_last_error).
void set_error(const char* fmt, ...);
void clear_error();

// Converts a CUDA error into a status code and records the message.
int cuda_status(cudaError_t e, const char* what);

#define QSG_CUDA(call)                                   \
  do {                                                   \
    cudaError_t e__ = (call);                            \
    if (e__ != cudaSuccess) return qsg::cuda_status(e__, #call); \
  } while (0)

#define QSG_LAUNCHED(ctx)                                \
  do {                                                   \
    cudaError_t e__ = cudaPeekAtLastError();             \
    if (e__ != cudaSuccess) return qsg::cuda_status(e__, "kernel launch"); \
    (ctx)->launches++;                                   \
  } while (0)

#define QSG_CHECK_ARG(cond, ...)                         \
  do {                                                   \
    if (!(cond)) {                                       \
      qsg::set_error(__VA_ARGS__);                       \
      return QSG_ERR_INVALID;                            \
    }                                                    \
  } while (0)

constexpr unsigned kMaxQubits = 40;   // 2^40 complex64 = 8 TiB: beyond HBM
constexpr unsigned kMaxTargets = 6;   // fused gates up to six qubits

inline uint64_t min_size(unsigned n) {
  uint64_t s = uint64_t{2} << n;
  return s < 64 ? 64 : s;
}

}  // namespace qsg

struct qsg_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int num_sms = 0;
  int max_smem_optin = 0;
  uint64_t launches = 0;

  // Device scratch for reductions / sampling, grown on demand.
  void* scratch = nullptr;
  size_t scratch_size = 0;
  // Pinned host scratch for small results.
  void* hscratch = nullptr;
  size_t hscratch_size = 0;

  cudaEvent_t ev0 = nullptr, ev1 = nullptr;

  // Ring of device slots (32 KiB each) for matrices of k >= 5 gates, fed
  // through pinned staging slots guarded by events.
  static constexpr int kRingSlots = 64;
  static constexpr size_t kRingSlotFloats = 8192;
  float* ring_dev = nullptr;
  float* ring_host = nullptr;
  cudaEvent_t ring_ev[kRingSlots] = {};
  bool ring_used[kRingSlots] = {};
  int ring_next = 0;

  // Device operands of single tensor-core gate calls.
  void* tc_slot = nullptr;
  size_t tc_slot_size = 0;

  // Ring of tensor-core operand slots (64 KiB each) for gates whose operands
  // are built on the host per call, fed asynchronously from pinned staging
  // slots guarded by events.
  static constexpr int kTcRingSlots = 8;
  unsigned char* tc_ring_dev = nullptr;
  unsigned char* tc_ring_host = nullptr;
  cudaEvent_t tc_ring_ev[kTcRingSlots] = {};
  bool tc_ring_used[kTcRingSlots] = {};
  int tc_ring_next = 0;
};

namespace qsg {

// Returns a device scratch pointer of at least `bytes` (synchronises the
// stream before replacing a smaller buffer).
int get_scratch(qsg_ctx* ctx, size_t bytes, void** out);
int get_hscratch(qsg_ctx* ctx, size_t bytes, void** out);
int get_tc_operand_slot(qsg_ctx* ctx, size_t bytes, void** out);

// Validates a qubit list: distinct, sorted ascending, < n.
bool valid_qubits(const unsigned* qs, unsigned k, unsigned n);

}  // namespace qsg
