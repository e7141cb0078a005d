// Context, allocation, copies, timing and error reporting of the C ABI.
// Replaces VectorSpaceCUDA (lib/vectorspace_cuda.h) and the ErrorCheck/exit
// convention of lib/util_cuda.h:31-39 with status codes.

#include <cstdarg>
#include <cstring>
#include <sys/syscall.h>
#include <unistd.h>

#include "common.cuh"
#include "internal.h"
#include "matring.cuh"

namespace qsg {

static thread_local char g_err[512] = {0};

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

void clear_error() { g_err[0] = 0; }

int cuda_status(cudaError_t e, const char* what) {
  set_error("CUDA error in %s: %s", what, cudaGetErrorString(e));
  if (e == cudaErrorMemoryAllocation) return QSG_ERR_OOM;
  return QSG_ERR_CUDA;
}

int get_scratch(qsg_ctx* ctx, size_t bytes, void** out) {
  if (bytes > ctx->scratch_size) {
    if (ctx->scratch) {
      QSG_CUDA(cudaStreamSynchronize(ctx->stream));
      QSG_CUDA(cudaFree(ctx->scratch));
      ctx->scratch = nullptr;
      ctx->scratch_size = 0;
    }
    size_t sz = bytes < 4096 ? 4096 : bytes;
    cudaError_t e = cudaMalloc(&ctx->scratch, sz);
    if (e != cudaSuccess) {
      ctx->scratch = nullptr;
      return cuda_status(e, "scratch allocation");
    }
    ctx->scratch_size = sz;
  }
  *out = ctx->scratch;
  return QSG_OK;
}

int get_hscratch(qsg_ctx* ctx, size_t bytes, void** out) {
  if (bytes > ctx->hscratch_size) {
    if (ctx->hscratch) {
      QSG_CUDA(cudaStreamSynchronize(ctx->stream));
      QSG_CUDA(cudaFreeHost(ctx->hscratch));
      ctx->hscratch = nullptr;
      ctx->hscratch_size = 0;
    }
    size_t sz = bytes < 4096 ? 4096 : bytes;
    cudaError_t e = cudaMallocHost(&ctx->hscratch, sz);
    if (e != cudaSuccess) {
      ctx->hscratch = nullptr;
      return cuda_status(e, "pinned scratch allocation");
    }
    ctx->hscratch_size = sz;
  }
  *out = ctx->hscratch;
  return QSG_OK;
}

int get_tc_operand_slot(qsg_ctx* ctx, size_t bytes, void** out) {
  if (bytes > ctx->tc_slot_size) {
    if (ctx->tc_slot) {
      QSG_CUDA(cudaStreamSynchronize(ctx->stream));
      QSG_CUDA(cudaFree(ctx->tc_slot));
      ctx->tc_slot = nullptr;
      ctx->tc_slot_size = 0;
    }
    QSG_CUDA(cudaMalloc(&ctx->tc_slot, bytes));
    ctx->tc_slot_size = bytes;
  }
  *out = ctx->tc_slot;
  return QSG_OK;
}

bool valid_qubits(const unsigned* qs, unsigned k, unsigned n) {
  if (k > 0 && qs == nullptr) return false;
  for (unsigned i = 0; i < k; ++i) {
    if (qs[i] >= n) return false;
    if (i > 0 && qs[i] <= qs[i - 1]) return false;
  }
  return true;
}

int dev_alloc(qsg_ctx* ctx, size_t bytes, void** out) {
  cudaSetDevice(ctx->device);
  cudaError_t e = cudaMalloc(out, bytes);
  if (e != cudaSuccess) {
    *out = nullptr;
    return cuda_status(e, "device allocation");
  }
  return QSG_OK;
}

int dev_free(qsg_ctx* ctx, void* p) {
  if (!p) return QSG_OK;
  QSG_CUDA(cudaStreamSynchronize(ctx->stream));
  QSG_CUDA(cudaFree(p));
  return QSG_OK;
}

int dev_upload(qsg_ctx* ctx, void* dst, const void* src, size_t bytes) {
  QSG_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice,
                           ctx->stream));
  QSG_CUDA(cudaStreamSynchronize(ctx->stream));
  return QSG_OK;
}

void* ctx_stream(qsg_ctx* ctx) { return ctx->stream; }
int ctx_device(qsg_ctx* ctx) { return ctx->device; }

}  // namespace qsg

using namespace qsg;

extern "C" {

const char* qsg_last_error(void) { return g_err; }

const char* qsg_version(void) { return "qsim_gb300 0.1 (sm_103a)"; }

int qsg_ctx_create(int device, void* stream, qsg_ctx** out) {
  clear_error();
  QSG_CHECK_ARG(out != nullptr, "qsg_ctx_create: null out");
  *out = nullptr;
  int count = 0;
  QSG_CUDA(cudaGetDeviceCount(&count));
  QSG_CHECK_ARG(device >= 0 && device < count,
                "qsg_ctx_create: device %d not present (%d devices)", device,
                count);
  QSG_CUDA(cudaSetDevice(device));
  qsg_ctx* ctx = new qsg_ctx();
  ctx->device = device;
  if (stream) {
    ctx->stream = static_cast<cudaStream_t>(stream);
  } else {
    cudaError_t e =
        cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      delete ctx;
      return cuda_status(e, "cudaStreamCreate");
    }
    ctx->own_stream = true;
  }
  cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount,
                         device);
  cudaDeviceGetAttribute(&ctx->max_smem_optin,
                         cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
  cudaEventCreate(&ctx->ev0);
  cudaEventCreate(&ctx->ev1);
  *out = ctx;
  return QSG_OK;
}

int qsg_ctx_destroy(qsg_ctx* ctx) {
  if (!ctx) return QSG_OK;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  matring_release(ctx);
  tcring_release(ctx);
  if (ctx->scratch) cudaFree(ctx->scratch);
  if (ctx->tc_slot) cudaFree(ctx->tc_slot);
  if (ctx->hscratch) cudaFreeHost(ctx->hscratch);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return QSG_OK;
}

int qsg_ctx_sync(qsg_ctx* ctx) {
  QSG_CHECK_ARG(ctx, "null context");
  QSG_CUDA(cudaStreamSynchronize(ctx->stream));
  return QSG_OK;
}

int qsg_ctx_num_sms(qsg_ctx* ctx, int* out) {
  QSG_CHECK_ARG(ctx && out, "null argument");
  *out = ctx->num_sms;
  return QSG_OK;
}

void* qsg_ctx_stream(qsg_ctx* ctx) { return ctx ? ctx->stream : nullptr; }

uint64_t qsg_ctx_launch_count(qsg_ctx* ctx) { return ctx ? ctx->launches : 0; }

int qsg_ctx_scratch_bytes(qsg_ctx* ctx, size_t* device_bytes,
                          size_t* pinned_bytes) {
  QSG_CHECK_ARG(ctx && device_bytes && pinned_bytes, "null argument");
  *device_bytes = ctx->scratch_size;
  *pinned_bytes = ctx->hscratch_size;
  return QSG_OK;
}

uint64_t qsg_min_size(unsigned num_qubits) { return min_size(num_qubits); }

int qsg_state_create(qsg_ctx* ctx, unsigned n, float** out) {
  clear_error();
  QSG_CHECK_ARG(ctx && out, "qsg_state_create: null argument");
  *out = nullptr;
  QSG_CHECK_ARG(n <= kMaxQubits, "qsg_state_create: %u qubits > %u", n,
                kMaxQubits);
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, min_size(n) * sizeof(float));
  if (e != cudaSuccess) {
    cudaGetLastError();  // clear the sticky-free allocation error
    set_error("not enough device memory for %u qubits", n);
    return QSG_ERR_OOM;
  }
  *out = static_cast<float*>(p);
  return QSG_OK;
}

int qsg_state_free(qsg_ctx* ctx, float* state) {
  QSG_CHECK_ARG(ctx, "null context");
  if (!state) return QSG_OK;
  QSG_CUDA(cudaStreamSynchronize(ctx->stream));
  QSG_CUDA(cudaFree(state));
  return QSG_OK;
}

int qsg_host_alloc(size_t bytes, void** out) {
  QSG_CHECK_ARG(out, "qsg_host_alloc: null out");
  *out = nullptr;
  cudaError_t e = cudaMallocHost(out, bytes);
  if (e != cudaSuccess) {
    *out = nullptr;
    cudaGetLastError();
    set_error("pinned host allocation of %zu bytes failed", bytes);
    return QSG_ERR_OOM;
  }
  return QSG_OK;
}

}  // extern "C"

namespace {

// cudaMallocHost with this thread's memory policy set to "preferred node"
// for the call (the pages are allocated and pinned inside it), then the
// previous policy restored.  Preferred, not bound: a full node falls back to
// another one instead of failing.
int host_alloc_on_node(int node, size_t bytes, void** out) {
#if defined(SYS_get_mempolicy) && defined(SYS_set_mempolicy)
  constexpr int kMpolPreferred = 1;
  constexpr int kMaskWords = 16;   // nodes 0..1023
  constexpr unsigned long kMaxNode = 64 * kMaskWords;
  if (node < 0 || node >= int(kMaxNode)) return QSG_ERR_UNSUPPORTED;
  int old_mode = 0;
  unsigned long old_mask[kMaskWords] = {};
  if (syscall(SYS_get_mempolicy, &old_mode, old_mask, kMaxNode, nullptr,
              0ul) != 0)
    return QSG_ERR_UNSUPPORTED;
  unsigned long mask[kMaskWords] = {};
  mask[node / 64] = 1ul << (node % 64);
  // maxnode counts one bit more than the mask holds (the kernel drops the
  // last one), as libnuma passes it.
  if (syscall(SYS_set_mempolicy, kMpolPreferred, mask, kMaxNode + 1) != 0)
    return QSG_ERR_UNSUPPORTED;
  const cudaError_t e = cudaMallocHost(out, bytes);
  syscall(SYS_set_mempolicy, old_mode, old_mode ? old_mask : nullptr,
          old_mode ? kMaxNode + 1 : 0ul);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *out = nullptr;
    return QSG_ERR_OOM;
  }
  return QSG_OK;
#else
  (void)node; (void)bytes; (void)out;
  return QSG_ERR_UNSUPPORTED;
#endif
}

}  // namespace

extern "C" {

int qsg_host_numa_node(int device, int* out) {
  QSG_CHECK_ARG(out, "qsg_host_numa_node: null out");
  *out = -1;
  if (cudaDeviceGetAttribute(out, cudaDevAttrHostNumaId, device) !=
      cudaSuccess) {
    cudaGetLastError();
    *out = -1;
  }
  return QSG_OK;
}

int qsg_host_alloc_near(int device, size_t bytes, void** out) {
  QSG_CHECK_ARG(out, "qsg_host_alloc_near: null out");
  *out = nullptr;
  int node = -1;
  if (cudaDeviceGetAttribute(&node, cudaDevAttrHostNumaId, device) !=
      cudaSuccess) {
    cudaGetLastError();
    node = -1;
  }
  if (node >= 0 && bytes > 0 &&
      host_alloc_on_node(node, bytes, out) == QSG_OK)
    return QSG_OK;
  return qsg_host_alloc(bytes, out);
}

int qsg_host_free(void* p) {
  if (p) QSG_CUDA(cudaFreeHost(p));
  return QSG_OK;
}

int qsg_copy_d2d(qsg_ctx* ctx, float* dest, const float* src, unsigned n) {
  QSG_CHECK_ARG(ctx && dest && src, "qsg_copy_d2d: null argument");
  QSG_CUDA(cudaMemcpyAsync(dest, src, min_size(n) * sizeof(float),
                           cudaMemcpyDeviceToDevice, ctx->stream));
  return QSG_OK;
}

int qsg_copy_d2h(qsg_ctx* ctx, float* host_dest, const float* src,
                 unsigned n) {
  QSG_CHECK_ARG(ctx && host_dest && src, "qsg_copy_d2h: null argument");
  QSG_CUDA(cudaMemcpyAsync(host_dest, src, min_size(n) * sizeof(float),
                           cudaMemcpyDeviceToHost, ctx->stream));
  QSG_CUDA(cudaStreamSynchronize(ctx->stream));
  return QSG_OK;
}

int qsg_copy_h2d(qsg_ctx* ctx, float* dest, const float* host_src,
                 unsigned n) {
  QSG_CHECK_ARG(ctx && dest && host_src, "qsg_copy_h2d: null argument");
  QSG_CUDA(cudaMemcpyAsync(dest, host_src, min_size(n) * sizeof(float),
                           cudaMemcpyHostToDevice, ctx->stream));
  QSG_CUDA(cudaStreamSynchronize(ctx->stream));
  return QSG_OK;
}

int qsg_copy_h2d_partial(qsg_ctx* ctx, float* dest, const float* host_src,
                         uint64_t size, unsigned n) {
  QSG_CHECK_ARG(ctx && dest && host_src, "qsg_copy_h2d_partial: null");
  uint64_t s = size < min_size(n) ? size : min_size(n);
  QSG_CUDA(cudaMemcpyAsync(dest, host_src, s * sizeof(float),
                           cudaMemcpyHostToDevice, ctx->stream));
  QSG_CUDA(cudaStreamSynchronize(ctx->stream));
  return QSG_OK;
}

int qsg_timer_start(qsg_ctx* ctx) {
  QSG_CHECK_ARG(ctx, "null context");
  QSG_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
  return QSG_OK;
}

int qsg_timer_stop(qsg_ctx* ctx, float* ms) {
  QSG_CHECK_ARG(ctx && ms, "null argument");
  QSG_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
  QSG_CUDA(cudaEventSynchronize(ctx->ev1));
  QSG_CUDA(cudaEventElapsedTime(ms, ctx->ev0, ctx->ev1));
  return QSG_OK;
}

unsigned qsg_simd_register_size(void) { return 32; }

}  // extern "C"
