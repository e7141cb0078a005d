// Cost-model network of the learned fusion planner: a 3-layer perceptron
// (16 inputs, two hidden layers of 64 ReLU units, one output) trained on the
// device by the kernels below.  It has no counterpart in the reference,
// whose fuser (lib/fuser_mqubit.h) uses a fixed maximum block size.
//
// Parameter vector layout (floats): W1 [16][64], b1 [64], W2 [64][64],
// b2 [64], W3 [64], b3 [1]; row i of W1 / W2 holds the weights from input
// (or hidden unit) i to every unit of the next layer.
//
// Training minimises the mean squared error of the prediction.  Gradients
// are formed per block of 64 samples in shared memory and summed over blocks
// in a fixed order, so a training run is deterministic; Adam updates the
// parameters on the device.

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "common.cuh"
#include "internal.h"
#include "mlp_dev.h"

namespace qsg {

namespace {

constexpr int kIn = kMlpInputs;
constexpr int kH = kMlpHidden;
constexpr int kW1 = 0;
constexpr int kB1 = kW1 + kIn * kH;
constexpr int kW2 = kB1 + kH;
constexpr int kB2 = kW2 + kH * kH;
constexpr int kW3 = kB2 + kH;
constexpr int kB3 = kW3 + kH;
constexpr int kP = kB3 + 1;
static_assert(kP == kMlpParams, "parameter count");

constexpr int kSamplesPerBlock = 64;
// Shared memory of the gradient kernel: parameters, then per sample the
// input, both hidden activations, their error terms and the output error.
constexpr size_t kGradSmemFloats =
    kP + kSamplesPerBlock * (kIn + 4 * kH + 1);

}  // namespace

// One thread per sample.
__global__ void __launch_bounds__(256)
    mlp_forward_kernel(const float* __restrict__ params,
                       const float* __restrict__ x, uint64_t n,
                       float* __restrict__ out) {
  __shared__ float p[kP];
  for (int i = threadIdx.x; i < kP; i += blockDim.x) p[i] = params[i];
  __syncthreads();
  for (uint64_t s = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; s < n;
       s += uint64_t(gridDim.x) * blockDim.x) {
    float xi[kIn];
#pragma unroll
    for (int i = 0; i < kIn; ++i) xi[i] = x[s * kIn + i];
    float h1[kH];
#pragma unroll 1
    for (int j = 0; j < kH; ++j) {
      float z = p[kB1 + j];
#pragma unroll
      for (int i = 0; i < kIn; ++i) z += xi[i] * p[kW1 + i * kH + j];
      h1[j] = z > 0.f ? z : 0.f;
    }
    float acc = p[kB3];
#pragma unroll 1
    for (int j2 = 0; j2 < kH; ++j2) {
      float z = p[kB2 + j2];
#pragma unroll 8
      for (int j = 0; j < kH; ++j) z += h1[j] * p[kW2 + j * kH + j2];
      acc += (z > 0.f ? z : 0.f) * p[kW3 + j2];
    }
    out[s] = acc;
  }
}

// Block b handles samples [b * 64, b * 64 + 64) of the index list (or of
// the data when idx is null) and writes its part of the gradient of
// (scale / 2) * sum(err^2) -- with scale = 2 / count, the gradient of the
// mean squared error -- and its sum of squared errors.
__global__ void __launch_bounds__(kSamplesPerBlock)
    mlp_grad_kernel(const float* __restrict__ params,
                    const float* __restrict__ x, const float* __restrict__ y,
                    const uint32_t* __restrict__ idx, uint64_t count,
                    float scale, float* __restrict__ partial,
                    double* __restrict__ sq_err) {
  extern __shared__ float sm[];
  float* p = sm;
  float* X = p + kP;                       // [64][16]
  float* H1 = X + kSamplesPerBlock * kIn;  // [64][64]
  float* D1 = H1 + kSamplesPerBlock * kH;
  float* H2 = D1 + kSamplesPerBlock * kH;
  float* D2 = H2 + kSamplesPerBlock * kH;
  float* D3 = D2 + kSamplesPerBlock * kH;  // [64]
  const int t = threadIdx.x;
  for (int i = t; i < kP; i += kSamplesPerBlock) p[i] = params[i];
  __syncthreads();

  const uint64_t s = uint64_t(blockIdx.x) * kSamplesPerBlock + t;
  double err2 = 0.0;
  if (s < count) {
    const uint64_t row = idx ? idx[s] : s;
#pragma unroll
    for (int i = 0; i < kIn; ++i) X[t * kIn + i] = x[row * kIn + i];
    float h1[kH];
#pragma unroll
    for (int j = 0; j < kH; ++j) {
      float z = p[kB1 + j];
#pragma unroll
      for (int i = 0; i < kIn; ++i) z += X[t * kIn + i] * p[kW1 + i * kH + j];
      h1[j] = z > 0.f ? z : 0.f;
      H1[t * kH + j] = h1[j];
    }
    float pred = p[kB3];
    for (int j2 = 0; j2 < kH; ++j2) {
      float z = p[kB2 + j2];
#pragma unroll
      for (int j = 0; j < kH; ++j) z += h1[j] * p[kW2 + j * kH + j2];
      const float h2 = z > 0.f ? z : 0.f;
      H2[t * kH + j2] = h2;
      pred += h2 * p[kW3 + j2];
    }
    const float err = pred - y[row];
    err2 = double(err) * double(err);
    const float d3 = scale * err;
    D3[t] = d3;
    for (int j2 = 0; j2 < kH; ++j2)
      D2[t * kH + j2] = H2[t * kH + j2] > 0.f ? d3 * p[kW3 + j2] : 0.f;
    for (int j = 0; j < kH; ++j) {
      float g = 0.f;
      if (h1[j] > 0.f) {
#pragma unroll 8
        for (int j2 = 0; j2 < kH; ++j2) g += p[kW2 + j * kH + j2] * D2[t * kH + j2];
      }
      D1[t * kH + j] = g;
    }
  } else {
    for (int i = 0; i < kIn; ++i) X[t * kIn + i] = 0.f;
    for (int j = 0; j < kH; ++j) {
      H1[t * kH + j] = 0.f;
      D1[t * kH + j] = 0.f;
      H2[t * kH + j] = 0.f;
      D2[t * kH + j] = 0.f;
    }
    D3[t] = 0.f;
  }
  __syncthreads();

  float* out = partial + size_t(blockIdx.x) * kP;
  for (int e = t; e < kP; e += kSamplesPerBlock) {
    float g = 0.f;
    if (e < kB1) {                       // W1[i][j]
      const int i = e / kH, j = e % kH;
      for (int u = 0; u < kSamplesPerBlock; ++u) g += X[u * kIn + i] * D1[u * kH + j];
    } else if (e < kW2) {                // b1[j]
      const int j = e - kB1;
      for (int u = 0; u < kSamplesPerBlock; ++u) g += D1[u * kH + j];
    } else if (e < kB2) {                // W2[j][j2]
      const int j = (e - kW2) / kH, j2 = (e - kW2) % kH;
      for (int u = 0; u < kSamplesPerBlock; ++u) g += H1[u * kH + j] * D2[u * kH + j2];
    } else if (e < kW3) {                // b2[j2]
      const int j2 = e - kB2;
      for (int u = 0; u < kSamplesPerBlock; ++u) g += D2[u * kH + j2];
    } else if (e < kB3) {                // W3[j2]
      const int j2 = e - kW3;
      for (int u = 0; u < kSamplesPerBlock; ++u) g += D3[u] * H2[u * kH + j2];
    } else {                             // b3
      for (int u = 0; u < kSamplesPerBlock; ++u) g += D3[u];
    }
    out[e] = g;
  }

  // Sum of squared errors of the block (fixed order).
  __shared__ double red[kSamplesPerBlock];
  red[t] = err2;
  __syncthreads();
  if (t == 0) {
    double a = 0.0;
    for (int u = 0; u < kSamplesPerBlock; ++u) a += red[u];
    sq_err[blockIdx.x] = a;
  }
}

// grad[e] = sum over blocks of partial[b][e], in block order.
__global__ void mlp_reduce_kernel(const float* __restrict__ partial,
                                  unsigned blocks, float* __restrict__ grad) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= kP) return;
  float g = 0.f;
  for (unsigned b = 0; b < blocks; ++b) g += partial[size_t(b) * kP + e];
  grad[e] = g;
}

// Adam (Kingma and Ba, 2015) with bias corrections c1 = 1 / (1 - beta1^t),
// c2 = 1 / (1 - beta2^t).
__global__ void mlp_adam_kernel(float* __restrict__ params,
                                float* __restrict__ m, float* __restrict__ v,
                                const float* __restrict__ grad, float lr,
                                float beta1, float beta2, float eps, float c1,
                                float c2) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= kP) return;
  const float g = grad[e];
  const float mm = beta1 * m[e] + (1.f - beta1) * g;
  const float vv = beta2 * v[e] + (1.f - beta2) * g * g;
  m[e] = mm;
  v[e] = vv;
  params[e] -= lr * (mm * c1) / (sqrtf(vv * c2) + eps);
}

// ---------------------------------------------------------------------------
// Host side: training, full-batch gradients and batched prediction.  The
// data arrive as host arrays and are uploaded once per call.

namespace {

struct DevBuf {
  qsg_ctx* ctx = nullptr;
  void* p = nullptr;
  ~DevBuf() {
    if (p) dev_free(ctx, p);
  }
  int alloc(qsg_ctx* c, size_t bytes) {
    ctx = c;
    return dev_alloc(c, bytes < 16 ? 16 : bytes, &p);
  }
  template <typename T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

unsigned grad_blocks(uint64_t count) {
  return unsigned((count + kSamplesPerBlock - 1) / kSamplesPerBlock);
}

int launch_grad(qsg_ctx* ctx, const float* params, const float* x,
                const float* y, const uint32_t* idx, uint64_t count,
                float* partial, double* sq_err, float* grad) {
  const unsigned blocks = grad_blocks(count);
  const size_t smem = kGradSmemFloats * sizeof(float);
  QSG_CUDA(cudaFuncSetAttribute(mlp_grad_kernel,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                int(smem)));
  mlp_grad_kernel<<<blocks, kSamplesPerBlock, smem, ctx->stream>>>(
      params, x, y, idx, count, 2.0f / float(count), partial, sq_err);
  QSG_LAUNCHED(ctx);
  mlp_reduce_kernel<<<(kP + 255) / 256, 256, 0, ctx->stream>>>(partial,
                                                              blocks, grad);
  QSG_LAUNCHED(ctx);
  return QSG_OK;
}

}  // namespace

int mlp_gradient(qsg_ctx* ctx, const float* params, const float* x,
                 const float* y, uint64_t n, float* grad_out, double* loss) {
  QSG_CHECK_ARG(n > 0 && n < (uint64_t{1} << 31), "mlp: 1..2^31 samples");
  DevBuf dp, dx, dy, dpart, dsq, dg;
  const unsigned blocks = grad_blocks(n);
  int rc;
  if ((rc = dp.alloc(ctx, kP * 4)) || (rc = dx.alloc(ctx, n * kIn * 4)) ||
      (rc = dy.alloc(ctx, n * 4)) ||
      (rc = dpart.alloc(ctx, size_t(blocks) * kP * 4)) ||
      (rc = dsq.alloc(ctx, blocks * 8)) || (rc = dg.alloc(ctx, kP * 4)))
    return rc;
  if ((rc = dev_upload(ctx, dp.p, params, kP * 4)) ||
      (rc = dev_upload(ctx, dx.p, x, n * kIn * 4)) ||
      (rc = dev_upload(ctx, dy.p, y, n * 4)))
    return rc;
  rc = launch_grad(ctx, dp.as<float>(), dx.as<float>(), dy.as<float>(),
                   nullptr, n, dpart.as<float>(), dsq.as<double>(),
                   dg.as<float>());
  if (rc) return rc;
  std::vector<double> sq(blocks);
  QSG_CUDA(cudaMemcpyAsync(grad_out, dg.p, kP * 4, cudaMemcpyDeviceToHost,
                           ctx->stream));
  QSG_CUDA(cudaMemcpyAsync(sq.data(), dsq.p, blocks * 8,
                           cudaMemcpyDeviceToHost, ctx->stream));
  QSG_CUDA(cudaStreamSynchronize(ctx->stream));
  double a = 0;
  for (double v : sq) a += v;
  if (loss) *loss = a / double(n);
  return QSG_OK;
}

int mlp_predict(qsg_ctx* ctx, const float* params, const float* x, uint64_t n,
                float* out) {
  QSG_CHECK_ARG(n > 0, "mlp: no samples");
  DevBuf dp, dx, dout;
  int rc;
  if ((rc = dp.alloc(ctx, kP * 4)) || (rc = dx.alloc(ctx, n * kIn * 4)) ||
      (rc = dout.alloc(ctx, n * 4)))
    return rc;
  if ((rc = dev_upload(ctx, dp.p, params, kP * 4)) ||
      (rc = dev_upload(ctx, dx.p, x, n * kIn * 4)))
    return rc;
  const unsigned grid =
      unsigned(std::min<uint64_t>((n + 255) / 256, uint64_t(ctx->num_sms) * 8));
  mlp_forward_kernel<<<grid, 256, 0, ctx->stream>>>(dp.as<float>(),
                                                    dx.as<float>(), n,
                                                    dout.as<float>());
  QSG_LAUNCHED(ctx);
  QSG_CUDA(cudaMemcpyAsync(out, dout.p, n * 4, cudaMemcpyDeviceToHost,
                           ctx->stream));
  QSG_CUDA(cudaStreamSynchronize(ctx->stream));
  return QSG_OK;
}

int mlp_train(qsg_ctx* ctx, float* params, const float* x, const float* y,
              uint64_t n, unsigned steps, unsigned batch, float lr,
              uint64_t seed, double* final_loss) {
  QSG_CHECK_ARG(n > 0 && n < (uint64_t{1} << 31), "mlp: 1..2^31 samples");
  QSG_CHECK_ARG(batch > 0 && lr > 0.f, "mlp: batch and lr must be positive");
  const uint64_t b = std::min<uint64_t>(batch, n);
  const unsigned blocks = grad_blocks(std::max<uint64_t>(b, n));
  DevBuf dp, dm, dv, dx, dy, didx, dpart, dsq, dg;
  int rc;
  if ((rc = dp.alloc(ctx, kP * 4)) || (rc = dm.alloc(ctx, kP * 4)) ||
      (rc = dv.alloc(ctx, kP * 4)) || (rc = dx.alloc(ctx, n * kIn * 4)) ||
      (rc = dy.alloc(ctx, n * 4)) || (rc = didx.alloc(ctx, n * 4)) ||
      (rc = dpart.alloc(ctx, size_t(blocks) * kP * 4)) ||
      (rc = dsq.alloc(ctx, blocks * 8)) || (rc = dg.alloc(ctx, kP * 4)))
    return rc;
  if ((rc = dev_upload(ctx, dp.p, params, kP * 4)) ||
      (rc = dev_upload(ctx, dx.p, x, n * kIn * 4)) ||
      (rc = dev_upload(ctx, dy.p, y, n * 4)))
    return rc;
  QSG_CUDA(cudaMemsetAsync(dm.p, 0, kP * 4, ctx->stream));
  QSG_CUDA(cudaMemsetAsync(dv.p, 0, kP * 4, ctx->stream));

  // Epochs over a fresh permutation of the samples (std::mt19937_64(seed)).
  std::mt19937_64 rng(seed);
  std::vector<uint32_t> perm(n);
  for (uint64_t i = 0; i < n; ++i) perm[i] = uint32_t(i);
  const float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
  uint64_t off = n;
  for (unsigned step = 1; step <= steps; ++step) {
    if (off + b > n) {
      for (uint64_t i = n - 1; i > 0; --i) {
        const uint64_t j = rng() % (i + 1);
        std::swap(perm[i], perm[j]);
      }
      // The upload must not overwrite indices that earlier launches still
      // read: wait for the stream before re-staging.
      QSG_CUDA(cudaStreamSynchronize(ctx->stream));
      if ((rc = dev_upload(ctx, didx.p, perm.data(), n * 4))) return rc;
      off = 0;
    }
    rc = launch_grad(ctx, dp.as<float>(), dx.as<float>(), dy.as<float>(),
                     didx.as<uint32_t>() + off, b, dpart.as<float>(),
                     dsq.as<double>(), dg.as<float>());
    if (rc) return rc;
    off += b;
    const float c1 = float(1.0 / (1.0 - std::pow(double(beta1), double(step))));
    const float c2 = float(1.0 / (1.0 - std::pow(double(beta2), double(step))));
    mlp_adam_kernel<<<(kP + 255) / 256, 256, 0, ctx->stream>>>(
        dp.as<float>(), dm.as<float>(), dv.as<float>(), dg.as<float>(), lr,
        beta1, beta2, eps, c1, c2);
    QSG_LAUNCHED(ctx);
  }
  QSG_CUDA(cudaMemcpyAsync(params, dp.p, kP * 4, cudaMemcpyDeviceToHost,
                           ctx->stream));
  QSG_CUDA(cudaStreamSynchronize(ctx->stream));
  if (final_loss) {
    std::vector<float> g(kP);
    rc = mlp_gradient(ctx, params, x, y, n, g.data(), final_loss);
    if (rc) return rc;
  }
  return QSG_OK;
}

}  // namespace qsg
