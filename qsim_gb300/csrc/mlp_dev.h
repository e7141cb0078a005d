// Cost-model network of the learned fusion planner: sizes and the device
// entry points of mlp.cu (plain C++ declarations).
#pragma once

#include <cstdint>

#include "qsim_gb300.h"

namespace qsg {

constexpr int kMlpInputs = 16;
constexpr int kMlpHidden = 64;
constexpr int kMlpParams =
    kMlpInputs * kMlpHidden + kMlpHidden + kMlpHidden * kMlpHidden +
    kMlpHidden + kMlpHidden + 1;

// All arrays are host arrays; x is [n][kMlpInputs], y and out are [n],
// params and grad are [kMlpParams].
//
// Gradient of the mean squared error over all n samples, and that error.
int mlp_gradient(qsg_ctx* ctx, const float* params, const float* x,
                 const float* y, uint64_t n, float* grad, double* loss);
// Predictions of the network for n samples.
int mlp_predict(qsg_ctx* ctx, const float* params, const float* x, uint64_t n,
                float* out);
// `steps` Adam steps (learning rate lr) on minibatches of `batch` samples
// drawn as successive slices of per-epoch permutations from
// std::mt19937_64(seed); params is updated in place; final_loss receives
// the mean squared error over all samples afterwards.
int mlp_train(qsg_ctx* ctx, float* params, const float* x, const float* y,
              uint64_t n, unsigned steps, unsigned batch, float lr,
              uint64_t seed, double* final_loss);

}  // namespace qsg
