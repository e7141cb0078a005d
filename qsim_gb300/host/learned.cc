// Learned cost model: features, host inference, and its C ABI
// (include/qsim_gb300.h, "learned fusion planner").

#include "learned.h"

#include <algorithm>
#include <cmath>
#include <new>
#include <random>

#include "internal.h"
#include "mlp_dev.h"
#include "runner.h"

namespace qsg {
namespace host {

static_assert(kFeatures == unsigned(kMlpInputs), "feature count");

std::vector<unsigned> tensor_core_qubits(unsigned n,
                                         const std::vector<unsigned>& qs) {
  std::vector<unsigned> all = qs;
  for (unsigned q = 0; all.size() < 6 && q < n; ++q)
    if (std::find(all.begin(), all.end(), q) == all.end()) all.push_back(q);
  std::sort(all.begin(), all.end());
  return all;
}

void block_features(unsigned n, const std::vector<unsigned>& qs,
                    unsigned ncontrols, Path path, float* f) {
  const unsigned k = unsigned(qs.size());
  f[0] = float(k) / 6.f;
  f[1] = float(ncontrols) / 4.f;
  f[2] = (float(n) - 24.f) / 8.f;
  f[3] = path == Path::kTensor ? 1.f : 0.f;
  for (unsigned j = 0; j < 6; ++j) f[4 + j] = j < k ? float(qs[j]) / 32.f : -0.25f;
  unsigned low3 = 0, low7 = 0, high3 = 0;
  for (unsigned q : qs) {
    low3 += q < 3;
    low7 += q < 7;
    high3 += q + 3 >= n;
  }
  f[10] = (k > 0 && qs[0] == 0) ? 1.f : 0.f;
  f[11] = float(low3) / 3.f;
  f[12] = float(low7) / 6.f;
  f[13] = float(high3) / 3.f;
  f[14] = float(1u << k) / 64.f;
  f[15] = k > 0 ? float(qs[k - 1] - qs[0]) / 32.f : 0.f;
}

double time_target(unsigned n, double us) {
  return std::log(us) - (double(n) - 24.0) * std::log(2.0);
}

double MlpCostModel::predict(const float* x) const {
  constexpr int kIn = kMlpInputs, kH = kMlpHidden;
  const float* W1 = params.data();
  const float* b1 = W1 + kIn * kH;
  const float* W2 = b1 + kH;
  const float* b2 = W2 + kH * kH;
  const float* W3 = b2 + kH;
  const float b3 = W3[kH];
  float h1[kH];
  for (int j = 0; j < kH; ++j) {
    float z = b1[j];
    for (int i = 0; i < kIn; ++i) z += x[i] * W1[i * kH + j];
    h1[j] = z > 0.f ? z : 0.f;
  }
  float acc = b3;
  for (int j2 = 0; j2 < kH; ++j2) {
    float z = b2[j2];
    for (int j = 0; j < kH; ++j) z += h1[j] * W2[j * kH + j2];
    acc += (z > 0.f ? z : 0.f) * W3[j2];
  }
  return acc;
}

double MlpCostModel::cost_us(unsigned n, const std::vector<unsigned>& qs,
                             unsigned ncontrols, Path path) const {
  float f[kFeatures];
  if (path == Path::kTensor) {
    block_features(n, tensor_core_qubits(n, qs), ncontrols, path, f);
  } else {
    block_features(n, qs, ncontrols, path, f);
  }
  return std::exp(predict(f) + (double(n) - 24.0) * std::log(2.0));
}

std::vector<float> mlp_init(uint64_t seed) {
  constexpr int kIn = kMlpInputs, kH = kMlpHidden;
  std::vector<float> p(kMlpParams, 0.f);
  std::mt19937_64 g(seed);
  auto fill = [&](float* w, int count, int fan_in) {
    const double a = std::sqrt(6.0 / fan_in);
    std::uniform_real_distribution<double> d(-a, a);
    for (int i = 0; i < count; ++i) w[i] = float(d(g));
  };
  float* W1 = p.data();
  float* W2 = W1 + kIn * kH + kH;
  float* W3 = W2 + kH * kH + kH;
  fill(W1, kIn * kH, kIn);
  fill(W2, kH * kH, kH);
  fill(W3, kH, kH);
  return p;
}

}  // namespace host
}  // namespace qsg

using namespace qsg;
using namespace qsg::host;

struct qsg_mlp {
  MlpCostModel model;
};

const CostModel* qsg::cost_model_from_handle(const void* h) {
  return h ? &static_cast<const qsg_mlp*>(h)->model : nullptr;
}

namespace {

int invalid(const char* msg) {
  set_error_msg(msg);
  return QSG_ERR_INVALID;
}

bool sorted_lt(const unsigned* qs, unsigned k, unsigned n) {
  for (unsigned i = 0; i < k; ++i) {
    if (qs[i] >= n) return false;
    if (i > 0 && qs[i] <= qs[i - 1]) return false;
  }
  return true;
}

}  // namespace

extern "C" {

uint64_t qsg_mlp_num_params(void) { return kMlpParams; }

int qsg_mlp_create(uint64_t seed, qsg_mlp** out) {
  if (!out) return invalid("null output");
  auto* m = new (std::nothrow) qsg_mlp();
  if (!m) return QSG_ERR_OOM;
  m->model.params = mlp_init(seed);
  *out = m;
  return QSG_OK;
}

int qsg_mlp_destroy(qsg_mlp* m) {
  delete m;
  return QSG_OK;
}

int qsg_mlp_get_params(const qsg_mlp* m, float* out) {
  if (!m || !out) return invalid("null argument");
  std::copy(m->model.params.begin(), m->model.params.end(), out);
  return QSG_OK;
}

int qsg_mlp_set_params(qsg_mlp* m, const float* in) {
  if (!m || !in) return invalid("null argument");
  m->model.params.assign(in, in + kMlpParams);
  return QSG_OK;
}

int qsg_mlp_gradient(qsg_ctx* ctx, const qsg_mlp* m, const float* x,
                     const float* y, uint64_t n, float* grad, double* loss) {
  if (!ctx || !m || !x || !y || !grad) return invalid("null argument");
  return mlp_gradient(ctx, m->model.params.data(), x, y, n, grad, loss);
}

int qsg_mlp_train(qsg_ctx* ctx, qsg_mlp* m, const float* x, const float* y,
                  uint64_t n, unsigned steps, unsigned batch, float lr,
                  uint64_t seed, double* final_loss) {
  if (!ctx || !m || !x || !y) return invalid("null argument");
  std::vector<float> p = m->model.params;
  int rc = mlp_train(ctx, p.data(), x, y, n, steps, batch, lr, seed,
                     final_loss);
  if (rc == QSG_OK) m->model.params = std::move(p);
  return rc;
}

int qsg_mlp_predict(qsg_ctx* ctx, const qsg_mlp* m, const float* x,
                    uint64_t n, float* out) {
  if (!ctx || !m || !x || !out) return invalid("null argument");
  return mlp_predict(ctx, m->model.params.data(), x, n, out);
}

int qsg_block_features(unsigned n, const unsigned* qs, unsigned k,
                       unsigned ncontrols, int path, float* out) {
  if ((k && !qs) || !out) return invalid("null argument");
  if (k > 6 || !sorted_lt(qs, k, n)) return invalid("bad qubits");
  block_features(n, std::vector<unsigned>(qs, qs + k), ncontrols,
                 path ? Path::kTensor : Path::kCudaCore, out);
  return QSG_OK;
}

int qsg_mlp_cost_us(const qsg_mlp* m, unsigned n, const unsigned* qs,
                    unsigned k, unsigned ncontrols, int path, double* out) {
  if (!m || (k && !qs) || !out) return invalid("null argument");
  if (k > 6 || !sorted_lt(qs, k, n)) return invalid("bad qubits");
  *out = m->model.cost_us(n, std::vector<unsigned>(qs, qs + k), ncontrols,
                          path ? Path::kTensor : Path::kCudaCore);
  return QSG_OK;
}

}  // extern "C"
