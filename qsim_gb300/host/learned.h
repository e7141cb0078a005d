// Learned cost model of the fusion planner.
//
// A small perceptron (csrc/mlp.cu) predicts the time of one fused-gate
// launch from features of the block; the planner (fuser.cc) uses it to
// choose block boundaries, block sizes and the path (CUDA cores or tensor
// cores) of each block.  The network is trained on the device on per-launch
// times the engine records itself (qsg_plan_profile).  It has no
// counterpart in the reference, whose MultiQubitGateFuser
// (lib/fuser_mqubit.h:282-526) fuses up to a fixed max_fused_size; that
// fuser's rule remains the fallback when no model is given.
#pragma once

#include <vector>

#include "engine.h"

namespace qsg {
namespace host {

constexpr unsigned kFeatures = 16;

// Qubits a tensor-core launch acts on: the block's qubits padded to six
// with the lowest free qubits (pad_block_to_6).
std::vector<unsigned> tensor_core_qubits(unsigned n,
                                         const std::vector<unsigned>& qs);

// Feature vector of one launch: n qubits in the state, sorted target qubits
// `qs` as launched (already padded for the tensor-core path), `ncontrols`
// control qubits, the path.
void block_features(unsigned n, const std::vector<unsigned>& qs,
                    unsigned ncontrols, Path path, float* out);

// Training target for a launch of `us` microseconds on n qubits:
// log(us) - (n - 24) log 2, the log-time per 2^24 amplitudes.
double time_target(unsigned n, double us);

struct MlpCostModel : CostModel {
  std::vector<float> params;  // kMlpParams values (mlp_dev.h layout)

  // Network output for one feature vector (host inference).
  double predict(const float* features) const;
  double cost_us(unsigned n, const std::vector<unsigned>& qs,
                 unsigned ncontrols, Path path) const override;
};

// He-uniform initialisation from std::mt19937_64(seed); biases zero.
std::vector<float> mlp_init(uint64_t seed);

}  // namespace host

// The cost model behind a qsg_fuse_options.cost_model handle (a qsg_mlp*),
// or null.
const host::CostModel* cost_model_from_handle(const void* handle);

}  // namespace qsg
