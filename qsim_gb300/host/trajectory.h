// Noisy circuits and quantum trajectories.
//
// Restates the reference's noise model (lib/channel.h:31-125,
// lib/channels_cirq.h, lib/circuit_noisy.h:33-64) and the sampling of
// QuantumTrajectorySimulator::RunIteration (lib/qtrajectory.h:240-387) on
// the GB300 engine, and runs batches of trajectories on concurrent streams.
//
// How a trajectory runs here.  The draws are the reference's: one
// std::mt19937(rep) per trajectory and one uniform_real_distribution<double>
// (0, 1) value per operation, so every choice that the reference makes from
// the lower probability bounds alone (all unitary channels, and the first
// Kraus operator of a weak non-unitary channel) is made identically on the
// host before anything runs.  The circuit is fused once per runner with each
// channel replaced by its first Kraus operator; a trajectory reuses that
// plan, recomputing only the blocks whose channel choice differs.  Where the
// bounds do not decide (the reference's second loop, :331-380), the plan is
// cut at that channel, the cut blocks are applied in two parts, and the
// choice is made on the device from the channel qubits' probabilities
// (traj.cu), without a host round trip.
#pragma once

#include <cstdint>
#include <memory>
#include <vector>

#include "batch_dev.h"
#include "engine.h"

namespace qsg {

struct TrajChannelDev;

namespace host {

// lib/channel.h:31-112.  `prob` is the probability of a unitary Kraus
// operator, or a lower bound of it for a non-unitary one.  `kdk` is
// K^dagger K on `qubits` (sorted), as the reference stores it.
struct KrausOp {
  bool unitary = true;
  double prob = 0;
  std::vector<Op> ops;
  std::vector<cplx> kdk;
  std::vector<unsigned> qubits;
};

enum class NoisyKind : int { kOp = 0, kChannel = 1 };

struct NoisyOp {
  NoisyKind kind = NoisyKind::kOp;
  Op op;                      // gate, controlled gate or measurement
  unsigned time = 0;          // channels
  std::vector<unsigned> qs;   // channels: qubits of the channel (sorted)
  std::vector<KrausOp> kops;  // channels
};

struct NoisyCircuit {
  unsigned num_qubits = 0;
  std::vector<NoisyOp> ops;
};

// Channels of lib/channels_cirq.h.  Matrices hold the single-precision
// values the reference's float channels hold.
NoisyOp depolarizing_channel(unsigned time, const std::vector<unsigned>& qs,
                             double p, bool register_qubits = false);
NoisyOp amplitude_damping_channel(unsigned time, unsigned q, double gamma);
NoisyOp phase_damping_channel(unsigned time, unsigned q, double gamma);
NoisyOp bit_flip_channel(unsigned time, unsigned q, double p);
NoisyOp phase_flip_channel(unsigned time, unsigned q, double p);
NoisyOp reset_channel(unsigned time, unsigned q);
// A general channel; kdk and qubits are computed as K^dagger K
// (KrausOperator::CalculateKdKMatrix, lib/channel.h:64-112).
void compute_kdk(KrausOp& k);

// lib/circuit_noisy.h:33-64: every op at time 2t, then a depolarizing(p)
// channel at time 2t+1 on each of its qubits (and controls).  With
// gamma > 0, an amplitude damping(gamma) channel on every qubit also follows
// the last op of each cycle, a cycle being `cycle_len` consecutive time
// steps of the clean circuit; op times are then 2(t + t / cycle_len) and the
// damping channels take the free step after each cycle.
NoisyCircuit make_noisy(const Circuit& c, double p_depol, double gamma,
                        unsigned cycle_len);

struct TrajectoryOptions {
  unsigned max_fused_size = 4;
  unsigned seeds = 12;
  bool collect_kop_stat = true;            // lib/qtrajectory.h:48-58
  bool collect_mea_stat = true;
  bool normalize_before_mea_gates = true;
  // Fused blocks of >= tc_min_k qubits on the tensor cores (padded to six
  // targets).  Their FP32 accumulation loses ~1e-6 of norm per pass, so
  // every trajectory is normalised at the end.
  bool tensor_path = false;
  unsigned tc_min_k = 5;
};

// Per-op statistics: entry i holds the Kraus-operator index chosen for op i
// (0 for a gate) or the measured bits of a measurement; kNoStat where the
// reference records nothing.  The reference's stat.samples is the sequence
// of entries that are not kNoStat.
constexpr uint64_t kNoStat = ~uint64_t{0};

// Device workspace of one stream: reduction partials, the chosen-operator
// matrix slot and the log of device-side choices.
struct TrajWorkspace {
  qsg_ctx* ctx = nullptr;
  double* partial = nullptr;
  float* dmat = nullptr;
  uint32_t* dlog = nullptr;
  uint32_t* hlog = nullptr;   // pinned
  size_t log_cap = 0, log_off = 0;
  struct Pending {
    uint64_t* stats;
    size_t op;
    size_t slot;
  };
  std::vector<Pending> pending;

  int init(qsg_ctx* ctx, size_t log_entries);
  void release();
  // Waits for the stream and writes the device-side choices into the stats.
  int resolve();
  ~TrajWorkspace() { release(); }
};

class TrajectoryRunner {
 public:
  // Validates the circuit and fuses it.  Fails (QSG_ERR_UNSUPPORTED) for a
  // non-unitary channel on more than two qubits or whose K^dagger K is not
  // diagonal.
  static int create(const NoisyCircuit& nc, const TrajectoryOptions& opt,
                    std::unique_ptr<TrajectoryRunner>* out);
  ~TrajectoryRunner();

  unsigned num_qubits() const { return nc_.num_qubits; }
  size_t num_ops() const { return nc_.ops.size(); }
  size_t num_fused_ops() const { return base_.ops.size(); }
  const Plan& base_plan() const { return base_; }

  // Enqueues one trajectory (repetition `rep`) on ws.ctx's stream:
  // |0..0> (or, with from_state, the state as given), the noisy circuit,
  // the final normalisation.  `stats` (num_ops() entries) is filled for
  // host-side choices now and for device-side ones by ws.resolve().
  // Measurements synchronise the stream.
  int enqueue(TrajWorkspace& ws, float* state, uint64_t rep,
              uint64_t* stats, bool from_state = false) const;

  // Device table of the channels sampled on the device (uploaded on first
  // use for the given context's device).
  int upload(qsg_ctx* ctx) const;
  // Tensor-core operands of the fused blocks on that path.
  int upload_tc(qsg_ctx* ctx) const;

  // True when every trajectory of this runner can run inside the packed
  // batch kernel: no measurements, fused blocks of at most kBatchMaxK
  // targets, at most kBatchMaxControls controls.
  bool packable() const;
  // upload() plus the fused plan's matrices, which packed programs point to.
  int upload_packed(qsg_ctx* ctx) const;

  // Compiles trajectory `rep` into packed-batch ops (see batch_dev.h):
  // appends to `ops`; matrices of blocks that differ from the fused plan go
  // to `extra` (float offsets are kept in `extra_refs` as (op index, offset)
  // pairs for the caller to turn into device pointers); CHANNEL ops get log
  // slots log_base, log_base + 1, ... and (stats, op) pairs in `log_refs`.
  // Requires upload() for the device first.
  struct LogRef {
    uint64_t* stats;
    size_t op;
  };
  int build_program(uint64_t rep, uint64_t* stats, std::vector<BatchOp>* ops,
                    std::vector<float>* extra,
                    std::vector<std::pair<size_t, size_t>>* extra_refs,
                    std::vector<LogRef>* log_refs) const;

 private:
  TrajectoryRunner() = default;
  template <class Sink>
  int walk(uint64_t rep, uint64_t* stats, Sink& sink) const;
  struct Channel;
  NoisyCircuit nc_;
  TrajectoryOptions opt_;
  Plan base_;
  std::vector<int> chan_of_op_;          // channel index or -1
  std::vector<Channel> chans_;
  std::vector<std::vector<Op>> kop_ops_;  // per channel, per kop: one op
  mutable TrajChannelDev* dev_table_ = nullptr;
  mutable float* dev_mats_ = nullptr;     // fused plan's matrices
  std::vector<size_t> mat_off_;           // per plan op: float offset
  mutable void* dev_tc_ = nullptr;        // tensor-core operands
  std::vector<size_t> tc_off_;            // per plan op (or size_t(-1))
  bool has_tc_ = false;
  mutable int dev_device_ = -1;
  size_t num_dev_channels_ = 0;
};

// One item of a batch: a runner and a repetition.  `stats` receives
// runner->num_ops() entries; `out_state`, when set, a device buffer of
// qsg_min_size(n) floats, receives the final state.
struct BatchItem {
  const TrajectoryRunner* runner = nullptr;
  uint64_t rep = 0;
  uint64_t* stats = nullptr;
  float* out_state = nullptr;
  float latency_ms = 0;   // device time from the item's first to last launch
};

struct BatchOptions {
  unsigned num_streams = 8;  // host threads, each with its own stream
  unsigned big_qubits = 0;   // circuits of >= big_qubits qubits run only on
  unsigned big_streams = 1;  // the first big_streams streams (0: no split)
};

// Runs the items on concurrent host threads, each with its own stream,
// state buffer and workspace on `device`; larger circuits are started
// first.  `wall_s` receives the elapsed wall time of the whole batch and
// `launches` the number of kernels launched.
int run_trajectory_batch(int device, std::vector<BatchItem>& items,
                         const BatchOptions& opt, double* wall_s,
                         uint64_t* launches);

struct PackedOptions {
  unsigned ctas_per_sm = 0;   // persistent CTAs per SM (0: 4, or fewer if
                              // the slot buffers do not fit)
  unsigned max_qubits = 30;   // larger circuits run on the stream path
  unsigned host_threads = 0;  // threads compiling programs (0: all cores)
  unsigned tile_kib = 0;      // tile buffers per CTA: 32, 64, 96 (0: 32)
  bool overlap = false;       // run the stream path while the kernel runs
  BatchOptions streams;       // the stream path for the other items
};

struct PackedStats {
  uint64_t packed_items = 0, stream_items = 0, ops = 0;
  unsigned ctas = 0, tile_kib = 0;
  double build_s = 0, upload_s = 0, kernel_s = 0, stream_s = 0;
};

// Runs the items that fit the packed kernel (packable runners of at most
// max_qubits qubits) as one persistent launch over a packed batch, largest
// circuits first, and the others on the stream path, after the launch or,
// with opt.overlap, concurrently with it.  Per-item latency is
// the item's device time inside the persistent kernel (%globaltimer).
int run_trajectory_batch_packed(int device, std::vector<BatchItem>& items,
                                const PackedOptions& opt, double* wall_s,
                                uint64_t* launches, PackedStats* stats);

}  // namespace host
}  // namespace qsg
