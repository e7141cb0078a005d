// Noisy circuits and the trajectory engine (declarations and the execution
// model in trajectory.h).

#include "trajectory.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <new>
#include <random>
#include <thread>

#include <cuda_runtime.h>

#include "internal.h"
#include "runner.h"
#include "traj_dev.h"

namespace qsg {
namespace host {

namespace {

using Mat = std::vector<cplx>;

Op gate_on(unsigned time, const std::vector<unsigned>& qs, Mat m) {
  Op op;
  op.kind = OpKind::kGate;
  op.time = time;
  op.qs = qs;
  op.m = std::move(m);
  return op;
}

// Pauli matrices of lib/gates_cirq.h (X, Y, Z).
const Mat kPauliX = {0, 1, 1, 0};
const Mat kPauliY = {0, cplx(0, -1), cplx(0, 1), 0};
const Mat kPauliZ = {1, 0, 0, -1};

// A one-qubit Kraus operator whose K and K^dagger K are given as
// single-precision values, as the reference's float channels store them.
KrausOp kop1(bool unitary, double prob, unsigned time, unsigned q,
             const float (&k)[8], const float (&kdk)[8]) {
  KrausOp o;
  o.unitary = unitary;
  o.prob = prob;
  Mat m(4), d(4);
  for (int i = 0; i < 4; ++i) {
    m[i] = cplx(k[2 * i], k[2 * i + 1]);
    d[i] = cplx(kdk[2 * i], kdk[2 * i + 1]);
  }
  o.ops.push_back(gate_on(time, {q}, std::move(m)));
  o.kdk = std::move(d);
  o.qubits = {q};
  return o;
}

NoisyOp channel_of(unsigned time, std::vector<unsigned> qs,
                   std::vector<KrausOp> kops) {
  NoisyOp c;
  c.kind = NoisyKind::kChannel;
  c.time = time;
  c.qs = std::move(qs);
  c.kops = std::move(kops);
  return c;
}

std::vector<unsigned> op_qubits(const Op& op) {
  std::vector<unsigned> q = op.qs;
  q.insert(q.end(), op.cqs.begin(), op.cqs.end());
  return q;
}

}  // namespace

void compute_kdk(KrausOp& k) {
  std::vector<unsigned> qs;
  for (const auto& op : k.ops) qs.insert(qs.end(), op.qs.begin(), op.qs.end());
  std::sort(qs.begin(), qs.end());
  qs.erase(std::unique(qs.begin(), qs.end()), qs.end());
  k.qubits = qs;
  std::vector<const Op*> ptrs;
  for (const auto& op : k.ops) ptrs.push_back(&op);
  Mat m = block_matrix_ops(ptrs, qs);
  const size_t d = size_t(1) << qs.size();
  k.kdk.assign(d * d, 0.0);
  for (size_t r = 0; r < d; ++r)
    for (size_t c = 0; c < d; ++c) {
      cplx acc = 0;
      for (size_t j = 0; j < d; ++j) acc += std::conj(m[j * d + r]) * m[j * d + c];
      k.kdk[r * d + c] = acc;
    }
}

NoisyOp depolarizing_channel(unsigned time, const std::vector<unsigned>& qs,
                             double p, bool register_qubits) {
  // lib/channels_cirq.h:127-199; the Pauli of index digit j acts on qs[j],
  // or, with register_qubits, on register qubit j as the reference's
  // multi-qubit factory places it (:147-189).  The channel then occupies
  // qubits 0..k-1, where its operators act.
  const double p1 = 1 - p, p2 = p / 3;
  const unsigned nq = qs.size();
  std::vector<KrausOp> kops;
  const uint64_t size = uint64_t{1} << (2 * nq);
  for (uint64_t i = 0; i < size; ++i) {
    KrausOp k;
    k.unitary = true;
    double prob = 1;
    for (unsigned j = 0; j < nq; ++j) {
      const unsigned pauli = unsigned(i >> (2 * j)) & 3;
      if (pauli == 0) {
        prob *= p1;
        continue;
      }
      prob *= p2;
      const Mat& m = pauli == 1 ? kPauliX : pauli == 2 ? kPauliY : kPauliZ;
      k.ops.push_back(gate_on(time, {register_qubits ? j : qs[j]}, m));
    }
    k.prob = prob;
    kops.push_back(std::move(k));
  }
  if (register_qubits) {
    std::vector<unsigned> acted(nq);
    for (unsigned j = 0; j < nq; ++j) acted[j] = j;
    return channel_of(time, acted, std::move(kops));
  }
  return channel_of(time, qs, std::move(kops));
}

NoisyOp amplitude_damping_channel(unsigned time, unsigned q, double gamma) {
  // lib/channels_cirq.h:274-300.
  const double p1 = 1 - gamma, p2 = 0;
  const float r = float(std::sqrt(p1)), s = float(std::sqrt(gamma));
  std::vector<KrausOp> kops;
  kops.push_back(kop1(false, p1, time, q, {1, 0, 0, 0, 0, 0, r, 0},
                      {1, 0, 0, 0, 0, 0, r * r, 0}));
  kops.push_back(kop1(false, p2, time, q, {0, 0, s, 0, 0, 0, 0, 0},
                      {0, 0, 0, 0, 0, 0, s * s, 0}));
  return channel_of(time, {q}, std::move(kops));
}

NoisyOp phase_damping_channel(unsigned time, unsigned q, double gamma) {
  // lib/channels_cirq.h:313-345.
  const double p1 = 1 - gamma, p2 = 0;
  const float r = float(std::sqrt(p1)), s = float(std::sqrt(gamma));
  std::vector<KrausOp> kops;
  kops.push_back(kop1(false, p1, time, q, {1, 0, 0, 0, 0, 0, r, 0},
                      {1, 0, 0, 0, 0, 0, r * r, 0}));
  kops.push_back(kop1(false, p2, time, q, {0, 0, 0, 0, 0, 0, s, 0},
                      {0, 0, 0, 0, 0, 0, s * s, 0}));
  return channel_of(time, {q}, std::move(kops));
}

NoisyOp reset_channel(unsigned time, unsigned q) {
  // lib/channels_cirq.h:359-380.
  std::vector<KrausOp> kops;
  kops.push_back(kop1(false, 0, time, q, {1, 0, 0, 0, 0, 0, 0, 0},
                      {1, 0, 0, 0, 0, 0, 0, 0}));
  kops.push_back(kop1(false, 0, time, q, {0, 0, 1, 0, 0, 0, 0, 0},
                      {0, 0, 0, 0, 0, 0, 1, 0}));
  return channel_of(time, {q}, std::move(kops));
}

NoisyOp bit_flip_channel(unsigned time, unsigned q, double p) {
  // lib/channels_cirq.h:425-447.
  std::vector<KrausOp> kops(2);
  kops[0].prob = 1 - p;
  kops[1].prob = p;
  kops[1].ops.push_back(gate_on(time, {q}, kPauliX));
  return channel_of(time, {q}, std::move(kops));
}

NoisyOp phase_flip_channel(unsigned time, unsigned q, double p) {
  // lib/channels_cirq.h:393-415.
  std::vector<KrausOp> kops(2);
  kops[0].prob = 1 - p;
  kops[1].prob = p;
  kops[1].ops.push_back(gate_on(time, {q}, kPauliZ));
  return channel_of(time, {q}, std::move(kops));
}

NoisyCircuit make_noisy(const Circuit& c, double p_depol, double gamma,
                        unsigned cycle_len) {
  NoisyCircuit nc;
  nc.num_qubits = c.num_qubits;
  if (cycle_len == 0) cycle_len = 1;
  // Op times become 2t and channel times 2t+1 (MakeNoisy).  With damping, a
  // free time step follows every cycle so that each qubit's times stay
  // strictly increasing, as the reference's fuser requires
  // (lib/fuser_mqubit.h:1210-1224).
  auto new_time = [&](unsigned t) {
    return gamma > 0 ? 2 * (t + t / cycle_len) : 2 * t;
  };
  for (size_t i = 0; i < c.ops.size(); ++i) {
    const Op& op = c.ops[i];
    const unsigned t2 = new_time(op.time);
    NoisyOp g;
    g.kind = NoisyKind::kOp;
    g.op = op;
    g.op.time = t2;
    nc.ops.push_back(std::move(g));
    if (p_depol > 0) {
      for (unsigned q : op_qubits(op)) {
        nc.ops.push_back(depolarizing_channel(t2 + 1, {q}, p_depol));
      }
    }
    const bool cycle_end = i + 1 == c.ops.size() ||
                           c.ops[i + 1].time / cycle_len != op.time / cycle_len;
    if (gamma > 0 && cycle_end) {
      for (unsigned q = 0; q < c.num_qubits; ++q) {
        nc.ops.push_back(amplitude_damping_channel(t2 + 2, q, gamma));
      }
    }
  }
  return nc;
}

// ---------------------------------------------------------------------------

struct TrajectoryRunner::Channel {
  size_t op = 0;
  std::vector<unsigned> qs;
  std::vector<double> prob;
  std::vector<char> unitary, identity;
  double cp_total = 0;
  bool any_nonunitary = false;
  int dev = -1;
};

namespace {

constexpr int kEscape = -1;  // decided on the device
constexpr int kNoOp = -2;    // bounds failed on an all-unitary channel

int unsupported(const char* msg) {
  set_error_msg(msg);
  return QSG_ERR_UNSUPPORTED;
}

int invalid(const char* msg) {
  set_error_msg(msg);
  return QSG_ERR_INVALID;
}

bool sorted_distinct_lt(const std::vector<unsigned>& qs, unsigned n) {
  for (size_t i = 0; i < qs.size(); ++i) {
    if (qs[i] >= n) return false;
    if (i > 0 && qs[i] <= qs[i - 1]) return false;
  }
  return true;
}

std::vector<float> to_f32(const Mat& m) {
  std::vector<float> out(2 * m.size());
  for (size_t i = 0; i < m.size(); ++i) {
    out[2 * i] = float(m[i].real());
    out[2 * i + 1] = float(m[i].imag());
  }
  return out;
}

}  // namespace

TrajectoryRunner::~TrajectoryRunner() {
  if (dev_table_ || dev_mats_ || dev_tc_) {
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(dev_device_);
    if (dev_table_) cudaFree(dev_table_);
    if (dev_mats_) cudaFree(dev_mats_);
    if (dev_tc_) cudaFree(dev_tc_);
    cudaSetDevice(cur);
  }
}

int TrajectoryRunner::upload_packed(qsg_ctx* ctx) const {
  int rc = upload(ctx);
  if (rc || dev_mats_) return rc;
  std::vector<float> all;
  for (const PlanOp& p : base_.ops) all.insert(all.end(), p.m32.begin(), p.m32.end());
  if (all.empty()) all.push_back(0.f);
  void* p = nullptr;
  rc = dev_alloc(ctx, all.size() * sizeof(float), &p);
  if (rc) return rc;
  rc = dev_upload(ctx, p, all.data(), all.size() * sizeof(float));
  if (rc) {
    dev_free(ctx, p);
    return rc;
  }
  dev_mats_ = static_cast<float*>(p);
  dev_device_ = ctx_device(ctx);
  return QSG_OK;
}

int TrajectoryRunner::create(const NoisyCircuit& nc,
                             const TrajectoryOptions& opt,
                             std::unique_ptr<TrajectoryRunner>* out) {
  if (!out) return invalid("null output");
  const unsigned n = nc.num_qubits;
  if (n < 1 || n > 40) return invalid("trajectories need 1..40 qubits");
  if (opt.max_fused_size < 1 || opt.max_fused_size > 6)
    return invalid("max_fused_size must be 1..6");
  std::unique_ptr<TrajectoryRunner> r(new TrajectoryRunner());
  r->nc_ = nc;
  r->opt_ = opt;
  Circuit slots;
  slots.num_qubits = n;
  r->chan_of_op_.assign(nc.ops.size(), -1);
  for (size_t i = 0; i < nc.ops.size(); ++i) {
    const NoisyOp& no = nc.ops[i];
    if (no.kind == NoisyKind::kOp) {
      std::vector<unsigned> all = op_qubits(no.op);
      std::vector<unsigned> s = all;
      std::sort(s.begin(), s.end());
      if (!sorted_distinct_lt(no.op.qs, n) || !sorted_distinct_lt(s, n) ||
          no.op.qs.size() > 6)
        return invalid("noisy circuit op with bad qubits");
      slots.ops.push_back(no.op);
      continue;
    }
    if (no.kops.empty()) return invalid("channel without Kraus operators");
    Channel ch;
    ch.op = i;
    std::vector<unsigned> qs = no.qs;
    for (const auto& k : no.kops) {
      for (const auto& g : k.ops) {
        if (g.kind != OpKind::kGate)
          return unsupported("Kraus operators must be matrix gates");
        qs.insert(qs.end(), g.qs.begin(), g.qs.end());
      }
      qs.insert(qs.end(), k.qubits.begin(), k.qubits.end());
    }
    std::sort(qs.begin(), qs.end());
    qs.erase(std::unique(qs.begin(), qs.end()), qs.end());
    if (qs.empty() || !sorted_distinct_lt(qs, n))
      return invalid("channel with bad qubits");
    if (qs.size() > 6) return unsupported("channels act on at most 6 qubits");
    ch.qs = qs;
    std::vector<Op> kops;
    for (const auto& k : no.kops) {
      std::vector<const Op*> ptrs;
      for (const auto& g : k.ops) ptrs.push_back(&g);
      kops.push_back(gate_on(no.time, qs, block_matrix_ops(ptrs, qs)));
      ch.prob.push_back(k.prob);
      ch.unitary.push_back(k.unitary);
      ch.identity.push_back(k.ops.empty());
      ch.cp_total += k.prob;
      if (!k.unitary) ch.any_nonunitary = true;
    }
    if (ch.any_nonunitary) {
      if (qs.size() > kTrajMaxChannelQubits || no.kops.size() > kTrajMaxKops)
        return unsupported(
            "non-unitary channels are supported on at most 2 qubits with at "
            "most 16 Kraus operators");
      // K^dagger K must be diagonal on the channel qubits.
      for (const auto& k : no.kops) {
        if (k.unitary) continue;
        const size_t kd = size_t(1) << k.qubits.size();
        if (k.kdk.size() != kd * kd)
          return invalid("Kraus operator without K^dagger K");
        for (size_t a = 0; a < kd; ++a)
          for (size_t b = 0; b < kd; ++b)
            if (a != b && k.kdk[a * kd + b] != 0.0)
              return unsupported(
                  "non-unitary Kraus operators need a diagonal K^dagger K");
      }
      ch.dev = int(r->num_dev_channels_++);
    }
    r->chan_of_op_[i] = int(r->chans_.size());
    // The fusion slot holds the first Kraus operator.
    slots.ops.push_back(kops[0]);
    r->kop_ops_.push_back(std::move(kops));
    r->chans_.push_back(std::move(ch));
  }
  FuseOptions fo;
  fo.max_fused_size = opt.max_fused_size;
  fo.seeds = opt.seeds ? opt.seeds : 12;
  fo.tensor_path = opt.tensor_path;
  fo.tc_min_k = opt.tc_min_k;
  r->base_ = fuse(slots, fo);
  for (auto& p : r->base_.ops) std::sort(p.members.begin(), p.members.end());
  size_t off = 0, toff = 0;
  r->mat_off_.assign(r->base_.ops.size(), 0);
  r->tc_off_.assign(r->base_.ops.size(), size_t(-1));
  for (size_t i = 0; i < r->base_.ops.size(); ++i) {
    const PlanOp& p = r->base_.ops[i];
    r->mat_off_[i] = off;
    off += p.m32.size();
    if (p.kind == OpKind::kGate && p.path == Path::kTensor) {
      r->tc_off_[i] = toff;
      toff += (tc_operand_bytes(p.qs.size()) + 1023) & ~size_t(1023);
      r->has_tc_ = true;
    }
  }
  *out = std::move(r);
  return QSG_OK;
}

int TrajectoryRunner::upload_tc(qsg_ctx* ctx) const {
  if (!has_tc_ || dev_tc_) return QSG_OK;
  int rc = tc_setup();
  if (rc) return rc;
  size_t total = 0;
  for (size_t i = 0; i < base_.ops.size(); ++i)
    if (tc_off_[i] != size_t(-1))
      total = tc_off_[i] + ((tc_operand_bytes(base_.ops[i].qs.size()) + 1023) &
                            ~size_t(1023));
  std::vector<unsigned char> host(total);
  for (size_t i = 0; i < base_.ops.size(); ++i)
    if (tc_off_[i] != size_t(-1))
      tc_build_operands(base_.ops[i].qs.size(), base_.ops[i].m32.data(),
                        host.data() + tc_off_[i]);
  void* p = nullptr;
  rc = dev_alloc(ctx, total, &p);
  if (rc) return rc;
  rc = dev_upload(ctx, p, host.data(), total);
  if (rc) {
    dev_free(ctx, p);
    return rc;
  }
  dev_tc_ = p;
  dev_device_ = ctx_device(ctx);
  return QSG_OK;
}

int TrajectoryRunner::upload(qsg_ctx* ctx) const {
  int rc0 = upload_tc(ctx);
  if (rc0) return rc0;
  if (num_dev_channels_ == 0 || dev_table_) return QSG_OK;
  std::vector<TrajChannelDev> table(num_dev_channels_);
  for (size_t c = 0; c < chans_.size(); ++c) {
    const Channel& ch = chans_[c];
    if (ch.dev < 0) continue;
    TrajChannelDev& t = table[ch.dev];
    std::memset(&t, 0, sizeof(t));
    t.nq = int(ch.qs.size());
    for (size_t j = 0; j < ch.qs.size(); ++j) t.q[j] = ch.qs[j];
    const NoisyOp& no = nc_.ops[ch.op];
    t.nkops = int(no.kops.size());
    const unsigned d = 1u << ch.qs.size();
    for (size_t k = 0; k < no.kops.size(); ++k) {
      const KrausOp& ko = no.kops[k];
      t.unitary[k] = ko.unitary ? 1 : 0;
      t.prob[k] = ko.prob;
      std::vector<float> m = to_f32(kop_ops_[c][k].m);
      std::memcpy(t.mat[k], m.data(), m.size() * sizeof(float));
      if (!ko.unitary) {
        // Diagonal of kd_k, expanded from its qubits to the channel's.
        for (unsigned b = 0; b < d; ++b) {
          unsigned sub = 0;
          for (size_t j = 0; j < ko.qubits.size(); ++j) {
            const size_t pos = size_t(
                std::find(ch.qs.begin(), ch.qs.end(), ko.qubits[j]) -
                ch.qs.begin());
            if ((b >> pos) & 1) sub |= 1u << j;
          }
          const size_t kd = size_t(1) << ko.qubits.size();
          t.kd[k][b] = float(ko.kdk[sub * kd + sub].real());
        }
      }
    }
  }
  const size_t bytes = table.size() * sizeof(TrajChannelDev);
  void* p = nullptr;
  int rc = dev_alloc(ctx, bytes, &p);
  if (rc) return rc;
  rc = dev_upload(ctx, p, table.data(), bytes);
  if (rc) {
    dev_free(ctx, p);
    return rc;
  }
  dev_table_ = static_cast<TrajChannelDev*>(p);
  dev_device_ = ctx_device(ctx);
  return QSG_OK;
}

// ---------------------------------------------------------------------------

int TrajWorkspace::init(qsg_ctx* c, size_t log_entries) {
  release();
  ctx = c;
  void* p = nullptr;
  int rc = dev_alloc(ctx, size_t(traj_max_parts(ctx)) * 4 * sizeof(double), &p);
  if (rc) return rc;
  partial = static_cast<double*>(p);
  rc = dev_alloc(ctx, 64 * sizeof(float), &p);
  if (rc) return rc;
  dmat = static_cast<float*>(p);
  rc = dev_alloc(ctx, log_entries * sizeof(uint32_t), &p);
  if (rc) return rc;
  dlog = static_cast<uint32_t*>(p);
  if (cudaMallocHost(&p, log_entries * sizeof(uint32_t)) != cudaSuccess) {
    set_error_msg("pinned allocation failed");
    return QSG_ERR_OOM;
  }
  hlog = static_cast<uint32_t*>(p);
  log_cap = log_entries;
  log_off = 0;
  pending.clear();
  return QSG_OK;
}

void TrajWorkspace::release() {
  if (ctx) {
    if (partial) dev_free(ctx, partial);
    if (dmat) dev_free(ctx, dmat);
    if (dlog) dev_free(ctx, dlog);
  }
  if (hlog) cudaFreeHost(hlog);
  partial = nullptr;
  dmat = nullptr;
  dlog = nullptr;
  hlog = nullptr;
  log_cap = log_off = 0;
  pending.clear();
}

int TrajWorkspace::resolve() {
  cudaStream_t s = static_cast<cudaStream_t>(ctx_stream(ctx));
  if (log_off > 0) {
    if (cudaMemcpyAsync(hlog, dlog, log_off * sizeof(uint32_t),
                        cudaMemcpyDeviceToHost, s) != cudaSuccess) {
      set_error_msg("choice log copy failed");
      return QSG_ERR_CUDA;
    }
  }
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    set_error_msg(cudaGetErrorString(e));
    return QSG_ERR_CUDA;
  }
  for (const auto& p : pending) {
    const uint32_t v = hlog[p.slot];
    if (p.stats) p.stats[p.op] = v == 0xffffffffu ? kNoStat : uint64_t(v);
  }
  pending.clear();
  log_off = 0;
  return QSG_OK;
}

template <class Sink>
int TrajectoryRunner::walk(uint64_t rep, uint64_t* stats, Sink& sink) const {
  const size_t nops = nc_.ops.size();
  int rc = QSG_OK;

  // Draws and host-side choices (lib/qtrajectory.h:265-331).
  thread_local std::vector<double> rr;
  thread_local std::vector<int> choice;
  thread_local std::vector<unsigned> seg;
  thread_local std::vector<size_t> escapes;
  thread_local std::vector<char> norm_before;
  norm_before.assign(nops, 0);
  rr.assign(nops, 0.0);
  choice.assign(nops, 0);
  seg.assign(nops, 0);
  escapes.clear();
  std::mt19937 rgen{static_cast<std::mt19937::result_type>(rep)};
  std::uniform_real_distribution<double> distr(0.0, 1.0);
  // `unitary` follows the reference's flag: false once a non-unitary
  // operator was applied and the state was not normalised since.
  bool unitary = true;
  for (size_t i = 0; i < nops; ++i) {
    const NoisyOp& no = nc_.ops[i];
    rr[i] = distr(rgen);
    seg[i] = unsigned(escapes.size());
    if (no.kind == NoisyKind::kOp) {
      if (no.op.kind == OpKind::kMeasure) {
        if (!unitary && opt_.normalize_before_mea_gates) {
          norm_before[i] = 1;
          unitary = true;
        }
        if (stats) stats[i] = kNoStat;
      } else if (stats) {
        stats[i] = opt_.collect_kop_stat ? 0 : kNoStat;
      }
      continue;
    }
    const Channel& ch = chans_[chan_of_op_[i]];
    double cp = 0;
    int chosen = -1;
    for (size_t k = 0; k < ch.prob.size(); ++k) {
      cp += ch.prob[k];
      if (rr[i] < cp) {
        chosen = int(k);
        break;
      }
    }
    if (chosen >= 0) {
      choice[i] = chosen;
      if (stats) stats[i] = opt_.collect_kop_stat ? uint64_t(chosen) : kNoStat;
      unitary = unitary && ch.unitary[chosen];
    } else if (ch.any_nonunitary) {
      choice[i] = kEscape;
      escapes.push_back(i);
      if (stats) stats[i] = kNoStat;
      unitary = false;
    } else {
      // The reference normalises here; the state is normalised at the end
      // (or before the next measurement) instead, which gives the same
      // state.
      choice[i] = kNoOp;
      if (stats) stats[i] = kNoStat;
    }
  }

  rc = sink.set_zero();
  if (rc) return rc;

  // Channel kops are fused slots of `base_`; a kop choice other than the
  // first, or a cut, makes the block's matrix be recomputed.
  thread_local std::vector<const Op*> ptrs;
  thread_local std::vector<unsigned> qs;
  const unsigned nseg = unsigned(escapes.size()) + 1;
  for (unsigned s = 0; s < nseg; ++s) {
    for (size_t pi = 0; pi < base_.ops.size(); ++pi) {
      const PlanOp& p = base_.ops[pi];
      if (p.kind == OpKind::kMeasure) {
        const int m = p.members[0];
        if (seg[m] != s) continue;
        if (norm_before[m]) {
          rc = sink.normalize();
          if (rc) return rc;
        }
        uint64_t mask = 0;
        for (unsigned q : nc_.ops[m].op.qs) mask |= uint64_t{1} << q;
        uint64_t bits = 0;
        rc = sink.measure(mask, rr[m], &bits);
        if (rc) return rc;
        if (stats) stats[m] = opt_.collect_mea_stat ? bits : kNoStat;
        continue;
      }
      ptrs.clear();
      size_t present = 0;
      bool all_default = true;
      for (int j : p.members) {
        if (seg[j] != s) continue;
        const int c = chan_of_op_[j];
        if (c < 0) {
          ++present;
          ptrs.push_back(&nc_.ops[j].op);
          continue;
        }
        const int ch = choice[j];
        if (ch == kEscape || ch == kNoOp) {
          all_default = false;
          continue;
        }
        ++present;
        if (ch != 0) all_default = false;
        if (!chans_[c].identity[ch]) ptrs.push_back(&kop_ops_[c][ch]);
      }
      if (present == 0) continue;
      if (p.kind == OpKind::kControlled) {
        rc = sink.gate(p.qs, &nc_.ops[p.members[0]].op, p.m32.data(),
                       ptrdiff_t(pi), nullptr);
        if (rc) return rc;
        continue;
      }
      if (present == p.members.size() && all_default) {
        rc = sink.gate(p.qs, nullptr, p.m32.data(), ptrdiff_t(pi),
                       tc_off_[pi] == size_t(-1)
                           ? nullptr
                           : static_cast<const unsigned char*>(dev_tc_) +
                                 tc_off_[pi]);
        if (rc) return rc;
        continue;
      }
      if (ptrs.empty()) continue;
      qs.clear();
      for (const Op* o : ptrs) qs.insert(qs.end(), o->qs.begin(), o->qs.end());
      std::sort(qs.begin(), qs.end());
      qs.erase(std::unique(qs.begin(), qs.end()), qs.end());
      std::vector<float> m32 = to_f32(block_matrix_ops(ptrs, qs));
      rc = sink.gate(qs, nullptr, m32.data(), -1, nullptr);
      if (rc) return rc;
    }
    if (s + 1 < nseg) {
      // The lower bounds did not decide: choose on the device
      // (lib/qtrajectory.h:331-380).
      const size_t e = escapes[s];
      const Channel& ch = chans_[chan_of_op_[e]];
      rc = sink.channel(ch.qs, dev_table_ + ch.dev, ch.cp_total, rr[e],
                        opt_.collect_kop_stat ? stats : nullptr, e);
      if (rc) return rc;
    }
  }
  if (!unitary || has_tc_) return sink.normalize();
  return QSG_OK;
}

namespace {

// Launches every op on the workspace's stream (RunOnce on the engine).
struct StreamSink {
  TrajWorkspace& ws;
  float* state;
  unsigned n;
  unsigned tc_min_k;  // recomputed blocks of >= tc_min_k qubits on tcgen05
                      // (0: never)
  bool keep_state = false;  // start from the state given, not |0..0>

  int set_zero() {
    return keep_state ? QSG_OK : qsg_set_state_zero(ws.ctx, state, n);
  }
  int gate(const std::vector<unsigned>& qs, const Op* ctl, const float* m32,
           ptrdiff_t, const void* tc_operands) {
    if (tc_operands)
      return apply_gate_tc(ws.ctx, state, n, qs.data(), qs.size(), m32,
                           tc_operands);
    // A block recomputed for a non-default Kraus choice or cut at a channel
    // takes the tensor cores like the plan's own blocks: a 5- or 6-qubit
    // CUDA-core pass costs several tensor-core passes.
    if (!ctl && tc_min_k && qs.size() >= tc_min_k && n >= 12)
      return apply_gate_tc_host(ws.ctx, state, n, qs.data(), qs.size(), m32);
    if (ctl)
      return apply_gate_ex(ws.ctx, state, n, qs.data(), qs.size(),
                           ctl->cqs.data(), ctl->cqs.size(), ctl->cvals, m32,
                           nullptr);
    return apply_gate_ex(ws.ctx, state, n, qs.data(), qs.size(), nullptr, 0,
                         0, m32, nullptr);
  }
  int measure(uint64_t mask, double u, uint64_t* bits) {
    return qsg_measure(ws.ctx, state, n, mask, u, 1, bits);
  }
  int normalize() {
    unsigned np = 0;
    int e = traj_channel_stats(ws.ctx, state, n, 0, nullptr, ws.partial, &np);
    if (e) return e;
    e = traj_choose(ws.ctx, ws.partial, np, nullptr, 0, 0, ws.dlog, ws.dmat);
    if (e) return e;
    return traj_apply(ws.ctx, state, n, 0, nullptr, ws.dmat);
  }
  int channel(const std::vector<unsigned>& qs, const TrajChannelDev* dev,
              double cp0, double r, uint64_t* stats, size_t op) {
    if (ws.log_off >= ws.log_cap) {
      const int e = ws.resolve();
      if (e) return e;
    }
    const size_t slot = ws.log_off++;
    unsigned np = 0;
    int e = traj_channel_stats(ws.ctx, state, n, qs.size(), qs.data(),
                               ws.partial, &np);
    if (e) return e;
    e = traj_choose(ws.ctx, ws.partial, np, dev, cp0, r, ws.dlog + slot,
                    ws.dmat);
    if (e) return e;
    e = traj_apply(ws.ctx, state, n, qs.size(), qs.data(), ws.dmat);
    if (e) return e;
    ws.pending.push_back({stats, op, slot});
    return QSG_OK;
  }
};

uint64_t mask_of(const std::vector<unsigned>& qs) {
  uint64_t m = 0;
  for (unsigned q : qs) m |= uint64_t{1} << q;
  return m;
}

// Appends packed-batch ops (batch_dev.h) instead of launching.
struct ProgramSink {
  std::vector<BatchOp>* ops;
  std::vector<float>* extra;
  std::vector<std::pair<size_t, size_t>>* extra_refs;
  std::vector<TrajectoryRunner::LogRef>* log_refs;
  const float* dev_mats;
  const std::vector<size_t>* mat_off;

  int set_zero() {
    BatchOp o{};
    o.kind = kBatchSetZero;
    ops->push_back(o);
    return QSG_OK;
  }
  int gate(const std::vector<unsigned>& qs, const Op* ctl, const float* m32,
           ptrdiff_t base, const void* tc_operands) {
    if (tc_operands)
      return unsupported("packed batch: tensor-core blocks run on streams");
    if (qs.empty() || qs.size() > kBatchMaxK ||
        (ctl && ctl->cqs.size() > kBatchMaxControls))
      return unsupported("packed batch: block too large");
    BatchOp o{};
    o.kind = kBatchGate;
    o.tmask = mask_of(qs);
    if (ctl) {
      o.cmask = mask_of(ctl->cqs);
      for (size_t i = 0; i < ctl->cqs.size(); ++i)
        if ((ctl->cvals >> i) & 1) o.cvals |= uint64_t{1} << ctl->cqs[i];
    }
    if (base >= 0) {
      o.mat = dev_mats + (*mat_off)[size_t(base)];
    } else {
      extra_refs->push_back({ops->size(), extra->size()});
      const size_t nf = size_t(2) << (2 * qs.size());
      extra->insert(extra->end(), m32, m32 + nf);
    }
    ops->push_back(o);
    return QSG_OK;
  }
  int measure(uint64_t, double, uint64_t*) {
    return unsupported("packed batch: measurements run on streams");
  }
  int normalize() {
    BatchOp o{};
    o.kind = kBatchNormalize;
    ops->push_back(o);
    return QSG_OK;
  }
  int channel(const std::vector<unsigned>& qs, const TrajChannelDev* dev,
              double cp0, double r, uint64_t* stats, size_t op) {
    if (qs.size() > kTrajMaxChannelQubits)
      return unsupported("packed batch: channel on too many qubits");
    BatchOp o{};
    o.kind = kBatchChannel;
    o.tmask = mask_of(qs);
    o.ch = dev;
    o.cp0 = cp0;
    o.r = r;
    ops->push_back(o);
    log_refs->push_back({stats, op});
    return QSG_OK;
  }
};

}  // namespace

int TrajectoryRunner::enqueue(TrajWorkspace& ws, float* state, uint64_t rep,
                              uint64_t* stats, bool from_state) const {
  const int rc = upload(ws.ctx);
  if (rc) return rc;
  StreamSink sink{ws, state, nc_.num_qubits,
                  has_tc_ ? std::max(opt_.tc_min_k, 1u) : 0u, from_state};
  return walk(rep, stats, sink);
}

bool TrajectoryRunner::packable() const {
  if (has_tc_) return false;
  for (const PlanOp& p : base_.ops) {
    if (p.kind == OpKind::kMeasure) return false;
    if (p.qs.size() > kBatchMaxK) return false;
    if (p.kind == OpKind::kControlled && p.cqs.size() > kBatchMaxControls)
      return false;
  }
  // A recomputed block holds the members of a fused block, so it has no
  // more targets than the block.
  return true;
}

int TrajectoryRunner::build_program(
    uint64_t rep, uint64_t* stats, std::vector<BatchOp>* ops,
    std::vector<float>* extra,
    std::vector<std::pair<size_t, size_t>>* extra_refs,
    std::vector<LogRef>* log_refs) const {
  if (!dev_mats_ && !base_.ops.empty())
    return invalid("packed batch: runner matrices not uploaded");
  ProgramSink sink{ops, extra, extra_refs, log_refs, dev_mats_, &mat_off_};
  return walk(rep, stats, sink);
}

// ---------------------------------------------------------------------------

int run_trajectory_batch(int device, std::vector<BatchItem>& items,
                         const BatchOptions& opt, double* wall_s,
                         uint64_t* launches) {
  if (wall_s) *wall_s = 0;
  if (launches) *launches = 0;
  if (items.empty()) return QSG_OK;
  unsigned max_n = 1;
  for (const auto& it : items) {
    if (!it.runner) return invalid("batch item without a runner");
    max_n = std::max(max_n, it.runner->num_qubits());
  }
  unsigned num_streams = opt.num_streams ? opt.num_streams : 8;
  num_streams = unsigned(std::min<size_t>(num_streams, items.size()));

  // Two queues, largest circuits first.  With big_qubits set, circuits of
  // at least that many qubits run only on the first big_streams streams,
  // one at a time per stream, so that a state that fits in L2 stays there
  // for its whole trajectory; the other streams take the small circuits.
  std::vector<size_t> big, small;
  for (size_t i = 0; i < items.size(); ++i) {
    if (opt.big_qubits && items[i].runner->num_qubits() >= opt.big_qubits)
      big.push_back(i);
    else
      small.push_back(i);
  }
  auto by_size = [&](size_t a, size_t b) {
    return items[a].runner->num_qubits() > items[b].runner->num_qubits();
  };
  std::stable_sort(big.begin(), big.end(), by_size);
  std::stable_sort(small.begin(), small.end(), by_size);
  unsigned num_big = 0;
  if (!big.empty()) {
    num_big = opt.big_streams ? opt.big_streams : 1;
    num_big = std::min(num_big, num_streams);
  }

  struct Worker {
    qsg_ctx* ctx = nullptr;
    float* state = nullptr;
    TrajWorkspace ws;
    std::vector<std::pair<size_t, std::pair<cudaEvent_t, cudaEvent_t>>> done;
    int rc = QSG_OK;
    bool serves_big = false;
  };
  std::vector<Worker> workers(num_streams);
  int rc = QSG_OK;
  for (unsigned wi = 0; wi < num_streams; ++wi) {
    Worker& w = workers[wi];
    w.serves_big = wi < num_big;
    rc = qsg_ctx_create(device, nullptr, &w.ctx);
    if (rc) break;
    void* p = nullptr;
    rc = dev_alloc(w.ctx, qsg_min_size(max_n) * sizeof(float), &p);
    if (rc) break;
    w.state = static_cast<float*>(p);
    rc = w.ws.init(w.ctx, size_t(1) << 16);
    if (rc) break;
  }
  if (rc == QSG_OK) {
    for (const auto& it : items) {
      rc = it.runner->upload(workers[0].ctx);
      if (rc) break;
    }
  }
  if (rc == QSG_OK) rc = qsg_ctx_sync(workers[0].ctx);

  std::atomic<size_t> next_big{0}, next_small{0};
  std::atomic<int> first_err{QSG_OK};
  const auto t0 = std::chrono::steady_clock::now();
  if (rc == QSG_OK) {
    std::vector<std::thread> threads;
    for (auto& w : workers) {
      threads.emplace_back([&, wp = &w]() {
        Worker& w = *wp;
        cudaSetDevice(device);
        cudaStream_t s = static_cast<cudaStream_t>(ctx_stream(w.ctx));
        // An exception may not leave a host thread (std::terminate): it
        // ends this worker with a status instead.
        try {
        for (;;) {
          if (first_err.load() != QSG_OK) break;
          size_t item = size_t(-1);
          if (w.serves_big) {
            const size_t b = next_big.fetch_add(1);
            if (b < big.size()) item = big[b];
          }
          if (item == size_t(-1)) {
            const size_t m = next_small.fetch_add(1);
            if (m < small.size()) item = small[m];
          }
          if (item == size_t(-1)) break;
          BatchItem& it = items[item];
          cudaEvent_t e0 = nullptr, e1 = nullptr;
          if (cudaEventCreate(&e0) != cudaSuccess ||
              cudaEventCreate(&e1) != cudaSuccess) {
            w.rc = QSG_ERR_CUDA;
            break;
          }
          cudaEventRecord(e0, s);
          int r = it.runner->enqueue(w.ws, w.state, it.rep, it.stats);
          if (r == QSG_OK && it.out_state) {
            const size_t bytes =
                qsg_min_size(it.runner->num_qubits()) * sizeof(float);
            if (cudaMemcpyAsync(it.out_state, w.state, bytes,
                                cudaMemcpyDeviceToDevice, s) != cudaSuccess)
              r = QSG_ERR_CUDA;
          }
          cudaEventRecord(e1, s);
          w.done.push_back({item, {e0, e1}});
          if (r != QSG_OK) {
            w.rc = r;
            break;
          }
        }
        } catch (const std::bad_alloc&) {
          w.rc = QSG_ERR_OOM;
        } catch (...) {
          w.rc = QSG_ERR_INVALID;
        }
        int r = w.ws.resolve();
        if (w.rc == QSG_OK) w.rc = r;
        for (auto& d : w.done) {
          float ms = 0;
          cudaEventElapsedTime(&ms, d.second.first, d.second.second);
          items[d.first].latency_ms = ms;
          cudaEventDestroy(d.second.first);
          cudaEventDestroy(d.second.second);
        }
        w.done.clear();
        if (w.rc != QSG_OK) {
          int expect = QSG_OK;
          first_err.compare_exchange_strong(expect, w.rc);
        }
      });
    }
    for (auto& t : threads) t.join();
    rc = first_err.load();
  }
  const auto t1 = std::chrono::steady_clock::now();
  if (wall_s) *wall_s = std::chrono::duration<double>(t1 - t0).count();
  for (auto& w : workers) {
    if (launches && w.ctx) *launches += qsg_ctx_launch_count(w.ctx);
    w.ws.release();
    if (w.state) dev_free(w.ctx, w.state);
    if (w.ctx) qsg_ctx_destroy(w.ctx);
  }
  return rc;
}

}  // namespace host
}  // namespace qsg
