// C ABI of noisy circuits and trajectories (include/qsim_gb300.h).

#include <algorithm>
#include <memory>
#include <new>
#include <vector>

#include "capi_types.h"
#include "engine.h"
#include "runner.h"
#include "trajectory.h"

using namespace qsg::host;

struct qsg_noisy {
  NoisyCircuit nc;
};

struct qsg_traj {
  std::unique_ptr<TrajectoryRunner> r;
};

namespace {

int invalid(const char* msg) {
  qsg::set_error_msg(msg);
  return QSG_ERR_INVALID;
}

bool distinct_lt(const unsigned* qs, unsigned k, unsigned n) {
  for (unsigned i = 0; i < k; ++i) {
    if (qs[i] >= n) return false;
    for (unsigned j = 0; j < i; ++j)
      if (qs[i] == qs[j]) return false;
  }
  return true;
}

}  // namespace

extern "C" {

int qsg_noisy_create(unsigned num_qubits, qsg_noisy** out) {
  if (!out) return invalid("null output");
  *out = nullptr;
  if (num_qubits < 1 || num_qubits > 40) return invalid("1..40 qubits");
  auto* h = new (std::nothrow) qsg_noisy();
  if (!h) return QSG_ERR_OOM;
  h->nc.num_qubits = num_qubits;
  *out = h;
  return QSG_OK;
}

int qsg_noisy_destroy(qsg_noisy* h) {
  delete h;
  return QSG_OK;
}

int qsg_noisy_info(const qsg_noisy* h, unsigned* num_qubits, uint64_t* num_ops,
                   uint64_t* num_channels) {
  if (!h) return invalid("null noisy circuit");
  if (num_qubits) *num_qubits = h->nc.num_qubits;
  if (num_ops) *num_ops = h->nc.ops.size();
  if (num_channels) {
    uint64_t c = 0;
    for (const auto& o : h->nc.ops) c += o.kind == NoisyKind::kChannel;
    *num_channels = c;
  }
  return QSG_OK;
}

int qsg_noisy_append_circuit(qsg_noisy* h, const qsg_circuit* c) {
  if (!h || !c) return invalid("null argument");
  if (c->c.num_qubits > h->nc.num_qubits)
    return invalid("circuit has more qubits than the noisy circuit");
  for (const auto& op : c->c.ops) {
    NoisyOp o;
    o.kind = NoisyKind::kOp;
    o.op = op;
    h->nc.ops.push_back(std::move(o));
  }
  return QSG_OK;
}

int qsg_noisy_add_channel(qsg_noisy* h, int kind, unsigned time,
                          const unsigned* qs, unsigned nq, double p) {
  if (!h || !qs || nq == 0) return invalid("null argument");
  if (!distinct_lt(qs, nq, h->nc.num_qubits)) return invalid("bad qubits");
  std::vector<unsigned> q(qs, qs + nq);
  std::sort(q.begin(), q.end());
  if (kind != QSG_CHANNEL_DEPOLARIZING &&
      kind != QSG_CHANNEL_DEPOLARIZING_REGISTER && nq != 1)
    return invalid("this channel acts on one qubit");
  if (kind != QSG_CHANNEL_RESET && !(p >= 0 && p <= 1))
    return invalid("channel parameter must lie in [0, 1]");
  switch (kind) {
    case QSG_CHANNEL_DEPOLARIZING:
      if (nq > 3) return invalid("depolarizing channels on at most 3 qubits");
      h->nc.ops.push_back(depolarizing_channel(time, q, p));
      break;
    case QSG_CHANNEL_DEPOLARIZING_REGISTER:
      if (nq > 3) return invalid("depolarizing channels on at most 3 qubits");
      if (nq > h->nc.num_qubits) return invalid("more channel qubits than qubits");
      h->nc.ops.push_back(depolarizing_channel(time, q, p, true));
      break;
    case QSG_CHANNEL_AMPLITUDE_DAMPING:
      h->nc.ops.push_back(amplitude_damping_channel(time, q[0], p));
      break;
    case QSG_CHANNEL_PHASE_DAMPING:
      h->nc.ops.push_back(phase_damping_channel(time, q[0], p));
      break;
    case QSG_CHANNEL_BIT_FLIP:
      h->nc.ops.push_back(bit_flip_channel(time, q[0], p));
      break;
    case QSG_CHANNEL_PHASE_FLIP:
      h->nc.ops.push_back(phase_flip_channel(time, q[0], p));
      break;
    case QSG_CHANNEL_RESET:
      h->nc.ops.push_back(reset_channel(time, q[0]));
      break;
    default:
      return invalid("unknown channel kind");
  }
  return QSG_OK;
}

int qsg_noisy_add_kraus_channel(qsg_noisy* h, unsigned time,
                                const unsigned* qs, unsigned nq,
                                unsigned num_kops, const int* unitary,
                                const double* probs, const double* matrices) {
  if (!h || !qs || !unitary || !probs || !matrices || nq == 0 || num_kops == 0)
    return invalid("null argument");
  if (nq > 6) return invalid("channels act on at most 6 qubits");
  if (!distinct_lt(qs, nq, h->nc.num_qubits)) return invalid("bad qubits");
  const size_t d = size_t(1) << nq;
  NoisyOp ch;
  ch.kind = NoisyKind::kChannel;
  ch.time = time;
  ch.qs.assign(qs, qs + nq);
  std::sort(ch.qs.begin(), ch.qs.end());
  for (unsigned k = 0; k < num_kops; ++k) {
    KrausOp ko;
    ko.unitary = unitary[k] != 0;
    ko.prob = probs[k];
    std::vector<cplx> m(d * d);
    const double* src = matrices + k * 2 * d * d;
    for (size_t i = 0; i < d * d; ++i) m[i] = cplx(src[2 * i], src[2 * i + 1]);
    ko.ops.push_back(make_gate(time, std::vector<unsigned>(qs, qs + nq), m));
    compute_kdk(ko);
    ch.kops.push_back(std::move(ko));
  }
  h->nc.ops.push_back(std::move(ch));
  return QSG_OK;
}

int qsg_noisy_make(const qsg_circuit* c, double p_depol, double gamma,
                   unsigned cycle_len, qsg_noisy** out) {
  if (!c || !out) return invalid("null argument");
  *out = nullptr;
  if (c->c.num_qubits < 1) return invalid("noisy circuits need qubits");
  if (!(p_depol >= 0 && p_depol <= 1 && gamma >= 0 && gamma <= 1))
    return invalid("noise parameters must lie in [0, 1]");
  auto* h = new (std::nothrow) qsg_noisy();
  if (!h) return QSG_ERR_OOM;
  h->nc = make_noisy(c->c, p_depol, gamma, cycle_len);
  *out = h;
  return QSG_OK;
}

int qsg_noisy_get_op(const qsg_noisy* h, uint64_t i, int* is_channel,
                     unsigned* time, unsigned* nq, unsigned* qs,
                     unsigned* num_kops) {
  if (!h) return invalid("null noisy circuit");
  if (i >= h->nc.ops.size()) return invalid("op index out of range");
  const NoisyOp& o = h->nc.ops[i];
  const bool ch = o.kind == NoisyKind::kChannel;
  if (is_channel) *is_channel = ch;
  if (time) *time = ch ? o.time : o.op.time;
  const std::vector<unsigned>& q = ch ? o.qs : o.op.qs;
  if (nq) *nq = unsigned(q.size());
  if (qs) std::copy(q.begin(), q.end(), qs);
  if (num_kops) *num_kops = ch ? unsigned(o.kops.size()) : 0;
  return QSG_OK;
}

int qsg_traj_create(const qsg_noisy* h, const qsg_traj_options* opts,
                    qsg_traj** out) {
  if (!h || !out) return invalid("null argument");
  *out = nullptr;
  TrajectoryOptions o;
  if (opts) {
    if (opts->max_fused_size) o.max_fused_size = opts->max_fused_size;
    if (opts->seeds) o.seeds = opts->seeds;
    o.collect_kop_stat = opts->collect_kop_stat != 0;
    o.collect_mea_stat = opts->collect_mea_stat != 0;
    o.normalize_before_mea_gates = opts->normalize_before_mea_gates != 0;
    o.tensor_path = opts->tensor_path != 0;
    if (opts->tc_min_k) o.tc_min_k = opts->tc_min_k;
  }
  auto* t = new (std::nothrow) qsg_traj();
  if (!t) return QSG_ERR_OOM;
  int rc = TrajectoryRunner::create(h->nc, o, &t->r);
  if (rc) {
    delete t;
    return rc;
  }
  *out = t;
  return QSG_OK;
}

int qsg_traj_destroy(qsg_traj* t) {
  delete t;
  return QSG_OK;
}

int qsg_traj_info(const qsg_traj* t, unsigned* num_qubits, uint64_t* num_ops,
                  uint64_t* num_fused_ops) {
  if (!t) return invalid("null trajectory runner");
  if (num_qubits) *num_qubits = t->r->num_qubits();
  if (num_ops) *num_ops = t->r->num_ops();
  if (num_fused_ops) *num_fused_ops = t->r->num_fused_ops();
  return QSG_OK;
}

int qsg_traj_run(qsg_ctx* ctx, qsg_traj* t, float* state, uint64_t rep,
                 uint64_t* stats) {
  if (!ctx || !t || !state) return invalid("null argument");
  TrajWorkspace ws;
  int rc = ws.init(ctx, 4096);
  if (rc) return rc;
  rc = t->r->enqueue(ws, state, rep, stats);
  int rc2 = ws.resolve();
  return rc ? rc : rc2;
}

int qsg_traj_run_from(qsg_ctx* ctx, qsg_traj* t, float* state, uint64_t rep,
                      uint64_t* stats) {
  if (!ctx || !t || !state) return invalid("null argument");
  TrajWorkspace ws;
  int rc = ws.init(ctx, 4096);
  if (rc) return rc;
  rc = t->r->enqueue(ws, state, rep, stats, /*from_state=*/true);
  int rc2 = ws.resolve();
  return rc ? rc : rc2;
}

int qsg_traj_run_batch(int device, qsg_traj* const* runners,
                       uint64_t num_runners, const uint32_t* item_runner,
                       const uint64_t* item_rep, uint64_t num_items,
                       const qsg_batch_options* opts, uint64_t* stats,
                       float* const* out_states, float* latency_ms,
                       double* wall_s, uint64_t* launches) {
  if (!runners || (num_items && (!item_runner || !item_rep)))
    return invalid("null argument");
  std::vector<BatchItem> items(num_items);
  uint64_t off = 0;
  for (uint64_t i = 0; i < num_items; ++i) {
    if (item_runner[i] >= num_runners || !runners[item_runner[i]])
      return invalid("batch item refers to no runner");
    const TrajectoryRunner* r = runners[item_runner[i]]->r.get();
    items[i].runner = r;
    items[i].rep = item_rep[i];
    items[i].stats = stats ? stats + off : nullptr;
    items[i].out_state = out_states ? out_states[i] : nullptr;
    off += r->num_ops();
  }
  BatchOptions o;
  if (opts) {
    o.num_streams = opts->num_streams;
    o.big_qubits = opts->big_qubits;
    o.big_streams = opts->big_streams;
  }
  int rc = run_trajectory_batch(device, items, o, wall_s, launches);
  if (latency_ms)
    for (uint64_t i = 0; i < num_items; ++i) latency_ms[i] = items[i].latency_ms;
  return rc;
}

int qsg_traj_run_packed(int device, qsg_traj* const* runners,
                        uint64_t num_runners, const uint32_t* item_runner,
                        const uint64_t* item_rep, uint64_t num_items,
                        const qsg_packed_options* opts, uint64_t* stats,
                        float* const* out_states, float* latency_ms,
                        double* wall_s, uint64_t* launches,
                        qsg_packed_info* info) {
  if (!runners || (num_items && (!item_runner || !item_rep)))
    return invalid("null argument");
  std::vector<BatchItem> items(num_items);
  uint64_t off = 0;
  for (uint64_t i = 0; i < num_items; ++i) {
    if (item_runner[i] >= num_runners || !runners[item_runner[i]])
      return invalid("batch item refers to no runner");
    const TrajectoryRunner* r = runners[item_runner[i]]->r.get();
    items[i].runner = r;
    items[i].rep = item_rep[i];
    items[i].stats = stats ? stats + off : nullptr;
    items[i].out_state = out_states ? out_states[i] : nullptr;
    off += r->num_ops();
  }
  PackedOptions o;
  if (opts) {
    o.ctas_per_sm = opts->ctas_per_sm;
    if (opts->max_qubits) o.max_qubits = opts->max_qubits;
    o.host_threads = opts->host_threads;
    o.tile_kib = opts->tile_kib;
    o.overlap = opts->overlap != 0;
    o.streams.num_streams = opts->streams.num_streams;
    o.streams.big_qubits = opts->streams.big_qubits;
    o.streams.big_streams = opts->streams.big_streams;
  }
  PackedStats ps;
  int rc = run_trajectory_batch_packed(device, items, o, wall_s, launches, &ps);
  if (latency_ms)
    for (uint64_t i = 0; i < num_items; ++i) latency_ms[i] = items[i].latency_ms;
  if (info) {
    info->packed_items = ps.packed_items;
    info->stream_items = ps.stream_items;
    info->ops = ps.ops;
    info->ctas = ps.ctas;
    info->tile_kib = ps.tile_kib;
    info->build_s = ps.build_s;
    info->upload_s = ps.upload_s;
    info->kernel_s = ps.kernel_s;
    info->stream_s = ps.stream_s;
  }
  return rc;
}

}  // extern "C"
