// Hybrid Schrodinger-Feynman simulation (qsimh): amplitudes of chosen
// bitstrings of a circuit cut into two parts of the qubits.
//
// The reference (lib/hybrid.h, lib/run_qsimh.h) splits the circuit
// (HybridSimulator::SplitLattice, :131-277): one-qubit gates and gates inside
// a part go to that part; a two-qubit gate across the cut is replaced by the
// operator Schmidt decomposition U = sum_k A_k (x) B_k, A_k on one part and
// B_k on the other.  A path chooses one term per cut gate; the amplitude of a
// bitstring is the sum over paths of the two parts' amplitudes,
// a0[path][i0] * a1[path][i1].  Paths are indexed as in the reference: the
// cut gates ordered by (time, circuit order), each taking 0, 1 or 2 path bits
// (Schmidt rank 1, 2, 3-4); the first num_prefix_gatexs gates are fixed by
// `prefix`, the next num_root_gatexs ("root") and the rest ("suffix") are
// summed over (Run, :290-437).  The reference runs the paths one after
// another, with checkpoints after the prefix and root gates.
//
// Here the suffix paths run as one batch: the part's state gets `batch_bits`
// extra high qubits ("path qubits", one per path bit), every amplitude block
// of the batch is one path, and a suffix cut gate on local qubit q becomes a
// gate on (q, its path qubits) whose matrix is block diagonal in the path
// qubits, block k = the gate's k-th Schmidt factor (zero for k >= rank: the
// reference skips such paths).  The fuser then treats path qubits as qubits,
// so cut gates fuse with their neighbours into the usual <= 6-qubit passes on
// the CUDA or tensor cores.  Per part and root path the state before the
// first suffix cut gate is computed once at 2^n_part amplitudes and
// broadcast to every block (the reference's second checkpoint); the
// amplitudes are then sum_b s0[i0 + b 2^n0] s1[i1 + b 2^n1] (one kernel,
// FP64 sums).  Root paths loop on the host, each one plan run per part on
// the checkpointed prefix state, as in the reference; suffix path bits that
// do not fit the device (max_batch_bits or 45 % of free HBM) loop on the host
// as well.

#include <algorithm>
#include <cstring>
#include <memory>
#include <string>
#include <future>
#include <vector>

#include <cuda_runtime.h>

#include "capi_types.h"
#include "engine.h"
#include "internal.h"
#include "runner.h"

namespace qsg {

// Device helpers (hybrid.cu).
int hybrid_broadcast(qsg_ctx* ctx, float* state, unsigned n, unsigned bits);
int hybrid_collect(qsg_ctx* ctx, const float* s0, unsigned n0, const float* s1,
                   unsigned n1, unsigned bits, const uint64_t* idx,
                   uint64_t m, double* acc);

namespace host {
namespace {

struct CutGate {
  unsigned time = 0;
  size_t order = 0;            // index of the gate in the circuit
  unsigned q[2] = {0, 0};      // local qubit in part 0 and part 1
  std::vector<cplx> f[2];      // per part: 4 values per Schmidt term
  unsigned terms = 0, bits = 0;
};

struct PartOp {
  unsigned time = 0;
  int cut = -1;                // >= 0: index into Split::cuts (path order)
  Op op;                       // plain ops, local qubits
};

struct Split {
  unsigned n[2] = {0, 0};
  std::vector<unsigned> local;
  std::vector<PartOp> ops[2];
  std::vector<CutGate> cuts;
};

int fail(int code, const std::string& msg) {
  set_error_msg(msg.c_str());
  return code;
}

unsigned schmidt_bits(unsigned terms) {
  return terms <= 1 ? 0 : terms == 2 ? 1 : terms <= 4 ? 2 : 99;
}

// HybridSimulator::SplitLattice (lib/hybrid.h:131-277).
int split_lattice(const Circuit& c, const unsigned* parts, unsigned np,
                  Split* sp) {
  if (np != c.num_qubits)
    return fail(QSG_ERR_INVALID, "parts size is not equal to the number of qubits");
  sp->local.assign(np, 0);
  for (unsigned q = 0; q < np; ++q) {
    if (parts[q] > 1) return fail(QSG_ERR_INVALID, "parts must be 0 or 1");
    sp->local[q] = sp->n[parts[q]]++;
  }
  if (sp->n[0] == 0 || sp->n[1] == 0)
    return fail(QSG_ERR_INVALID, "both parts need at least one qubit");
  std::vector<CutGate> cuts;
  for (size_t i = 0; i < c.ops.size(); ++i) {
    const Op& op = c.ops[i];
    if (op.kind != OpKind::kGate)
      return fail(QSG_ERR_UNSUPPORTED,
                  "measurement, controlled or other non-matrix gates are not "
                  "supported by the hybrid simulator");
    if (op.qs.size() != 1 && op.qs.size() != 2)
      return fail(QSG_ERR_UNSUPPORTED,
                  "only one- and two-qubit gates are supported by the hybrid "
                  "simulator");
    const unsigned p0 = parts[op.qs[0]];
    if (op.qs.size() == 1 || parts[op.qs[1]] == p0) {
      PartOp po;
      po.time = op.time;
      po.op = op;
      for (auto& q : po.op.qs) q = sp->local[q];
      sp->ops[p0].push_back(std::move(po));
      continue;
    }
    if (op.schmidt.empty())
      return fail(QSG_ERR_UNSUPPORTED,
                  "no Schmidt decomposition for a gate on the cut (named "
                  "two-qubit gates only)");
    CutGate g;
    g.time = op.time;
    g.order = i;
    g.terms = unsigned(op.schmidt.size() / 8);
    g.bits = schmidt_bits(g.terms);
    if (g.bits > 2)
      return fail(QSG_ERR_UNSUPPORTED, "Schmidt rank is too large");
    // Factor A (on qs[0]) goes to qs[0]'s part.
    for (unsigned t = 0; t < g.terms; ++t) {
      const cplx* a = &op.schmidt[8 * t];
      g.f[p0].insert(g.f[p0].end(), a, a + 4);
      g.f[1 - p0].insert(g.f[1 - p0].end(), a + 4, a + 8);
    }
    g.q[p0] = sp->local[op.qs[0]];
    g.q[1 - p0] = sp->local[op.qs[1]];
    cuts.push_back(std::move(g));
  }
  // Path order: by time, then circuit order (the reference sorts part 0's
  // operations this way and numbers the cut gates in that order).
  std::stable_sort(cuts.begin(), cuts.end(),
                   [](const CutGate& a, const CutGate& b) {
                     return a.time < b.time;
                   });
  sp->cuts = std::move(cuts);
  for (size_t j = 0; j < sp->cuts.size(); ++j) {
    for (int p = 0; p < 2; ++p) {
      PartOp po;
      po.time = sp->cuts[j].time;
      po.cut = int(j);
      sp->ops[p].push_back(std::move(po));
    }
  }
  // Each part in time order, plain ops before cut gates of the same time,
  // cut gates in path order.
  for (int p = 0; p < 2; ++p) {
    std::stable_sort(sp->ops[p].begin(), sp->ops[p].end(),
                     [](const PartOp& a, const PartOp& b) {
                       if (a.time != b.time) return a.time < b.time;
                       if ((a.cut >= 0) != (b.cut >= 0)) return b.cut >= 0;
                       return a.cut < b.cut;
                     });
  }
  return QSG_OK;
}

// Term k of cut gate g on part p as a one-qubit gate.
Op term_gate(const CutGate& g, int p, unsigned k, unsigned time) {
  Op op;
  op.time = time;
  op.qs = {g.q[p]};
  op.m.assign(g.f[p].begin() + 4 * k, g.f[p].begin() + 4 * k + 4);
  return op;
}

// Cut gate g on part p with its `g.bits` path qubits starting at `pq`:
// block diagonal over the path value k, block k = term k (zero when k is
// not a term).  Qubits (q, pq, pq + 1) are sorted since q < n <= pq.
Op path_gate(const CutGate& g, int p, unsigned pq, unsigned time) {
  Op op;
  op.time = time;
  op.qs = {g.q[p]};
  for (unsigned b = 0; b < g.bits; ++b) op.qs.push_back(pq + b);
  const unsigned d = 2u << g.bits;
  op.m.assign(size_t(d) * d, 0.0);
  for (unsigned k = 0; k < (1u << g.bits) && k < g.terms; ++k)
    for (unsigned r = 0; r < 2; ++r)
      for (unsigned cc = 0; cc < 2; ++cc)
        op.m[(2 * k + r) * d + 2 * k + cc] = g.f[p][4 * k + 2 * r + cc];
  return op;
}

struct PathSel {
  // Per cut gate: fixed term (>= 0), or -1 for a batched (path-qubit) gate.
  std::vector<int> k;
  std::vector<unsigned> pq;  // first path qubit offset of batched gates
};

// Picks the terms of cut gates [i0, i1) from `path` (the reference's
// SetSchmidtMatrices, lib/hybrid.h:512-541): false when a gate's index is
// not one of its terms.
bool select(const Split& sp, size_t i0, size_t i1, uint64_t path,
            PathSel* sel, size_t* bad) {
  unsigned sh = 0;
  for (size_t i = i0; i < i1; ++i) {
    const CutGate& g = sp.cuts[i];
    if (g.bits == 0) {
      sel->k[i] = 0;
      continue;
    }
    const unsigned k = unsigned(path >> sh) & ((1u << g.bits) - 1);
    sh += g.bits;
    if (k >= g.terms) {
      if (bad) *bad = i;
      return false;
    }
    sel->k[i] = int(k);
  }
  return true;
}

// Circuit of part p's ops [a, b) on `nq` qubits with the cut gates as `sel`
// says.
Circuit portion(const Split& sp, int p, size_t a, size_t b, unsigned nq,
                const PathSel& sel) {
  Circuit c;
  c.num_qubits = nq;
  for (size_t i = a; i < b; ++i) {
    const PartOp& po = sp.ops[p][i];
    if (po.cut < 0) {
      c.ops.push_back(po.op);
      continue;
    }
    const CutGate& g = sp.cuts[po.cut];
    if (sel.k[po.cut] >= 0)
      c.ops.push_back(term_gate(g, p, unsigned(sel.k[po.cut]), po.time));
    else
      c.ops.push_back(path_gate(g, p, sp.n[p] + sel.pq[po.cut], po.time));
  }
  return c;
}

// First position in part p's op list of a cut gate with index >= j.
size_t first_cut_at_least(const Split& sp, int p, size_t j) {
  for (size_t i = 0; i < sp.ops[p].size(); ++i)
    if (sp.ops[p][i].cut >= 0 && size_t(sp.ops[p][i].cut) >= j) return i;
  return sp.ops[p].size();
}

struct DevBuf {
  qsg_ctx* ctx = nullptr;
  float* p = nullptr;
  ~DevBuf() {
    if (p) qsg_state_free(ctx, p);
  }
};

int run_plan(qsg_ctx* ctx, Plan plan, float* state) {
  PlanRuntime rt;
  rt.plan = std::move(plan);
  return rt.run(ctx, state, 0, nullptr);
}

// Fuses the two parts' circuits, part 1 on a host thread of its own (a
// future, so an exception on either thread reaches the caller).
void fuse_parts(const Circuit& c0, const Circuit& c1, const FuseOptions& fo,
                Plan* out) {
  auto part1 = std::async(std::launch::async, [&] { return fuse(c1, fo); });
  out[0] = fuse(c0, fo);
  out[1] = part1.get();
}

}  // namespace

}  // namespace host
}  // namespace qsg

using namespace qsg;
using namespace qsg::host;

namespace {

void fill_info(const Split& sp, const qsg_hybrid_options* o,
               qsg_hybrid_info* info) {
  std::memset(info, 0, sizeof(*info));
  info->num_qubits0 = sp.n[0];
  info->num_qubits1 = sp.n[1];
  info->num_ops0 = unsigned(sp.ops[0].size());
  info->num_ops1 = unsigned(sp.ops[1].size());
  info->num_gatexs = unsigned(sp.cuts.size());
  const size_t np = o ? std::min<size_t>(o->num_prefix_gatexs, sp.cuts.size()) : 0;
  const size_t nr =
      o ? std::min<size_t>(np + o->num_root_gatexs, sp.cuts.size()) : np;
  for (size_t i = 0; i < sp.cuts.size(); ++i) {
    const unsigned b = sp.cuts[i].bits;
    if (i < np) info->prefix_bits += b;
    else if (i < nr) info->root_bits += b;
    else info->suffix_bits += b;
  }
}

}  // namespace

extern "C" {

int qsg_hybrid_split(const qsg_circuit* c, const unsigned* parts,
                     unsigned num_parts, qsg_hybrid_info* info) {
  if (!c || !parts || !info) {
    set_error_msg("qsg_hybrid_split: null argument");
    return QSG_ERR_INVALID;
  }
  Split sp;
  int rc = split_lattice(c->c, parts, num_parts, &sp);
  if (rc) return rc;
  fill_info(sp, nullptr, info);
  return QSG_OK;
}

int qsg_hybrid_run(qsg_ctx* ctx, const qsg_circuit* c, const unsigned* parts,
                   unsigned num_parts, const qsg_hybrid_options* o,
                   const uint64_t* bitstrings, uint64_t m, double* results,
                   qsg_hybrid_info* info_out) {
  if (!ctx || !c || !parts || !o || (m && (!bitstrings || !results))) {
    set_error_msg("qsg_hybrid_run: null argument");
    return QSG_ERR_INVALID;
  }
  Split sp;
  int rc = split_lattice(c->c, parts, num_parts, &sp);
  if (rc) return rc;
  const size_t G = sp.cuts.size();
  const size_t P = o->num_prefix_gatexs, PR = P + o->num_root_gatexs;
  if (PR > G)
    return fail(QSG_ERR_INVALID,
                "num_prefix_gatexs plus num_root_gatexs is greater than the "
                "number of gates on the cut");
  qsg_hybrid_info info;
  fill_info(sp, o, &info);
  FuseOptions fo;
  fo.max_fused_size = o->max_fused_size ? o->max_fused_size : 4;
  if (fo.max_fused_size > 6)
    return fail(QSG_ERR_INVALID, "max_fused_size must be 1..6");
  fo.tensor_path = o->tensor_path != 0;
  // On the tensor cores, consecutive blocks share two-gate passes where
  // their tile allows (from 2 run bits, weighed by the measured saving).
  fo.tc_pair_bits = fo.tensor_path ? 2 : 0;

  // Suffix gates batched on the device: the first ones whose bits fit.
  unsigned cap = o->max_batch_bits;
  if (cap == 0) {
    size_t free_b = 0, total_b = 0;
    cudaSetDevice(ctx_device(ctx));
    cudaMemGetInfo(&free_b, &total_b);
    const double budget = 0.45 * double(free_b);
    cap = 0;
    while (cap < 40 &&
           8.0 * (std::ldexp(1.0, int(sp.n[0] + cap + 1)) +
                  std::ldexp(1.0, int(sp.n[1] + cap + 1))) <= budget)
      ++cap;
  }
  if (sp.n[0] + cap > 40 || sp.n[1] + cap > 40)
    cap = 40 - std::max(sp.n[0], sp.n[1]);
  PathSel sel;
  sel.k.assign(G, 0);
  sel.pq.assign(G, 0);
  unsigned dev_bits = 0;
  size_t S_dev_end = PR;  // suffix gates [PR, S_dev_end) batched
  for (size_t i = PR; i < G; ++i) {
    if (dev_bits + sp.cuts[i].bits > cap) break;
    sel.pq[i] = dev_bits;
    dev_bits += sp.cuts[i].bits;
    S_dev_end = i + 1;
  }
  unsigned host_bits = 0;
  for (size_t i = S_dev_end; i < G; ++i) host_bits += sp.cuts[i].bits;
  info.batch_bits = dev_bits;
  if (info.root_bits + host_bits > 40)
    return fail(QSG_ERR_INVALID, "too many path bits outside the batch");

  size_t bad = 0;
  if (!select(sp, 0, P, o->prefix, &sel, &bad)) {
    return fail(QSG_ERR_INVALID, "invalid prefix " + std::to_string(o->prefix) +
                                     " for prefix gate index " +
                                     std::to_string(bad));
  }

  // Device buffers: per part the prefix state, the root state and the batch.
  DevBuf st_p[2], st_r[2], big[2];
  for (int p = 0; p < 2; ++p) {
    st_p[p].ctx = st_r[p].ctx = big[p].ctx = ctx;
    if ((rc = qsg_state_create(ctx, sp.n[p], &st_p[p].p))) return rc;
    if ((rc = qsg_state_create(ctx, sp.n[p], &st_r[p].p))) return rc;
    if ((rc = qsg_state_create(ctx, sp.n[p] + dev_bits, &big[p].p))) return rc;
  }
  std::vector<uint64_t> idx(2 * std::max<uint64_t>(m, 1), 0);
  for (uint64_t i = 0; i < m; ++i) {
    for (unsigned q = 0; q < num_parts; ++q) {
      const uint64_t bit = (bitstrings[i] >> q) & 1;
      idx[2 * i + parts[q]] |= bit << sp.local[q];
    }
  }
  void* d_idx = nullptr;
  void* d_acc = nullptr;
  if ((rc = dev_alloc(ctx, idx.size() * 8, &d_idx))) return rc;
  if ((rc = dev_alloc(ctx, idx.size() * 8, &d_acc))) {
    dev_free(ctx, d_idx);
    return rc;
  }
  auto cleanup = [&]() {
    dev_free(ctx, d_idx);
    dev_free(ctx, d_acc);
  };
  cudaStream_t s = static_cast<cudaStream_t>(ctx_stream(ctx));
  if ((rc = dev_upload(ctx, d_idx, idx.data(), idx.size() * 8))) {
    cleanup();
    return rc;
  }
  cudaMemsetAsync(d_acc, 0, idx.size() * 8, s);

  size_t c1[2], c2[2];
  for (int p = 0; p < 2; ++p) {
    c1[p] = first_cut_at_least(sp, p, P);
    c2[p] = first_cut_at_least(sp, p, PR);
  }
  // Prefix: once per part.
  {
    Plan pl[2];
    fuse_parts(portion(sp, 0, 0, c1[0], sp.n[0], sel),
               portion(sp, 1, 0, c1[1], sp.n[1], sel), fo, pl);
    for (int p = 0; p < 2 && !rc; ++p) {
      rc = qsg_set_state_zero(ctx, st_p[p].p, sp.n[p]);
      if (!rc) rc = run_plan(ctx, std::move(pl[p]), st_p[p].p);
    }
  }
  // Suffix plans of batched gates; host-looped gates fixed per s_host.
  for (size_t i = PR; i < S_dev_end; ++i) sel.k[i] = -1;
  const uint64_t rmax = uint64_t{1} << info.root_bits;
  const uint64_t hmax = uint64_t{1} << host_bits;
  // Suffix plans (one per host-looped suffix path), kept with their device
  // matrices across root paths.
  std::vector<std::unique_ptr<PlanRuntime>> suffix_rts[2];
  for (auto& v : suffix_rts) v.resize(hmax);
  auto suffix_plans = [&](uint64_t sh, PlanRuntime** out) -> bool {
    if (!suffix_rts[0][sh]) {
      if (!select(sp, S_dev_end, G, sh, &sel, nullptr)) return false;
      Plan pl[2];
      fuse_parts(portion(sp, 0, c2[0], sp.ops[0].size(), sp.n[0] + dev_bits, sel),
                 portion(sp, 1, c2[1], sp.ops[1].size(), sp.n[1] + dev_bits, sel),
                 fo, pl);
      for (int p = 0; p < 2; ++p) {
        suffix_rts[p][sh] = std::make_unique<PlanRuntime>();
        suffix_rts[p][sh]->plan = std::move(pl[p]);
      }
    }
    out[0] = suffix_rts[0][sh].get();
    out[1] = suffix_rts[1][sh].get();
    return true;
  };
  uint64_t paths = 0;
  for (uint64_t r = 0; r < rmax && !rc; ++r) {
    if (!select(sp, P, PR, r, &sel, nullptr)) continue;
    Plan pl[2];
    fuse_parts(portion(sp, 0, c1[0], c2[0], sp.n[0], sel),
               portion(sp, 1, c1[1], c2[1], sp.n[1], sel), fo, pl);
    for (int p = 0; p < 2 && !rc; ++p) {
      rc = qsg_copy_d2d(ctx, st_r[p].p, st_p[p].p, sp.n[p]);
      if (!rc) rc = run_plan(ctx, std::move(pl[p]), st_r[p].p);
    }
    for (uint64_t sh = 0; sh < hmax && !rc; ++sh) {
      PlanRuntime* srt[2];
      if (!suffix_plans(sh, srt)) continue;
      for (int p = 0; p < 2 && !rc; ++p) {
        rc = qsg_copy_d2d(ctx, big[p].p, st_r[p].p, sp.n[p]);
        if (!rc) rc = hybrid_broadcast(ctx, big[p].p, sp.n[p], dev_bits);
        if (!rc) rc = srt[p]->run(ctx, big[p].p, 0, nullptr);
      }
      if (!rc)
        rc = hybrid_collect(ctx, big[0].p, sp.n[0], big[1].p, sp.n[1],
                            dev_bits, static_cast<const uint64_t*>(d_idx), m,
                            static_cast<double*>(d_acc));
      paths += uint64_t{1} << dev_bits;
    }
  }
  std::vector<double> acc(2 * m);
  if (!rc && m) {
    if (cudaMemcpyAsync(acc.data(), d_acc, 16 * m, cudaMemcpyDeviceToHost, s) !=
            cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      rc = fail(QSG_ERR_CUDA, "qsg_hybrid_run: result copy failed");
  }
  cleanup();
  if (rc) return rc;
  for (uint64_t i = 0; i < 2 * m; ++i) results[i] += acc[i];
  info.paths_run = paths;
  if (info_out) *info_out = info;
  return QSG_OK;
}

}  // extern "C"
