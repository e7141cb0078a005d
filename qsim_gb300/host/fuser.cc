// Fusion planner.
//
// The reference's MultiQubitGateFuser (lib/fuser_mqubit.h:185-526) groups
// one- and two-qubit gates into blocks of at most max_fused_size qubits,
// passes controlled gates through unfused (:408-421), splits at measurement
// times, and multiplies each block's matrices on the host
// (CalculateFusedMatrix, lib/fuser.h:149-179).  This planner keeps that
// contract (same inputs, same kinds of outputs, blocks <= max_fused_size)
// with its own search: a block grows from a seed gate by scanning the
// remaining gates in order and absorbing every gate whose qubits fit and
// whose unscheduled predecessors are already in the block.  Qubits touched by
// a skipped gate are blocked for the rest of the scan, which keeps the block
// order-preserving.  Several front gates are tried as seeds and the best
// block is kept: by default the one absorbing the most gates; with a cost
// model, the one with the largest (cost of its gates applied alone) minus
// (cost of the block) per block, i.e. the most time saved.

#include <algorithm>
#include <cmath>
#include <future>
#include <unordered_map>
#include <utility>
#include <vector>
#include <cstring>

#include "engine.h"

namespace qsg {
// Run bits of the two-gate tensor-core tile of two padded 6-qubit gates, or
// -1 if they cannot share a pass (tc_gate.cu).
int tc2_run_bits(unsigned n, const unsigned* qa6, const unsigned* qb6);
}

namespace qsg {
namespace host {

unsigned Plan::max_k() const {
  unsigned k = 0;
  for (const auto& op : ops) k = std::max<unsigned>(k, op.qs.size());
  return k;
}

std::vector<cplx> block_matrix(const Circuit& c, const std::vector<int>& members,
                               const std::vector<unsigned>& qs) {
  std::vector<const Op*> ops;
  ops.reserve(members.size());
  for (int idx : members) ops.push_back(&c.ops[idx]);
  return block_matrix_ops(ops, qs);
}

std::vector<cplx> block_matrix_ops(const std::vector<const Op*>& ops,
                                   const std::vector<unsigned>& qs) {
  const unsigned k = qs.size();
  const unsigned d = 1u << k;
  // Columns of the block matrix evolve as k-qubit states.  Real and
  // imaginary parts are kept apart, so the update of a row runs along
  // contiguous columns (vectorisable); every element gets the same sums in
  // the same order as a complex column-by-column update.
  std::vector<double> re(size_t(d) * d, 0.0), im(size_t(d) * d, 0.0);
  for (unsigned i = 0; i < d; ++i) re[size_t(i) * d + i] = 1.0;
  std::vector<double> tre(size_t(d) * d), tim(size_t(d) * d);
  for (const Op* opp : ops) {
    const Op& op = *opp;
    const unsigned gk = op.qs.size();
    const unsigned gd = 1u << gk;
    // Positions of the gate's qubits inside the block.
    unsigned pos[6], gmask = 0;
    for (unsigned j = 0; j < gk; ++j) {
      pos[j] = unsigned(std::find(qs.begin(), qs.end(), op.qs[j]) - qs.begin());
      gmask |= 1u << pos[j];
    }
    unsigned off[64];
    for (unsigned gi = 0; gi < gd; ++gi) {
      unsigned r = 0;
      for (unsigned j = 0; j < gk; ++j)
        if ((gi >> j) & 1) r |= 1u << pos[j];
      off[gi] = r;
    }
    const cplx* g = op.m.data();
    for (unsigned base = 0; base < d; ++base) {
      if (base & gmask) continue;
      for (unsigned go = 0; go < gd; ++go) {
        double* ar = &tre[size_t(go) * d];
        double* ai = &tim[size_t(go) * d];
        for (unsigned col = 0; col < d; ++col) ar[col] = ai[col] = 0.0;
        for (unsigned gi = 0; gi < gd; ++gi) {
          const double gr = g[go * gd + gi].real(), gm = g[go * gd + gi].imag();
          const double* xr = &re[size_t(base | off[gi]) * d];
          const double* xi = &im[size_t(base | off[gi]) * d];
          for (unsigned col = 0; col < d; ++col) {
            ar[col] += gr * xr[col] - gm * xi[col];
            ai[col] += gr * xi[col] + gm * xr[col];
          }
        }
      }
      for (unsigned go = 0; go < gd; ++go) {
        std::memcpy(&re[size_t(base | off[go]) * d], &tre[size_t(go) * d],
                    d * sizeof(double));
        std::memcpy(&im[size_t(base | off[go]) * d], &tim[size_t(go) * d],
                    d * sizeof(double));
      }
    }
  }
  std::vector<cplx> m(size_t(d) * d);
  for (size_t i = 0; i < m.size(); ++i) m[i] = cplx(re[i], im[i]);
  return m;
}

namespace {

uint64_t qmask(const std::vector<unsigned>& qs) {
  uint64_t m = 0;
  for (unsigned q : qs) m |= uint64_t{1} << q;
  return m;
}

// The 12-qubit tile of two sorted 6-qubit target sets: the mask of their
// union completed with the lowest other qubits (0 when the union has more
// than 12), without the kernel geometry: a quick filter before
// tc2_run_bits, which also builds the geometry and its swizzles.
uint64_t pair_tile(unsigned n, const std::vector<unsigned>& a,
                   const std::vector<unsigned>& b) {
  uint64_t u = 0;
  for (unsigned q : a) u |= uint64_t{1} << q;
  for (unsigned q : b) u |= uint64_t{1} << q;
  int cnt = __builtin_popcountll(u);
  if (cnt > 12) return 0;
  for (unsigned q = 0; cnt < 12 && q < n; ++q)
    if (!((u >> q) & 1)) {
      u |= uint64_t{1} << q;
      ++cnt;
    }
  return u;
}

// Run bits of a tile mask: the length of its prefix of qubits 0, 1, ...
int tile_run_bits(uint64_t tile) {
  int run = 0;
  while (run < 64 && ((tile >> run) & 1)) ++run;
  return run;
}

// M^dagger M = 1 within 1e-5 per entry (M row-major, d x d).
bool unitary_matrix(const std::vector<cplx>& m) {
  const size_t d = size_t(std::sqrt(double(m.size())) + 0.5);
  for (size_t r = 0; r < d; ++r)
    for (size_t c = r; c < d; ++c) {
      cplx a = 0;
      for (size_t j = 0; j < d; ++j) a += std::conj(m[j * d + r]) * m[j * d + c];
      if (std::abs(a - (r == c ? 1.0 : 0.0)) > 1e-5) return false;
    }
  return true;
}

void finish(const Circuit& c, PlanOp& p) {
  // A block is unitary when every member gate is: the members are small
  // (usually 1-2 qubits), the block up to 64 x 64.
  p.unitary = p.kind != OpKind::kMeasure && !p.members.empty();
  for (int mi : p.members)
    if (!unitary_matrix(c.ops[mi].m)) {
      p.unitary = false;
      break;
    }
  if (p.kind == OpKind::kGate) {
    if (p.members.size() == 1 && c.ops[p.members[0]].qs == p.qs) {
      p.m = c.ops[p.members[0]].m;
    } else {
      p.m = block_matrix(c, p.members, p.qs);
    }
  }
  p.m32.resize(2 * p.m.size());
  for (size_t i = 0; i < p.m.size(); ++i) {
    p.m32[2 * i] = float(p.m[i].real());
    p.m32[2 * i + 1] = float(p.m[i].imag());
  }
}

struct Block {
  std::vector<int> members;
  uint64_t mask = 0;
  double score = -1e300;
  Path path = Path::kCudaCore;
};

// One absorb scan over the unscheduled ops of [first, end): ops whose qubits
// lie in `mask` and whose unscheduled predecessors are all in the block are
// absorbed (in_block set, appended to `members` when `commit`).  Returns the
// count absorbed and fills `cands` with expansion candidates: fusible ops
// that are not blocked but need qubits outside `mask`, with
// popcount(mask | q) <= f, in scan order.
constexpr size_t kCandWindow = 256;

// Per-op qubit masks (targets | controls) and fusibility of a circuit,
// computed once per planning run.
struct OpInfo {
  std::vector<uint64_t> mask;
  std::vector<char> fusible;
};

size_t absorb_scan(const OpInfo& info, const std::vector<char>& done,
                   std::vector<char>& in_block, size_t first, size_t end,
                   uint64_t mask, unsigned f, bool commit,
                   std::vector<int>* members, std::vector<size_t>* cands,
                   size_t max_cands) {
  // The scan visits each op once, so a trial scan (commit false) needs no
  // marks; a committed one marks its ops for the scans that follow.
  uint64_t blocked = 0;
  size_t absorbed = 0;
  for (size_t i = first; i < end; ++i) {
    if (done[i] || in_block[i]) continue;
    const uint64_t m = info.mask[i];
    const bool fus = info.fusible[i] != 0;
    if (m & blocked) {
      blocked |= m;
    } else if (fus && (m & ~mask) == 0) {
      ++absorbed;
      if (commit) {
        members->push_back(int(i));
        in_block[i] = 1;
      }
    } else {
      if (cands && fus && cands->size() < max_cands &&
          unsigned(__builtin_popcountll(mask | m)) <= f)
        cands->push_back(i);
      blocked |= m;
    }
    // Once every qubit of the block is blocked nothing more can be absorbed;
    // the candidate scan then goes on only while it has found fewer than
    // max_cands candidates and stays within a window of ops.
    if ((mask & ~blocked) == 0 &&
        (!cands || cands->size() >= max_cands || i - first > kCandWindow))
      break;
  }
  return absorbed;
}

// Grows a block from `seed`: absorb everything inside the current qubit
// set, then expand the set by the candidate whose expanded set absorbs the
// most ops (one-step lookahead), until the set has f qubits or no
// candidate fits.
Block grow_block(const Circuit& c, const OpInfo& info,
                 const std::vector<char>& done, size_t first, size_t end,
                 size_t seed, unsigned f) {
  // All zero between calls: each call clears the marks it set (its
  // members), also when it leaves by an exception.
  static thread_local std::vector<char> in_block;
  if (in_block.size() < c.ops.size()) in_block.assign(c.ops.size(), 0);
  Block b;
  struct Unmark {
    std::vector<char>& v;
    const std::vector<int>& m;
    ~Unmark() {
      for (int i : m) v[size_t(i)] = 0;
    }
  } unmark{in_block, b.members};
  b.members.push_back(int(seed));
  in_block[seed] = 1;
  b.mask = qmask(c.ops[seed].qs);
  constexpr size_t kMaxCands = 12;
  std::vector<size_t> cands;
  for (;;) {
    cands.clear();
    absorb_scan(info, done, in_block, first, end, b.mask, f, true,
                &b.members, &cands, kMaxCands);
    if (unsigned(__builtin_popcountll(b.mask)) >= f || cands.empty()) break;
    size_t best = cands[0];
    long best_score = -1;
    for (size_t cand : cands) {
      const uint64_t m2 = b.mask | qmask(c.ops[cand].qs);
      const size_t got = absorb_scan(info, done, in_block, first, end, m2, f,
                                     false, nullptr, nullptr, 0);
      // Prefer more absorbed ops, then fewer new qubits.
      const long score =
          long(got) * 8 - long(__builtin_popcountll(m2 & ~b.mask));
      if (score > best_score) {
        best_score = score;
        best = cand;
      }
    }
    b.mask |= qmask(c.ops[best].qs);
  }
  std::sort(b.members.begin(), b.members.end());
  return b;
}

}  // namespace

// Pads a block to 6 targets with the identity on the lowest free qubits
// (the tensor-core kernel's fixed shape).
void pad_block_to_6(unsigned n, PlanOp& po) {
  const unsigned k = po.qs.size();
  if (k >= 6 || n < 6) return;
  std::vector<unsigned> all = po.qs;
  for (unsigned q = 0; all.size() < 6 && q < n; ++q)
    if (std::find(all.begin(), all.end(), q) == all.end()) all.push_back(q);
  std::sort(all.begin(), all.end());
  unsigned pos[6];
  unsigned tmask = 0;
  for (unsigned j = 0; j < k; ++j) {
    pos[j] = unsigned(std::find(all.begin(), all.end(), po.qs[j]) - all.begin());
    tmask |= 1u << pos[j];
  }
  auto sub = [&](unsigned i) {
    unsigned r = 0;
    for (unsigned j = 0; j < k; ++j) r |= ((i >> pos[j]) & 1) << j;
    return r;
  };
  const unsigned d = 1u << k;
  std::vector<cplx> m6(64 * 64, 0.0);
  for (unsigned r = 0; r < 64; ++r)
    for (unsigned cc = 0; cc < 64; ++cc)
      if ((r & ~tmask) == (cc & ~tmask)) m6[r * 64 + cc] = po.m[sub(r) * d + sub(cc)];
  po.qs = all;
  po.m = std::move(m6);
  po.m32.resize(2 * po.m.size());
  for (size_t i = 0; i < po.m.size(); ++i) {
    po.m32[2 * i] = float(po.m[i].real());
    po.m32[2 * i + 1] = float(po.m[i].imag());
  }
}

Plan unfused(const Circuit& c) {
  Plan p;
  p.num_qubits = c.num_qubits;
  for (size_t i = 0; i < c.ops.size(); ++i) {
    const Op& op = c.ops[i];
    PlanOp po;
    po.kind = op.kind;
    po.time = op.time;
    po.qs = op.qs;
    po.cqs = op.cqs;
    po.cvals = op.cvals;
    po.m = op.m;
    po.members = {int(i)};
    finish(c, po);
    p.ops.push_back(std::move(po));
  }
  return p;
}

namespace {

// One greedy pass with block-size limit f.  Without a cost model (and with
// per_gate false) every block grows to f qubits, the candidate absorbing the
// most gates wins and blocks of >= tc_min_k qubits take the tensor-core
// path.  With a cost model each block's path is the one with the lower
// predicted time; with per_gate, blocks of every size limit from the seed's
// size to f compete and the lowest predicted time per absorbed gate wins.
Plan fuse_greedy(const Circuit& c, const FuseOptions& opt, unsigned f,
                 bool per_gate) {
  Plan plan;
  plan.num_qubits = c.num_qubits;
  const size_t nops = c.ops.size();
  std::vector<char> done(nops, 0);

  auto fusible = [&](const Op& op) {
    return op.kind == OpKind::kGate && op.qs.size() <= f;
  };
  OpInfo info;
  info.mask.resize(nops);
  info.fusible.resize(nops);
  for (size_t i = 0; i < nops; ++i) {
    info.mask[i] = qmask(c.ops[i].qs) | qmask(c.ops[i].cqs);
    info.fusible[i] = fusible(c.ops[i]) ? 1 : 0;
  }
  // With a cost model: the cheaper path for a block (tensor cores only for
  // blocks of >= tc_min_k qubits on >= 12-qubit states) and its cost.
  auto cost_of = [&](const std::vector<unsigned>& qs, Path* path) {
    double best = opt.cost->cost_us(c.num_qubits, qs, 0, Path::kCudaCore);
    *path = Path::kCudaCore;
    if (opt.tensor_path && qs.size() >= opt.tc_min_k && c.num_qubits >= 12) {
      const double t = opt.cost->cost_us(c.num_qubits, qs, 0, Path::kTensor);
      if (t < best) {
        best = t;
        *path = Path::kTensor;
      }
    }
    return best;
  };

  size_t seg_begin = 0;
  while (seg_begin < nops) {
    // Segment: up to and including the next measurement (a full barrier).
    size_t seg_end = seg_begin;
    while (seg_end < nops && c.ops[seg_end].kind != OpKind::kMeasure) ++seg_end;

    size_t first = seg_begin;
    for (;;) {
      while (first < seg_end && done[first]) ++first;
      if (first >= seg_end) break;
      const Op& op0 = c.ops[first];
      if (!fusible(op0)) {
        PlanOp po;
        po.kind = op0.kind;
        po.time = op0.time;
        po.qs = op0.qs;
        po.cqs = op0.cqs;
        po.cvals = op0.cvals;
        po.m = op0.m;
        po.members = {int(first)};
        finish(c, po);
        plan.ops.push_back(std::move(po));
        done[first] = 1;
        continue;
      }
      // Seeds: front gates (no unscheduled predecessor) among the first few
      // unscheduled fusible gates.
      std::vector<size_t> seeds;
      {
        uint64_t touched = 0;
        for (size_t i = first; i < seg_end && seeds.size() < opt.seeds; ++i) {
          if (done[i]) continue;
          const Op& op = c.ops[i];
          const uint64_t m = qmask(op.qs) | qmask(op.cqs);
          if (fusible(op) && (m & touched) == 0) seeds.push_back(i);
          touched |= m;
          if (touched == (c.num_qubits >= 64 ? ~uint64_t{0}
                                             : (uint64_t{1} << c.num_qubits) - 1))
            break;
        }
      }
      Block best;
      for (size_t seed : seeds) {
        // Without a cost model every block grows to f qubits and the one
        // absorbing the most gates wins.  With one, blocks of every size
        // limit from the seed's size to f compete, and the one with the
        // lowest predicted time per absorbed gate wins: the model chooses
        // the block boundaries, the block size and the path.
        const unsigned lo = (opt.cost && per_gate)
                                ? std::max<unsigned>(
                                      1, unsigned(c.ops[seed].qs.size()))
                                : f;
        for (unsigned lim = lo; lim <= f; ++lim) {
          Block b = grow_block(c, info, done, first, seg_end, seed, lim);
          std::vector<unsigned> qs;
          for (unsigned q = 0; q < c.num_qubits; ++q)
            if ((b.mask >> q) & 1) qs.push_back(q);
          if (opt.cost && per_gate) {
            b.score = -cost_of(qs, &b.path) / double(b.members.size());
          } else if (opt.cost) {
            b.score = double(b.members.size()) - 1e-3 * double(qs.size());
            cost_of(qs, &b.path);
          } else {
            b.score = double(b.members.size()) - 1e-3 * double(qs.size());
            b.path = (opt.tensor_path && qs.size() >= opt.tc_min_k &&
                      c.num_qubits >= 12)
                         ? Path::kTensor
                         : Path::kCudaCore;
          }
          if (b.score > best.score) best = std::move(b);
        }
      }
      PlanOp po;
      po.kind = OpKind::kGate;
      po.time = c.ops[best.members.front()].time;
      for (unsigned q = 0; q < c.num_qubits; ++q)
        if ((best.mask >> q) & 1) po.qs.push_back(q);
      po.members = best.members;
      for (int mi : best.members) done[mi] = 1;
      finish(c, po);
      if (best.path == Path::kTensor) {
        pad_block_to_6(c.num_qubits, po);
        po.path = Path::kTensor;
      }
      plan.ops.push_back(std::move(po));
    }
    if (seg_end < nops) {
      const Op& m = c.ops[seg_end];
      PlanOp po;
      po.kind = OpKind::kMeasure;
      po.time = m.time;
      po.qs = m.qs;
      po.members = {int(seg_end)};
      plan.ops.push_back(std::move(po));
      done[seg_end] = 1;
    }
    seg_begin = seg_end + 1;
  }
  return plan;
}

// A cost model's answers memoised by (qubit set, controls, path): the greedy
// search prices the same blocks many times over.  Not thread-safe: one per
// planning thread.
class MemoCost : public CostModel {
 public:
  explicit MemoCost(const CostModel* m) : m_(m) {}
  double cost_us(unsigned n, const std::vector<unsigned>& qs,
                 unsigned ncontrols, Path path) const override {
    uint64_t mask = 0;
    bool sorted = n <= 64;
    for (size_t i = 0; sorted && i < qs.size(); ++i) {
      sorted = qs[i] < 64 && (i == 0 || qs[i - 1] < qs[i]);
      if (sorted) mask |= uint64_t{1} << qs[i];
    }
    if (!sorted) return m_->cost_us(n, qs, ncontrols, path);
    const Key k{mask, (uint64_t(n) << 40) | (uint64_t(ncontrols) << 8) |
                          uint64_t(path == Path::kTensor)};
    auto it = memo_.find(k);
    if (it != memo_.end()) return it->second;
    const double v = m_->cost_us(n, qs, ncontrols, path);
    memo_.emplace(k, v);
    return v;
  }

 private:
  struct Key {
    uint64_t mask, rest;
    bool operator==(const Key& o) const {
      return mask == o.mask && rest == o.rest;
    }
  };
  struct KeyHash {
    size_t operator()(const Key& k) const {
      return size_t(k.mask * 0x9E3779B97F4A7C15ull ^ (k.rest + (k.rest << 17)));
    }
  };
  const CostModel* m_;
  mutable std::unordered_map<Key, double, KeyHash> memo_;
};

// Predicted time of a plan; a two-gate tensor-core pass costs
// tc_pair_cost_factor(tile) of its two blocks' one-gate passes.
double plan_cost(const Circuit& c, const Plan& p, const CostModel& m) {
  double t = 0;
  for (size_t i = 0; i < p.ops.size(); ++i) {
    const auto& op = p.ops[i];
    if (op.kind == OpKind::kMeasure) continue;
    double ti = m.cost_us(c.num_qubits, op.qs, unsigned(op.cqs.size()), op.path);
    if (op.tc_pair_next) {
      const auto& nx = p.ops[i + 1];
      ti += m.cost_us(c.num_qubits, nx.qs, unsigned(nx.cqs.size()), nx.path);
      ti *= tc_pair_cost_factor(pair_tile(c.num_qubits, op.qs, nx.qs));
      ++i;
    }
    t += ti;
  }
  return t;
}

// Passes over the state in units of one pass: a two-gate pass counts
// 2 tc_pair_cost_factor(tile).
double plan_passes(const Plan& p) {
  double t = 0;
  for (size_t i = 0; i < p.ops.size(); ++i) {
    const auto& op = p.ops[i];
    if (op.kind == OpKind::kMeasure) continue;
    if (op.tc_pair_next) {
      t += 2.0 * tc_pair_cost_factor(
                     pair_tile(p.num_qubits, op.qs, p.ops[i + 1].qs));
      ++i;
    } else {
      t += 1.0;
    }
  }
  return t;
}

}  // namespace

// A controlled op as a plain gate on its targets and controls (sorted):
// the identity except on the rows and columns whose control bits equal
// cvals, where the target matrix acts.  Same op index, so block members
// still name circuit ops.
namespace {

Op expand_controlled_op(const Op& op) {
  Op e;
  e.kind = OpKind::kGate;
  e.time = op.time;
  e.qs = op.qs;
  e.qs.insert(e.qs.end(), op.cqs.begin(), op.cqs.end());
  std::sort(e.qs.begin(), e.qs.end());
  const unsigned k = op.qs.size(), nc = op.cqs.size(), u = e.qs.size();
  auto pos = [&](unsigned q) {
    return unsigned(std::find(e.qs.begin(), e.qs.end(), q) - e.qs.begin());
  };
  unsigned tpos[6], cpos[6];
  for (unsigned j = 0; j < k; ++j) tpos[j] = pos(op.qs[j]);
  for (unsigned i = 0; i < nc; ++i) cpos[i] = pos(op.cqs[i]);
  const unsigned d = 1u << u, dk = 1u << k;
  auto tidx = [&](unsigned x) {
    unsigned t = 0;
    for (unsigned j = 0; j < k; ++j) t |= ((x >> tpos[j]) & 1u) << j;
    return t;
  };
  auto cval = [&](unsigned x) {
    uint64_t v = 0;
    for (unsigned i = 0; i < nc; ++i) v |= uint64_t((x >> cpos[i]) & 1u) << i;
    return v;
  };
  e.m.assign(size_t(d) * d, 0.0);
  for (unsigned r = 0; r < d; ++r) {
    for (unsigned col = 0; col < d; ++col) {
      if (cval(r) != cval(col)) continue;
      const unsigned tr = tidx(r), tc = tidx(col);
      if (cval(r) == op.cvals) {
        e.m[size_t(r) * d + col] = op.m[size_t(tr) * dk + tc];
      } else if (tr == tc) {
        e.m[size_t(r) * d + col] = 1.0;
      }
    }
  }
  return e;
}

// The circuit with every controlled op on at most f qubits (targets and
// controls) expanded to a plain gate; op indices unchanged.
Circuit expand_controlled(const Circuit& c, unsigned f) {
  Circuit e = c;
  for (auto& op : e.ops)
    if (op.kind == OpKind::kControlled && op.qs.size() + op.cqs.size() <= f)
      op = expand_controlled_op(op);
  return e;
}

// A plan of the expanded circuit with every block that holds one expanded
// controlled op alone turned back into that controlled op (a controlled
// pass touches only the amplitudes its controls select).
Plan restore_lone_controlled(const Circuit& c, Plan p) {
  for (auto& po : p.ops) {
    if (po.kind != OpKind::kGate || po.members.size() != 1) continue;
    const Op& op = c.ops[po.members[0]];
    if (op.kind != OpKind::kControlled) continue;
    PlanOp r;
    r.kind = op.kind;
    r.time = op.time;
    r.qs = op.qs;
    r.cqs = op.cqs;
    r.cvals = op.cvals;
    r.m = op.m;
    r.members = po.members;
    finish(c, r);
    po = std::move(r);
  }
  return p;
}

}  // namespace

// Seed windows tried by the multi-start search: the greedy rule is not
// monotonic in the window (on the 30-qubit depth-20 grid circuit at f = 6,
// windows of 3 and 4 gates give 36 blocks, 12 gives 37, 5 gives 41).
constexpr unsigned kStartWindows[] = {2, 3, 4, 6, 8};

size_t pair_tensor_ops(Plan& plan, unsigned bits) {
  const size_t n = plan.ops.size();
  for (auto& op : plan.ops) op.tc_pair_next = false;
  if (bits == 0 || n < 2) return 0;
  auto tensor6 = [&](const PlanOp& op) {
    return op.kind == OpKind::kGate && op.path == Path::kTensor &&
           op.qs.size() == 6 && op.cqs.empty();
  };
  // gain[i] > 0: ops i, i + 1 fit one pass, predicted faster than two (in
  // units of one pass).  best[i]: the largest total gain among ops >= i.
  std::vector<double> gain(n, 0.0);
  for (size_t i = 0; i + 1 < n; ++i) {
    if (!tensor6(plan.ops[i]) || !tensor6(plan.ops[i + 1])) continue;
    const uint64_t tile = pair_tile(plan.num_qubits, plan.ops[i].qs,
                                    plan.ops[i + 1].qs);
    if (!tile || tile_run_bits(tile) < int(bits)) continue;
    const double g = 2.0 * (1.0 - tc_pair_cost_factor(tile));
    if (g <= 0) continue;
    if (tc2_run_bits(plan.num_qubits, plan.ops[i].qs.data(),
                     plan.ops[i + 1].qs.data()) < int(bits))
      continue;
    gain[i] = g;
  }
  std::vector<double> best(n + 2, 0.0);
  for (size_t i = n; i-- > 0;) {
    best[i] = best[i + 1];
    if (gain[i] > 0) best[i] = std::max(best[i], gain[i] + best[i + 2]);
  }
  size_t pairs = 0;
  for (size_t i = 0; i < n;) {
    if (gain[i] > 0 && gain[i] + best[i + 2] >= best[i + 1]) {
      plan.ops[i].tc_pair_next = true;
      ++pairs;
      i += 2;
    } else {
      ++i;
    }
  }
  return pairs;
}

Plan fuse(const Circuit& c, const FuseOptions& opt) {
  const unsigned f = std::max(1u, std::min(6u, opt.max_fused_size));
  if (!opt.cost) {
    if (!opt.tensor_path) return fuse_greedy(c, opt, f, false);
    // Tensor-core plans cost about the same per block, so their run time is
    // their block count: keep the greedy result with the fewest blocks (the
    // first of equal ones, in window order).  The runs are independent and
    // run on host threads of their own.
    std::vector<unsigned> windows{opt.seeds};
    for (unsigned w : kStartWindows)
      if (w != opt.seeds) windows.push_back(w);
    // std::async futures carry a worker's exception (bad_alloc, say) to
    // get() on this thread, and their destructors wait for the worker, so
    // an exception here never leaves a joinable thread behind.
    // With two-gate passes a pair counts as its measured cost in passes.
    std::vector<Plan> plans(windows.size());
    std::vector<std::future<Plan>> pool;
    for (size_t i = 1; i < windows.size(); ++i) {
      pool.push_back(std::async(std::launch::async, [&, i] {
        FuseOptions o = opt;
        o.seeds = windows[i];
        Plan p = fuse_greedy(c, o, f, false);
        pair_tensor_ops(p, opt.tc_pair_bits);
        return p;
      }));
    }
    plans[0] = fuse_greedy(c, opt, f, false);
    pair_tensor_ops(plans[0], opt.tc_pair_bits);
    for (size_t i = 1; i < windows.size(); ++i) plans[i] = pool[i - 1].get();
    size_t best = 0;
    for (size_t i = 1; i < plans.size(); ++i)
      if (plan_passes(plans[i]) < plan_passes(plans[best])) best = i;
    return std::move(plans[best]);
  }
  // Learned planner: candidate plans for every block-size limit up to f,
  // grown by gate count and by predicted time per gate (for limits >= 5
  // also with a 3-gate seed window), each block on its predicted-faster
  // path; the plan of lowest predicted total time wins.
  // The fixed-size plans of the gate-count rule are among the candidates.
  // Circuits with controlled ops also get candidates in which those ops are
  // plain gates on targets and controls that blocks may absorb (the
  // reference's fuser always passes them through unfused), each lone one
  // turned back into a controlled pass; the predicted times decide.
  //
  // The candidates are independent: each runs on a host thread of its own
  // (futures), and the lowest predicted time wins, the first in candidate
  // order on ties, so the result does not depend on the threads.
  bool has_controlled = false;
  for (const auto& op : c.ops) has_controlled |= op.kind == OpKind::kControlled;
  std::vector<Circuit> expanded(f + 1);
  if (has_controlled)
    for (unsigned ff = 2; ff <= f; ++ff) expanded[ff] = expand_controlled(c, ff);
  struct Cand {
    unsigned ff, w;
    int pg;
    bool expand;
  };
  std::vector<Cand> cands;
  for (int ex = 0; ex < (has_controlled ? 2 : 1); ++ex) {
    for (unsigned ff = 1; ff <= f; ++ff) {
      if (ex && ff < 2) continue;
      for (int pg = 0; pg < 2; ++pg) {
        if (ff == 1 && pg) continue;
        for (unsigned w : {opt.seeds, 3u}) {
          if (w == 3u && (opt.seeds == 3u || ff < 5)) continue;
          cands.push_back({ff, w, pg, ex != 0});
        }
        // The gate-count rule at the full block size also from the other
        // start windows of the fixed tensor-core planner.
        if (opt.tensor_path && ff == f && f >= 5 && !pg)
          for (unsigned w : kStartWindows)
            if (w != opt.seeds && w != 3u) cands.push_back({ff, w, pg, ex != 0});
      }
    }
  }
  std::vector<std::future<std::pair<Plan, double>>> runs;
  for (const Cand& cd : cands) {
    const Circuit& cc = cd.expand ? expanded[cd.ff] : c;
    runs.push_back(std::async(std::launch::async, [&c, &cc, &opt, cd] {
      MemoCost memo(opt.cost);   // one per candidate: no shared state
      FuseOptions o = opt;
      o.seeds = cd.w;
      o.cost = &memo;
      Plan p = fuse_greedy(cc, o, cd.ff, cd.pg != 0);
      if (cd.expand) p = restore_lone_controlled(c, std::move(p));
      if (opt.tensor_path) pair_tensor_ops(p, opt.tc_pair_bits);
      const double t = plan_cost(c, p, memo);
      return std::make_pair(std::move(p), t);
    }));
  }
  Plan best;
  double best_t = 0;
  bool have = false;
  for (auto& r : runs) {
    auto pt = r.get();
    if (!have || pt.second < best_t) {
      best = std::move(pt.first);
      best_t = pt.second;
      have = true;
    }
  }
  return best;
}

}  // namespace host
}  // namespace qsg
