// Packed trajectory batches: compile every trajectory to a device program
// on the host cores, upload the batch once and run it with one persistent
// launch (batch.cu).  The reference's RunBatch (lib/qtrajectory.h:141-236)
// runs the same trajectories one after another with host synchronisations
// at every non-unitary channel.

#include <algorithm>
#include <chrono>
#include <cstring>
#include <new>
#include <thread>

#include <cuda_runtime.h>

#include "batch_dev.h"
#include "internal.h"
#include "runner.h"
#include "trajectory.h"

namespace qsg {
namespace host {

namespace {

int fail(int rc, const char* msg) {
  set_error_msg(msg);
  return rc;
}

struct Program {
  std::vector<BatchOp> ops;
  std::vector<float> extra;
  std::vector<std::pair<size_t, size_t>> extra_refs;
  std::vector<TrajectoryRunner::LogRef> log_refs;
  int rc = QSG_OK;
};

// Device buffers of one packed launch, freed on scope exit.
struct DeviceBatch {
  qsg_ctx* ctx = nullptr;
  void* ops = nullptr;
  void* items = nullptr;
  void* extra = nullptr;
  void* log = nullptr;
  void* times = nullptr;
  void* counter = nullptr;  // uint32 counter + int error flag
  void* slots = nullptr;
  void* geoms = nullptr;
  ~DeviceBatch() {
    for (void* p : {ops, items, extra, log, times, counter, slots, geoms})
      if (p) dev_free(ctx, p);
  }
};

double seconds_since(std::chrono::steady_clock::time_point t) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t)
      .count();
}

}  // namespace

int run_trajectory_batch_packed(int device, std::vector<BatchItem>& items,
                                const PackedOptions& opt, double* wall_s,
                                uint64_t* launches, PackedStats* stats) {
  PackedStats st;
  if (wall_s) *wall_s = 0;
  if (launches) *launches = 0;
  const auto t_start = std::chrono::steady_clock::now();
  std::vector<size_t> packed, rest;
  for (size_t i = 0; i < items.size(); ++i) {
    const TrajectoryRunner* r = items[i].runner;
    if (!r) return fail(QSG_ERR_INVALID, "batch item without a runner");
    if (r->packable() && r->num_qubits() <= opt.max_qubits)
      packed.push_back(i);
    else
      rest.push_back(i);
  }
  // Largest circuits first (longest-processing-time order over the CTAs).
  std::stable_sort(packed.begin(), packed.end(), [&](size_t a, size_t b) {
    return items[a].runner->num_qubits() > items[b].runner->num_qubits();
  });
  int rc = QSG_OK;
  uint64_t nlaunch = 0;
  // The other items run on the stream path: after the packed launch, or
  // while it runs (opt.overlap), on their own streams.
  bool rest_done = false;
  auto run_rest = [&]() -> int {
    rest_done = true;
    auto t_r = std::chrono::steady_clock::now();
    std::vector<BatchItem> sub;
    sub.reserve(rest.size());
    for (size_t i : rest) sub.push_back(items[i]);
    double w = 0;
    uint64_t l = 0;
    const int r = run_trajectory_batch(device, sub, opt.streams, &w, &l);
    for (size_t j = 0; j < rest.size(); ++j)
      items[rest[j]].latency_ms = sub[j].latency_ms;
    nlaunch += l;
    st.stream_items = rest.size();
    st.stream_s = seconds_since(t_r);
    return r;
  };
  if (!packed.empty()) {
    qsg_ctx* ctx = nullptr;
    rc = qsg_ctx_create(device, nullptr, &ctx);
    if (rc) return rc;
    struct CtxGuard {
      qsg_ctx* c;
      ~CtxGuard() { qsg_ctx_destroy(c); }
    } guard{ctx};
    DeviceBatch db;
    db.ctx = ctx;
    unsigned max_n = 1;
    for (size_t i : packed) {
      rc = items[i].runner->upload_packed(ctx);
      if (rc) return rc;
      max_n = std::max(max_n, items[i].runner->num_qubits());
    }

    // Compile the programs on the host cores.
    auto t_build = std::chrono::steady_clock::now();
    std::vector<Program> progs(packed.size());
    unsigned nthreads = opt.host_threads ? opt.host_threads
                                         : std::thread::hardware_concurrency();
    nthreads = std::max(1u, std::min<unsigned>(nthreads, 64));
    nthreads = unsigned(std::min<size_t>(nthreads, packed.size()));
    {
      std::vector<std::thread> pool;
      for (unsigned t = 0; t < nthreads; ++t) {
        pool.emplace_back([&, t]() {
          for (size_t j = t; j < packed.size(); j += nthreads) {
            const BatchItem& it = items[packed[j]];
            Program& p = progs[j];
            // An exception may not leave a host thread (std::terminate):
            // it becomes this program's status.
            try {
              p.rc = it.runner->build_program(it.rep, it.stats, &p.ops,
                                              &p.extra, &p.extra_refs,
                                              &p.log_refs);
            } catch (const std::bad_alloc&) {
              p.rc = QSG_ERR_OOM;
            } catch (...) {
              p.rc = QSG_ERR_INVALID;
            }
          }
        });
      }
      for (auto& th : pool) th.join();
    }
    size_t nops = 0, nextra = 0, nlog = 0;
    for (const Program& p : progs) {
      if (p.rc) return p.rc;
      nops += p.ops.size();
      nextra += p.extra.size();
      nlog += p.log_refs.size();
    }
    if (packed.size() > 0xffffffffu || nlog > 0xffffffffu)
      return fail(QSG_ERR_INVALID, "packed batch too large");
    st.build_s = seconds_since(t_build);

    // Device buffers.
    auto t_up = std::chrono::steady_clock::now();
    bool need_slots = false;
    for (size_t i : packed)
      if (!items[i].out_state) need_slots = true;
    int sms = 0;
    rc = qsg_ctx_num_sms(ctx, &sms);
    if (rc) return rc;
    int occ = 0;
    const unsigned tile_kib = opt.tile_kib ? opt.tile_kib : 32;
    rc = batch_max_ctas_per_sm(128, tile_kib, &occ);
    if (rc) return rc;
    unsigned per_sm = opt.ctas_per_sm ? opt.ctas_per_sm : 4;
    per_sm = std::max(1u, std::min<unsigned>(per_sm, unsigned(std::max(occ, 1))));
    uint64_t ctas = uint64_t(sms) * per_sm;
    const uint64_t slot_floats = qsg_min_size(max_n);
    if (need_slots) {
      size_t free_b = 0, total_b = 0;
      if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess)
        return fail(QSG_ERR_CUDA, "cudaMemGetInfo failed");
      const uint64_t slot_bytes = slot_floats * sizeof(float);
      const uint64_t fit = uint64_t(0.8 * double(free_b)) / slot_bytes;
      if (fit == 0)
        return fail(QSG_ERR_OOM, "packed batch: no room for one state slot");
      ctas = std::min(ctas, fit);
    }
    ctas = std::min<uint64_t>(ctas, packed.size());
    st.ctas = unsigned(ctas);
    st.tile_kib = tile_kib;

    std::vector<BatchItemDev> hitems(packed.size());
    std::vector<BatchOp> hops;
    hops.reserve(nops);
    std::vector<float> hextra;
    hextra.reserve(nextra);
    std::vector<std::pair<size_t, size_t>> patch;  // (op index, extra offset)
    uint32_t log_base = 0;
    for (size_t j = 0; j < packed.size(); ++j) {
      Program& p = progs[j];
      BatchItemDev& d = hitems[j];
      d.op_begin = hops.size();
      d.num_ops = uint32_t(p.ops.size());
      d.n = items[packed[j]].runner->num_qubits();
      d.state = items[packed[j]].out_state;
      d.log_begin = log_base;
      log_base += uint32_t(p.log_refs.size());
      for (const auto& r : p.extra_refs)
        patch.push_back({d.op_begin + r.first, hextra.size() + r.second});
      hops.insert(hops.end(), p.ops.begin(), p.ops.end());
      hextra.insert(hextra.end(), p.extra.begin(), p.extra.end());
    }
    rc = dev_alloc(ctx, std::max<size_t>(hops.size(), 1) * sizeof(BatchOp), &db.ops);
    if (!rc) rc = dev_alloc(ctx, hitems.size() * sizeof(BatchItemDev), &db.items);
    if (!rc) rc = dev_alloc(ctx, std::max<size_t>(hextra.size(), 1) * sizeof(float), &db.extra);
    if (!rc) rc = dev_alloc(ctx, std::max<size_t>(nlog, 1) * sizeof(uint32_t), &db.log);
    if (!rc) rc = dev_alloc(ctx, hitems.size() * 2 * sizeof(unsigned long long), &db.times);
    if (!rc) rc = dev_alloc(ctx, 16, &db.counter);
    if (!rc && need_slots)
      rc = dev_alloc(ctx, ctas * slot_floats * sizeof(float), &db.slots);
    if (rc) return rc;
    const float* dextra = static_cast<const float*>(db.extra);
    for (const auto& pr : patch) hops[pr.first].mat = dextra + pr.second;
    std::vector<unsigned char> gtab;
    rc = batch_plan_geometries(hitems.data(), hitems.size(), hops.data(), &gtab);
    if (!rc) rc = dev_alloc(ctx, gtab.size(), &db.geoms);
    if (!rc) rc = dev_upload(ctx, db.geoms, gtab.data(), gtab.size());
    if (rc) return rc;
    rc = dev_upload(ctx, db.ops, hops.data(), hops.size() * sizeof(BatchOp));
    if (!rc) rc = dev_upload(ctx, db.items, hitems.data(),
                             hitems.size() * sizeof(BatchItemDev));
    if (!rc && !hextra.empty())
      rc = dev_upload(ctx, db.extra, hextra.data(), hextra.size() * sizeof(float));
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(ctx_stream(ctx));
    if (cudaMemsetAsync(db.counter, 0, 16, s) != cudaSuccess)
      return fail(QSG_ERR_CUDA, "memset failed");
    st.upload_s = seconds_since(t_up);

    // One persistent launch.
    auto t_k = std::chrono::steady_clock::now();
    BatchLaunch l;
    l.ctas = unsigned(ctas);
    l.threads = 128;
    l.slots = static_cast<float*>(db.slots);
    l.slot_floats = slot_floats;
    l.geoms = db.geoms;
    l.tile_kib = tile_kib;
    uint32_t* counter = static_cast<uint32_t*>(db.counter);
    int* error = reinterpret_cast<int*>(counter + 1);
    rc = batch_launch(s, l, static_cast<const BatchItemDev*>(db.items),
                      uint32_t(hitems.size()),
                      static_cast<const BatchOp*>(db.ops),
                      static_cast<uint32_t*>(db.log),
                      static_cast<unsigned long long*>(db.times), counter,
                      error);
    if (rc) return rc;
    nlaunch += 1;
    std::vector<uint32_t> hlog(std::max<size_t>(nlog, 1));
    std::vector<unsigned long long> htimes(2 * hitems.size());
    int herr = 0;
    if (cudaMemcpyAsync(hlog.data(), db.log, hlog.size() * sizeof(uint32_t),
                        cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpyAsync(htimes.data(), db.times,
                        htimes.size() * sizeof(unsigned long long),
                        cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpyAsync(&herr, error, sizeof(int), cudaMemcpyDeviceToHost,
                        s) != cudaSuccess)
      return fail(QSG_ERR_CUDA, "packed batch: result copy failed");
    int rc_rest = QSG_OK;
    if (opt.overlap && !rest.empty()) rc_rest = run_rest();
    const cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(QSG_ERR_CUDA, cudaGetErrorString(e));
    if (rc_rest) return rc_rest;
    if (herr) return fail(QSG_ERR_INVALID, "packed batch: malformed op");
    st.kernel_s = seconds_since(t_k);
    for (size_t j = 0; j < packed.size(); ++j) {
      const Program& p = progs[j];
      for (size_t q = 0; q < p.log_refs.size(); ++q) {
        const auto& r = p.log_refs[q];
        const uint32_t v = hlog[hitems[j].log_begin + q];
        if (r.stats) r.stats[r.op] = v == 0xffffffffu ? kNoStat : uint64_t(v);
      }
      items[packed[j]].latency_ms =
          float(double(htimes[2 * j + 1] - htimes[2 * j]) * 1e-6);
    }
    st.packed_items = packed.size();
    st.ops = hops.size();
  }
  if (!rest.empty() && !rest_done) {
    rc = run_rest();
    if (rc) return rc;
  }
  if (wall_s) *wall_s = seconds_since(t_start);
  if (launches) *launches = nlaunch;
  if (stats) *stats = st;
  return QSG_OK;
}

}  // namespace host
}  // namespace qsg
