// Fused-plan cache keyed by circuit content, with CUDA-graph replay.
//
// The reference fuses the circuit again on every run: QSimRunner::Run
// (lib/run_qsim.h:225-289) calls the fuser, then applies each fused gate,
// and a text circuit is parsed by CircuitQsimParser::FromStream
// (lib/circuit_qsim_parser.h:52-153) before that.  Here a run looks its
// circuit up first: the key is the circuit's operations (or, for a text
// circuit, the text itself and maxtime) together with the fusion options,
// hashed to 64 bits and compared in full on a hash match, so a collision
// never returns another circuit's plan.  A hit skips parsing and fusion; a
// plan without measurements is captured once per (context, state) into a
// CUDA graph, and later runs on that state replay the graph (one launch on
// the host).  Plans with measurements run op by op, their measurements
// drawing from std::mt19937(seed) as in qsg_plan_run.  Least recently used
// entries are evicted beyond `capacity`.

#include <algorithm>
#include <cstring>
#include <list>
#include <memory>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "capi_types.h"
#include "engine.h"
#include "internal.h"
#include "runner.h"

using namespace qsg;
using namespace qsg::host;

namespace {

struct Entry {
  uint64_t hash = 0;
  std::string key;
  std::unique_ptr<PlanRuntime> rt;
  bool has_measure = false;
};

template <typename T>
void put(std::string* s, const T& v) {
  s->append(reinterpret_cast<const char*>(&v), sizeof(v));
}

void put_options(std::string* s, const FuseOptions& fo) {
  put(s, fo.max_fused_size);
  put(s, fo.seeds);
  put(s, uint8_t(fo.tensor_path));
  put(s, fo.tc_min_k);
  put(s, fo.tc_pair_bits);
  // A cost model is keyed by its identity: a model changed in place (more
  // training) needs qsg_plan_cache_clear.
  put(s, reinterpret_cast<uintptr_t>(fo.cost));
}

std::string circuit_key(const Circuit& c, const FuseOptions& fo) {
  std::string s;
  size_t bytes = 64;
  for (const Op& op : c.ops)
    bytes += 32 + 4 * (op.qs.size() + op.cqs.size()) + 16 * op.m.size();
  s.reserve(bytes);
  s.push_back('C');
  put_options(&s, fo);
  put(&s, c.num_qubits);
  put(&s, uint64_t(c.ops.size()));
  for (const Op& op : c.ops) {
    put(&s, int(op.kind));
    put(&s, op.time);
    put(&s, uint32_t(op.qs.size()));
    s.append(reinterpret_cast<const char*>(op.qs.data()),
             op.qs.size() * sizeof(unsigned));
    put(&s, uint32_t(op.cqs.size()));
    s.append(reinterpret_cast<const char*>(op.cqs.data()),
             op.cqs.size() * sizeof(unsigned));
    put(&s, op.cvals);
    put(&s, uint64_t(op.m.size()));
    s.append(reinterpret_cast<const char*>(op.m.data()),
             op.m.size() * sizeof(cplx));
  }
  return s;
}

std::string text_key(const char* text, unsigned maxtime,
                     const FuseOptions& fo) {
  std::string s;
  const size_t len = std::strlen(text);
  s.reserve(len + 64);
  s.push_back('T');
  put_options(&s, fo);
  put(&s, maxtime);
  s.append(text, len);
  return s;
}

// 64-bit hash of a byte string: 8-byte words multiplied into the state and
// folded (a multiply-rotate mix), then a final avalanche (the 64-bit
// finaliser of MurmurHash3).
uint64_t hash_bytes(const std::string& s) {
  const uint64_t k1 = 0x9e3779b97f4a7c15ull, k2 = 0xc2b2ae3d27d4eb4full;
  uint64_t h = 0x243f6a8885a308d3ull ^ (uint64_t(s.size()) * k1);
  const char* p = s.data();
  size_t n = s.size();
  for (; n >= 8; p += 8, n -= 8) {
    uint64_t w;
    std::memcpy(&w, p, 8);
    h ^= w * k2;
    h = ((h << 31) | (h >> 33)) * k1;
  }
  uint64_t tail = 0;
  std::memcpy(&tail, p, n);
  h ^= tail * k2;
  h ^= h >> 33;
  h *= 0xff51afd7ed558ccdull;
  h ^= h >> 33;
  h *= 0xc4ceb9fe1a85ec53ull;
  h ^= h >> 33;
  return h;
}

int invalid(const char* msg) {
  set_error_msg(msg);
  return QSG_ERR_INVALID;
}

}  // namespace

struct qsg_plan_cache {
  std::mutex mu;
  size_t capacity = 0;
  uint64_t hits = 0, misses = 0, evictions = 0, captures = 0;
  std::list<Entry> lru;  // front: most recently used
  std::unordered_multimap<uint64_t, std::list<Entry>::iterator> index;

  // The entry of `key`, moved to the front; null when absent.
  Entry* find(uint64_t h, const std::string& key) {
    auto range = index.equal_range(h);
    for (auto it = range.first; it != range.second; ++it) {
      if (it->second->key == key) {
        lru.splice(lru.begin(), lru, it->second);
        return &*lru.begin();
      }
    }
    return nullptr;
  }

  Entry* insert(uint64_t h, std::string key, Plan plan) {
    while (capacity && lru.size() >= capacity) {
      auto last = std::prev(lru.end());
      auto range = index.equal_range(last->hash);
      for (auto it = range.first; it != range.second; ++it) {
        if (it->second == last) {
          index.erase(it);
          break;
        }
      }
      lru.pop_back();
      ++evictions;
    }
    Entry e;
    e.hash = h;
    e.key = std::move(key);
    e.rt = std::make_unique<PlanRuntime>();
    for (const auto& op : plan.ops) e.has_measure |= op.kind == OpKind::kMeasure;
    e.rt->plan = std::move(plan);
    lru.push_front(std::move(e));
    index.emplace(h, lru.begin());
    return &*lru.begin();
  }

  int run(qsg_ctx* ctx, Entry* e, float* state, unsigned seed, uint64_t* mbits,
          uint64_t mbits_cap, uint64_t* num_meas) {
    PlanRuntime& rt = *e->rt;
    if (rt.ctx && rt.ctx != ctx) {
      // Device resources belong to the context that uploaded them: start
      // over for another context, keeping the fused plan.
      auto fresh = std::make_unique<PlanRuntime>();
      fresh->plan = std::move(rt.plan);
      e->rt = std::move(fresh);
      return run(ctx, e, state, seed, mbits, mbits_cap, num_meas);
    }
    if (e->has_measure) {
      std::vector<uint64_t> bits;
      const int rc = rt.run(ctx, state, seed, &bits);
      if (num_meas) *num_meas = bits.size();
      if (mbits)
        std::copy(bits.begin(),
                  bits.begin() + std::min<size_t>(bits.size(), mbits_cap), mbits);
      return rc;
    }
    if (num_meas) *num_meas = 0;
    if (!rt.graph_exec || rt.captured_state != state) {
      const int rc = rt.capture(ctx, state);
      if (rc) return rc;
      ++captures;
    }
    return rt.replay(ctx);
  }
};

extern "C" {

int qsg_plan_cache_create(unsigned capacity, qsg_plan_cache** out) {
  if (!out) return invalid("qsg_plan_cache_create: null argument");
  auto* c = new qsg_plan_cache();
  c->capacity = capacity;
  *out = c;
  return QSG_OK;
}

int qsg_plan_cache_destroy(qsg_plan_cache* c) {
  delete c;
  return QSG_OK;
}

int qsg_plan_cache_clear(qsg_plan_cache* c) {
  if (!c) return invalid("qsg_plan_cache_clear: null cache");
  std::lock_guard<std::mutex> lk(c->mu);
  c->index.clear();
  c->lru.clear();
  return QSG_OK;
}

int qsg_plan_cache_stats(qsg_plan_cache* c, uint64_t* hits,
                         uint64_t* misses, uint64_t* evictions,
                         uint64_t* captures, uint64_t* size) {
  if (!c) return invalid("qsg_plan_cache_stats: null cache");
  std::lock_guard<std::mutex> lk(c->mu);
  if (hits) *hits = c->hits;
  if (misses) *misses = c->misses;
  if (evictions) *evictions = c->evictions;
  if (captures) *captures = c->captures;
  if (size) *size = c->lru.size();
  return QSG_OK;
}

int qsg_plan_cache_run(qsg_ctx* ctx, qsg_plan_cache* cache,
                       const qsg_circuit* circuit,
                       const qsg_fuse_options* opts, float* state,
                       unsigned seed, uint64_t* mbits, uint64_t mbits_cap,
                       uint64_t* num_meas, int* hit) {
  if (!ctx || !cache || !circuit || !state)
    return invalid("qsg_plan_cache_run: null argument");
  FuseOptions fo;
  if (!fuse_options_from(opts, &fo))
    return invalid("qsg_plan_cache_run: max_fused_size must be 1..6");
  std::string key = circuit_key(circuit->c, fo);
  const uint64_t h = hash_bytes(key);
  std::lock_guard<std::mutex> lk(cache->mu);
  Entry* e = cache->find(h, key);
  if (hit) *hit = e != nullptr;
  if (e) {
    ++cache->hits;
  } else {
    ++cache->misses;
    e = cache->insert(h, std::move(key), fuse(circuit->c, fo));
  }
  return cache->run(ctx, e, state, seed, mbits, mbits_cap, num_meas);
}

int qsg_plan_cache_run_text(qsg_ctx* ctx, qsg_plan_cache* cache,
                            const char* text, unsigned maxtime,
                            const qsg_fuse_options* opts, float* state,
                            unsigned seed, uint64_t* mbits,
                            uint64_t mbits_cap, uint64_t* num_meas,
                            int* hit) {
  if (!ctx || !cache || !text || !state)
    return invalid("qsg_plan_cache_run_text: null argument");
  FuseOptions fo;
  if (!fuse_options_from(opts, &fo))
    return invalid("qsg_plan_cache_run_text: max_fused_size must be 1..6");
  std::string key = text_key(text, maxtime, fo);
  const uint64_t h = hash_bytes(key);
  std::lock_guard<std::mutex> lk(cache->mu);
  Entry* e = cache->find(h, key);
  if (hit) *hit = e != nullptr;
  if (e) {
    ++cache->hits;
  } else {
    Circuit c;
    std::string err;
    if (!parse_qsim_text(text, maxtime, &c, &err)) return invalid(err.c_str());
    ++cache->misses;
    e = cache->insert(h, std::move(key), fuse(c, fo));
  }
  return cache->run(ctx, e, state, seed, mbits, mbits_cap, num_meas);
}

}  // extern "C"
