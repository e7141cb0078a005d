// statespace_gb300.h — header-only StateSpace over the GB300 engine's C ABI.
//
// Drop-in for qsim's StateSpaceCUDA<float> (lib/statespace_cuda.h:43-472)
// with the vector space of lib/vectorspace_cuda.h:44-165 and the
// measurement members of the CRTP base (lib/statespace.h:32-141).  Every
// member keeps the reference's name, signature and error convention:
//
//   * Create returns Null() when the device is out of memory;
//   * Add returns false and InnerProduct / RealInnerProduct return NaN on
//     qubit-count mismatch;
//   * VirtualMeasure returns valid = false for an out-of-range qubit;
//   * CUDA errors that the reference would answer with exit() throw
//     qsim_gb300::Error here (the process keeps running).
//
// The internal order of the engine is the normal (interleaved re/im) order,
// so InternalToNormalOrder / NormalToInternalOrder only validate.
#ifndef QSIM_GB300_STATESPACE_GB300_H_
#define QSIM_GB300_STATESPACE_GB300_H_

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <memory>
#include <random>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "../qsim_gb300.h"

namespace qsim_gb300 {

struct Error : std::runtime_error {
  int status;
  Error(int s, const std::string& m) : std::runtime_error(m), status(s) {}
};

inline void check(int status) {
  if (status != QSG_OK) throw Error(status, qsg_last_error());
}

// A CUDA stream plus device workspaces; shared by a state space and a
// simulator so their work is ordered on one stream (the reference orders
// everything on the legacy default stream).
class Context {
 public:
  explicit Context(int device = 0, void* stream = nullptr) {
    check(qsg_ctx_create(device, stream, &ctx_));
  }
  ~Context() { qsg_ctx_destroy(ctx_); }
  Context(const Context&) = delete;
  Context& operator=(const Context&) = delete;
  qsg_ctx* get() const { return ctx_; }

  // Process-wide context of device 0, created on first use.
  static std::shared_ptr<Context> Default() {
    static std::shared_ptr<Context> c = std::make_shared<Context>(0);
    return c;
  }

 private:
  qsg_ctx* ctx_ = nullptr;
};

template <typename FP = float>
class StateSpaceGB300 {
  static_assert(std::is_same<FP, float>::value,
                "the GB300 engine stores complex64 states (FP = float)");

 public:
  using fp_type = FP;

  // VectorSpaceCUDA::Vector (lib/vectorspace_cuda.h:51-82).
  class Vector {
   public:
    Vector() = delete;
    Vector(fp_type* p, unsigned n, std::shared_ptr<Context> ctx, bool owned)
        : ptr_(p), num_qubits_(n), ctx_(std::move(ctx)), owned_(owned) {}
    Vector(Vector&& o) noexcept
        : ptr_(o.ptr_), num_qubits_(o.num_qubits_), ctx_(std::move(o.ctx_)),
          owned_(o.owned_) {
      o.ptr_ = nullptr;
      o.owned_ = false;
    }
    Vector& operator=(Vector&& o) noexcept {
      if (this != &o) {
        reset();
        ptr_ = o.ptr_;
        num_qubits_ = o.num_qubits_;
        ctx_ = std::move(o.ctx_);
        owned_ = o.owned_;
        o.ptr_ = nullptr;
        o.owned_ = false;
      }
      return *this;
    }
    Vector(const Vector&) = delete;
    Vector& operator=(const Vector&) = delete;
    ~Vector() { reset(); }

    fp_type* get() { return ptr_; }
    const fp_type* get() const { return ptr_; }
    fp_type* release() {
      num_qubits_ = 0;
      owned_ = false;
      fp_type* p = ptr_;
      ptr_ = nullptr;
      return p;
    }
    unsigned num_qubits() const { return num_qubits_; }
    static constexpr bool requires_copy_to_host() { return true; }

   private:
    void reset() {
      if (owned_ && ptr_ && ctx_) qsg_state_free(ctx_->get(), ptr_);
      ptr_ = nullptr;
      owned_ = false;
    }
    fp_type* ptr_;
    unsigned num_qubits_;
    std::shared_ptr<Context> ctx_;
    bool owned_;
  };

  using State = Vector;

  // lib/statespace_cuda.h:59-70; accepted for compatibility (the engine
  // sizes its own grids).
  struct Parameter {
    unsigned num_threads = 512;
    unsigned num_dblocks = 16;
  };

  // lib/statespace.h:45-68.
  struct MeasurementResult {
    uint64_t mask;
    uint64_t bits;
    std::vector<unsigned> bitstring;
    bool valid;
  };

  explicit StateSpaceGB300(const Parameter& param = Parameter(),
                           std::shared_ptr<Context> ctx = Context::Default())
      : param_(param), ctx_(std::move(ctx)) {}

  qsg_ctx* context() const { return ctx_->get(); }
  const std::shared_ptr<Context>& shared_context() const { return ctx_; }

  // ---- vector space --------------------------------------------------------
  static uint64_t MinSize(unsigned num_qubits) { return qsg_min_size(num_qubits); }

  State Create(unsigned num_qubits) const {
    float* p = nullptr;
    int rc = qsg_state_create(ctx_->get(), num_qubits, &p);
    if (rc == QSG_ERR_OOM) return Null();
    check(rc);
    return State(p, num_qubits, ctx_, true);
  }
  // Non-owning view; `p` must hold MinSize(num_qubits) floats on the device.
  static State Create(fp_type* p, unsigned num_qubits) {
    return State(p, num_qubits, nullptr, false);
  }
  static State Null() { return State(nullptr, 0, nullptr, false); }
  static bool IsNull(const State& s) { return s.get() == nullptr; }
  void Free(fp_type* p) const { check(qsg_state_free(ctx_->get(), p)); }

  bool Copy(const State& src, State& dest) const {
    if (src.num_qubits() != dest.num_qubits()) return false;
    check(qsg_copy_d2d(ctx_->get(), dest.get(), src.get(), src.num_qubits()));
    return true;
  }
  bool Copy(const State& src, fp_type* dest) const {
    check(qsg_copy_d2h(ctx_->get(), dest, src.get(), src.num_qubits()));
    return true;
  }
  bool Copy(const fp_type* src, State& dest) const {
    check(qsg_copy_h2d(ctx_->get(), dest.get(), src, dest.num_qubits()));
    return true;
  }
  bool Copy(const fp_type* src, uint64_t size, State& dest) const {
    check(qsg_copy_h2d_partial(ctx_->get(), dest.get(), src, size,
                               dest.num_qubits()));
    return true;
  }
  void DeviceSync() const { check(qsg_ctx_sync(ctx_->get())); }

  // ---- state space ---------------------------------------------------------
  void InternalToNormalOrder(State& s) const {
    check(qsg_internal_to_normal(ctx_->get(), s.get(), s.num_qubits()));
  }
  void NormalToInternalOrder(State& s) const {
    check(qsg_normal_to_internal(ctx_->get(), s.get(), s.num_qubits()));
  }
  void SetAllZeros(State& s) const {
    check(qsg_set_all_zeros(ctx_->get(), s.get(), s.num_qubits()));
  }
  void SetStateUniform(State& s) const {
    check(qsg_set_state_uniform(ctx_->get(), s.get(), s.num_qubits()));
  }
  void SetStateZero(State& s) const {
    check(qsg_set_state_zero(ctx_->get(), s.get(), s.num_qubits()));
  }
  std::complex<fp_type> GetAmpl(const State& s, uint64_t i) const {
    float v[2];
    check(qsg_get_ampl(ctx_->get(), s.get(), s.num_qubits(), i, v));
    return {v[0], v[1]};
  }
  void SetAmpl(State& s, uint64_t i, const std::complex<fp_type>& a) const {
    SetAmpl(s, i, a.real(), a.imag());
  }
  void SetAmpl(State& s, uint64_t i, fp_type re, fp_type im) const {
    check(qsg_set_ampl(ctx_->get(), s.get(), s.num_qubits(), i, re, im));
  }
  void BulkSetAmpl(State& s, uint64_t mask, uint64_t bits,
                   const std::complex<fp_type>& v, bool exclude = false) const {
    BulkSetAmpl(s, mask, bits, v.real(), v.imag(), exclude);
  }
  void BulkSetAmpl(State& s, uint64_t mask, uint64_t bits, fp_type re,
                   fp_type im, bool exclude = false) const {
    check(qsg_bulk_set_ampl(ctx_->get(), s.get(), s.num_qubits(), mask, bits,
                            re, im, exclude ? 1 : 0));
  }
  bool Add(const State& src, State& dest) const {
    if (src.num_qubits() != dest.num_qubits()) return false;
    check(qsg_add(ctx_->get(), src.get(), dest.get(), src.num_qubits()));
    return true;
  }
  void Multiply(fp_type a, State& s) const {
    check(qsg_multiply(ctx_->get(), a, s.get(), s.num_qubits()));
  }
  std::complex<double> InnerProduct(const State& a, const State& b) const {
    if (a.num_qubits() != b.num_qubits()) return std::nan("");
    double r[2];
    check(qsg_inner_product(ctx_->get(), a.get(), b.get(), a.num_qubits(), r));
    return {r[0], r[1]};
  }
  double RealInnerProduct(const State& a, const State& b) const {
    if (a.num_qubits() != b.num_qubits()) return std::nan("");
    double r;
    check(qsg_real_inner_product(ctx_->get(), a.get(), b.get(),
                                 a.num_qubits(), &r));
    return r;
  }
  double Norm(const State& s) const {
    double r;
    check(qsg_norm(ctx_->get(), s.get(), s.num_qubits(), &r));
    return r;
  }

  // lib/statespace_cuda.h:243-312: the same uniforms as the reference
  // (std::mt19937(seed), uniform_real_distribution<DistrRealType>(0, norm),
  // sorted), CDF search on the device.  For double the library draws them
  // (the same libstdc++ algorithm); for any other DistrRealType they are
  // drawn here with the caller's std::uniform_real_distribution, in that
  // type, as the reference's GenerateRandomValues (lib/util.h:67-85) does.
  template <typename DistrRealType = double>
  std::vector<uint64_t> Sample(const State& s, uint64_t num_samples,
                               unsigned seed) const {
    std::vector<uint64_t> out(num_samples);
    if (num_samples == 0) return out;
    if (std::is_same<DistrRealType, double>::value) {
      check(qsg_sample(ctx_->get(), s.get(), s.num_qubits(), num_samples,
                       seed, out.data()));
      return out;
    }
    const DistrRealType norm = DistrRealType(Norm(s));
    std::mt19937 rgen(seed);
    std::uniform_real_distribution<DistrRealType> distr(0.0, norm);
    std::vector<DistrRealType> rs(num_samples);
    for (auto& r : rs) r = distr(rgen);
    std::sort(rs.begin(), rs.end());
    std::vector<double> r64(rs.begin(), rs.end());
    check(qsg_sample_thresholds(ctx_->get(), s.get(), s.num_qubits(),
                                num_samples, r64.data(), out.data()));
    return out;
  }

  void Collapse(const MeasurementResult& mr, State& s) const {
    check(qsg_collapse(ctx_->get(), s.get(), s.num_qubits(), mr.mask,
                       mr.bits));
  }

  std::vector<double> PartialNorms(const State& s) const {
    std::vector<double> out(qsg_num_chunks(s.num_qubits()));
    check(qsg_partial_norms(ctx_->get(), s.get(), s.num_qubits(), out.data()));
    return out;
  }

  uint64_t FindMeasuredBits(unsigned m, double r, uint64_t mask,
                            const State& s) const {
    uint64_t out;
    check(qsg_find_measured_bits(ctx_->get(), s.get(), s.num_qubits(), m, r,
                                 mask, &out));
    return out;
  }

  // lib/statespace.h:97-140.  One draw of uniform_real_distribution<double>
  // from rgen (r = u * norm, the value RandomValue(rgen, norm) returns);
  // the CDF search over the whole state runs on the device.
  template <typename RGen>
  MeasurementResult VirtualMeasure(const std::vector<unsigned>& qubits,
                                   RGen& rgen, const State& s) const {
    MeasurementResult res;
    res.valid = true;
    res.mask = 0;
    for (unsigned q : qubits) {
      if (q >= s.num_qubits()) {
        res.valid = false;
        return res;
      }
      res.mask |= uint64_t{1} << q;
    }
    std::uniform_real_distribution<double> distr(0.0, 1.0);
    const double u = distr(rgen);
    check(qsg_measure(ctx_->get(), const_cast<float*>(s.get()),
                      s.num_qubits(), res.mask, u, 0, &res.bits));
    res.bitstring.reserve(qubits.size());
    for (unsigned q : qubits) res.bitstring.push_back((res.bits >> q) & 1);
    return res;
  }

  // lib/statespace.h:84-95.
  template <typename RGen>
  MeasurementResult Measure(const std::vector<unsigned>& qubits, RGen& rgen,
                            State& s) const {
    auto res = VirtualMeasure(qubits, rgen, s);
    if (res.valid) Collapse(res, s);
    return res;
  }

 private:
  Parameter param_;
  std::shared_ptr<Context> ctx_;
};

}  // namespace qsim_gb300

#endif  // QSIM_GB300_STATESPACE_GB300_H_
