// unitary_gb300.h — header-only unitary space and unitary calculator over
// the GB300 engine's C ABI.
//
// Drop-in for qsim's UnitarySpaceBasic (lib/unitaryspace_basic.h:34-100)
// and UnitaryCalculatorBasic (lib/unitary_calculator_basic.h:33-124):
// the same member names, signatures and storage convention (entry (i, j) at
// complex index i * 2^n + j; a gate mixes every row's entries over the
// column bits at its qubits), so qsim's gate_appl.h templates
// (ApplyGate(calculator, gate, unitary), lib/gate_appl.h) run on the GPU:
//
//   qsim_gb300::UnitaryCalculatorGB300<float> calc;
//   qsim_gb300::UnitarySpaceGB300<float> us;
//   auto u = us.CreateUnitary(n);
//   us.SetIdentity(u);
//   for (const auto& gate : circuit.gates) qsim::ApplyGate(calc, gate, u);
#ifndef QSIM_GB300_UNITARY_GB300_H_
#define QSIM_GB300_UNITARY_GB300_H_

#include <complex>
#include <cstdint>
#include <memory>
#include <vector>

#include "../qsim_gb300.h"
#include "statespace_gb300.h"

namespace qsim_gb300 {

template <typename FP = float>
class UnitarySpaceGB300 {
  static_assert(std::is_same<FP, float>::value,
                "the GB300 engine stores complex64 unitaries (FP = float)");

 public:
  using fp_type = FP;
  // Owning device buffer with the reference's Unitary interface (get(),
  // release(), num_qubits()); num_qubits() is the unitary's n.
  using Unitary = typename StateSpaceGB300<FP>::Vector;

  explicit UnitarySpaceGB300(std::shared_ptr<Context> ctx = Context::Default())
      : ctx_(std::move(ctx)) {}

  // lib/unitaryspace.h:41-55 and lib/unitaryspace_basic.h:45-51.
  Unitary CreateUnitary(unsigned num_qubits) const {
    float* p = nullptr;
    const int rc = qsg_unitary_create(ctx_->get(), num_qubits, &p);
    if (rc == QSG_ERR_OOM) return NullUnitary();
    check(rc);
    return Unitary(p, num_qubits, ctx_, true);
  }
  Unitary CreateUnitary(fp_type* p, unsigned num_qubits) const {
    return Unitary(p, num_qubits, ctx_, false);
  }
  Unitary NullUnitary() const { return Unitary(nullptr, 0, ctx_, false); }
  static bool IsNull(const Unitary& u) { return u.get() == nullptr; }
  static uint64_t Size(unsigned num_qubits) { return uint64_t{1} << num_qubits; }
  static uint64_t MinRowSize(unsigned num_qubits) {
    return 2 * (uint64_t{1} << num_qubits);
  }
  static uint64_t MinSize(unsigned num_qubits) {
    return qsg_unitary_min_size(num_qubits);
  }
  void CopyUnitary(const Unitary& src, Unitary& dest) const {
    check(qsg_copy_d2d(ctx_->get(), dest.get(), src.get(),
                       2 * src.num_qubits()));
  }

  // lib/unitaryspace_basic.h:53-96.
  void SetAllZeros(Unitary& u) const {
    check(qsg_unitary_set_all_zeros(ctx_->get(), u.get(), u.num_qubits()));
  }
  void SetIdentity(Unitary& u) const {
    check(qsg_unitary_set_identity(ctx_->get(), u.get(), u.num_qubits()));
  }
  std::complex<fp_type> GetEntry(const Unitary& u, uint64_t i,
                                 uint64_t j) const {
    float v[2];
    check(qsg_unitary_get_entry(ctx_->get(), u.get(), u.num_qubits(), i, j, v));
    return {v[0], v[1]};
  }
  void SetEntry(Unitary& u, uint64_t i, uint64_t j,
                const std::complex<fp_type>& a) const {
    SetEntry(u, i, j, a.real(), a.imag());
  }
  void SetEntry(Unitary& u, uint64_t i, uint64_t j, fp_type re,
                fp_type im) const {
    check(qsg_unitary_set_entry(ctx_->get(), u.get(), u.num_qubits(), i, j,
                                re, im));
  }

  const std::shared_ptr<Context>& context() const { return ctx_; }

 private:
  std::shared_ptr<Context> ctx_;
};

template <typename FP = float>
class UnitaryCalculatorGB300 {
 public:
  using UnitarySpace = UnitarySpaceGB300<FP>;
  using Unitary = typename UnitarySpace::Unitary;
  using fp_type = typename UnitarySpace::fp_type;
  using StateSpace = UnitarySpace;
  using State = Unitary;

  explicit UnitaryCalculatorGB300(
      std::shared_ptr<Context> ctx = Context::Default())
      : ctx_(std::move(ctx)) {}

  // lib/unitary_calculator_basic.h:51-79.
  void ApplyGate(const std::vector<unsigned>& qs, const fp_type* matrix,
                 Unitary& u) const {
    check(qsg_unitary_apply_gate(ctx_->get(), u.get(), u.num_qubits(),
                                 qs.data(), unsigned(qs.size()), matrix));
  }

  // lib/unitary_calculator_basic.h:88-117.
  void ApplyControlledGate(const std::vector<unsigned>& qs,
                           const std::vector<unsigned>& cqs, uint64_t cvals,
                           const fp_type* matrix, Unitary& u) const {
    check(qsg_unitary_apply_controlled_gate(
        ctx_->get(), u.get(), u.num_qubits(), qs.data(), unsigned(qs.size()),
        cqs.data(), unsigned(cqs.size()), cvals, matrix));
  }

  // lib/unitary_calculator_basic.h:120-122.
  static unsigned SIMDRegisterSize() { return 1; }

 private:
  std::shared_ptr<Context> ctx_;
};

}  // namespace qsim_gb300

#endif  // QSIM_GB300_UNITARY_GB300_H_
