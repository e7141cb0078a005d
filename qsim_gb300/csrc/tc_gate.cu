// Tensor-core path for fused gates of k = 5, 6 qubits (placeholder until the
// tcgen05 kernel lands: reports the path as unsupported).

#include "common.cuh"
#include "internal.h"

namespace qsg {

size_t tc_operand_bytes(unsigned k) { return size_t(2) << (2 * k + 2); }

void tc_build_operands(unsigned, const float*, void*) {}

int apply_gate_tc(qsg_ctx*, float*, unsigned, const unsigned*, unsigned,
                  const float*, const void*) {
  set_error("the tensor-core path is not available in this build");
  return QSG_ERR_UNSUPPORTED;
}

void set_error_msg(const char* msg) { set_error("%s", msg); }

}  // namespace qsg
