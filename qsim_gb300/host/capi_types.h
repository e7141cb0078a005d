// Definitions of the C ABI's opaque handles shared by the host translation
// units.
#pragma once

#include "engine.h"
#include "qsim_gb300.h"

struct qsg_circuit {
  qsg::host::Circuit c;
};

namespace qsg {
namespace host {

// qsg_fuse_options -> FuseOptions (zeros select the defaults; null: all
// defaults).  Returns false for a max_fused_size outside 1..6.
bool fuse_options_from(const qsg_fuse_options* o, FuseOptions* out);

}  // namespace host
}  // namespace qsg
