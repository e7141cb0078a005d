// Definitions of the C ABI's opaque handles shared by the host translation
// units.
#pragma once

#include "engine.h"

struct qsg_circuit {
  qsg::host::Circuit c;
};
