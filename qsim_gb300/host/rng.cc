// Host random numbers with the reference's generator conventions:
// std::mt19937 and uniform_real_distribution<double> (lib/util.h:61-85,
// lib/qtrajectory.h:268-302).  Exposed through the C ABI so Python callers
// and the C++ adapters draw the same streams as the reference.

#include <algorithm>
#include <random>

#include "qsim_gb300.h"

struct qsg_rng {
  std::mt19937 g;
};

extern "C" {

qsg_rng* qsg_rng_create(unsigned seed) { return new qsg_rng{std::mt19937(seed)}; }

void qsg_rng_destroy(qsg_rng* r) { delete r; }

uint32_t qsg_rng_next_u32(qsg_rng* r) { return r->g(); }

double qsg_rng_uniform(qsg_rng* r, double max_value) {
  std::uniform_real_distribution<double> d(0.0, max_value);
  return d(r->g);
}

void qsg_generate_random_values(uint64_t num, unsigned seed, double max_value,
                                double* out) {
  std::mt19937 g(seed);
  std::uniform_real_distribution<double> d(0.0, max_value);
  for (uint64_t i = 0; i < num; ++i) out[i] = d(g);
  std::sort(out, out + num);
}

}  // extern "C"
