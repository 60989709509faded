/* Oracle test infrastructure: a stand-in for the handful of GSL RNG names the
   SOUFFLE sources call.  GSL draws only initial velocities and Brownian noise;
   both are off the checked path (states are injected through restart files),
   so this is a plain std::mt19937 with uniform = draw / 2^32. */
#ifndef ORACLE_SHIM_GSL_RNG_H
#define ORACLE_SHIM_GSL_RNG_H
#include <random>

struct gsl_rng_type {
  int unused;
};
struct gsl_rng {
  std::mt19937 eng;
};

static const gsl_rng_type oracle_shim_mt_type = {0};
static const gsl_rng_type* gsl_rng_default = &oracle_shim_mt_type;

inline gsl_rng* gsl_rng_alloc(const gsl_rng_type*) { return new gsl_rng(); }
inline void gsl_rng_free(gsl_rng* r) { delete r; }
inline const gsl_rng_type* gsl_rng_env_setup(void) { return gsl_rng_default; }
inline void gsl_rng_set(gsl_rng* r, unsigned long s) {
  r->eng.seed(static_cast<std::mt19937::result_type>(s));
}
inline double gsl_rng_uniform(gsl_rng* r) { return r->eng() / 4294967296.0; }

#endif
