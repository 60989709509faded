/* Oracle test infrastructure: the SOUFFLE sources include this header but call
   nothing from it on the paths the checker exercises. */
#include <gsl/gsl_rng.h>
