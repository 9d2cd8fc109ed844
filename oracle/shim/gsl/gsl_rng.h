/* Stand-in for the GSL random-number interface the reference calls
   (gsl_rng_alloc/set/uniform/free with gsl_rng_ranlxd1), backed by the
   oracle's RANLUX restatement.  Test infrastructure only. */
#ifndef AAR_SHIM_GSL_RNG_H
#define AAR_SHIM_GSL_RNG_H
#include "aar_oracle.h"
typedef struct { int luxury; } gsl_rng_type;
typedef struct { orc_rlx s; } gsl_rng;
extern const gsl_rng_type *gsl_rng_ranlxd1;
gsl_rng *gsl_rng_alloc(const gsl_rng_type *t);
void gsl_rng_set(gsl_rng *r, unsigned long seed);
double gsl_rng_uniform(gsl_rng *r);
void gsl_rng_free(gsl_rng *r);
#endif
