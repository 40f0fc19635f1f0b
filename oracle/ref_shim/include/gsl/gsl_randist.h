/* Stub of gsl/gsl_randist.h (oracle test infrastructure): binomial and
 * hypergeometric draws from the per-node stream, see gsl_rng.h. */
#ifndef SHIM_GSL_RANDIST_H
#define SHIM_GSL_RANDIST_H
#include "gsl_rng.h"
unsigned int shim_binomial(const gsl_rng *r, double p, unsigned int n, long node);
unsigned int shim_hypergeometric(const gsl_rng *r, unsigned int n1, unsigned int n2,
                                 unsigned int t, long node);
#define gsl_ran_binomial(r, p, n) shim_binomial((r), (p), (n), (long) (node))
#define gsl_ran_hypergeometric(r, n1, n2, t) shim_hypergeometric((r), (n1), (n2), (t), (long) (node))
#endif
