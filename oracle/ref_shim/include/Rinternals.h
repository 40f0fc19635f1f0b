/* Stub of Rinternals.h (oracle test infrastructure): only what the solver
 * sources and the model files reference. */
#ifndef SHIM_RINTERNALS_H
#define SHIM_RINTERNALS_H
#include "R.h"
#include <math.h>
typedef void *SEXP;
typedef void *(*DL_FUNC)(void);
#define R_FINITE(x) isfinite(x)
#endif
