/* Stub of R.h for compiling the reference solver sources without R
 * (oracle test infrastructure).  Console output goes to stderr only when
 * SIMINF_REF_VERBOSE is set. */
#ifndef SHIM_R_H
#define SHIM_R_H
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <limits.h>
#include <stddef.h>
void REprintf(const char *fmt, ...);
void Rprintf(const char *fmt, ...);
void R_FlushConsole(void);
#endif
