/*
 * ref_particle_filter.c -- the reference's systematic resampling
 * (src/misc/SimInf_particle_filter.c), compiled unmodified by including it
 * (oracle test infrastructure).
 *
 * The R API calls of the file act on a plain (pointer, length) record
 * here: REAL/INTEGER give the pointer, XLENGTH the length, Rf_allocVector
 * hands out the caller's output buffer, unif_rand() returns the uniform the
 * caller passes (R's generator state calls do nothing), and Rf_error
 * formats its message and jumps back to the wrapper, which returns -1 with
 * it.
 */
#include <setjmp.h>
#include <stdarg.h>
#include <stddef.h>
#include <stdio.h>
#include <string.h>

#include "R.h"
#include "Rinternals.h"

typedef ptrdiff_t R_xlen_t;
typedef struct {
    void *data;
    ptrdiff_t len;
} shim_vec;

static jmp_buf shim_jump;
static char shim_msg[256];
static shim_vec shim_out;
static double shim_unif;

static void shim_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(shim_msg, sizeof(shim_msg), fmt, ap);
    va_end(ap);
    longjmp(shim_jump, 1);
}

#define INTSXP 13
#define REAL(x) ((double *) ((shim_vec *) (x))->data)
#define INTEGER(x) ((int *) ((shim_vec *) (x))->data)
#define XLENGTH(x) (((shim_vec *) (x))->len)
#define Rf_allocVector(type, n) ((void) (type), (void) (n), (SEXP) &shim_out)
#define Rf_allocMatrix(type, r, c) ((void) (type), (void) (r), (void) (c), (SEXP) &shim_out)
#define PROTECT(x) (x)
#define UNPROTECT(n) ((void) (n))
#define GetRNGstate() ((void) 0)
#define PutRNGstate() ((void) 0)
#define unif_rand() (shim_unif)
#define Rf_error shim_error

#include "misc/SimInf_particle_filter.c"

/* SimInf_systematic_resampling on w[0 .. n) with the uniform unif: idx
 * receives the one-based ancestors.  The reference's search may read one
 * weight past the end (it stops on u > the running sum, not on j); the
 * caller's w must hold one readable element more.  Returns 0, or -1 with
 * the reference's message in msg. */
int ref_systematic_resampling(double *w, long long n, double unif, int *idx, char *msg,
                              int msg_len)
{
    shim_vec v_w = {w, n};
    shim_out.data = idx;
    shim_out.len = n;
    shim_unif = unif;
    shim_msg[0] = 0;
    int rc = 0;
    if (setjmp(shim_jump) == 0)
        SimInf_systematic_resampling(&v_w);
    else
        rc = -1;
    if (msg && msg_len > 0)
        snprintf(msg, (size_t) msg_len, "%s", shim_msg);
    return rc;
}
