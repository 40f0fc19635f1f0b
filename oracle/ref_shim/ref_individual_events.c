/*
 * ref_individual_events.c -- the reference's cleaning of individual-based
 * event data (src/misc/SimInf_individual_events.c), compiled unmodified by
 * including it (oracle test infrastructure).
 *
 * The few R API calls the file makes act on a plain (pointer, length)
 * record here: INTEGER/LOGICAL give the pointer, XLENGTH the length,
 * Rf_allocVector hands out the caller's keep buffer, R_alloc is malloc
 * (freed by the wrapper), and Rf_error formats its message and jumps back
 * to ref_individual_events(), which returns -1 with the message.
 */
#include <setjmp.h>
#include <stdarg.h>
#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define LONG_VECTOR_SUPPORT 1
#include "SimInf.h"
#include "SimInf_internal.h"

int shim_configure(uint64_t seed, int Nn, int Nthread, int Nrep, int threads);

typedef ptrdiff_t R_xlen_t;
typedef struct {
    void *data;
    ptrdiff_t len;
} shim_vec;

static jmp_buf shim_jump;
static char shim_msg[256];
static shim_vec shim_keep;
static void *shim_scratch[8];
static int shim_nscratch;

static void shim_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(shim_msg, sizeof(shim_msg), fmt, ap);
    va_end(ap);
    longjmp(shim_jump, 1);
}

static char *shim_alloc(size_t n, int size)
{
    void *p = calloc(n > 0 ? n : 1, (size_t) size);
    if (!p || shim_nscratch == 8)
        shim_error("out of memory");
    shim_scratch[shim_nscratch++] = p;
    return (char *) p;
}

int SimInf_set_num_threads(int threads)
{
    (void) threads;
    return SimInf_num_threads();
}

#define LGLSXP 10
#define INTEGER(x) ((int *) ((shim_vec *) (x))->data)
#define LOGICAL(x) ((int *) ((shim_vec *) (x))->data)
#define XLENGTH(x) (((shim_vec *) (x))->len)
#define Rf_allocVector(type, n) ((void) (type), (void) (n), (SEXP) &shim_keep)
#define R_alloc(n, size) shim_alloc((size_t) (n), (int) (size))
#define PROTECT(x) (x)
#define UNPROTECT(n) ((void) (n))
#define Rf_error shim_error

#include "misc/SimInf_individual_events.c"

/* keep[0 .. len) for the sorted, de-duplicated events; returns 0, or -1
 * with the reference's message in msg (msg_len bytes). */
int ref_individual_events(long long len, int *id, int *event, int *time, int *node, int *dest,
                          int *keep, int threads, char *msg, int msg_len)
{
    shim_vec v_id = {id, len}, v_event = {event, len}, v_time = {time, len},
             v_node = {node, len}, v_dest = {dest, len};
    shim_keep.data = keep;
    shim_keep.len = len;
    shim_nscratch = 0;
    shim_msg[0] = 0;
    if (shim_configure(0, 1, 1, 1, threads))
        return -2;
    int rc = 0;
    if (setjmp(shim_jump) == 0)
        SimInf_individual_events(&v_id, &v_event, &v_time, &v_node, &v_dest);
    else
        rc = -1;
    for (int k = 0; k < shim_nscratch; k++)
        free(shim_scratch[k]);
    shim_nscratch = 0;
    if (msg && msg_len > 0)
        snprintf(msg, (size_t) msg_len, "%s", shim_msg);
    return rc;
}
