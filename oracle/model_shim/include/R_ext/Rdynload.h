/* Stub of R_ext/Rdynload.h for building model C code on the host without
 * R (oracle test infrastructure): the names the generated run function
 * and registration code use.  R_GetCCallable("SimInf", "SimInf_run")
 * returns the capture function of model_shim.c. */
#ifndef SHIM_RDYNLOAD_H
#define SHIM_RDYNLOAD_H
#include <stddef.h>
typedef void *SEXP;
typedef struct DllInfo DllInfo;
typedef void *(*DL_FUNC)(void);
typedef struct {
    const char *name;
    DL_FUNC fun;
    int numArgs;
} R_CallMethodDef;
#ifndef TRUE
#define TRUE 1
#define FALSE 0
#endif
DL_FUNC R_GetCCallable(const char *package, const char *name);
int R_registerRoutines(DllInfo *info, const void *c, const R_CallMethodDef *call,
                       const void *f, const void *e);
int R_useDynamicSymbols(DllInfo *info, int value);
int R_forceSymbols(DllInfo *info, int value);
void Rf_error(const char *fmt, ...);
#endif
