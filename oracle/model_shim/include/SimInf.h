/* Host stand-in of the reference's inst/include/SimInf.h for building
 * model C code without R (oracle test infrastructure): the macro, error
 * code and function-type names model code uses, with the reference's
 * values, and the two helpers it exports to model code. */
#ifndef SHIM_SIMINF_H
#define SHIM_SIMINF_H
#include <math.h>
#include <R_ext/Rdynload.h>
#define SIMINF_UNUSED(x) ((void) (x))
#define SIMINF_STR(name) #name
#define SIMINF_CALLDEF(name, n) {SIMINF_STR(name), (DL_FUNC) &(name), (n)}
#define R_FINITE(x) isfinite(x)
enum {
    SIMINF_ERR_NEGATIVE_STATE = -1, SIMINF_ERR_ALLOC_MEMORY_BUFFER = -2,
    SIMINF_UNDEFINED_EVENT = -3, SIMINF_INVALID_EDGE_PROBABILITY = -4,
    SIMINF_ERR_V_IS_NOT_FINITE = -7, SIMINF_ERR_SAMPLE_SELECT = -8,
    SIMINF_ERR_INVALID_MODEL = -9, SIMINF_ERR_V_IS_NEGATIVE = -10,
    SIMINF_ERR_INVALID_RATE = -11
};
typedef double (*TRFun)(const int *u, const double *v, const double *ldata,
                        const double *gdata, double t);
typedef int (*PTSFun)(double *v_new, const int *u, const double *v, const double *ldata,
                      const double *gdata, int node, double t);
SEXP SimInf_run(SEXP model, SEXP solver, TRFun *tr_fun, PTSFun pts_fun);
double SimInf_forward_euler_linear_decay(double phi, int day, int end_t1, int end_t2,
                                         int end_t3, int end_t4, double beta_t1,
                                         double beta_t2, double beta_t3, double beta_t4);
double SimInf_local_spread(const double *neighbors, const double *phi, const int *u,
                           const double N_i, const double phi_i, const int Nc,
                           const double D);
#endif
