/*
 * siminf_model_code.h -- what model C code written for SimInf may use, for
 * that code compiled as device functions (siminf_gb300/devmodel.py).
 *
 * Model files (mparse output, R/C-generator.R:204-297, and hand-written
 * models like src/models/SISe_sp.c) include the reference's
 * inst/include/SimInf.h and R's headers.  Compiled for the device they get
 * this header instead: the same macro and error-code names with the same
 * values (inst/include/SimInf.h:61-89), the TRFun/PTSFun types
 * (:92-107), R_FINITE, and device versions of the two helpers SimInf.h
 * exports to model code, SimInf_forward_euler_linear_decay (:148-158) and
 * SimInf_local_spread (:169-176), with the reference's signatures.
 */
#ifndef SIMINF_MODEL_CODE_H
#define SIMINF_MODEL_CODE_H

#include <math.h>

#include "siminf_kernels.cuh"

#define SIMINF_UNUSED(x) ((void) (x))
#define R_FINITE(x) isfinite(x)
#define attribute_hidden

typedef enum {
    SIMINF_ERR_NEGATIVE_STATE = -1,
    SIMINF_ERR_ALLOC_MEMORY_BUFFER = -2,
    SIMINF_UNDEFINED_EVENT = -3,
    SIMINF_INVALID_EDGE_PROBABILITY = -4,
    SIMINF_ERR_V_IS_NOT_FINITE = -7,
    SIMINF_ERR_SAMPLE_SELECT = -8,
    SIMINF_ERR_INVALID_MODEL = -9,
    SIMINF_ERR_V_IS_NEGATIVE = -10,
    SIMINF_ERR_INVALID_RATE = -11,
    SIMINF_ERR_UNKNOWN_SOLVER = -12,
    SIMINF_ERR_DEST_OUT_OF_BOUNDS = -13,
    SIMINF_ERR_NODE_OUT_OF_BOUNDS = -14,
    SIMINF_ERR_EVENTS_N = -15,
    SIMINF_ERR_EVENT_SHIFT = -16,
    SIMINF_ERR_SHIFT_OUT_OF_BOUNDS = -17,
    SIMINF_ERR_INVALID_PROPORTION = -18,
    SIMINF_ERR_AEM_REPLICATED_MODEL = -19,
    SIMINF_ERR_SPARSE_MODEL = -20,
    SIMINF_ERR_INVALID_OPTIONS = -21,
    SIMINF_ERR_INVALID_SEED = -22,
    SIMINF_ERR_INVALID_CRN = -23,
    SIMINF_ERR_INVALID_RNG_TYPE = -24
} SimInf_error_code;

typedef double (*TRFun)(const int *u, const double *v, const double *ldata,
                        const double *gdata, double t);
typedef int (*PTSFun)(double *v_new, const int *u, const double *v, const double *ldata,
                      const double *gdata, int node, double t);

__device__ __forceinline__ double SimInf_forward_euler_linear_decay(
    double phi, int day, int end_t1, int end_t2, int end_t3, int end_t4, double beta_t1,
    double beta_t2, double beta_t3, double beta_t4)
{
    return siminf::forward_euler_linear_decay(phi, day, end_t1, end_t2, end_t3, end_t4, beta_t1,
                                              beta_t2, beta_t3, beta_t4);
}

__device__ __forceinline__ double SimInf_local_spread(const double *neighbors, const double *phi,
                                                      const int *u, const double N_i,
                                                      const double phi_i, const int Nc,
                                                      const double D)
{
    return siminf::local_spread(neighbors, phi, u, N_i, phi_i, Nc, D);
}

#endif
