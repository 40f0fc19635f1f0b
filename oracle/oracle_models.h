/*
 * oracle_models.h -- host versions of the models the GPU library ships,
 * for the oracle only (test infrastructure, never linked into the product).
 *
 * Each rate function evaluates the same C expression, in the same order,
 * as the reference model file it names, so that IEEE double arithmetic
 * gives the same bits.  The device versions live in
 * siminf_gb300/csrc/siminf_models.cuh.
 */
#ifndef ORACLE_MODELS_H
#define ORACLE_MODELS_H

typedef double (*oracle_trfun)(const int *u, const double *v,
                               const double *ldata, const double *gdata,
                               double t);
typedef int (*oracle_ptsfun)(double *v_new, const int *u, const double *v,
                             const double *ldata, const double *gdata,
                             int node, double t);

typedef struct oracle_model {
    const char *name;
    int Nc, Nt, Nd;
    oracle_trfun tr[32];
    oracle_ptsfun pts;
} oracle_model;

const oracle_model *oracle_model_lookup(const char *name);

#endif
