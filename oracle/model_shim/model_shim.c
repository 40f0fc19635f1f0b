/*
 * model_shim.c -- the R and SimInf symbols model C code needs when it is
 * built on the host without R (oracle test infrastructure): mparse output
 * (R/C-generator.R) or a hand-written model file compiled by gcc as R CMD
 * SHLIB would compile it, so that the oracle and the reference's solver
 * can run the model's own trFun/ptsFun.
 *
 * The model's run function hands tr_fun and its post-time-step function to
 * SimInf_run, which it finds through R_GetCCallable("SimInf", "SimInf_run")
 * (mparse output) or calls directly (model files); here SimInf_run only
 * records the two, and shim_model_capture() runs the run function to get
 * them.  The helpers SimInf.h exports to model code are restated from
 * src/misc/SimInf_forward_euler_linear_decay.c:57-93 and
 * src/misc/SimInf_local_spread.c:43-71.
 */
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include "SimInf.h"

static TRFun g_tr[32];
static PTSFun g_pts;
static int g_nt;

SEXP SimInf_run(SEXP model, SEXP solver, TRFun *tr_fun, PTSFun pts_fun)
{
    (void) model;
    (void) solver;
    for (int k = 0; k < g_nt && k < 32; k++)
        g_tr[k] = tr_fun[k];
    g_pts = pts_fun;
    return NULL;
}

DL_FUNC R_GetCCallable(const char *package, const char *name)
{
    (void) package;
    (void) name;
    return (DL_FUNC) &SimInf_run;
}

int R_registerRoutines(DllInfo *info, const void *c, const R_CallMethodDef *call,
                       const void *f, const void *e)
{
    (void) info; (void) c; (void) call; (void) f; (void) e;
    return 1;
}

int R_useDynamicSymbols(DllInfo *info, int value) { (void) info; return value; }
int R_forceSymbols(DllInfo *info, int value) { (void) info; return value; }

void Rf_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vfprintf(stderr, fmt, ap);
    va_end(ap);
    abort();
}

int shim_model_capture(SEXP (*run)(SEXP, SEXP), int nt, TRFun *tr, PTSFun *pts)
{
    if (nt < 1 || nt > 32)
        return -1;
    g_nt = nt;
    g_pts = NULL;
    run(NULL, NULL);
    for (int k = 0; k < nt; k++)
        tr[k] = g_tr[k];
    *pts = g_pts;
    return g_pts ? 0 : -1;
}

double SimInf_forward_euler_linear_decay(double phi, int day, int end_t1, int end_t2,
                                         int end_t3, int end_t4, double beta_t1,
                                         double beta_t2, double beta_t3, double beta_t4)
{
    if (day < end_t2) {
        if (day < end_t1) {
            if (end_t1 < end_t4)
                return phi * (1.0 - beta_t1);
            if (day < end_t4) {
                if (end_t4 < end_t3)
                    return phi * (1.0 - beta_t4);
                if (day < end_t3)
                    return phi * (1.0 - beta_t3);
                return phi * (1.0 - beta_t4);
            }
            return phi * (1.0 - beta_t1);
        }
        return phi * (1.0 - beta_t2);
    }
    if (end_t3 < end_t1 || day < end_t3)
        return phi * (1.0 - beta_t3);
    if (end_t4 < end_t1 || day < end_t4)
        return phi * (1.0 - beta_t4);
    return phi * (1.0 - beta_t1);
}

double SimInf_local_spread(const double *neighbors, const double *phi, const int *u,
                           const double N_i, const double phi_i, const int Nc,
                           const double D)
{
    double ls = 0.0;
    const double phi_i_N_i = phi_i * N_i;
    for (int j = (int) neighbors[0]; j >= 0; j = (int) neighbors[0]) {
        double N_j = 0;
        for (int k = j * Nc; k < (j + 1) * Nc; k++)
            N_j += u[k];
        if (N_j > 0.0)
            ls += ((phi[j] * N_j - phi_i_N_i) * D) / (N_i * neighbors[1]);
        neighbors += 2;
    }
    return ls;
}
