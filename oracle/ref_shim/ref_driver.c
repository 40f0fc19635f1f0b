/*
 * ref_driver.c -- fills the reference's SimInf_solver_args
 * (src/SimInf_internal.h:44-200) from the layout-identical
 * siminf_gpu_solver_args and calls the reference solvers directly,
 * bypassing SimInf_run's SEXP marshalling (src/SimInf.c:224-409).
 * Oracle test infrastructure only.
 */
#include <string.h>
#include "SimInf.h"
#include "SimInf_internal.h"
#include "../../include/siminf_gb300.h"
#include "../oracle_models.h"

int shim_configure(uint64_t seed, int Nn, int Nthread, int Nrep, int threads);
void shim_release(void);

extern TRFun ref_SIR_tr[], ref_SEIR_tr[], ref_SIS_tr[], ref_SISe_tr[], ref_SISe3_tr[];
extern PTSFun ref_SIR_pts, ref_SEIR_pts, ref_SIS_pts, ref_SISe_pts, ref_SISe3_pts;
extern TRFun ref_SISe_sp_tr[], ref_SISe3_sp_tr[];
extern PTSFun ref_SISe_sp_pts, ref_SISe3_sp_pts;

_Static_assert(sizeof(SimInf_solver_args) == sizeof(siminf_gpu_solver_args),
               "siminf_gpu_solver_args must stay layout-identical to SimInf_solver_args");

int ref_run(const siminf_gpu_solver_args *ga, const char *model, int threads)
{
    SimInf_solver_args a;
    TRFun tr[32];
    PTSFun pts;
    int Nt = ga->Nt;

    if (strcmp(model, "SIR") == 0) {
        memcpy(tr, ref_SIR_tr, 2 * sizeof(TRFun)); pts = ref_SIR_pts;
    } else if (strcmp(model, "SEIR") == 0) {
        memcpy(tr, ref_SEIR_tr, 3 * sizeof(TRFun)); pts = ref_SEIR_pts;
    } else if (strcmp(model, "SIS") == 0) {
        memcpy(tr, ref_SIS_tr, 2 * sizeof(TRFun)); pts = ref_SIS_pts;
    } else if (strcmp(model, "SISe") == 0) {
        memcpy(tr, ref_SISe_tr, 2 * sizeof(TRFun)); pts = ref_SISe_pts;
    } else if (strcmp(model, "SISe3") == 0) {
        memcpy(tr, ref_SISe3_tr, 6 * sizeof(TRFun)); pts = ref_SISe3_pts;
    } else if (strcmp(model, "SISe_sp") == 0) {
        memcpy(tr, ref_SISe_sp_tr, 2 * sizeof(TRFun)); pts = ref_SISe_sp_pts;
    } else if (strcmp(model, "SISe3_sp") == 0) {
        memcpy(tr, ref_SISe3_sp_tr, 6 * sizeof(TRFun)); pts = ref_SISe3_sp_pts;
    } else {
        /* mparse models have no source in the reference tree: use the
         * oracle's host versions of the generated code. */
        const oracle_model *m = oracle_model_lookup(model);
        if (!m)
            return -32;
        for (int j = 0; j < Nt && j < 32; j++)
            tr[j] = (TRFun) m->tr[j];
        pts = (PTSFun) m->pts;
    }

    memcpy(&a, ga, sizeof(a));
    a.tr_fun = tr;
    a.pts_fun = pts;
    if (threads < 1)
        threads = 1;
    if (a.Nrep > 1) {
        a.Nthread = a.Nrep;
    } else {
        a.Nrep = 1;
        a.Nthread = threads < a.Nn ? threads : a.Nn;
        if (a.Nthread < 1)
            a.Nthread = 1;
    }
    if (shim_configure((uint64_t) a.seed, a.Nn, a.Nthread, a.Nrep, threads))
        return -2;
    int err;
    /* the dispatch of src/SimInf.c:383-399 */
    if (a.solver == 1)            /* aem: one replicate */
        err = a.Nrep > 1 ? -19 : SimInf_run_solver_aem(&a);
    else if (a.Nrep > 1)
        err = a.crn == 1 ? SimInf_run_solver_mssm_crn(&a) : SimInf_run_solver_mssm(&a);
    else
        err = SimInf_run_solver_ssm(&a);
    shim_release();
    return err;
}

/* The model files' <Model>_run glue calls SimInf_run; it is never called
 * here, but the symbol must resolve. */
SEXP SimInf_run(SEXP model, SEXP solver, TRFun *tr_fun, PTSFun pts_fun)
{
    (void) model; (void) solver; (void) tr_fun; (void) pts_fun;
    return NULL;
}
