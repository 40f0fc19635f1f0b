/*
 * siminf_launch.h -- per-model kernel launchers (defined in
 * siminf_kernels.cu, called by the host planner in siminf_capi.cpp).
 */
#ifndef SIMINF_LAUNCH_H
#define SIMINF_LAUNCH_H

#include <cuda_runtime.h>
#include "siminf_plan.h"

namespace siminf {

struct Launchers {
    int Nc, Nt, Nd;
    int Ngd;            /* gdata entries the model reads */
    bool pts_local;     /* post-time-step reads only its own node */
    bool time_invariant;    /* rates ignore t (the heavy part of the work queue applies) */
    cudaError_t (*init)(const DevState &s, double tt0, cudaStream_t st);
    cudaError_t (*horizon)(const DevState &s, const DayInfo *days, int ndays, cudaStream_t st);
    /* the first pass of a two-pass day (k_quick); ssa_e1 is the second */
    cudaError_t (*quick)(const DevState &s, int day, double tt, double next, cudaStream_t st);
    cudaError_t (*ssa_e1)(const DevState &s, int day, double tt, double next, cudaStream_t st);
    cudaError_t (*e2_wave)(const DevState &s, const E2Rec *ev, int count, int day, double tt,
                           cudaStream_t st);
    cudaError_t (*pts_store)(const DevState &s, int day, double tt, int c0, int c1,
                             const double *v_in, double *v_out, cudaStream_t st);
    /* the all-events method's initialisation, day and day end */
    cudaError_t (*aem_init)(const DevState &s, double tt0, cudaStream_t st);
    cudaError_t (*aem_day)(const DevState &s, int day, double tt, double next, cudaStream_t st);
    cudaError_t (*aem_pts)(const DevState &s, int day, double tt, int c0, int c1,
                           const double *v_in, double *v_out, cudaStream_t st);
    /* a day's last, small wavefronts in one launch */
    cudaError_t (*e2_tail)(const DevState &s, const E2Rec *ev, const E2Tail &tail, int day,
                           double tt, cudaStream_t st);
};

/* Particle-filter kernels (model independent). */
cudaError_t pf_weights(const int *U, int tlen, int Nn, int Nc, int Np, const int *obs_row,
                       int obs_c, const double *lfact, int tablen, double logp, double logq,
                       double *w, cudaStream_t st, const int *interval = nullptr);
cudaError_t pf_finalize(double *w, int Np, double log_np, double *loglik, double *ess, int i,
                        uint64_t seed, uint64_t sid, int *anc, int *anc_out, cudaStream_t st,
                        int *interval = nullptr, const uint64_t *seed_dev = nullptr);
cudaError_t pf_gather(const int *U, const double *V, int tlen, long long nu, long long nv,
                      const int *anc, int Np, int *u0, double *v0, cudaStream_t st);

/* The launcher table of a built-in device model, or nullptr. */
const Launchers *launchers_for(const char *name);

/* A device model compiled from model C code into a library of its own
 * (siminf_gb300/devmodel.py) exports its launcher table and this version
 * as siminf_model_launchers() and siminf_model_abi(); the loader compares
 * the version with its own, which changes whenever the table or the device
 * state it passes changes layout. */
#define SIMINF_MODEL_ABI \
    (20261204 + (int) sizeof(siminf::DevState) + (int) sizeof(siminf::Launchers))

}  // namespace siminf

#endif
