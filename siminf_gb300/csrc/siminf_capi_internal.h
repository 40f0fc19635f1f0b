/*
 * siminf_capi_internal.h -- what the translation units behind the C ABI
 * share: the model handle and the argument check and per-thread status of
 * siminf_capi.cpp.
 */
#ifndef SIMINF_CAPI_INTERNAL_H
#define SIMINF_CAPI_INTERNAL_H

#include <memory>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/siminf_gb300.h"
#include "siminf_launch.h"
#include "siminf_plan.h"

/* A device model: its name and the launchers of its kernels. */
struct siminf_gpu_model {
    char name[64];
    const siminf::Launchers *L;
};

using siminf::DayInfo;
using siminf::DevState;
using siminf::E2Rec;
using siminf::Launchers;

/* A planned failure: an event the device cannot apply (bad node, dest or
 * kind) that the reference would reject when it reaches it. */
struct PlannedErr {
    int day, code, index, node, phase;
};

struct siminf_gpu_plan {
    const Launchers *L = nullptr;
    DevState s{};
    cudaStream_t stream = nullptr;      /* copies and kernels of create, run, download */
    bool async_alloc = false;           /* buffers from the stream-ordered allocator */
    std::vector<void *> owned;

    int ndays = 0;
    std::vector<DayInfo> days;
    DayInfo *d_days = nullptr;
    bool horizon = false;

    /* E2 waves */
    E2Rec *d_e2 = nullptr;
    std::vector<long long> wave_ptr;    /* offsets into d_e2, one past the last */
    std::vector<int> day_wave;          /* ndays + 1 */
    uint64_t e1_count = 0, e2_count = 0;

    std::vector<PlannedErr> planned;

    /* host-side copies needed to write results back */
    size_t U_len = 0, V_len = 0, prU_len = 0, prV_len = 0;
    int *d_u0 = nullptr;            /* device copy of the initial state */
    double *d_v0 = nullptr;
    double tt0 = 0;

    siminf_gpu_stats stats{};
    bool ran = false;
    int days_cap = 0;
    int max_days = 0;                   /* > 0: runs stop after this many days (tuning) */
    /* A run that repeats the previous one unchanged replays it from a CUDA
     * graph (the reset copies and every kernel launch of the run). */
    cudaGraphExec_t run_graph = nullptr;
    int runs_unchanged = 0;             /* runs since the last change of the plan */
    int *d_init_flags = nullptr;        /* {0, INT_MAX, INT_MAX}: the error counters' reset */

    /* E2 planning state: events of day d go to positions e2_day_off[d] ..
     * e2_day_off[d + 1] of d_e2 and come from input range e2_lo[d] ..
     * e2_hi[d]; day_waves[d] holds the day's wave sizes. */
    int nsel = 0;
    int max_select = 0, max_shift = 0;  /* largest select / shift of any event */
    std::vector<long long> e2_day_off, e2_lo, e2_hi;
    std::vector<std::vector<long long>> day_waves;
    /* Streamed runs: the waves are planned on host threads while the GPU
     * runs earlier days; the caller's arrays stay valid until the run. */
    bool e2_pending = false;
    /* Streamed runs whose events the device plans (siminf_schedule.cu):
     * e2_lo / e2_hi are the days' input ranges; dev_bad is the first event
     * out of order the planner found, or -1.  dev_levels: host threads
     * plan the transfers' levels and the device the rest (classification,
     * order check, E1 lists, wave order); otherwise the device plans the
     * levels too. */
    bool dev_plan = false;
    bool dev_levels = false;
    /* Streamed runs planned on host threads without a scan of the whole
     * table first (siminf_capi.cpp, scan_free_for): e2_lo / e2_hi are the
     * days' input ranges; the first run fills e2_day_off, the E1 lists,
     * the planned failures and dev_bad. */
    bool scan_free = false;
    long long dev_bad = -1;
    siminf_gpu_solver_args args{};
    std::unique_ptr<E2Rec[]> h_e2;
    /* Streamed runs with pinned output arrays: each chunk's finished
     * columns of U/V go back to out_args while later days run; columns
     * [0, cols_sent) of every replicate are copied or on their way. */
    siminf_gpu_solver_args *out_args = nullptr;
    int cols_sent = 0;
};

namespace siminf {

/* Create a plan: validate, plan the schedule and upload.  stream: leave
 * the external transfers' waves to the first run, which plans them beside
 * the GPU.  no_output: allocate no U/V (the caller reads results some
 * other way), whatever args->U says. */
int plan_create_internal(const siminf_gpu_solver_args *a, const siminf_gpu_model *model,
                         const siminf_gpu_options *opt, siminf_gpu_plan **out, bool stream,
                         bool no_output);

/* Run a plan on stream st (waits for it; returns 0 or the run's error). */
int plan_run_internal(siminf_gpu_plan *p, cudaStream_t st);

/* Upload n elements into a new device buffer the plan owns. */
int plan_upload(siminf_gpu_plan *p, void **dst, const void *src, size_t bytes);

/* The day schedule of tspan (src/solvers/SimInf_solver_ssm.c:305-334). */
int plan_days(const double *tspan, int tlen, std::vector<DayInfo> &days);

/* Plans created by the calling thread from now on put their copies and
 * kernels on `stream` and, if async, take their buffers from the
 * stream-ordered allocator on it (nullptr, false: the defaults). */
void plan_thread_stream(cudaStream_t stream, bool async);

/* The checks siminf_gpu_run_solver_ssm applies to its arguments. */
int capi_validate(const siminf_gpu_solver_args *a, const Launchers *L);

/* Record the calling thread's status (read by siminf_gpu_last_status). */
void capi_set_status(int code, int node, int tr, int evi, double time, double rate,
                     const char *msg);
void capi_clear_status();

/* Record the calling thread's run statistics (siminf_gpu_last_stats). */
void capi_set_stats(const siminf_gpu_stats &st);

/* Record a failed CUDA call; returns SIMINF_GPU_ERR_CUDA. */
int capi_cuda_fail(cudaError_t e, const char *what);

}  // namespace siminf

#endif
