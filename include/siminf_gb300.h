/*
 * siminf_gb300.h -- C ABI of the GB300 ssm/mssm solver.
 *
 * The library replaces the reference's solver entry points behind the
 * dispatch in SimInf_run (src/SimInf.c:382-399).  All pointers in the
 * argument struct are host pointers owned by the caller, exactly as in the
 * reference; the library copies what it needs to the GPU, runs there, and
 * writes U/V back into the caller's buffers before returning.  No torch
 * types and no CUDA types appear in any signature.
 *
 * Threading and errors follow the reference's convention: every call
 * returns 0 or a negative SimInf error code, never longjmps, and frees and
 * synchronises everything it allocated before returning.  Diagnostics of
 * the last failing call on the calling thread are kept for
 * siminf_gpu_last_status().
 */
#ifndef SIMINF_GB300_H
#define SIMINF_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Transition-rate and post-time-step callback types, unchanged from
 * inst/include/SimInf.h:92-107.  The GPU solver never calls host
 * callbacks; the fields are kept so that the struct below stays
 * layout-identical to SimInf_solver_args. */
typedef double (*siminf_gpu_trfun)(const int *u, const double *v,
                                   const double *ldata, const double *gdata,
                                   double t);
typedef int (*siminf_gpu_ptsfun)(double *v_new, const int *u, const double *v,
                                 const double *ldata, const double *gdata,
                                 int node, double t);

/* Event kinds, inst/include/SimInf.h:56-59. */
enum {
    SIMINF_GPU_EXIT_EVENT = 0,
    SIMINF_GPU_ENTER_EVENT = 1,
    SIMINF_GPU_INTERNAL_TRANSFER_EVENT = 2,
    SIMINF_GPU_EXTERNAL_TRANSFER_EVENT = 3
};

/* Error codes: the reference's SimInf_error_code values
 * (inst/include/SimInf.h:66-89) keep their numbers; codes from -30 down are
 * new and only the GPU path returns them. */
enum {
    SIMINF_GPU_ERR_NEGATIVE_STATE = -1,
    SIMINF_GPU_ERR_ALLOC_MEMORY_BUFFER = -2,
    SIMINF_GPU_UNDEFINED_EVENT = -3,
    SIMINF_GPU_ERR_SAMPLE_SELECT = -8,
    SIMINF_GPU_ERR_INVALID_MODEL = -9,
    SIMINF_GPU_ERR_INVALID_RATE = -11,
    SIMINF_GPU_ERR_UNKNOWN_SOLVER = -12,
    SIMINF_GPU_ERR_DEST_OUT_OF_BOUNDS = -13,
    SIMINF_GPU_ERR_NODE_OUT_OF_BOUNDS = -14,
    SIMINF_GPU_ERR_EVENTS_N = -15,
    SIMINF_GPU_ERR_EVENT_SHIFT = -16,
    SIMINF_GPU_ERR_SHIFT_OUT_OF_BOUNDS = -17,
    SIMINF_GPU_ERR_INVALID_PROPORTION = -18,
    SIMINF_GPU_ERR_AEM_REPLICATED_MODEL = -19,
    SIMINF_GPU_ERR_CUDA = -30,              /* a CUDA runtime call failed */
    SIMINF_GPU_ERR_EVENTS_UNSORTED = -31,   /* events not sorted by time, E1 before E2 */
    SIMINF_GPU_ERR_UNKNOWN_MODEL = -32,     /* no device model of that name */
    SIMINF_GPU_ERR_TIMEOUT = -33,           /* a bounded device wait gave up */
    SIMINF_GPU_ERR_NO_DEVICE = -34,         /* no CUDA device is visible */
    SIMINF_GPU_ERR_SCRATCH_LIMIT = -35      /* too large for siminf_gpu_run_solver_ssm_noalloc */
};

/*
 * Solver arguments.  Field for field the same struct as
 * SimInf_solver_args (src/SimInf_internal.h:44-200): the same types in the
 * same order, so SimInf_run can pass its own struct by pointer cast.
 * Node, dest, select and shift in the event arrays are one-based as in the
 * reference; events must be sorted by time with, within a time, the E1
 * events (exit, enter, internal transfer) before the external transfers --
 * the order R/SimInf_events.R:398 produces.
 */
typedef struct siminf_gpu_solver_args {
    const int *u0;              /* Nc x (Nn * Nrep) */
    const double *v0;           /* Nd x (Nn * Nrep) */
    const int *irG;             /* dependency graph G (Nt x Nt), CSC */
    const int *jcG;
    const int *irS;             /* state-change matrix S (Nc x Nt), CSC */
    const int *jcS;
    const int *prS;
    const double *tspan;
    int tlen;
    int *U;                     /* dense (Nn*Nc) x (Nrep*tlen), or NULL */
    const int *irU;             /* sparse U pattern when U is NULL */
    const int *jcU;
    double *prU;
    double *V;                  /* dense (Nn*Nd) x (Nrep*tlen), or NULL */
    const int *irV;
    const int *jcV;
    double *prV;
    const double *ldata;        /* Nld x Nn */
    const double *gdata;
    int Nn;
    int Nc;
    int Nt;
    int Nd;
    int Nld;
    int Nrep;
    const int *irE;             /* select matrix E, CSC */
    const int *jcE;
    double *prE;
    const int *N;               /* shift matrix, Nc x Nshift, or NULL */
    int len;                    /* number of scheduled events */
    const int *event;
    const int *time;
    const int *node;
    const int *dest;
    const int *n;
    const double *proportion;
    const int *select;
    const int *shift;
    int Nthread;                /* ignored on the GPU */
    int solver;                 /* 0 = ssm/mssm, 1 = aem (one replicate) */
    int crn;                    /* common random numbers (mssm) */
    int rng_type;               /* ignored: the GPU stream is Philox4x32-10 */
    unsigned long int seed;     /* Philox key */
    siminf_gpu_trfun *tr_fun;   /* ignored on the GPU */
    siminf_gpu_ptsfun pts_fun;  /* ignored on the GPU */
} siminf_gpu_solver_args;

/* A compiled device model: the __device__ transition-rate functions and
 * post-time-step function of one model.  Opaque. */
typedef struct siminf_gpu_model siminf_gpu_model;

/*
 * Look up a device model compiled into the library by name.  Replaces the
 * construction of `TRFun tr_fun[]` and the PTSFun pointer in each
 * <Model>_run (e.g. src/models/SEIR.c:157-165, src/models/SIR.c,
 * src/models/SISe.c) and the mparse-generated SIMINF_MODEL_RUN
 * (R/C-generator.R:304-332) for the models the library ships.
 * Names: "SIR" (SIR.c), "SEIR" (SEIR.c), "SIS" (SIS.c), "SISe" (SISe.c),
 * "SISe3" (SISe3.c),
 * "SIR_mparse" (mparse "S -> beta*S*I/N -> I", "I -> gamma*I -> R",
 * N <- S+I+R, beta/gamma in gdata), "SISe_pf" (mparse
 * "S -> upsilon*phi*S -> I", "I -> gamma*I -> S" with the pts_fun
 * phi <- phi*(1-0.03) + 0.05*I/(S+I); upsilon/gamma in gdata).
 * Returns 0 or SIMINF_GPU_ERR_UNKNOWN_MODEL.
 */
int siminf_gpu_model_builtin(const char *name, siminf_gpu_model **out);

/*
 * A device model compiled from model C code: the mparse output of
 * R/C-generator.R:204-297 (trFun1..trFunK and ptsFun) or a hand-written
 * model file with TRFun/PTSFun functions (inst/include/SimInf.h:92-107),
 * whose functions were compiled for the GPU with their signatures
 * unchanged into a library of their own (siminf_gb300/devmodel.py does it
 * with nvcc, caching the library by a digest of the C code as
 * R/run.R:93-98 caches the host build).  Replaces the dyn.load of the
 * compiled model in R/run.R:22-98 that SimInf_run then calls through
 * tr_fun/pts_fun.  path names that library; it stays loaded until the
 * process exits.  Returns 0 or SIMINF_GPU_ERR_UNKNOWN_MODEL (not found, or
 * built against another version of this library).
 */
int siminf_gpu_model_load(const char *path, siminf_gpu_model **out);

/* Number of transitions (Nt), compartments (Nc) and continuous state
 * variables (Nd) the model expects; any pointer may be NULL. */
int siminf_gpu_model_dims(const siminf_gpu_model *model, int *Nc, int *Nt, int *Nd);

void siminf_gpu_model_free(siminf_gpu_model *model);

/*
 * Run one replicate (Nrep == 1) with the split-step method.  Replaces
 * int SimInf_run_solver_ssm(SimInf_solver_args *args)
 * (src/SimInf_internal.h:418-420, src/solvers/SimInf_solver_ssm.c:381-414).
 * Writes U (dense) or prU (sparse) and V or prV.  Returns 0 or an error.
 */
int siminf_gpu_run_solver_ssm(siminf_gpu_solver_args *args,
                              const siminf_gpu_model *model);

/*
 * Run Nrep >= 1 replicates in one batched launch.  Replaces
 * int SimInf_run_solver_mssm(SimInf_solver_args *args)
 * (src/SimInf_internal.h:410-412, src/solvers/SimInf_solver_mssm.c:410-443).
 * Replicate r owns columns [r*tlen, (r+1)*tlen) of U/V and draws from the
 * streams r*Nn + node.
 */
int siminf_gpu_run_solver_mssm(siminf_gpu_solver_args *args,
                               const siminf_gpu_model *model);

/*
 * Options of the GPU path that the reference does not have.  Zero-filled
 * options give exactly the reference's semantics.
 *
 * cap_transfers: an exit, internal-transfer or external-transfer event that
 * asks for more individuals than the selected compartments hold takes all of
 * them instead of stopping the run with SIMINF_ERR_SAMPLE_SELECT
 * (src/solvers/SimInf_solver.c:102-105).  Synthetic schedules whose sizes
 * are drawn without knowledge of the state need it.
 *
 * heavy_rate: a tuning knob, not a semantic option -- nodes whose rate sum
 * at the start of a day reaches it are queued and simulated first, 32 to a
 * warp (results are identical either way); 0 takes the default (8), a
 * negative value turns the queue off.
 *
 * two_pass: a tuning knob, not a semantic option -- each day first
 * finishes, one node per thread, every node whose day has no transition,
 * and steps only the others in the work queue (results are identical
 * either way).  It pays where most node-days are quiet and the plan holds
 * many nodes, which is when the default turns it on.
 *
 * gdata_per_replicate: args->gdata holds one gdata vector per replicate
 * (Nrep rows of the model's gdata length); replicate r reads row r.  The
 * reference shares one gdata among replicates; particle filters and ABC
 * batches over parameter sets need one per replicate.
 *
 * max_node_day_transitions: the most transitions one node may fire in one
 * unit of time; a node that would fire more stops the run with
 * SIMINF_GPU_ERR_TIMEOUT instead of holding the GPU (the reference loops
 * until its rate sum runs out).  0 takes the default, 2^28.
 */
typedef struct siminf_gpu_options {
    int cap_transfers;
    int heavy_rate;     /* rate sum from which a node is queued first (0 = default 8, < 0 = off) */
    int gdata_per_replicate;
    int two_pass;       /* > 0 on, < 0 off, 0 = on from 500,000 nodes (all replicates) */
    int max_node_day_transitions;   /* > 0: the bound; 0: 2^28 */
    int streamed;       /* siminf_gpu_plan_create_ex: plan the events during the first run,
                         * beside the GPU, as the run entry points do (on host threads;
                         * SIMINF_DEVICE_PLANNER=1 or 2 selects the device planner); 0:
                         * before the plan returns */
    int ssa_variant;    /* SSA kernel register budget: 0 the model's default, 1 more
                         * registers a thread and fewer resident warps (see the autotuner) */
    int wave_block;     /* threads per block of the wavefront kernel: 128, 256 or 512 (0: 256) */
    int heavy_lanes;    /* lanes of a warp that take nodes of the heaviest class (rate sum
                         * >= 16 x heavy_rate), 1..32 (0: 32) */
} siminf_gpu_options;

/* The default of siminf_gpu_options.max_node_day_transitions. */
#define SIMINF_GPU_MAX_NODE_DAY_TRANSITIONS (1u << 28)

/* siminf_gpu_run_solver_mssm with options (NULL = all zero). */
int siminf_gpu_run_solver_ex(siminf_gpu_solver_args *args,
                             const siminf_gpu_model *model,
                             const siminf_gpu_options *options);

/*
 * No counterpart in the reference.  The run entry points keep the pinned
 * host buffers through which they stage external transfers (at most four,
 * 4 GiB in all) for the next run, and copy U/V back during the run when
 * those arrays are pinned.  This frees the kept buffers.
 */
void siminf_gpu_release_cached(void);

/*
 * Many independent models of one device model in one run -- different node
 * counts, tspan lengths (prefixes of one grid from the same tspan[0]),
 * events, parameters (ldata/gdata) and seeds -- each reduced on the device
 * to its prevalence series (sum over its nodes of the compartments in
 * prevalence_num_mask over those in prevalence_den_mask, at every tspan
 * point) and the L2 distance of that series to a target.  Replaces the
 * simulate-then-measure loop of the reference's ABC samplers
 * (R/abc.R:589-628 for gdata proposals, :675-729 for ldata proposals),
 * which calls run() once per proposal.  Each model's trajectory is the one
 * siminf_gpu_run_solver_ssm gives it alone with its own seed; the models
 * must share E and N (the model's select and shift matrices).  Returns 0
 * or an error code; an error in one model stops the batch and the status
 * names the model.
 */
typedef struct siminf_gpu_batch_job {
    siminf_gpu_solver_args *args;   /* one model, Nrep = 1; its U/V are not written */
    const double *target;           /* tlen prevalence values, or NULL */
    double *prevalence;             /* out: tlen values, or NULL */
    double *distance;               /* out: L2 distance to target (0 without one), or NULL */
} siminf_gpu_batch_job;

typedef struct siminf_gpu_batch_options {
    unsigned prevalence_num_mask;   /* compartments (bit c) summed in the numerator */
    unsigned prevalence_den_mask;   /* compartments summed in the denominator */
    int cap_transfers;              /* as in siminf_gpu_options */
    int heavy_rate;                 /* as in siminf_gpu_options */
    int reserved[4];
} siminf_gpu_batch_options;

int siminf_gpu_run_batch(siminf_gpu_batch_job *jobs, int njobs, const siminf_gpu_model *model,
                         const siminf_gpu_batch_options *options);

/*
 * siminf_gpu_run_solver_ssm without allocating: no counterpart in the
 * reference, which allocates its solver state on every run.  For callers
 * that cannot allocate when they run a trajectory: a process whose device
 * memory is held by another allocator (cudaMalloc would fail or fragment
 * it), or a loop that runs trajectories between its own kernels on other
 * streams and cannot afford cudaFree, which waits for the whole device.
 * Same arguments and results as siminf_gpu_run_solver_ssm for one
 * replicate without scheduled events (Nrep = 1, len = 0) and a dense U;
 * every buffer of the run lives in one static device array of
 * SIMINF_GPU_NOALLOC_SCRATCH_BYTES, and a run that does not fit returns
 * SIMINF_GPU_ERR_SCRATCH_LIMIT.  The call calls no allocator, runs on
 * cuda_stream (a cudaStream_t, or NULL) and returns when U and V are
 * written.  The first call on a device looks up the array's address on
 * that device (the current one): make it before any stream capture.  All
 * calls on a device share the array and each clears what must start at
 * zero; calls that overlap on the GPU race on it.
 */
#define SIMINF_GPU_NOALLOC_SCRATCH_BYTES (16u * 1024u * 1024u)
int siminf_gpu_run_solver_ssm_noalloc(siminf_gpu_solver_args *args,
                                      const siminf_gpu_model *model,
                                      void *cuda_stream);

/*
 * Plan an event schedule on the host only (no GPU is touched): checks the
 * event order and splits each day's external transfers into the
 * conflict-free wavefronts the GPU runs, exactly as siminf_gpu_plan_create
 * does.  days, waves, e1_events, e2_events receive counts (any may be
 * NULL); wave, if not NULL, must hold args->len ints and receives per event
 * the zero-based wavefront of an external transfer within its day, or -1.
 * Returns 0 or an error code.  This is the planning half of the
 * reference's SimInf_scheduled_events_create
 * (src/solvers/SimInf_solver.c:443-510) and SimInf_split_events (:353-385).
 */
int siminf_gpu_schedule(const siminf_gpu_solver_args *args, int *days, int *waves,
                        long long *e1_events, long long *e2_events, int *wave);

/*
 * The same schedule planned on the GPU (siminf_schedule.cu), with the same
 * outputs as siminf_gpu_schedule: the events are classified, ordered and
 * levelled a chunk of days at a time by rounds of relaxation over per-node
 * event lists, the planner the streamed runs use.  Days whose wavefronts
 * run deeper than the rounds allow are levelled by the host planner.
 */
int siminf_gpu_schedule_device(const siminf_gpu_solver_args *args, int *days, int *waves,
                               long long *e1_events, long long *e2_events, int *wave);

/*
 * Bootstrap particle filter on the GPU: the loop of pfilter_internal
 * (R/pfilter.R:315-499) with SimInf_systematic_resampling
 * (src/misc/SimInf_particle_filter.c:33-67).  args describes one particle's
 * model (Nrep is ignored; events are not supported yet); every interval
 * (R/pfilter.R:177-193) runs all particles as replicates of one plan,
 * resident on the device, then weights, resamples and copies the ancestors'
 * states without leaving the GPU.  The observation process is
 * Binomial(x, detect_p) of one compartment per node, log-density floored at
 * -690 per node for impossible observations (the reference stops on
 * non-finite weights, R/pfilter.R:438-442).  Interval i runs with seed
 * seed + (i+1) * 0x9E3779B97F4A7C15 and resamples with draw 0 of stream
 * 2^62 + i under seed.
 */
typedef struct siminf_gpu_pfilter_args {
    int n_particles;
    int gdata_per_particle;     /* args->gdata holds n_particles rows */
    int n_obs;
    const int *obs_time;        /* n_obs increasing times >= tspan[0] */
    const int *obs;             /* n_obs x Nn observed counts, row-major */
    int obs_compartment;        /* zero-based */
    double detect_p;
    unsigned long seed;
    double *loglik;             /* out: log-likelihood */
    double *ess;                /* out: n_obs effective sample sizes */
    int *ancestors;             /* out (or NULL): n_obs x n_particles, one-based */
    double ms_total;            /* out: wall time of the filter */
} siminf_gpu_pfilter_args;

int siminf_gpu_pfilter(const siminf_gpu_solver_args *args, const siminf_gpu_model *model,
                       siminf_gpu_pfilter_args *pf);

/*
 * Particle-marginal Metropolis-Hastings with the particle filter above:
 * the chain of pmcmc() and continue_pmcmc() (R/pmcmc.R:470-600).  The
 * chain is resident: siminf_gpu_pmcmc_create keeps the filter's plan,
 * observations and buffers on the device, and every siminf_gpu_pmcmc_run
 * call continues the chain where the last one stopped, so that n calls of
 * k iterations give the rows of one call of n k iterations.  Row 1 is the
 * initial theta; each later row proposes theta + z Q (z standard normal,
 * Q = chol, the upper Cholesky factor of the proposal covariance, as
 * R/pmcmc.R:423-437 with the adaptive part off), runs one filter pass when
 * the prior density is positive, and accepts with probability
 * exp(logLik' + logPrior' - logLik - logPrior).  Parameters are gdata
 * entries with uniform priors; args->gdata holds the other entries.
 * Draws come from counter-based streams keyed by (seed, iteration), so a
 * continued chain equals an uninterrupted one.  The pfilter arguments'
 * outputs (loglik, ess, ancestors) are not used.
 */
typedef struct siminf_gpu_pmcmc_args {
    int n_pars;
    const int *gdata_index;     /* zero-based gdata entry of each parameter */
    const double *theta;        /* initial values */
    const double *prior_lo;     /* uniform priors U(lo, hi) */
    const double *prior_hi;
    const double *chol;         /* n_pars x n_pars, row-major, upper triangular */
    unsigned long seed;
    int reserved[4];
} siminf_gpu_pmcmc_args;

typedef struct siminf_gpu_pmcmc siminf_gpu_pmcmc;

int siminf_gpu_pmcmc_create(const siminf_gpu_solver_args *args, const siminf_gpu_model *model,
                            const siminf_gpu_pfilter_args *pf, const siminf_gpu_pmcmc_args *pm,
                            siminf_gpu_pmcmc **out);
/* n_iterations more rows; rows (or NULL) receives n_iterations x
 * (4 + n_pars) doubles, row-major: logPost, logLik, logPrior, accept,
 * theta -- the columns of the reference's chain. */
int siminf_gpu_pmcmc_run(siminf_gpu_pmcmc *chain, int n_iterations, double *rows);
long long siminf_gpu_pmcmc_length(const siminf_gpu_pmcmc *chain);
void siminf_gpu_pmcmc_free(siminf_gpu_pmcmc *chain);

/* Diagnostics of the last failing call on the calling thread: the fields
 * SimInf_print_status (src/solvers/SimInf_solver.c:1191-1249) and
 * SimInf_print_event (src/solvers/SimInf_solver.c:550-645) print. */
typedef struct siminf_gpu_status {
    int error;                  /* the returned code */
    int node;                   /* zero-based node of the failure, or -1 */
    int transition;             /* zero-based transition, or -1 */
    int event_index;            /* zero-based index into the event arrays, or -1 */
    double time;                /* simulation time of the failure */
    double rate;                /* the offending rate for INVALID_RATE */
    char message[512];          /* one human-readable line */
} siminf_gpu_status;

int siminf_gpu_last_status(siminf_gpu_status *out);

/* Counters and timings of the last successful run on the calling thread. */
typedef struct siminf_gpu_stats {
    uint64_t transitions;       /* SSA transitions fired */
    uint64_t node_days;         /* node x unit-time steps simulated */
    uint64_t e1_events;         /* exit/enter/internal events applied */
    uint64_t e2_events;         /* external transfers applied */
    int e2_waves;               /* conflict-free wavefronts executed */
    int days;                   /* unit-time steps simulated */
    double ms_upload;           /* planning and host -> device copies */
    double ms_plan;             /* of which: host-side event planning */
    double ms_solve;            /* device time of the day loop */
    double ms_download;         /* device -> host copies of U/V */
} siminf_gpu_stats;

int siminf_gpu_last_stats(siminf_gpu_stats *out);

/*
 * Device-resident plans, for callers that keep a model on the GPU across
 * runs (particle filters, ABC, serving).  plan_create copies the model,
 * the event schedule and its per-day wave plan to the device; plan_run
 * runs the whole horizon from u0/v0 on the given CUDA stream (a
 * cudaStream_t passed as void*, NULL for the default stream) without any
 * host copy; plan_download writes U/V into the args' buffers.
 */
typedef struct siminf_gpu_plan siminf_gpu_plan;

int siminf_gpu_plan_create(const siminf_gpu_solver_args *args,
                           const siminf_gpu_model *model,
                           siminf_gpu_plan **out);
int siminf_gpu_plan_create_ex(const siminf_gpu_solver_args *args,
                              const siminf_gpu_model *model,
                              const siminf_gpu_options *options,
                              siminf_gpu_plan **out);
int siminf_gpu_plan_run(siminf_gpu_plan *plan, void *cuda_stream);
int siminf_gpu_plan_download(siminf_gpu_plan *plan, siminf_gpu_solver_args *args);
/* plan_run once recording, per day, the most transitions any node fired
 * that day (day_max: one entry per day of the plan; the days' sum is the
 * run's critical path: every day lasts at least as long as its busiest
 * node's chain of transitions).  Recorded by the direct method's work
 * queue; plans without external transfers and aem plans report zeros.
 * For profiling. */
int siminf_gpu_plan_day_max(siminf_gpu_plan *plan, void *cuda_stream, unsigned *day_max);

/* plan_run with a CUDA event pair around every launch: device milliseconds
 * and launch counts per kernel kind, [0] initialisation, [1] SSA + E1,
 * [2] E2 wavefront, [3] post time step + store, [4] whole-horizon kernel,
 * [5] first pass of a two-pass day (entries 6..7 are zero).  For
 * profiling; slower than plan_run. */
int siminf_gpu_plan_profile(siminf_gpu_plan *plan, void *cuda_stream, double ms[8],
                            long long launches[8]);
int siminf_gpu_plan_stats(const siminf_gpu_plan *plan, siminf_gpu_stats *out);

/*
 * Autotuner (no counterpart in the reference): times the plan's first
 * probe_days days (0: 16) for candidate launch layouts and keeps the
 * fastest in the plan, reporting every candidate's time.  Stage 1: the
 * SSA work queue's heavy-part threshold (rate sum from which a node is
 * queued first and run 32 to a warp; 0 turns the part off: 0, 2, 8, 32),
 * with one-pass and with two-pass days (siminf_gpu_options.two_pass).
 * Stage 2, from the best of stage 1: the SSA kernel's other register
 * budget (ssa_variant 1: more registers a thread, fewer resident warps),
 * then, for a plan of one model and one replicate with the heavy part on,
 * 8 lanes a warp for the heaviest class (heavy_lanes; 32 otherwise).  Stage 3, for plans with external transfers: the wavefront kernel's block
 * of 128 and 512 threads (256 otherwise).  The three fastest are then
 * timed again as repeated runs execute them (the third run of each, which
 * replays the run's CUDA graph), and their times replace the probes'; the
 * fastest of those is kept.  The choice is kept per device
 * model and size class (node count and day count to a power of two,
 * transfers or not): a later plan of the same class takes it without
 * probing (cached = 1; probe_days < 0 forces a new search).  Results never
 * depend on the layout; only the order in which nodes are simulated does.
 */
#define SIMINF_GPU_TUNE_CANDIDATES 16
typedef struct siminf_gpu_tune_result {
    double heavy_rate[SIMINF_GPU_TUNE_CANDIDATES];
    int two_pass[SIMINF_GPU_TUNE_CANDIDATES];   /* 1: two-pass days */
    int ssa_variant[SIMINF_GPU_TUNE_CANDIDATES];    /* SSA kernel register budget */
    int wave_block[SIMINF_GPU_TUNE_CANDIDATES];     /* threads per wavefront block */
    int heavy_lanes[SIMINF_GPU_TUNE_CANDIDATES];    /* lanes a warp for the heaviest class */
    double ms[SIMINF_GPU_TUNE_CANDIDATES];     /* device time of the probe days */
    int n_candidates;                           /* candidates timed */
    int chosen;                                 /* index of the kept candidate */
    int probe_days;
    int cached;                                 /* 1: taken from an earlier plan's search */
} siminf_gpu_tune_result;

int siminf_gpu_plan_tune(siminf_gpu_plan *plan, void *cuda_stream, int probe_days,
                         siminf_gpu_tune_result *out);
void siminf_gpu_plan_free(siminf_gpu_plan *plan);

/*
 * Serving: a request loop that runs simulations, particle filters and
 * re-runs of device-resident plans as they arrive.  No counterpart in the
 * reference, where each run() call simulates on the calling thread
 * (R/run.R:178-283).  The server keeps `slots` requests on the GPU at once,
 * each on its own stream with stream-ordered allocation, and admits a
 * request when its estimated device bytes fit the HBM budget (oldest first;
 * a younger one that fits may pass an older one waiting for memory).
 * siminf_gpu_server_submit returns at once; the request and every buffer it
 * points to must stay valid until siminf_gpu_server_wait reports it
 * finished.  Results are those of the same call made alone
 * (siminf_gpu_run_solver_ex, siminf_gpu_pfilter, siminf_gpu_plan_run).
 */
enum {
    SIMINF_GPU_REQUEST_RUN = 0,         /* args + model + options: U/V written */
    SIMINF_GPU_REQUEST_PFILTER = 1,     /* args + model + pfilter */
    SIMINF_GPU_REQUEST_PLAN = 2,        /* plan: run again, results stay on the device */
    SIMINF_GPU_REQUEST_PMCMC = 3        /* pmcmc: continue a resident chain by
                                         * pmcmc_iterations rows into pmcmc_rows
                                         * (continue_pmcmc, R/pmcmc.R:474-600) */
};

typedef struct siminf_gpu_request {
    int kind;
    siminf_gpu_solver_args *args;
    const siminf_gpu_model *model;
    siminf_gpu_options options;
    siminf_gpu_pfilter_args *pfilter;
    siminf_gpu_plan *plan;
    long long bytes;                    /* device bytes to admit (0: estimated) */
    /* set by the server */
    int status;                         /* 0 or an error code */
    int finished;
    double ms_wait;                     /* from submission to the start on a slot */
    double ms_run;                      /* on the slot */
    long long submit_ns;
    siminf_gpu_stats stats;             /* runs and plans */
    char message[200];                  /* the error's diagnostics */
    /* SIMINF_GPU_REQUEST_PMCMC */
    siminf_gpu_pmcmc *pmcmc;
    int pmcmc_iterations;
    double *pmcmc_rows;
} siminf_gpu_request;

typedef struct siminf_gpu_server_options {
    int slots;                          /* requests on the GPU at once (0: 8) */
    int reserved0;
    long long hbm_budget_bytes;         /* admission budget (0: 90% of free memory) */
    int reserved[4];
} siminf_gpu_server_options;

typedef struct siminf_gpu_server siminf_gpu_server;

int siminf_gpu_server_create(const siminf_gpu_server_options *options,
                             siminf_gpu_server **out);
int siminf_gpu_server_submit(siminf_gpu_server *server, siminf_gpu_request *request);
/* 1 when the request has finished, 0 on timeout (timeout_ms < 0: wait). */
int siminf_gpu_server_wait(siminf_gpu_server *server, siminf_gpu_request *request,
                           double timeout_ms);
int siminf_gpu_server_load(siminf_gpu_server *server, int *pending, int *running,
                           long long *bytes_in_use);
/* Finishes every submitted request, then stops the slots. */
void siminf_gpu_server_free(siminf_gpu_server *server);

/*
 * Trajectory consumers on the device, reading U or V where a run left them
 * in HBM (a plan's outputs, siminf_gpu_plan_outputs, or any device copy of
 * a dense U/V): the caller copies back the series it asks for, not the
 * trajectory.  U is (Nn * Nc) x ncol and V (Nn * Nd) x ncol, column-major
 * as the solver writes them (ncol = Nrep * tlen, replicate-major).  Node
 * identifiers are one-based (NULL: every node in order); outputs are host
 * arrays; the call waits for its stream.
 */
typedef struct siminf_gpu_reduce_stats {
    double ms_kernel;           /* device time of the reduction kernels */
    double ms_total;            /* the whole call, copies included */
    long long bytes_read;       /* U/V bytes the kernels read */
    long long bytes_written;    /* output bytes */
} siminf_gpu_reduce_stats;

/*
 * The long format of SimInf_trajectory for dense U
 * (src/misc/SimInf_trajectory.c:566-620, SimInf_u_dense2df): for each of
 * the n_compartments one-based compartments, ncol * n rows (n = n_id, or
 * Nn), row col * n + l holding node id[l] in column col.  out receives
 * n_compartments such columns, one after the other.
 */
int siminf_gpu_trajectory_u(const int *d_U, int Nn, int Nc, int ncol,
                            const int *compartments, int n_compartments,
                            const int *id, int n_id, int *out, void *cuda_stream,
                            siminf_gpu_reduce_stats *stats);

/* The same for dense V (SimInf_v_dense2df, src/misc/SimInf_trajectory.c:652-706). */
int siminf_gpu_trajectory_v(const double *d_V, int Nn, int Nd, int ncol,
                            const int *variables, int n_variables,
                            const int *id, int n_id, double *out, void *cuda_stream,
                            siminf_gpu_reduce_stats *stats);

/*
 * prevalence(model, formula, level, index) (R/prevalence.R:72-96): cases
 * and population are bit masks of zero-based compartments (the formula's
 * left- and right-hand sides); the optional condition (the formula's
 * "| ..." part) is a postfix program of n_condition (operator, argument)
 * pairs over the node's compartments, evaluated in 64-bit integers;
 * comparisons and logical operators give 0 or 1, and the program must end
 * in one.  Where it is false a node counts neither as a case nor in the
 * population.  Level 1: sum(cases) / sum(population) per column; level 2:
 * #(cases > 0) / #(population > 0); level 3: cases / population per node,
 * out[col * n + l].  0 / 0 gives NaN as in R.
 */
enum {
    SIMINF_GPU_COND_COMPARTMENT = 1,    /* push u[argument] (zero-based) */
    SIMINF_GPU_COND_CONST = 2,          /* push the argument */
    SIMINF_GPU_COND_ADD = 3,
    SIMINF_GPU_COND_SUB = 4,
    SIMINF_GPU_COND_MUL = 5,
    SIMINF_GPU_COND_NEG = 6,            /* unary minus */
    SIMINF_GPU_COND_EQ = 7,
    SIMINF_GPU_COND_NE = 8,
    SIMINF_GPU_COND_LT = 9,
    SIMINF_GPU_COND_LE = 10,
    SIMINF_GPU_COND_GT = 11,
    SIMINF_GPU_COND_GE = 12,
    SIMINF_GPU_COND_AND = 13,
    SIMINF_GPU_COND_OR = 14,
    SIMINF_GPU_COND_NOT = 15
};

typedef struct siminf_gpu_prevalence_spec {
    unsigned int cases;                 /* bit c: compartment c is a case */
    unsigned int population;            /* bit c: compartment c is in the population */
    int level;                          /* 1, 2 or 3 */
    int n_condition;                    /* 0: no condition */
    const int *condition;               /* 2 * n_condition ints: (operator, argument) */
} siminf_gpu_prevalence_spec;

int siminf_gpu_prevalence(const int *d_U, int Nn, int Nc, int ncol,
                          const siminf_gpu_prevalence_spec *spec,
                          const int *id, int n_id, double *out, void *cuda_stream,
                          siminf_gpu_reduce_stats *stats);

/*
 * The ordering SimInf_events gives a scheduled-event table
 * (R/SimInf_events.R:396): events sorted by (time, event, select), equal
 * keys in input order, done on the device (an LSD radix sort of the packed
 * key and the input position, then a gather of every column).  The len
 * events of the eight host columns are reordered in place; the solver
 * entry points expect this order.  No counterpart in the reference's C.
 */
int siminf_gpu_sort_events(long long len, int *event, int *time, int *node, int *dest,
                           int *n, double *proportion, int *select, int *shift,
                           void *cuda_stream, siminf_gpu_reduce_stats *stats);

/*
 * SimInf_individual_events (src/misc/SimInf_individual_events.c:167-249):
 * the cleaning of individual-based event data.  The len events of the host
 * columns are sorted by (id, time, event, node, dest) with exact duplicates
 * removed (R/SimInf_individual_events.R:397-410 does both before its C
 * call); event is 0 (exit), 1 (enter) or 3 (external transfer) and dest is
 * NA (INT_MIN) for the first two.  keep[i] becomes 1 for the events on each
 * individual's longest consistent path and 0 for the rest, with the
 * reference's search order and tie rule.  Runs on the device: one thread
 * per individual over its slice of the columns.
 * Returns 0, SIMINF_GPU_UNDEFINED_EVENT for an event type other than
 * 0, 1 or 3 (message "'event[i]' is invalid." with the reference's
 * one-based i; siminf_gpu_status.event_index holds it zero-based; keep is
 * then all 0), SIMINF_GPU_ERR_INVALID_MODEL for a negative len, len above
 * INT_MAX or a NULL column, or SIMINF_GPU_ERR_CUDA.
 */
int siminf_gpu_individual_events(long long len, const int *id, const int *event,
                                 const int *time, const int *node, const int *dest,
                                 int *keep, void *cuda_stream, siminf_gpu_reduce_stats *stats);

/*
 * siminf_gpu_individual_events with a bound on each individual's search
 * (no counterpart in the reference).  The depth-first search can take time
 * exponential in an individual's event count -- branches that rejoin while
 * the exits present cannot be reached, so nothing prunes it -- and here it
 * holds a GPU thread.  max_steps bounds the candidate events one
 * individual's search examines (<= 0: SIMINF_GPU_INDIVIDUAL_MAX_STEPS,
 * which siminf_gpu_individual_events uses).  An individual that runs out
 * keeps none of its events and the call returns SIMINF_GPU_ERR_TIMEOUT,
 * siminf_gpu_status.event_index holding the zero-based first event of the
 * lowest such individual; every other individual's keep is computed.
 */
#define SIMINF_GPU_INDIVIDUAL_MAX_STEPS (1LL << 26)
int siminf_gpu_individual_events_ex(long long len, const int *id, const int *event,
                                    const int *time, const int *node, const int *dest,
                                    int *keep, long long max_steps, void *cuda_stream,
                                    siminf_gpu_reduce_stats *stats);

/* The device U/V of a plan that has run (d_V NULL without V), and ncol. */
int siminf_gpu_plan_outputs(const siminf_gpu_plan *plan, const int **d_U,
                            const double **d_V, int *ncol);

#ifdef __cplusplus
}
#endif

#endif /* SIMINF_GB300_H */
