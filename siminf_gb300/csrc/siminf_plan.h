/*
 * siminf_plan.h -- device-side data layout of one solver run, shared by the
 * host planner (siminf_capi.cpp) and the kernels (siminf_kernels.cu).
 *
 * HBM layout, for Ntot = Nrep * Nn (replicate-major, g = rep * Nn + node):
 *   u        int32  [Ntot][Nc]     node-major, the layout of one U column
 *   v, v_new double [Ntot][Nd]     double-buffered, swapped every day
 *   t_rate   double [Nt][Ntot]     transition-major (coalesced per warp)
 *   sum_rate double [Ntot], t_time double [Ntot]
 *   ctr      uint64 [Ntot]         next draw index of stream g
 *   update   uint8  [Ntot]         node flagged by an event this day
 *   U        int32  [(Nrep*tlen)][Nn*Nc]   the reference's column-major U
 *   V        double [(Nrep*tlen)][Nn*Nd]
 * Events are copied once per plan:
 *   E1 (exit/enter/internal): e1[] sorted by (node, day, array order), with
 *     e1_ptr[node] .. e1_ptr[node+1] the events of node.
 *   E2 (external transfers): e2[] sorted by (day, wave, array order), with
 *     the waves of day d in wave_ptr[day_wave[d]] .. wave_ptr[day_wave[d+1]].
 */
#ifndef SIMINF_PLAN_H
#define SIMINF_PLAN_H

#include <stdint.h>

namespace siminf {

enum { MAX_NC = 16, MAX_NT = 32, MAX_ERR = 1024 };

/* k_ssa_e1 is a persistent grid fed by a per-day work queue of nodes: first
 * the heavy nodes (rate sum >= heavy_rate at the start of the day, listed by
 * k_pts_store or k_init in classes sum >= 16, 4 and 1 times heavy_rate,
 * heaviest first), then every node in index order, heavy ones skipped.  So
 * the day's longest chains start first, and a thread whose node is done
 * takes the next one.  At most MAX_HEAVY nodes per class and day are
 * listed; the rest come in index order. */
enum { SSA_BLOCK = 128, HEAVY_CLASSES = 3, MAX_HEAVY = 32768 };

enum { PHASE_INIT = 0, PHASE_SSA = 1, PHASE_E1 = 2, PHASE_E2 = 3, PHASE_PTS = 4 };

struct E1Rec {          /* 32 bytes */
    int day;
    int kind;
    int n;
    int select;         /* zero-based column of E */
    int shift;          /* zero-based column of N, or -1 */
    int index;          /* position in the caller's event arrays */
    double proportion;
};

struct E2Rec {          /* 32 bytes */
    int src;            /* zero-based */
    int dst;
    int n;
    int select;
    int shift;
    int index;
    double proportion;
};

/* A day's last, small wavefronts, run by one block (k_e2_tail): wave w
 * holds count[w] events from off[w] of the wave list (at most
 * E2_TAIL_WAVES waves of at most E2_TAIL_ITEMS events x replicates). */
enum { E2_TAIL_WAVES = 32, E2_TAIL_ITEMS = 1024 };
struct E2Tail {
    int n;
    int count[E2_TAIL_WAVES];
    long long off[E2_TAIL_WAVES];
};

struct ErrRec {
    int code;
    int phase;
    int day;
    int rep;
    int node;
    int transition;
    int event_index;
    int pad;
    double time;
    double rate;
};

struct DayInfo {
    double tt;          /* time at the start of the day */
    double next;        /* next unit of time */
    int c0, c1;         /* U/V columns stored after this day */
};

struct DevState {
    int Nn, Nc, Nt, Nd, Nld, Nrep, tlen;
    long long Ntot;
    uint64_t seed;
    int cap;                /* cap sampled sizes at what the node holds */
    unsigned max_fired;     /* transitions one node may fire in one unit of
                             * time before the run stops with a timeout */

    /* model matrices */
    const int *S;           /* dense, Nt rows of Nc */
    const uint32_t *Gmask;  /* Nt: bit k set if rate k is refreshed after transition j */
    const int *irE, *jcE;
    const double *prE;
    const int *Nshift;      /* Nc x Nshift */
    int hasN;               /* the caller passed N */
    const double *ldata, *gdata;
    int gdata_stride;       /* 0: one gdata; else replicate r reads gdata + r * stride */

    /* state */
    int *u;
    double *vA, *vB;
    double *t_rate, *sum_rate, *t_time;
    uint64_t *ctr;
    uint8_t *update;
    /* common random numbers (mssm_crn, replicated models): the SSA draws of
     * node g come from stream SI_CRN_SID | g, whose next draw index is
     * crn_ctr[g]; ctr[g] then counts the draws of its events only.
     * nullptr: the SSA and the events share stream g. */
    uint64_t *crn_ctr;

    /* events */
    const int *e1_ptr;
    const E1Rec *e1;

    /* outputs: dense or sparse (pattern on the device) */
    int *U;
    double *V;
    const int *irU, *jcU;
    double *prU;
    const int *irV, *jcV;
    double *prV;

    /* errors and counters */
    ErrRec *err;
    int *err_count;
    int *err_day;           /* first day with an error (INT_MAX if none) */
    int *err_day_pre_e2;    /* first day with an SSA or E1 error */
    unsigned long long *fired;

    /* heavy nodes of the next two days:
     * list[((d & 1) * HEAVY_CLASSES + class) * MAX_HEAVY + i] */
    int *heavy_list;
    int *heavy_count;       /* [2][HEAVY_CLASSES] */
    unsigned long long *queue_next;  /* [day parity][heavy, ordinary]: next queue entries,
                                      * then [4 + day parity]: length of `active` */
    int *heavy_mark;        /* per g: day + 1 when listed for that day */
    double heavy_rate;      /* <= 0: no heavy part in the queue */

    /* Two-pass days: k_quick finishes every ordinary node whose day has no
     * transition and lists the others in `active` (Ntot entries), the
     * ordinary part of k_ssa_e1's queue. */
    int two_pass;
    int *active;

    /* Launch layout the autotuner picks: the SSA kernel's register budget
     * (0: the model's default, 1: more registers a thread and fewer
     * resident warps) and the external-transfer wave kernel's block size
     * (128, 256 or 512; 0: 256). */
    int ssa_variant;
    int wave_block;
    /* Lanes of a warp that take nodes of the heaviest class (1..32; 0:
     * 32): a warp that holds the day's longest chains shares its issue
     * slots and FP64 pipe with fewer lanes. */
    int heavy_lanes;

    /* Profiling: per day, the most transitions any node fired that day
     * (nullptr: not recorded). */
    unsigned *day_max;

    /* All-events method (one replicate): per transition j of node g, in
     * [j][Ntot] order, the next event time, the time left when its rate
     * fell to zero, and the draw index of its own stream. */
    int aem;
    double *react_time, *react_inf;
    uint64_t *react_ctr;

    /* Batches of independent models (siminf_gpu_run_batch); job_of is NULL
     * for a single model.  Node g belongs to job j = job_of[g], whose nodes
     * start at job_node0[j]: its stream key is (job_seed[j], g -
     * job_node0[j]), as in a run of that model alone, its gdata row is j,
     * and it runs job_ndays[j] days.  At every stored column col <
     * job_tlen[j], the sums over the job's nodes of the compartments in
     * prev_num_mask and prev_den_mask are added to prev[2 * (job_col0[j] +
     * col)] and prev[2 * (job_col0[j] + col) + 1]. */
    const int *job_of;
    const long long *job_node0;
    const uint64_t *job_seed;
    const int *job_ndays;
    const int *job_tlen;
    const long long *job_col0;
    unsigned long long *prev;
    uint32_t prev_num_mask, prev_den_mask;

    /* Particle-filter intervals replayed from one CUDA graph: the interval
     * index lives on the device (*pf_interval), and with it the interval's
     * seed (pf_seeds[i]) and day schedule (pf_days + i * pf_days_stride),
     * which k_init and k_horizon read instead of their arguments. */
    const int *pf_interval;
    const uint64_t *pf_seeds;
    const DayInfo *pf_days;
    int pf_days_stride;
};

}  // namespace siminf

#endif
