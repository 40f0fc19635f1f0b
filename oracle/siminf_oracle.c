/*
 * siminf_oracle.c -- CPU restatement of SimInf's ssm/mssm day loop and
 * scheduled-event engine.  TEST INFRASTRUCTURE: only the test suite, the
 * smoke check and the CPU-baseline leg of the benchmark load this file's
 * library; the product (siminf_gb300/) never links it.
 *
 * What it restates, in the reference's order of operations:
 *   - rate initialisation          src/solvers/SimInf_solver_ssm.c:96-117
 *   - direct-method SSA per node    src/solvers/SimInf_solver_ssm.c:144-235
 *   - events (E1 then E2, array order, time <= tt)
 *                                   src/solvers/SimInf_solver.c:658-919
 *   - sample_select                 src/solvers/SimInf_solver.c:62-214
 *   - sample_select_enter           src/solvers/SimInf_solver.c:243-324
 *   - post time step + rate refresh src/solvers/SimInf_solver_ssm.c:262-302
 *   - time advance and dense store  src/solvers/SimInf_solver_ssm.c:305-334
 *   - sparse store                  src/solvers/SimInf_solver.c:929-950,
 *                                   src/solvers/SimInf_solver_mssm.c:332-371
 *   - replicate loop (mssm)         src/solvers/SimInf_solver_mssm.c:105-384
 *   - all-events method (aem)       src/solvers/SimInf_solver_aem.c:52-75
 *                                   (calcTimes), :113-158 (initial times),
 *                                   :179-307 (a node's day), :329-381
 *                                   (rate refresh with time rescaling)
 *
 * Random draws come from siminf_stream.h, keyed by (seed, replicate * Nn +
 * node, draw index) instead of one GSL generator per thread, so results do
 * not depend on the thread count.  With sorted events (R/SimInf_events.R:
 * 398) the reference's ssm with any thread count and its mssm process a
 * day's events in array order after the day's SSA, which is what
 * process_events() below does.
 *
 * The SSA, E1 and post-time-step phases run OpenMP-parallel over nodes
 * (one replicate) or over replicates (Nrep > 1), and the external
 * transfers run serially, as in the reference, so that this file doubles
 * as the CPU baseline.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#  include <omp.h>
#endif

#include "../include/siminf_gb300.h"
#include "../siminf_gb300/csrc/siminf_stream.h"
#include "oracle_models.h"

typedef struct oracle_result {
    int error;
    int err_node;
    int err_transition;
    int err_event;
    double err_time;
    double err_rate;
    uint64_t transitions;
    uint64_t node_days;
    uint64_t e1_events;
    uint64_t e2_events;
    double seconds_e2;          /* wall time of the serial E2 phase */
} oracle_result;

typedef struct ev {
    int event, time, node, dest, n;
    double proportion;
    int select, shift;
} ev;

typedef struct ctx {
    const siminf_gpu_solver_args *a;
    const oracle_model *m;
    ev *events;
    int Nn, Nc, Nt, Nd, Nld;
    uint64_t seed;
    int gdata_stride;           /* 0: one gdata; else replicate r uses gdata + r * stride */
    int aem;                    /* all-events method instead of the direct method */
    int crn;                    /* mssm_crn: SSA draws from a stream of their own */
} ctx;

static const double *gdata_of(const ctx *c, int r)
{
    return c->a->gdata + (size_t) r * c->gdata_stride;
}

typedef struct rep {
    int *u;
    double *v, *v_new;
    double *t_rate, *sum_t_rate, *t_time;
    int *update_node;
    uint64_t *ctr;              /* next draw index of each node's stream */
    uint64_t *crn_ctr;          /* mssm_crn: next draw index of its SSA stream */
    int *node_err;              /* per-node error of the current phase */
    double *node_err_time, *node_err_rate;
    int *node_err_tr;
    int error, err_node, err_transition, err_event;
    double err_time, err_rate;
    size_t events_index;
    int *individuals;
    /* aem: per (node, transition) the next event time, the time left
     * when its rate fell to zero, and the draw index of its stream */
    double *react_time, *react_inf;
    uint64_t *react_ctr;
} rep;

static double now_seconds(void)
{
#ifdef _OPENMP
    return omp_get_wtime();
#else
    return 0.0;
#endif
}

static void set_err(rep *s, int code, int node, int tr, int evi, double t, double rate)
{
    s->error = code;
    s->err_node = node;
    s->err_transition = tr;
    s->err_event = evi;
    s->err_time = t;
    s->err_rate = rate;
}

/* ------------------------------------------------------------------ */
/* Direct-method SSA of one node up to next_unit_of_time              */
/* (src/solvers/SimInf_solver_ssm.c:144-235).                          */
/* Returns the number of transitions fired.                            */
/* ------------------------------------------------------------------ */
/* Optional per-(replicate, node) transition counts and per-day maximum
 * over nodes, for workload analysis. */
static uint64_t *g_node_fired = NULL;
static uint64_t *g_day_max = NULL;

static uint64_t ssa_node(const ctx *c, rep *s, int r, int node, double next)
{
    const int Nc = c->Nc, Nt = c->Nt, Nd = c->Nd, Nld = c->Nld;
    const siminf_gpu_solver_args *a = c->a;
    int *u = &s->u[(size_t) node * Nc];
    const double *v = &s->v[(size_t) node * Nd];
    const double *ld = &a->ldata[(size_t) node * Nld];
    double *t_rate = &s->t_rate[(size_t) node * Nt];
    uint64_t fired = 0;
    si_rng rng;

    /* mssm_crn (src/solvers/SimInf_solver_mssm_crn.c:185,196): the two
     * draws of a transition come from a generator per (replicate, node),
     * apart from the one the node's events draw from */
    if (c->crn)
        si_rng_init(&rng, c->seed, SI_CRN_SID | ((uint64_t) r * c->Nn + node), s->crn_ctr[node]);
    else
        si_rng_init(&rng, c->seed, (uint64_t) r * c->Nn + node, s->ctr[node]);
    for (;;) {
        double cum, rand, tau, delta = 0.0;
        int tr;

        if (s->sum_t_rate[node] <= 0.0) {
            s->t_time[node] = next;
            break;
        }
        /* -log(u) of the stream's uniform, by the 32-bit-input logarithm
         * (within 0.54 ulp, like si_log). */
        tau = si_neglog_u32(si_next_u32(&rng)) / s->sum_t_rate[node];
        if ((tau + s->t_time[node]) >= next) {
            s->t_time[node] = next;
            break;
        }
        s->t_time[node] += tau;

        rand = si_uniform_pos(&rng) * s->sum_t_rate[node];
        tr = 0;
        cum = t_rate[0];
        while (tr < Nt && rand > cum) {
            tr++;
            if (tr < Nt)
                cum += t_rate[tr];
        }
        if (tr >= Nt)
            tr = Nt - 1;
        if (t_rate[tr] == 0.0) {
            for (; tr > 0 && t_rate[tr] == 0.0; tr--);
            if (t_rate[tr] == 0.0) {
                s->sum_t_rate[node] = 0.0;
                break;
            }
        }

        fired++;
        for (int j = a->jcS[tr]; j < a->jcS[tr + 1]; j++) {
            u[a->irS[j]] += a->prS[j];
            if (u[a->irS[j]] < 0) {
                s->node_err[node] = SIMINF_GPU_ERR_NEGATIVE_STATE;
                s->node_err_time[node] = s->t_time[node];
                s->node_err_rate[node] = 0;
                s->node_err_tr[node] = tr;
            }
        }

        for (int j = a->jcG[tr]; j < a->jcG[tr + 1]; j++) {
            const int k = a->irG[j];
            const double old = t_rate[k];
            const double rate = c->m->tr[k](u, v, ld, gdata_of(c, r), s->t_time[node]);
            t_rate[k] = rate;
            delta += rate - old;
            if (!isfinite(rate) || rate < 0.0) {
                s->node_err[node] = SIMINF_GPU_ERR_INVALID_RATE;
                s->node_err_time[node] = s->t_time[node];
                s->node_err_rate[node] = rate;
                s->node_err_tr[node] = k;
            }
        }
        s->sum_t_rate[node] += delta;
    }
    if (c->crn)
        s->crn_ctr[node] = rng.ctr;
    else
        s->ctr[node] = rng.ctr;
    if (g_node_fired)
        g_node_fired[(size_t) r * c->Nn + node] += fired;
    return fired;
}

/* ------------------------------------------------------------------ */
/* Event sampling (src/solvers/SimInf_solver.c:62-324).                 */
/* ------------------------------------------------------------------ */
static int g_cap_transfers = 0;

static int sample_select(const siminf_gpu_solver_args *a, int Nc, const int *u,
                         int node, int select, int n, double proportion,
                         int *individuals, si_rng *rng)
{
    const int *irE = a->irE, *jcE = a->jcE;
    const double *prE = a->prE;
    int i, Nstates, Nindividuals = 0, Nkinds = 0;

    memset(individuals, 0, Nc * sizeof(int));
    for (i = jcE[select]; i < jcE[select + 1]; i++) {
        const int nk = u[node * Nc + irE[i]];
        if (nk > 0)
            Nkinds++;
        Nindividuals += nk;
    }
    Nstates = jcE[select + 1] - jcE[select];

    if (n == 0) {
        if (proportion < 0 || proportion > 1)
            return SIMINF_GPU_ERR_INVALID_PROPORTION;
        n = si_binomial(rng, proportion, Nindividuals);
    }
    /* Extension (siminf_gpu_options.cap_transfers): take what is there. */
    if (g_cap_transfers && n > Nindividuals)
        n = Nindividuals;
    if (Nstates <= 0 || n > Nindividuals || n < 0)
        return SIMINF_GPU_ERR_SAMPLE_SELECT;

    if (n == 0)
        return 0;
    if (Nindividuals == n) {
        for (i = jcE[select]; i < jcE[select + 1]; i++)
            individuals[irE[i]] = u[node * Nc + irE[i]];
        return 0;
    }
    if (Nstates == 1) {
        individuals[irE[jcE[select]]] = n;
        return 0;
    }
    if (Nkinds == 1) {
        for (i = jcE[select]; i < jcE[select + 1]; i++) {
            if (u[node * Nc + irE[i]] > 0) {
                individuals[irE[i]] = n;
                break;
            }
        }
        return 0;
    }

    for (i = jcE[select] + 1; i < jcE[select + 1]; i++) {
        if (prE[i] != prE[i - 1])
            goto biased_urn;
    }

    /* Equal weights: sequential multivariate hypergeometric. */
    for (i = jcE[select]; i < jcE[select + 1] - 1; i++) {
        if (n == 0)
            break;
        const int nk = u[node * Nc + irE[i]];
        individuals[irE[i]] = si_hypergeometric(rng, nk, Nindividuals - nk, n);
        Nindividuals -= nk;
        n -= individuals[irE[i]];
    }
    individuals[irE[i]] = n;
    return 0;

biased_urn:
    /* Wallenius' noncentral hypergeometric by an urn with bias. */
    while (n > 0) {
        double rand, cum = 0;
        for (i = jcE[select]; i < jcE[select + 1]; i++)
            cum += prE[i] * (u[node * Nc + irE[i]] - individuals[irE[i]]);
        rand = si_uniform_pos(rng) * cum;
        i = jcE[select];
        cum = prE[i] * (u[node * Nc + irE[i]] - individuals[irE[i]]);
        while (i < jcE[select + 1] && rand > cum) {
            i++;
            if (i < jcE[select + 1])
                cum += prE[i] * (u[node * Nc + irE[i]] - individuals[irE[i]]);
        }
        if (i >= jcE[select + 1])
            i = jcE[select + 1] - 1;
        if ((prE[i] * (u[node * Nc + irE[i]] - individuals[irE[i]])) == 0.0) {
            for (; i > jcE[select] &&
                     (prE[i] * (u[node * Nc + irE[i]] - individuals[irE[i]])) == 0.0;
                 i--);
            if ((prE[i] * (u[node * Nc + irE[i]] - individuals[irE[i]])) == 0.0)
                return SIMINF_GPU_ERR_SAMPLE_SELECT;
        }
        individuals[irE[i]] += 1;
        n--;
    }
    return 0;
}

static int sample_select_enter(const siminf_gpu_solver_args *a, int Nc,
                               const int *u, int node, int select, int n,
                               double proportion, int *individuals, si_rng *rng)
{
    const int *irE = a->irE, *jcE = a->jcE;
    const double *prE = a->prE;
    int i, Nstates = jcE[select + 1] - jcE[select];
    double w_cum = 0;

    memset(individuals, 0, Nc * sizeof(int));
    if (n == 0) {
        if (proportion < 0 || proportion > 1)
            return SIMINF_GPU_ERR_INVALID_PROPORTION;
        for (i = jcE[select]; i < jcE[select + 1]; i++)
            n += u[node * Nc + irE[i]];
        n = si_binomial(rng, proportion, n);
    }
    if (Nstates <= 0 || n < 0)
        return SIMINF_GPU_ERR_SAMPLE_SELECT;
    if (n == 0)
        return 0;
    if (Nstates == 1) {
        individuals[irE[jcE[select]]] = n;
        return 0;
    }
    for (i = jcE[select]; i < jcE[select + 1]; i++)
        w_cum += prE[i];
    while (n > 0) {
        double cum, rand = si_uniform_pos(rng) * w_cum;
        i = jcE[select];
        cum = prE[i];
        while (i < jcE[select + 1] && rand > cum) {
            i++;
            if (i < jcE[select + 1])
                cum += prE[i];
        }
        if (i >= jcE[select + 1])
            i = jcE[select + 1] - 1;
        if (prE[i] == 0.0) {
            for (; i > jcE[select] && prE[i] == 0.0; i--);
            if (prE[i] == 0.0)
                return SIMINF_GPU_ERR_SAMPLE_SELECT;
        }
        individuals[irE[i]] += 1;
        n--;
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* Scheduled events with time <= tt, in array order                     */
/* (src/solvers/SimInf_solver.c:658-919 with process_E2 = 1).           */
/* ------------------------------------------------------------------ */
static void process_events(const ctx *c, rep *s, int r, double tt,
                           oracle_result *res, double *e2_seconds)
{
    const siminf_gpu_solver_args *a = c->a;
    const int Nc = c->Nc, Ntot = c->Nn;
    double t0 = 0.0;
    int in_e2 = 0;

    while (s->events_index < (size_t) a->len && !s->error) {
        const ev *ee = &c->events[s->events_index];
        const int evi = (int) s->events_index;
        int *ind = s->individuals;
        int err;
        si_rng rng;

        if (ee->time > tt)
            break;
        if (ee->node < 0 || ee->node >= Ntot) {
            set_err(s, SIMINF_GPU_ERR_NODE_OUT_OF_BOUNDS, ee->node, -1, evi, tt, 0);
            break;
        }
        if (ee->event == SIMINF_GPU_EXTERNAL_TRANSFER_EVENT && !in_e2) {
            in_e2 = 1;
            t0 = now_seconds();
        }
        si_rng_init(&rng, c->seed, (uint64_t) r * c->Nn + ee->node, s->ctr[ee->node]);

        switch (ee->event) {
        case SIMINF_GPU_EXIT_EVENT:
            err = sample_select(a, Nc, s->u, ee->node, ee->select, ee->n,
                                ee->proportion, ind, &rng);
            if (err) {
                set_err(s, err, ee->node, -1, evi, tt, 0);
                goto done;
            }
            for (int i = a->jcE[ee->select]; i < a->jcE[ee->select + 1]; i++) {
                const int jj = a->irE[i];
                const int kn = ee->node * Nc + jj;
                s->u[kn] -= ind[jj];
                if (s->u[kn] < 0) {
                    set_err(s, SIMINF_GPU_ERR_NEGATIVE_STATE, ee->node, -1, evi, tt, 0);
                    goto done;
                }
            }
            break;

        case SIMINF_GPU_ENTER_EVENT:
            err = sample_select_enter(a, Nc, s->u, ee->node, ee->select, ee->n,
                                      ee->proportion, ind, &rng);
            if (err) {
                set_err(s, err, ee->node, -1, evi, tt, 0);
                goto done;
            }
            for (int i = a->jcE[ee->select]; i < a->jcE[ee->select + 1]; i++) {
                const int jj = a->irE[i];
                const int kn = ee->node * Nc + jj;
                if (ee->shift < 0) {
                    s->u[kn] += ind[jj];
                    if (s->u[kn] < 0) {
                        set_err(s, SIMINF_GPU_ERR_NEGATIVE_STATE, ee->node, -1, evi, tt, 0);
                        goto done;
                    }
                } else if (!a->N) {
                    set_err(s, SIMINF_GPU_ERR_EVENTS_N, ee->node, -1, evi, tt, 0);
                    goto done;
                } else {
                    const int ll = a->N[ee->shift * Nc + jj];
                    if (jj + ll < 0 || jj + ll >= Nc) {
                        set_err(s, SIMINF_GPU_ERR_SHIFT_OUT_OF_BOUNDS, ee->node, -1, evi, tt, 0);
                        goto done;
                    }
                    s->u[kn + ll] += ind[jj];
                    if (s->u[kn + ll] < 0) {
                        set_err(s, SIMINF_GPU_ERR_NEGATIVE_STATE, ee->node, -1, evi, tt, 0);
                        goto done;
                    }
                }
            }
            break;

        case SIMINF_GPU_INTERNAL_TRANSFER_EVENT:
            if (!a->N) {
                set_err(s, SIMINF_GPU_ERR_EVENTS_N, ee->node, -1, evi, tt, 0);
                goto done;
            }
            if (ee->shift < 0) {
                set_err(s, SIMINF_GPU_ERR_EVENT_SHIFT, ee->node, -1, evi, tt, 0);
                goto done;
            }
            err = sample_select(a, Nc, s->u, ee->node, ee->select, ee->n,
                                ee->proportion, ind, &rng);
            if (err) {
                set_err(s, err, ee->node, -1, evi, tt, 0);
                goto done;
            }
            for (int i = a->jcE[ee->select]; i < a->jcE[ee->select + 1]; i++) {
                const int jj = a->irE[i];
                const int kn = ee->node * Nc + jj;
                const int ll = a->N[ee->shift * Nc + jj];
                if (jj + ll < 0 || jj + ll >= Nc) {
                    set_err(s, SIMINF_GPU_ERR_SHIFT_OUT_OF_BOUNDS, ee->node, -1, evi, tt, 0);
                    goto done;
                }
                s->u[kn + ll] += ind[jj];
                if (s->u[kn + ll] < 0) {
                    set_err(s, SIMINF_GPU_ERR_NEGATIVE_STATE, ee->node, -1, evi, tt, 0);
                    goto done;
                }
                s->u[kn] -= ind[jj];
                if (s->u[kn] < 0) {
                    set_err(s, SIMINF_GPU_ERR_NEGATIVE_STATE, ee->node, -1, evi, tt, 0);
                    goto done;
                }
            }
            break;

        case SIMINF_GPU_EXTERNAL_TRANSFER_EVENT:
            if (ee->dest < 0 || ee->dest >= Ntot) {
                set_err(s, SIMINF_GPU_ERR_DEST_OUT_OF_BOUNDS, ee->node, -1, evi, tt, 0);
                goto done;
            }
            err = sample_select(a, Nc, s->u, ee->node, ee->select, ee->n,
                                ee->proportion, ind, &rng);
            if (err) {
                set_err(s, err, ee->node, -1, evi, tt, 0);
                goto done;
            }
            for (int i = a->jcE[ee->select]; i < a->jcE[ee->select + 1]; i++) {
                const int jj = a->irE[i];
                const int kd = ee->dest * Nc + jj;
                const int kn = ee->node * Nc + jj;
                if (ee->shift < 0) {
                    s->u[kd] += ind[jj];
                    if (s->u[kd] < 0) {
                        set_err(s, SIMINF_GPU_ERR_NEGATIVE_STATE, ee->node, -1, evi, tt, 0);
                        goto done;
                    }
                } else if (!a->N) {
                    set_err(s, SIMINF_GPU_ERR_EVENTS_N, ee->node, -1, evi, tt, 0);
                    goto done;
                } else {
                    const int ll = a->N[ee->shift * Nc + jj];
                    if (jj + ll < 0 || jj + ll >= Nc) {
                        set_err(s, SIMINF_GPU_ERR_SHIFT_OUT_OF_BOUNDS, ee->node, -1, evi, tt, 0);
                        goto done;
                    }
                    s->u[kd + ll] += ind[jj];
                    if (s->u[kd + ll] < 0) {
                        set_err(s, SIMINF_GPU_ERR_NEGATIVE_STATE, ee->node, -1, evi, tt, 0);
                        goto done;
                    }
                }
                s->u[kn] -= ind[jj];
                if (s->u[kn] < 0) {
                    set_err(s, SIMINF_GPU_ERR_NEGATIVE_STATE, ee->node, -1, evi, tt, 0);
                    goto done;
                }
            }
            s->update_node[ee->dest] = 1;
            break;

        default:
            set_err(s, SIMINF_GPU_UNDEFINED_EVENT, ee->node, -1, evi, tt, 0);
            break;
        }

        s->ctr[ee->node] = rng.ctr;
        s->update_node[ee->node] = 1;
        if (ee->event == SIMINF_GPU_EXTERNAL_TRANSFER_EVENT)
            res->e2_events++;
        else
            res->e1_events++;
        s->events_index++;
        continue;
done:
        s->ctr[ee->node] = rng.ctr;
        break;
    }
    if (in_e2 && e2_seconds)
        *e2_seconds += now_seconds() - t0;
}

/* Rate refresh of one node after the post-time-step function
 * (src/solvers/SimInf_solver_ssm.c:262-301).  Returns the pts rc. */
static int pts_node(const ctx *c, rep *s, int r, int node, double tt)
{
    const int Nc = c->Nc, Nt = c->Nt, Nd = c->Nd, Nld = c->Nld;
    const siminf_gpu_solver_args *a = c->a;
    const double *gd = gdata_of(c, r);
    const int rc = c->m->pts(&s->v_new[(size_t) node * Nd], &s->u[(size_t) node * Nc],
                             &s->v[(size_t) node * Nd], &a->ldata[(size_t) node * Nld],
                             gd, node, tt);
    if (rc < 0) {
        s->node_err[node] = rc;
        s->node_err_time[node] = tt;
        s->node_err_tr[node] = -1;
        s->node_err_rate[node] = 0;
        return rc;
    }
    if (rc > 0 || s->update_node[node]) {
        double delta = 0.0;
        double *t_rate = &s->t_rate[(size_t) node * Nt];
        for (int j = 0; j < Nt; j++) {
            const double old = t_rate[j];
            const double rate = c->m->tr[j](&s->u[(size_t) node * Nc],
                                            &s->v_new[(size_t) node * Nd],
                                            &a->ldata[(size_t) node * Nld],
                                            gd, tt);
            t_rate[j] = rate;
            delta += rate - old;
            if (!isfinite(rate) || rate < 0.0) {
                s->node_err[node] = SIMINF_GPU_ERR_INVALID_RATE;
                s->node_err_time[node] = tt;
                s->node_err_rate[node] = rate;
                s->node_err_tr[node] = j;
            }
        }
        s->sum_t_rate[node] += delta;
        s->update_node[node] = 0;
    }
    return rc;
}

static void store(const ctx *c, rep *s, int r, int *U_it, int *V_it, double tt)
{
    const siminf_gpu_solver_args *a = c->a;
    const size_t Nn = (size_t) c->Nn, Nc = (size_t) c->Nc, Nd = (size_t) c->Nd;
    const size_t col0 = (size_t) r * a->tlen;

    while (*U_it < a->tlen && tt > a->tspan[*U_it]) {
        if (a->U) {
            memcpy(&a->U[(col0 + *U_it) * Nn * Nc], s->u, Nn * Nc * sizeof(int));
        } else if (a->jcU) {
            for (int j = a->jcU[col0 + *U_it]; j < a->jcU[col0 + *U_it + 1]; j++)
                a->prU[j] = s->u[a->irU[j]];
        }
        (*U_it)++;
    }
    while (*V_it < a->tlen && tt > a->tspan[*V_it]) {
        if (a->V) {
            if (Nd > 0)
                memcpy(&a->V[(col0 + *V_it) * Nn * Nd], s->v_new, Nn * Nd * sizeof(double));
        } else if (a->jcV) {
            for (int j = a->jcV[col0 + *V_it]; j < a->jcV[col0 + *V_it + 1]; j++)
                a->prV[j] = s->v_new[a->irV[j]];
        }
        (*V_it)++;
    }
}

/* Lowest node with an error in the SSA phase decides the code, as with
 * one reference thread: later nodes of that day are not simulated. */
static void resolve_ssa_errors(const ctx *c, rep *s)
{
    for (int node = 0; node < c->Nn; node++) {
        if (s->node_err[node]) {
            set_err(s, s->node_err[node], node, s->node_err_tr[node], -1,
                    s->node_err_time[node], s->node_err_rate[node]);
            return;
        }
    }
}

/* One reference thread walks the post-time-step loop in node order: a
 * negative rc stops it, an invalid rate is recorded and the walk goes on. */
static void resolve_pts_errors(const ctx *c, rep *s)
{
    for (int node = 0; node < c->Nn; node++) {
        const int e = s->node_err[node];
        if (!e)
            continue;
        set_err(s, e, node, s->node_err_tr[node], -1, s->node_err_time[node],
                s->node_err_rate[node]);
        if (e != SIMINF_GPU_ERR_INVALID_RATE)
            return;
    }
}

/* ------------------------------------------------------------------ */
/* All-events method (src/solvers/SimInf_solver_aem.c).                */
/* Transition j of node g draws from its own stream, keyed (seed,      */
/* AEM_SID | (g * Nt + j)), where the reference gives every (node,     */
/* transition) its own generator (:465-481).  The next event is the    */
/* smallest time, the lowest transition among equal times, where the   */
/* reference's binary heap (src/misc/binheap.c) may break an exact tie */
/* the other way.                                                      */
/* ------------------------------------------------------------------ */
#define AEM_SID (1ULL << 63)

static double aem_neglog(const ctx *c, int node, int j, uint64_t *ctr)
{
    si_rng rng;
    si_rng_init(&rng, c->seed, AEM_SID | ((uint64_t) node * c->Nt + j), *ctr);
    const double x = si_neglog_u32(si_next_u32(&rng));
    *ctr = rng.ctr;
    return x;
}

/* calcTimes (src/solvers/SimInf_solver_aem.c:52-75). */
static void aem_calc_times(const ctx *c, int node, int j, double *time, double *inf,
                           double tt, double old_rate, double new_rate, uint64_t *ctr)
{
    const double oldtime = *time;
    if (isinf(oldtime)) {
        if (*inf == 0.0)
            *time = aem_neglog(c, node, j, ctr) / new_rate + tt;
        else if (new_rate > 0.0)
            *time = tt + (*inf / new_rate);
    } else if (new_rate >= DBL_MIN) {
        if (oldtime == tt)
            *time = aem_neglog(c, node, j, ctr) / new_rate + tt;
        else
            *time = ((old_rate / new_rate) * (oldtime - tt)) + tt;
    } else {
        *inf = (oldtime - tt) * old_rate;
        *time = INFINITY;
    }
}

/* A rate of transition j refreshed at time t, then its event time. */
static void aem_refresh(const ctx *c, rep *s, int r, int node, int j, const double *v,
                        double t_rate_time, double t_calc)
{
    const siminf_gpu_solver_args *a = c->a;
    const int Nc = c->Nc, Nt = c->Nt, Nld = c->Nld;
    double *t_rate = &s->t_rate[(size_t) node * Nt];
    const double old = t_rate[j];
    const double rate = c->m->tr[j](&s->u[(size_t) node * Nc], v,
                                    &a->ldata[(size_t) node * Nld], gdata_of(c, r),
                                    t_rate_time);
    t_rate[j] = rate;
    if (!isfinite(rate) || rate < 0.0) {
        s->node_err[node] = SIMINF_GPU_ERR_INVALID_RATE;
        s->node_err_time[node] = t_rate_time;
        s->node_err_rate[node] = rate;
        s->node_err_tr[node] = j;
    }
    const size_t k = (size_t) node * Nt + j;
    aem_calc_times(c, node, j, &s->react_time[k], &s->react_inf[k], t_calc, old, rate,
                   &s->react_ctr[k]);
}

/* Initial rates and event times (src/solvers/SimInf_solver_aem.c:113-158). */
static int aem_init_node(const ctx *c, rep *s, int r, int node, double tt)
{
    const siminf_gpu_solver_args *a = c->a;
    const int Nc = c->Nc, Nt = c->Nt, Nd = c->Nd, Nld = c->Nld;
    int err = 0;
    for (int j = 0; j < Nt; j++) {
        const double rate = c->m->tr[j](&s->u[(size_t) node * Nc], &s->v[(size_t) node * Nd],
                                        &a->ldata[(size_t) node * Nld], gdata_of(c, r), tt);
        const size_t k = (size_t) node * Nt + j;
        s->t_rate[k] = rate;
        if (!isfinite(rate) || rate < 0.0) {
            s->node_err[node] = SIMINF_GPU_ERR_INVALID_RATE;
            s->node_err_time[node] = tt;
            s->node_err_rate[node] = rate;
            s->node_err_tr[node] = j;
            err = 1;
        }
        s->react_ctr[k] = 0;
        s->react_inf[k] = 0.0;
        s->react_time[k] = aem_neglog(c, node, j, &s->react_ctr[k]) / rate + tt;
        if (s->react_time[k] <= 0.0)
            s->react_time[k] = INFINITY;
    }
    s->t_time[node] = tt;
    return err;
}

/* One node's day (src/solvers/SimInf_solver_aem.c:179-307).  Returns the
 * number of transitions fired. */
static uint64_t aem_node(const ctx *c, rep *s, int r, int node, double next)
{
    const siminf_gpu_solver_args *a = c->a;
    const int Nc = c->Nc, Nt = c->Nt, Nd = c->Nd;
    int *u = &s->u[(size_t) node * Nc];
    const double *v = &s->v[(size_t) node * Nd];
    const double *times = &s->react_time[(size_t) node * Nt];
    uint64_t fired = 0;
    for (;;) {
        int tr = 0;
        double t = times[0];
        for (int j = 1; j < Nt; j++) {
            if (times[j] < t) {
                t = times[j];
                tr = j;
            }
        }
        s->t_time[node] = t;
        if (isinf(t) || t >= next) {
            s->t_time[node] = next;
            break;
        }
        fired++;
        for (int j = a->jcS[tr]; j < a->jcS[tr + 1]; j++) {
            u[a->irS[j]] += a->prS[j];
            if (u[a->irS[j]] < 0) {
                s->node_err[node] = SIMINF_GPU_ERR_NEGATIVE_STATE;
                s->node_err_time[node] = t;
                s->node_err_rate[node] = 0;
                s->node_err_tr[node] = tr;
            }
        }
        for (int ii = a->jcG[tr]; ii < a->jcG[tr + 1]; ii++) {
            const int j = a->irG[ii];
            if (j != tr)
                aem_refresh(c, s, r, node, j, v, t, t);
        }
        aem_refresh(c, s, r, node, tr, v, t, t);
    }
    if (g_node_fired)
        g_node_fired[(size_t) r * c->Nn + node] += fired;
    return fired;
}

/* Post time step and, where needed, every rate refreshed with v_new at tt
 * and its event time rescaled at the node's time
 * (src/solvers/SimInf_solver_aem.c:329-381).  Returns the pts rc. */
static int aem_pts_node(const ctx *c, rep *s, int r, int node, double tt)
{
    const siminf_gpu_solver_args *a = c->a;
    const int Nc = c->Nc, Nt = c->Nt, Nd = c->Nd, Nld = c->Nld;
    const int rc = c->m->pts(&s->v_new[(size_t) node * Nd], &s->u[(size_t) node * Nc],
                             &s->v[(size_t) node * Nd], &a->ldata[(size_t) node * Nld],
                             gdata_of(c, r), node, tt);
    if (rc < 0) {
        s->node_err[node] = rc;
        s->node_err_time[node] = tt;
        s->node_err_tr[node] = -1;
        s->node_err_rate[node] = 0;
        return rc;
    }
    if (rc > 0 || s->update_node[node]) {
        for (int j = 0; j < Nt; j++)
            aem_refresh(c, s, r, node, j, &s->v_new[(size_t) node * Nd], tt, s->t_time[node]);
        s->update_node[node] = 0;
    }
    return rc;
}

static int run_replicate(const ctx *c, rep *s, int r, int parallel_nodes,
                         oracle_result *res)
{
    const siminf_gpu_solver_args *a = c->a;
    const int Nn = c->Nn, Nc = c->Nc, Nt = c->Nt, Nd = c->Nd, Nld = c->Nld;
    double tt = a->tspan[0];
    double next = floor(tt) + 1.0;
    int U_it = 0, V_it = 0;
    uint64_t fired = 0;
    int any_err = 0;
    int day = 0;

    memcpy(s->u, &a->u0[(size_t) r * Nn * Nc], (size_t) Nn * Nc * sizeof(int));
    if (Nd > 0) {
        memcpy(s->v, &a->v0[(size_t) r * Nn * Nd], (size_t) Nn * Nd * sizeof(double));
        memcpy(s->v_new, &a->v0[(size_t) r * Nn * Nd], (size_t) Nn * Nd * sizeof(double));
    }
    memset(s->update_node, 0, Nn * sizeof(int));
    memset(s->ctr, 0, Nn * sizeof(uint64_t));
    memset(s->crn_ctr, 0, Nn * sizeof(uint64_t));
    memset(s->node_err, 0, Nn * sizeof(int));
    s->error = 0;
    s->events_index = 0;

    /* Rates at the start (src/solvers/SimInf_solver_ssm.c:96-117). */
#pragma omp parallel for schedule(static) if (parallel_nodes) reduction(|:any_err)
    for (int node = 0; node < Nn; node++) {
        if (c->aem) {
            any_err |= aem_init_node(c, s, r, node, tt);
            continue;
        }
        s->sum_t_rate[node] = 0.0;
        for (int j = 0; j < Nt; j++) {
            const double rate = c->m->tr[j](&s->u[(size_t) node * Nc], &s->v[(size_t) node * Nd],
                                            &a->ldata[(size_t) node * Nld], gdata_of(c, r), tt);
            s->t_rate[(size_t) node * Nt + j] = rate;
            s->sum_t_rate[node] += rate;
            if (!isfinite(rate) || rate < 0.0) {
                s->node_err[node] = SIMINF_GPU_ERR_INVALID_RATE;
                s->node_err_time[node] = tt;
                s->node_err_rate[node] = rate;
                s->node_err_tr[node] = j;
                any_err = 1;
            }
        }
        s->t_time[node] = tt;
    }
    if (any_err) {
        /* Every node is initialised; the last failing node's message is
         * printed last, the code is the same for all. */
        resolve_ssa_errors(c, s);
        return s->error;
    }

    for (;;) {
        /* (1) SSA per node. */
        any_err = 0;
        uint64_t day_max = 0;
#pragma omp parallel for schedule(static) if (parallel_nodes) reduction(+:fired) reduction(|:any_err) reduction(max:day_max)
        for (int node = 0; node < Nn; node++) {
            const uint64_t f = c->aem ? aem_node(c, s, r, node, next)
                                      : ssa_node(c, s, r, node, next);
            fired += f;
            if (f > day_max)
                day_max = f;
            any_err |= (s->node_err[node] != 0);
        }
        if (g_day_max && r == 0)
            g_day_max[day] = day_max;
        day++;
        res->node_days += (uint64_t) Nn;
        if (any_err)
            resolve_ssa_errors(c, s);

        /* (2, 3) Scheduled events. */
        process_events(c, s, r, tt, res, &res->seconds_e2);

        /* (4) Post time step and rate refresh for every node. */
        memset(s->node_err, 0, Nn * sizeof(int));
        any_err = 0;
#pragma omp parallel for schedule(static) if (parallel_nodes) reduction(|:any_err)
        for (int node = 0; node < Nn; node++) {
            if (c->aem)
                aem_pts_node(c, s, r, node, tt);
            else
                pts_node(c, s, r, node, tt);
            any_err |= (s->node_err[node] != 0);
        }
        if (any_err)
            resolve_pts_errors(c, s);

        /* (5) Advance time, (6) store. */
        tt = next;
        next += 1.0;
        store(c, s, r, &U_it, &V_it, tt);

        double *tmp = s->v;
        s->v = s->v_new;
        s->v_new = tmp;

        if (s->error)
            break;
        if (U_it >= a->tlen)
            break;
    }
    res->transitions += fired;
    return s->error;
}

static int rep_alloc(rep *s, int Nn, int Nc, int Nt, int Nd)
{
    memset(s, 0, sizeof(*s));
    s->u = malloc((size_t) Nn * Nc * sizeof(int) + 1);
    s->v = malloc((size_t) Nn * Nd * sizeof(double) + 8);
    s->v_new = malloc((size_t) Nn * Nd * sizeof(double) + 8);
    s->t_rate = malloc((size_t) Nn * Nt * sizeof(double) + 8);
    s->sum_t_rate = malloc((size_t) Nn * sizeof(double) + 8);
    s->t_time = malloc((size_t) Nn * sizeof(double) + 8);
    s->update_node = malloc((size_t) Nn * sizeof(int) + 4);
    s->ctr = malloc((size_t) Nn * sizeof(uint64_t) + 8);
    s->crn_ctr = malloc((size_t) Nn * sizeof(uint64_t) + 8);
    s->node_err = malloc((size_t) Nn * sizeof(int) + 4);
    s->node_err_time = malloc((size_t) Nn * sizeof(double) + 8);
    s->node_err_rate = malloc((size_t) Nn * sizeof(double) + 8);
    s->node_err_tr = malloc((size_t) Nn * sizeof(int) + 4);
    s->individuals = malloc((size_t) Nc * sizeof(int) + 4);
    s->react_time = malloc((size_t) Nn * Nt * sizeof(double) + 8);
    s->react_inf = malloc((size_t) Nn * Nt * sizeof(double) + 8);
    s->react_ctr = malloc((size_t) Nn * Nt * sizeof(uint64_t) + 8);
    return (s->react_time && s->react_inf && s->react_ctr && s->u && s->v && s->v_new && s->t_rate && s->sum_t_rate && s->t_time &&
            s->update_node && s->ctr && s->crn_ctr && s->node_err && s->node_err_time &&
            s->node_err_rate && s->node_err_tr && s->individuals) ? 0 : -1;
}

static void rep_free(rep *s)
{
    free(s->u); free(s->v); free(s->v_new); free(s->t_rate); free(s->sum_t_rate);
    free(s->t_time); free(s->update_node); free(s->ctr); free(s->crn_ctr); free(s->node_err);
    free(s->node_err_time); free(s->node_err_rate); free(s->node_err_tr);
    free(s->individuals);
    free(s->react_time); free(s->react_inf); free(s->react_ctr);
}

/*
 * Run every replicate of args with the named host model.  nthreads <= 0
 * uses the OpenMP default; cap_transfers mirrors siminf_gpu_options.  Returns 0 or the first failing replicate's
 * error code; res receives counters and the failure's diagnostics.
 */
static int oracle_run_impl(const siminf_gpu_solver_args *args, const char *model_name,
                           int nthreads, int cap_transfers, int gdata_stride,
                           oracle_result *res)
{
    ctx c;
    int err = 0;

    g_cap_transfers = cap_transfers;
    c.gdata_stride = gdata_stride;

    memset(res, 0, sizeof(*res));
    c.m = oracle_model_lookup(model_name);
    if (!c.m)
        return SIMINF_GPU_ERR_UNKNOWN_MODEL;
    if (args->Nc != c.m->Nc || args->Nt != c.m->Nt || args->Nd != c.m->Nd)
        return SIMINF_GPU_ERR_INVALID_MODEL;
    c.a = args;
    c.Nn = args->Nn;
    c.Nc = args->Nc;
    c.Nt = args->Nt;
    c.Nd = args->Nd;
    c.Nld = args->Nld;
    c.seed = (uint64_t) args->seed;
    c.aem = args->solver == 1;
    if (args->solver != 0 && args->solver != 1)
        return SIMINF_GPU_ERR_UNKNOWN_SOLVER;
    if (c.aem && args->Nrep > 1)
        return SIMINF_GPU_ERR_AEM_REPLICATED_MODEL;  /* src/SimInf.c:393-396 */
    /* crn selects SimInf_run_solver_mssm_crn for replicated models only
     * (src/SimInf.c:385-389) */
    c.crn = !c.aem && args->Nrep > 1 && args->crn == 1;
#ifdef _OPENMP
    if (nthreads > 0)
        omp_set_num_threads(nthreads);
#else
    (void) nthreads;
#endif

    /* Zero-based events (src/solvers/SimInf_solver.c:371-374). */
    c.events = malloc(((size_t) args->len + 1) * sizeof(ev));
    if (!c.events)
        return SIMINF_GPU_ERR_ALLOC_MEMORY_BUFFER;
    for (int i = 0; i < args->len; i++) {
        ev e = {args->event[i], args->time[i], args->node[i] - 1, args->dest[i] - 1,
                args->n[i], args->proportion[i], args->select[i] - 1, args->shift[i] - 1};
        c.events[i] = e;
    }

    const int Nrep = args->Nrep > 0 ? args->Nrep : 1;
    if (Nrep == 1) {
        rep s;
        if (rep_alloc(&s, c.Nn, c.Nc, c.Nt, c.Nd)) {
            rep_free(&s);
            free(c.events);
            return SIMINF_GPU_ERR_ALLOC_MEMORY_BUFFER;
        }
        err = run_replicate(&c, &s, 0, 1, res);
        if (err) {
            res->err_node = s.err_node;
            res->err_transition = s.err_transition;
            res->err_event = s.err_event;
            res->err_time = s.err_time;
            res->err_rate = s.err_rate;
        }
        rep_free(&s);
    } else {
        int *errs = calloc((size_t) Nrep, sizeof(int));
        oracle_result *rr = calloc((size_t) Nrep, sizeof(oracle_result));
        rep *ss = calloc((size_t) Nrep, sizeof(rep));
#pragma omp parallel for schedule(dynamic, 1)
        for (int r = 0; r < Nrep; r++) {
            if (rep_alloc(&ss[r], c.Nn, c.Nc, c.Nt, c.Nd)) {
                errs[r] = SIMINF_GPU_ERR_ALLOC_MEMORY_BUFFER;
            } else {
                errs[r] = run_replicate(&c, &ss[r], r, 0, &rr[r]);
                rr[r].err_node = ss[r].err_node;
                rr[r].err_transition = ss[r].err_transition;
                rr[r].err_event = ss[r].err_event;
                rr[r].err_time = ss[r].err_time;
                rr[r].err_rate = ss[r].err_rate;
            }
            rep_free(&ss[r]);
        }
        for (int r = 0; r < Nrep; r++) {
            res->transitions += rr[r].transitions;
            res->node_days += rr[r].node_days;
            res->e1_events += rr[r].e1_events;
            res->e2_events += rr[r].e2_events;
            res->seconds_e2 += rr[r].seconds_e2;
            if (!err && errs[r]) {
                err = errs[r];
                res->err_node = rr[r].err_node;
                res->err_transition = rr[r].err_transition;
                res->err_event = rr[r].err_event;
                res->err_time = rr[r].err_time;
                res->err_rate = rr[r].err_rate;
            }
        }
        free(errs);
        free(rr);
        free(ss);
    }
    free(c.events);
    res->error = err;
    return err;
}

int oracle_run_ex(const siminf_gpu_solver_args *args, const char *model_name,
                  int nthreads, int cap_transfers, oracle_result *res)
{
    return oracle_run_impl(args, model_name, nthreads, cap_transfers, 0, res);
}

int oracle_run(const siminf_gpu_solver_args *args, const char *model_name,
               int nthreads, oracle_result *res)
{
    return oracle_run_ex(args, model_name, nthreads, 0, res);
}

/* ------------------------------------------------------------------ */
/* Bootstrap particle filter (R/pfilter.R:315-499) over one model whose   */
/* replicates are the particles, with a Binomial(count, p) observation of */
/* one compartment per node.                                            */
/* ------------------------------------------------------------------ */

/* ln Binomial(k; n, p) from a log-factorial table, with a floor for
 * impossible observations (the reference rejects non-finite weights,
 * R/pfilter.R:438-442).  The same expression runs on the GPU. */
#define PF_LOG_FLOOR (-690.0)
static double pf_logdens(const double *lfact, int tablen, int k, int n, double logp, double logq)
{
    if (k < 0 || n < 0 || k > n || n >= tablen)
        return PF_LOG_FLOOR;
    return (((lfact[n] - lfact[k]) - lfact[n - k]) + (double) k * logp) +
           (double) (n - k) * logq;
}

/* Systematic resampling, src/misc/SimInf_particle_filter.c:33-67, with the
 * uniform from the stream (seed, sid); idx receives zero-based ancestors. */
static int pf_resample(const double *w, int n, double unif, int *idx)
{
    double cumsum_w = 0;
    for (int i = 0; i < n; i++) {
        if (!isfinite(w[i]) || w[i] < 0.0)
            return -1;
        cumsum_w += w[i];
    }
    if (cumsum_w <= 0.0)
        return -1;
    const double du = cumsum_w / (double) n;
    double u = du * unif;
    cumsum_w = w[0];
    for (int i = 0, j = 0; i < n; i++) {
        while (u > cumsum_w && j < n - 1)
            cumsum_w += w[++j];
        idx[i] = j;
        u += du;
    }
    return 0;
}

/* pf_resample on its own, with one-based ancestors as the reference's
 * function returns them; -1 on invalid weights. */
int oracle_systematic_resampling(const double *w, int n, double unif, int *idx)
{
    if (pf_resample(w, n, unif, idx))
        return -1;
    for (int i = 0; i < n; i++)
        idx[i] += 1;
    return 0;
}

/* Seeds of interval i and of its resampling draw. */
#define PF_SEED(seed, i) ((uint64_t) (seed) + ((uint64_t) (i) + 1) * 0x9E3779B97F4A7C15ULL)
#define PF_RESAMPLE_SID (((uint64_t) 1) << 62)

int oracle_pfilter(const siminf_gpu_solver_args *a1, const char *model_name, int Np,
                   int gdata_stride, int n_obs, const int *obs_time, const int *obs,
                   int obs_c, double p_detect, uint64_t seed, int nthreads,
                   double *loglik_out, double *ess, int *ancestors)
{
    const int Nn = a1->Nn, Nc = a1->Nc, Nd = a1->Nd;
    const size_t nu = (size_t) Nn * Nc, nv = (size_t) Nn * Nd;
    int err = 0, tablen = 1;
    for (int node = 0; node < Nn; node++) {
        int tot = 0;
        for (int c = 0; c < Nc; c++)
            tot += a1->u0[(size_t) node * Nc + c];
        if (tot + 1 > tablen)
            tablen = tot + 1;
    }
    double *lfact = malloc((size_t) tablen * sizeof(double));
    int *u0 = malloc((size_t) Np * nu * sizeof(int) + 4);
    double *v0 = malloc((size_t) Np * nv * sizeof(double) + 8);
    int *U = malloc((size_t) Np * 2 * nu * sizeof(int) + 4);
    double *V = malloc((size_t) Np * 2 * nv * sizeof(double) + 8);
    int *ulast = malloc((size_t) Np * nu * sizeof(int) + 4);
    double *vlast = malloc((size_t) Np * nv * sizeof(double) + 8);
    double *w = malloc((size_t) Np * sizeof(double));
    int *anc = malloc((size_t) Np * sizeof(int));
    si_lfact_fill(lfact, tablen);
    for (int p = 0; p < Np; p++) {
        memcpy(&u0[p * nu], a1->u0, nu * sizeof(int));
        if (nv)
            memcpy(&v0[p * nv], a1->v0, nv * sizeof(double));
        anc[p] = p;
    }
    const double logp = si_log(p_detect), logq = si_log(1.0 - p_detect);
    const double log_np = si_log((double) Np);
    double loglik = 0.0;
    for (int i = 0; i < n_obs && !err; i++) {
        /* interval tspan, R/pfilter.R:177-193 */
        double tsp[2];
        int tlen;
        const double prev = (i == 0) ? a1->tspan[0] : (double) obs_time[i - 1];
        if ((i == 0 && prev < obs_time[0]) || (i > 0 && obs_time[i] - obs_time[i - 1] > 1)) {
            tsp[0] = prev;
            tsp[1] = obs_time[i];
            tlen = 2;
        } else {
            tsp[0] = obs_time[i];
            tlen = 1;
        }
        /* ancestors' states: u0[p] = last[anc[p]] (R/pfilter.R:384-398) */
        if (i > 0) {
            for (int p = 0; p < Np; p++) {
                memcpy(&u0[p * nu], &ulast[(size_t) anc[p] * nu], nu * sizeof(int));
                if (nv)
                    memcpy(&v0[p * nv], &vlast[(size_t) anc[p] * nv], nv * sizeof(double));
            }
        }
        siminf_gpu_solver_args a = *a1;
        a.u0 = u0;
        a.v0 = v0;
        a.tspan = tsp;
        a.tlen = tlen;
        a.U = U;
        a.V = V;
        a.Nrep = Np;
        a.len = 0;
        a.seed = PF_SEED(seed, i);
        oracle_result res;
        err = oracle_run_impl(&a, model_name, nthreads, 0, gdata_stride, &res);
        if (err)
            break;
        for (int p = 0; p < Np; p++) {
            memcpy(&ulast[p * nu], &U[((size_t) p * tlen + tlen - 1) * nu], nu * sizeof(int));
            if (nv)
                memcpy(&vlast[p * nv], &V[((size_t) p * tlen + tlen - 1) * nv], nv * sizeof(double));
        }
        /* log-weights: sum over nodes in order */
        for (int p = 0; p < Np; p++) {
            double acc = 0.0;
            for (int node = 0; node < Nn; node++)
                acc = acc + pf_logdens(lfact, tablen, obs[(size_t) i * Nn + node],
                                       ulast[(size_t) p * nu + (size_t) node * Nc + obs_c], logp, logq);
            w[p] = acc;
        }
        /* R/pfilter.R:444-452 */
        double max_w = w[0];
        for (int p = 1; p < Np; p++)
            if (w[p] > max_w)
                max_w = w[p];
        double sum_w = 0.0;
        for (int p = 0; p < Np; p++) {
            w[p] = si_exp(w[p] - max_w);
            sum_w = sum_w + w[p];
        }
        loglik = ((loglik + max_w) + si_log(sum_w)) - log_np;
        double sq = 0.0;
        for (int p = 0; p < Np; p++) {
            w[p] = w[p] / sum_w;
            sq = sq + w[p] * w[p];
        }
        ess[i] = 1.0 / sq;
        si_rng rr;
        si_rng_init(&rr, seed, PF_RESAMPLE_SID + (uint64_t) i, 0);
        if (pf_resample(w, Np, si_uniform_pos(&rr), anc)) {
            err = SIMINF_GPU_ERR_INVALID_MODEL;
            break;
        }
        if (ancestors)
            for (int p = 0; p < Np; p++)
                ancestors[(size_t) i * Np + p] = anc[p] + 1;
    }
    *loglik_out = loglik;
    free(lfact); free(u0); free(v0); free(U); free(V); free(ulast); free(vlast);
    free(w); free(anc);
    return err;
}

/* Set (or clear with NULL) a caller-owned array of Nrep * Nn counters that
 * accumulates the transitions each node fires. */
void oracle_set_node_counters(uint64_t *counts)
{
    g_node_fired = counts;
}

/* Set (or clear) a caller-owned array, one entry per day, that receives the
 * largest number of transitions any node of replicate 0 fired that day. */
void oracle_set_day_max(uint64_t *day_max)
{
    g_day_max = day_max;
}

/* ------------------------------------------------------------------ */
/* Wrappers of the shared random source, for the test suite.            */
/* ------------------------------------------------------------------ */
double oracle_si_log(double x) { return si_log(x); }

void oracle_neglog_u32(const uint32_t *w, double *out, int64_t n)
{
    for (int64_t i = 0; i < n; i++)
        out[i] = si_neglog_u32(w[i]);
}

void oracle_philox(uint32_t *ctr4, uint32_t k0, uint32_t k1)
{
    si_philox4x32_10(&ctr4[0], &ctr4[1], &ctr4[2], &ctr4[3], k0, k1);
}

void oracle_uniform_pos(uint64_t seed, uint64_t sid, uint64_t ctr, int n, double *out)
{
    si_rng r;
    si_rng_init(&r, seed, sid, ctr);
    for (int i = 0; i < n; i++)
        out[i] = si_uniform_pos(&r);
}

void oracle_hypergeometric(uint64_t seed, uint64_t sid, int n1, int n2, int t,
                           int count, int *out)
{
    si_rng r;
    si_rng_init(&r, seed, sid, 0);
    for (int i = 0; i < count; i++)
        out[i] = si_hypergeometric(&r, n1, n2, t);
}

void oracle_binomial(uint64_t seed, uint64_t sid, double p, int n, int count, int *out)
{
    si_rng r;
    si_rng_init(&r, seed, sid, 0);
    for (int i = 0; i < count; i++)
        out[i] = si_binomial(&r, p, n);
}

int oracle_result_size(void) { return (int) sizeof(oracle_result); }
int oracle_args_size(void) { return (int) sizeof(siminf_gpu_solver_args); }
