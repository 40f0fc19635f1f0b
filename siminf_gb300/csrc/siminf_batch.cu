/*
 * siminf_batch.cu -- siminf_gpu_run_batch: many independent models of one
 * device model (different node counts, tspan lengths, events, parameters
 * and seeds) run as one plan, with each model's prevalence series and its
 * L2 distance to a target reduced on the device.
 *
 * Replaces the loop of the reference's ABC samplers, which run one
 * simulation per proposal and compute the distance on the host
 * (R/abc.R:589-628 with gdata proposals, :675-729 with ldata proposals).
 * Here the models' nodes are laid end to end: the merged plan runs the
 * longest model's days, the kernels skip a model's nodes once its days are
 * over, and every node draws from the stream keyed by its own model's seed
 * and its index within that model, so each model's trajectory is the one
 * it has when run alone (siminf_gpu_run_solver_ssm with that seed).
 *
 * Events of the models are merged into one schedule by (time, E1 before
 * E2), keeping each model's own order; the models touch disjoint nodes, so
 * the merged order changes no model's result.  An error in any model stops
 * the batch; the status names the model and its local node.
 */
#include <algorithm>
#include <atomic>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/siminf_gb300.h"
#include "siminf_capi_internal.h"

using namespace siminf;

namespace {

/* Prevalence num/den of every stored column of every model (den 0 gives
 * 0) and the L2 distance to the model's target, summed over columns in
 * order: the same IEEE operations as the host restatement. */
__global__ void k_batch_distance(const unsigned long long *prev, const long long *col0,
                                 const int *tlen, const double *target, const int *has_target,
                                 int njobs, double *prevalence, double *distance)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= njobs)
        return;
    double acc = 0.0;
    for (int col = 0; col < tlen[j]; col++) {
        const long long k = col0[j] + col;
        const unsigned long long num = prev[2 * k], den = prev[2 * k + 1];
        const double p = den ? (double) num / (double) den : 0.0;
        prevalence[k] = p;
        if (has_target[j]) {
            const double d = p - target[k];
            acc = acc + d * d;
        }
    }
    distance[j] = has_target[j] ? sqrt(acc) : 0.0;
}

int fail(int code, const char *msg)
{
    capi_set_status(code, -1, -1, -1, 0, 0, msg);
    return code;
}

/* Columns of E (and of N) that a model's events use. */
void used_columns(const siminf_gpu_solver_args *a, int &nsel, int &nshift)
{
    nsel = 0;
    nshift = 0;
    for (int i = 0; i < a->len; i++) {
        nsel = std::max(nsel, a->select[i]);
        nshift = std::max(nshift, a->shift[i]);
    }
}

}  // namespace

extern "C" int siminf_gpu_run_batch(siminf_gpu_batch_job *jobs, int njobs,
                                    const siminf_gpu_model *model,
                                    const siminf_gpu_batch_options *opt)
{
    capi_clear_status();
    const auto t0 = std::chrono::steady_clock::now();
    auto ms_since = [](std::chrono::steady_clock::time_point a) {
        return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - a)
            .count();
    };
    if (!jobs || njobs < 1 || !model || !model->L)
        return fail(SIMINF_GPU_ERR_INVALID_MODEL, "no jobs or no device model");
    const Launchers *L = model->L;
    const int Nc = L->Nc, Nd = L->Nd;
    char msg[256];

    /* Check every model; find the longest tspan and the reference E/N. */
    int longest = 0, eref = -1, eref_sel = 0, nref = -1, nref_shift = 0;
    for (int j = 0; j < njobs; j++) {
        siminf_gpu_solver_args a = jobs[j].args ? *jobs[j].args : siminf_gpu_solver_args{};
        static int stand_in;
        a.U = &stand_in;                       /* the batch writes no U */
        int rc = jobs[j].args ? capi_validate(&a, L) : SIMINF_GPU_ERR_INVALID_MODEL;
        if (!rc && a.solver != 0) {
            capi_set_status(SIMINF_GPU_ERR_UNKNOWN_SOLVER, -1, -1, -1, 0, 0,
                            "a batch runs the ssm solver");
            rc = SIMINF_GPU_ERR_UNKNOWN_SOLVER;
        }
        /* a post-time-step that reads other nodes indexes them within its
         * own model, which a batch's node numbering does not keep */
        if (!rc && (a.Nrep != 1 || a.Nld != jobs[0].args->Nld || !L->pts_local))
            rc = SIMINF_GPU_ERR_INVALID_MODEL;
        if (rc) {
            snprintf(msg, sizeof(msg), "batch job %d: not a valid one-replicate model like job 0",
                     j);
            return fail(rc, msg);
        }
        if (a.tspan[0] != jobs[0].args->tspan[0]) {
            snprintf(msg, sizeof(msg), "batch job %d: tspan starts at %g, job 0 at %g", j,
                     a.tspan[0], jobs[0].args->tspan[0]);
            return fail(SIMINF_GPU_ERR_INVALID_MODEL, msg);
        }
        if (a.tlen > jobs[longest].args->tlen)
            longest = j;
        if (a.len > 0) {
            int ns, nh;
            used_columns(&a, ns, nh);
            if (eref < 0 || ns > eref_sel) {
                eref = j;
                eref_sel = ns;
            }
            if (a.N && (nref < 0 || nh > nref_shift)) {
                nref = j;
                nref_shift = nh;
            }
        }
    }
    const siminf_gpu_solver_args *T = jobs[longest].args;
    for (int j = 0; j < njobs; j++) {
        const siminf_gpu_solver_args *a = jobs[j].args;
        for (int k = 0; k < a->tlen; k++)
            if (a->tspan[k] != T->tspan[k]) {
                snprintf(msg, sizeof(msg),
                         "batch job %d: tspan is not a prefix of the longest one's", j);
                return fail(SIMINF_GPU_ERR_INVALID_MODEL, msg);
            }
        if (a->len > 0) {
            /* the models share E and N: compare the columns this one uses */
            const siminf_gpu_solver_args *E = jobs[eref].args;
            int ns, nh;
            used_columns(a, ns, nh);
            bool same = a->jcE[0] == E->jcE[0];
            for (int c = 0; same && c < ns; c++) {
                same = a->jcE[c + 1] == E->jcE[c + 1];
                for (int k = a->jcE[c]; same && k < a->jcE[c + 1]; k++)
                    same = a->irE[k] == E->irE[k] && a->prE[k] == E->prE[k];
            }
            if (same && nh > 0 && a->N) {
                const siminf_gpu_solver_args *Nr = jobs[nref].args;
                for (int k = 0; same && k < nh * Nc; k++)
                    same = a->N[k] == Nr->N[k];
            }
            if (!same) {
                snprintf(msg, sizeof(msg), "batch job %d: its E or N differs from the others'",
                         j);
                return fail(SIMINF_GPU_ERR_INVALID_MODEL, msg);
            }
        }
    }

    /* Node offsets, days, columns. */
    std::vector<long long> node0(njobs + 1, 0), col0(njobs + 1, 0);
    std::vector<int> ndays(njobs), tlen(njobs), has_target(njobs);
    std::vector<uint64_t> seeds(njobs);
    for (int j = 0; j < njobs; j++) {
        const siminf_gpu_solver_args *a = jobs[j].args;
        node0[j + 1] = node0[j] + a->Nn;
        col0[j + 1] = col0[j] + a->tlen;
        std::vector<DayInfo> days;
        if (plan_days(a->tspan, a->tlen, days))
            return fail(SIMINF_GPU_ERR_INVALID_MODEL, "tspan too long");
        ndays[j] = (int) days.size();
        tlen[j] = a->tlen;
        seeds[j] = (uint64_t) a->seed;
        has_target[j] = jobs[j].target != nullptr;
    }
    const long long Ntot = node0[njobs];
    if (Ntot > INT_MAX)
        return fail(SIMINF_GPU_ERR_INVALID_MODEL, "batch has more than 2^31 nodes");
    const double tt0 = T->tspan[0];
    auto event_day = [tt0](int time) -> long long {
        return (double) time <= tt0 ? 0 : (long long) time - (long long) std::floor(tt0);
    };

    /* Merged inputs. */
    const int Nld = T->Nld;
    std::vector<int> u0((size_t) Ntot * Nc), job_of((size_t) Ntot);
    std::vector<double> v0((size_t) Ntot * Nd + 1), ldata((size_t) Ntot * (Nld > 0 ? Nld : 0) + 1);
    std::vector<double> gdata((size_t) njobs * (L->Ngd > 0 ? L->Ngd : 1), 0.0);
    for (int j = 0; j < njobs; j++) {
        const siminf_gpu_solver_args *a = jobs[j].args;
        const size_t n = (size_t) a->Nn;
        memcpy(&u0[(size_t) node0[j] * Nc], a->u0, n * Nc * sizeof(int));
        if (Nd > 0)
            memcpy(&v0[(size_t) node0[j] * Nd], a->v0, n * Nd * sizeof(double));
        if (Nld > 0)
            memcpy(&ldata[(size_t) node0[j] * Nld], a->ldata, n * Nld * sizeof(double));
        if (L->Ngd > 0 && a->gdata)
            memcpy(&gdata[(size_t) j * L->Ngd], a->gdata, (size_t) L->Ngd * sizeof(double));
        std::fill(job_of.begin() + node0[j], job_of.begin() + node0[j + 1], j);
    }

    /* Events: stable counting sort by (time, E2 after E1), each model's own
     * order kept, events past a model's horizon dropped.  Keys are counted
     * per model on host threads, offsets run key-major then model-major,
     * and every model then writes its own events. */
    const int nthreads = std::max(1, std::min(njobs, (int) std::thread::hardware_concurrency()));
    std::vector<int> jmin(njobs, INT_MAX), jmax(njobs, INT_MIN), jbad(njobs, 0);
    std::vector<long long> jcount(njobs, 0);
    auto for_jobs = [&](auto &&f) {
        std::atomic<int> next(0);
        std::vector<std::thread> th;
        for (int t = 0; t < nthreads; t++)
            th.emplace_back([&]() {
                for (int j = next++; j < njobs; j = next++)
                    f(j);
            });
        for (auto &x : th)
            x.join();
    };
    for_jobs([&](int j) {
        const siminf_gpu_solver_args *a = jobs[j].args;
        for (int i = 0; i < a->len; i++) {
            if (event_day(a->time[i]) >= ndays[j])
                continue;
            const bool e2 = a->event[i] == SIMINF_GPU_EXTERNAL_TRANSFER_EVENT;
            if (a->node[i] < 1 || a->node[i] > a->Nn ||
                (e2 && (a->dest[i] < 1 || a->dest[i] > a->Nn))) {
                if (!jbad[j])
                    jbad[j] = (e2 && a->node[i] >= 1 && a->node[i] <= a->Nn) ? -(i + 1) : i + 1;
                continue;
            }
            jmin[j] = std::min(jmin[j], a->time[i]);
            jmax[j] = std::max(jmax[j], a->time[i]);
            jcount[j]++;
        }
    });
    long long nev = 0;
    int tmin = INT_MAX, tmax = INT_MIN;
    for (int j = 0; j < njobs; j++) {
        if (jbad[j]) {
            snprintf(msg, sizeof(msg), "batch job %d: event %d names a node outside it", j,
                     std::abs(jbad[j]));
            return fail(jbad[j] < 0 ? SIMINF_GPU_ERR_DEST_OUT_OF_BOUNDS
                                    : SIMINF_GPU_ERR_NODE_OUT_OF_BOUNDS, msg);
        }
        nev += jcount[j];
        tmin = std::min(tmin, jmin[j]);
        tmax = std::max(tmax, jmax[j]);
    }
    std::vector<int> ev_event(nev), ev_time(nev), ev_node(nev), ev_dest(nev), ev_n(nev),
        ev_select(nev), ev_shift(nev);
    std::vector<double> ev_prop(nev);
    if (nev > 0) {
        const long long nkeys = 2 * ((long long) tmax - tmin + 1);
        if (nkeys * njobs > 400000000LL)
            return fail(SIMINF_GPU_ERR_INVALID_MODEL, "batch event times span too wide a range");
        auto key = [&](const siminf_gpu_solver_args *a, int i) {
            return 2 * ((long long) a->time[i] - tmin) +
                   (a->event[i] == SIMINF_GPU_EXTERNAL_TRANSFER_EVENT ? 1 : 0);
        };
        /* off[key * njobs + j]: first position of model j's events with key */
        std::vector<long long> off((size_t) nkeys * njobs, 0);
        for_jobs([&](int j) {
            const siminf_gpu_solver_args *a = jobs[j].args;
            for (int i = 0; i < a->len; i++)
                if (event_day(a->time[i]) < ndays[j])
                    off[(size_t) key(a, i) * njobs + j]++;
        });
        long long run = 0;
        for (size_t k = 0; k < off.size(); k++) {
            const long long c = off[k];
            off[k] = run;
            run += c;
        }
        for_jobs([&](int j) {
            const siminf_gpu_solver_args *a = jobs[j].args;
            const int base = (int) node0[j];
            for (int i = 0; i < a->len; i++) {
                if (event_day(a->time[i]) >= ndays[j])
                    continue;
                const long long at = off[(size_t) key(a, i) * njobs + j]++;
                const bool e2 = a->event[i] == SIMINF_GPU_EXTERNAL_TRANSFER_EVENT;
                ev_event[at] = a->event[i];
                ev_time[at] = a->time[i];
                ev_node[at] = a->node[i] + base;
                ev_dest[at] = e2 ? a->dest[i] + base : a->dest[i];
                ev_n[at] = a->n[i];
                ev_prop[at] = a->proportion[i];
                ev_select[at] = a->select[i];
                ev_shift[at] = a->shift[i];
            }
        });
    }

    siminf_gpu_solver_args m = *T;
    m.u0 = u0.data();
    m.v0 = Nd > 0 ? v0.data() : nullptr;
    m.ldata = Nld > 0 ? ldata.data() : T->ldata;
    m.gdata = gdata.data();
    m.Nn = (int) Ntot;
    m.Nrep = 1;
    m.U = nullptr;
    m.V = nullptr;
    m.irU = m.jcU = m.irV = m.jcV = nullptr;
    m.prU = m.prV = nullptr;
    m.len = (int) nev;
    m.event = ev_event.data();
    m.time = ev_time.data();
    m.node = ev_node.data();
    m.dest = ev_dest.data();
    m.n = ev_n.data();
    m.proportion = ev_prop.data();
    m.select = ev_select.data();
    m.shift = ev_shift.data();
    if (eref >= 0) {
        m.irE = jobs[eref].args->irE;
        m.jcE = jobs[eref].args->jcE;
        m.prE = jobs[eref].args->prE;
    }
    m.N = nref >= 0 ? jobs[nref].args->N : (eref >= 0 ? jobs[eref].args->N : nullptr);
    if (nev == 0)
        m.len = 0;

    siminf_gpu_options o{};
    o.cap_transfers = opt ? opt->cap_transfers : 0;
    o.heavy_rate = opt ? opt->heavy_rate : 0;
    const double ms_merge = ms_since(t0);
    siminf_gpu_plan *p = nullptr;
    /* streamed: the external transfers' waves are planned beside the GPU */
    int rc = plan_create_internal(&m, model, &o, &p, true, true);
    if (rc)
        return rc;

    /* The models' tables. */
    std::vector<double> targets((size_t) col0[njobs] + 1, 0.0);
    for (int j = 0; j < njobs; j++)
        if (jobs[j].target)
            memcpy(&targets[(size_t) col0[j]], jobs[j].target, (size_t) tlen[j] * sizeof(double));
    std::vector<unsigned long long> zeros(2 * (size_t) col0[njobs] + 2, 0ULL);
    void *d_job_of, *d_node0, *d_seed, *d_ndays, *d_tlen, *d_col0, *d_prev, *d_gdata, *d_target,
        *d_has, *d_prevalence, *d_distance;
    const size_t ncols = (size_t) col0[njobs];
    if (!rc) rc = plan_upload(p, &d_job_of, job_of.data(), job_of.size() * sizeof(int));
    if (!rc) rc = plan_upload(p, &d_node0, node0.data(), node0.size() * sizeof(long long));
    if (!rc) rc = plan_upload(p, &d_seed, seeds.data(), seeds.size() * sizeof(uint64_t));
    if (!rc) rc = plan_upload(p, &d_ndays, ndays.data(), ndays.size() * sizeof(int));
    if (!rc) rc = plan_upload(p, &d_tlen, tlen.data(), tlen.size() * sizeof(int));
    if (!rc) rc = plan_upload(p, &d_col0, col0.data(), col0.size() * sizeof(long long));
    if (!rc) rc = plan_upload(p, &d_prev, zeros.data(), zeros.size() * sizeof(unsigned long long));
    if (!rc) rc = plan_upload(p, &d_gdata, gdata.data(), gdata.size() * sizeof(double));
    if (!rc) rc = plan_upload(p, &d_target, targets.data(), targets.size() * sizeof(double));
    if (!rc) rc = plan_upload(p, &d_has, has_target.data(), has_target.size() * sizeof(int));
    if (!rc) rc = plan_upload(p, &d_prevalence, nullptr, (ncols + 1) * sizeof(double));
    if (!rc) rc = plan_upload(p, &d_distance, nullptr, (size_t) njobs * sizeof(double));
    if (!rc) {
        DevState &s = p->s;
        s.job_of = (const int *) d_job_of;
        s.job_node0 = (const long long *) d_node0;
        s.job_seed = (const uint64_t *) d_seed;
        s.job_ndays = (const int *) d_ndays;
        s.job_tlen = (const int *) d_tlen;
        s.job_col0 = (const long long *) d_col0;
        s.prev = (unsigned long long *) d_prev;
        s.prev_num_mask = opt ? opt->prevalence_num_mask : 0;
        s.prev_den_mask = opt ? opt->prevalence_den_mask : 0;
        s.gdata = (const double *) d_gdata;
        s.gdata_stride = L->Ngd;
        p->horizon = false;                /* the prevalence sums come from k_pts_store */
        rc = plan_run_internal(p, nullptr);
        if (rc) {
            /* name the model and its own node */
            siminf_gpu_status st;
            siminf_gpu_last_status(&st);
            if (st.node >= 0) {
                const int j = (int) (std::upper_bound(node0.begin(), node0.end(),
                                                      (long long) st.node) - node0.begin()) - 1;
                char m2[300];
                snprintf(m2, sizeof(m2), "batch job %d, node %lld (one-based): %.200s", j,
                         (long long) st.node - node0[j] + 1, st.message);
                capi_set_status(st.error, (int) (st.node - node0[j]), st.transition,
                                st.event_index, st.time, st.rate, m2);
            }
        }
    }
    if (!rc) {
        k_batch_distance<<<(njobs + 127) / 128, 128>>>(
            (const unsigned long long *) d_prev, (const long long *) d_col0, (const int *) d_tlen,
            (const double *) d_target, (const int *) d_has, njobs, (double *) d_prevalence,
            (double *) d_distance);
        std::vector<double> hp(ncols + 1), hd(njobs);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess)
            e = cudaMemcpy(hp.data(), d_prevalence, ncols * sizeof(double), cudaMemcpyDeviceToHost);
        if (e == cudaSuccess)
            e = cudaMemcpy(hd.data(), d_distance, (size_t) njobs * sizeof(double),
                           cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) {
            rc = capi_cuda_fail(e, "batch distances");
        } else {
            for (int j = 0; j < njobs; j++) {
                if (jobs[j].prevalence)
                    memcpy(jobs[j].prevalence, &hp[(size_t) col0[j]],
                           (size_t) tlen[j] * sizeof(double));
                if (jobs[j].distance)
                    *jobs[j].distance = hd[j];
            }
        }
    }
    siminf_gpu_stats st = p->stats;
    st.ms_plan += ms_merge;
    st.ms_upload += ms_merge;
    st.ms_download = ms_since(t0) - st.ms_upload - st.ms_solve;
    capi_set_stats(st);
    siminf_gpu_plan_free(p);
    return rc;
}
