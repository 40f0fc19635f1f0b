/*
 * siminf_capi.cpp -- host side of the C ABI in include/siminf_gb300.h.
 *
 * Replaces, behind SimInf_run's dispatch (src/SimInf.c:382-399), the
 * reference's SimInf_run_solver_ssm / _mssm
 * (src/solvers/SimInf_solver_ssm.c:381-414, _mssm.c:410-443).  What the
 * reference does in SimInf_compartment_model_create and
 * SimInf_scheduled_events_create (src/solvers/SimInf_solver.c:443-510,
 * 998-1173) happens here as a plan:
 *
 *  - the day schedule: tt starts at tspan[0], next = floor(tt) + 1, and
 *    column k of U/V is written after the first day whose end time is past
 *    tspan[k] (src/solvers/SimInf_solver_ssm.c:305-334);
 *  - E1 events (exit, enter, internal transfer) bucketed per node in array
 *    order, each tagged with the day whose event pass applies it (events
 *    with time <= tt, src/solvers/SimInf_solver.c:671);
 *  - E2 events (external transfers) of each day split into conflict-free
 *    wavefronts: an event waits for every earlier event of the day that
 *    touched its source, and for every earlier event whose source was its
 *    destination.  Adds into a common destination commute and share a wave.
 *    Running the waves in order reproduces the reference's serial array
 *    order (src/solvers/SimInf_solver_ssm.c:244-250) exactly.
 *
 * Errors follow the reference: a negative SimInf code, diagnostics kept per
 * calling thread, every device buffer freed before returning.
 */
#include <algorithm>
#include <array>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <atomic>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <tuple>
#include <vector>

#include <cuda_runtime.h>
#include <dlfcn.h>

#include "../../include/siminf_gb300.h"
#include "siminf_capi_internal.h"
#include "siminf_launch.h"
#include "siminf_plan.h"
#include "siminf_schedule.h"
#include "siminf_stream.h"

using namespace siminf;

namespace {

thread_local siminf_gpu_status g_status;
thread_local siminf_gpu_stats g_stats;

void set_status(int code, int node, int tr, int evi, double time, double rate, const char *msg)
{
    g_status.error = code;
    g_status.node = node;
    g_status.transition = tr;
    g_status.event_index = evi;
    g_status.time = time;
    g_status.rate = rate;
    snprintf(g_status.message, sizeof(g_status.message), "%s", msg ? msg : "");
}

int cuda_fail(cudaError_t e, const char *what)
{
    char buf[400];
    snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
    set_status(SIMINF_GPU_ERR_CUDA, -1, -1, -1, 0, 0, buf);
    return SIMINF_GPU_ERR_CUDA;
}

/* Where the calling thread's plans live: the stream their copies and
 * kernels go to, and whether their buffers come from the stream-ordered
 * allocator (no device-wide synchronisation when they are freed). */
thread_local cudaStream_t g_plan_stream = nullptr;
thread_local bool g_plan_async = false;

template <class T>
int dalloc(T **p, size_t n, std::vector<void *> &owned)
{
    *p = nullptr;
    if (n == 0)
        n = 1;
    cudaError_t e = g_plan_async ? cudaMallocAsync((void **) p, n * sizeof(T), g_plan_stream)
                                 : cudaMalloc((void **) p, n * sizeof(T));
    if (e != cudaSuccess) {
        *p = nullptr;
        return cuda_fail(e, "cudaMalloc");
    }
    owned.push_back(*p);
    return 0;
}

template <class T>
int upload(T **p, const T *src, size_t n, std::vector<void *> &owned, cudaStream_t st)
{
    int rc = dalloc(p, n, owned);
    if (rc)
        return rc;
    if (n && src) {
        cudaError_t e = cudaMemcpyAsync(*p, src, n * sizeof(T), cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess)
            return cuda_fail(e, "cudaMemcpyAsync H2D");
    }
    return 0;
}

double ms_since(std::chrono::steady_clock::time_point t0)
{
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

/* Pinned host staging buffers kept between runs.  Pinning the gigabyte
 * that a streamed run of 10^6 nodes stages its external transfers
 * through takes longer than several days of the GPU's work, so
 * a buffer a run releases is kept for the next run: at most PINNED_KEEP
 * buffers and PINNED_KEEP_BYTES in all, freed by
 * siminf_gpu_release_cached. */
enum { PINNED_KEEP = 4 };
constexpr size_t PINNED_KEEP_BYTES = (size_t) 4 << 30;

struct PinnedCache {
    std::mutex mu;
    std::vector<std::pair<void *, size_t>> free_list;
};

PinnedCache &pinned_cache()
{
    static PinnedCache c;
    return c;
}

/* A pinned buffer of at least `bytes`: the smallest cached one that
 * fits, else a new one. */
cudaError_t pinned_acquire(size_t bytes, void **out, size_t *got)
{
    PinnedCache &c = pinned_cache();
    {
        std::lock_guard<std::mutex> lk(c.mu);
        int best = -1;
        for (size_t i = 0; i < c.free_list.size(); i++)
            if (c.free_list[i].second >= bytes &&
                (best < 0 || c.free_list[i].second < c.free_list[best].second))
                best = (int) i;
        if (best >= 0) {
            *out = c.free_list[best].first;
            *got = c.free_list[best].second;
            c.free_list.erase(c.free_list.begin() + best);
            return cudaSuccess;
        }
    }
    *got = bytes;
    return cudaHostAlloc(out, bytes, cudaHostAllocPortable);
}

/* Return a buffer of pinned_acquire: kept if the cache has room, the
 * smallest buffers leaving first. */
void pinned_release(void *ptr, size_t bytes)
{
    if (!ptr)
        return;
    PinnedCache &c = pinned_cache();
    std::vector<void *> drop;
    {
        std::lock_guard<std::mutex> lk(c.mu);
        c.free_list.emplace_back(ptr, bytes);
        std::sort(c.free_list.begin(), c.free_list.end(),
                  [](const std::pair<void *, size_t> &x, const std::pair<void *, size_t> &y) {
                      return x.second > y.second;
                  });
        size_t total = 0, keep = 0;
        while (keep < c.free_list.size() && keep < PINNED_KEEP &&
               total + c.free_list[keep].second <= PINNED_KEEP_BYTES)
            total += c.free_list[keep++].second;
        for (size_t i = keep; i < c.free_list.size(); i++)
            drop.push_back(c.free_list[i].first);
        c.free_list.resize(keep);
    }
    for (void *q : drop)
        cudaFreeHost(q);
}

/* True if host pointer q is pinned (page-locked or registered), so that an
 * asynchronous copy to it does not hold the calling thread. */
bool host_pinned(const void *q)
{
    if (!q)
        return false;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, q) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeHost;
}

}  // namespace

static int validate(const siminf_gpu_solver_args *a, const Launchers *L)
{
    char msg[256];
    if (!a || !L)
        return SIMINF_GPU_ERR_INVALID_MODEL;
    if (a->solver != 0 && a->solver != 1) {
        set_status(SIMINF_GPU_ERR_UNKNOWN_SOLVER, -1, -1, -1, 0, 0, "Invalid 'solver' value.");
        return SIMINF_GPU_ERR_UNKNOWN_SOLVER;
    }
    if (a->solver == 1 && a->Nrep > 1) {
        /* src/SimInf.c:393-396 */
        set_status(SIMINF_GPU_ERR_AEM_REPLICATED_MODEL, -1, -1, -1, 0, 0,
                   "Cannot run the 'aem' solver on a replicated model.");
        return SIMINF_GPU_ERR_AEM_REPLICATED_MODEL;
    }
    if (a->Nc != L->Nc || a->Nt != L->Nt || a->Nd != L->Nd || a->Nn < 1 || a->tlen < 1 ||
        (a->Nrep < 1) || !a->u0 || !a->tspan || !a->irG || !a->jcG || !a->irS || !a->jcS ||
        !a->prS || (a->Nld > 0 && !a->ldata) || (a->Nd > 0 && !a->v0)) {
        snprintf(msg, sizeof(msg),
                 "invalid model: Nc=%d Nt=%d Nd=%d (device model wants %d, %d, %d), Nn=%d, tlen=%d",
                 a->Nc, a->Nt, a->Nd, L->Nc, L->Nt, L->Nd, a->Nn, a->tlen);
        set_status(SIMINF_GPU_ERR_INVALID_MODEL, -1, -1, -1, 0, 0, msg);
        return SIMINF_GPU_ERR_INVALID_MODEL;
    }
    if (!a->U && !a->jcU) {
        set_status(SIMINF_GPU_ERR_INVALID_MODEL, -1, -1, -1, 0, 0, "neither U nor a U_sparse pattern");
        return SIMINF_GPU_ERR_INVALID_MODEL;
    }
    /* G and S: CSC with row indices in range and ascending per column (the
     * dgCMatrix invariant the refresh order relies on). */
    for (int j = 0; j < a->Nt; j++) {
        for (int k = a->jcG[j]; k < a->jcG[j + 1]; k++) {
            if (a->irG[k] < 0 || a->irG[k] >= a->Nt ||
                (k > a->jcG[j] && a->irG[k] <= a->irG[k - 1])) {
                set_status(SIMINF_GPU_ERR_INVALID_MODEL, -1, j, -1, 0, 0, "invalid G");
                return SIMINF_GPU_ERR_INVALID_MODEL;
            }
        }
        for (int k = a->jcS[j]; k < a->jcS[j + 1]; k++) {
            if (a->irS[k] < 0 || a->irS[k] >= a->Nc) {
                set_status(SIMINF_GPU_ERR_INVALID_MODEL, -1, j, -1, 0, 0, "invalid S");
                return SIMINF_GPU_ERR_INVALID_MODEL;
            }
        }
    }
    if (a->len > 0 && (!a->event || !a->time || !a->node || !a->dest || !a->n ||
                       !a->proportion || !a->select || !a->shift || !a->jcE || !a->irE ||
                       !a->prE)) {
        set_status(SIMINF_GPU_ERR_INVALID_MODEL, -1, -1, -1, 0, 0, "incomplete event arrays");
        return SIMINF_GPU_ERR_INVALID_MODEL;
    }
    return 0;
}

extern "C" {
static int plan_create_impl(const siminf_gpu_solver_args *a, const siminf_gpu_model *model,
                            const siminf_gpu_options *opt, siminf_gpu_plan **out, bool stream,
                            bool no_output);
static int plan_run_impl(siminf_gpu_plan *p, cudaStream_t st, struct KernelProfile *kp);
}
static int make_days(siminf_gpu_plan *p, const siminf_gpu_solver_args *a);
/* Something a run depends on changed: the next run goes launch by launch
 * and a later unchanged one captures a new graph. */
static void plan_changed(siminf_gpu_plan *p)
{
    p->runs_unchanged = 0;
    if (p->run_graph) {
        cudaGraphExecDestroy(p->run_graph);
        p->run_graph = nullptr;
    }
}

template <class T>
static int upload_owned(siminf_gpu_plan *p, T **dst, const T *src, size_t n);

namespace siminf {

int plan_create_internal(const siminf_gpu_solver_args *a, const siminf_gpu_model *model,
                         const siminf_gpu_options *opt, siminf_gpu_plan **out, bool stream,
                         bool no_output)
{
    return plan_create_impl(a, model, opt, out, stream, no_output);
}

void plan_thread_stream(cudaStream_t stream, bool async)
{
    g_plan_stream = stream;
    g_plan_async = async;
}

int plan_run_internal(siminf_gpu_plan *p, cudaStream_t st)
{
    return plan_run_impl(p, st, nullptr);
}

int plan_upload(siminf_gpu_plan *p, void **dst, const void *src, size_t bytes)
{
    unsigned char *d = nullptr;
    const int rc = upload_owned(p, &d, (const unsigned char *) src, bytes);
    *dst = d;
    return rc;
}

int plan_days(const double *tspan, int tlen, std::vector<DayInfo> &days)
{
    siminf_gpu_plan p;
    siminf_gpu_solver_args a{};
    a.tspan = tspan;
    a.tlen = tlen;
    const int rc = make_days(&p, &a);
    days = p.days;
    return rc;
}

int capi_validate(const siminf_gpu_solver_args *a, const Launchers *L)
{
    return validate(a, L);
}

void capi_set_status(int code, int node, int tr, int evi, double time, double rate,
                     const char *msg)
{
    set_status(code, node, tr, evi, time, rate, msg);
}

void capi_set_stats(const siminf_gpu_stats &st)
{
    g_stats = st;
}

void capi_clear_status()
{
    memset(&g_status, 0, sizeof(g_status));
}

int capi_cuda_fail(cudaError_t e, const char *what)
{
    return cuda_fail(e, what);
}

}  // namespace siminf

template <class T>
static int upload_owned(siminf_gpu_plan *p, T **dst, const T *src, size_t n)
{
    const int rc = upload(dst, src, n, p->owned, p->stream);
    if (rc)
        return rc;
    const cudaError_t e = cudaStreamSynchronize(p->stream);
    return e == cudaSuccess ? 0 : cuda_fail(e, "upload");
}

/* Day index whose event pass applies an event at `time`. */
static inline long long event_day(int time, double tt0)
{
    if ((double) time <= tt0)
        return 0;
    return (long long) time - (long long) std::floor(tt0);
}

/* How a streamed plan plans its events: 0 (the default) on host threads
 * after a scan of the whole table; 1 on the device (siminf_schedule.cu),
 * levels included; 2 the device's planner with the levels from host
 * threads (SIMINF_DEVICE_PLANNER=1 or 2).  The device planner equals the
 * host one and starts the first day without the host's scan, but during a
 * run its kernels wait for the SSA kernel, whose persistent grid holds
 * every SM, so its work adds to the run's device time; the host threads
 * are otherwise idle. */
static int device_planner_for(long long len)
{
    if (len <= 0)
        return 0;
    if (const char *ev = getenv("SIMINF_DEVICE_PLANNER"))
        return ev[0] == '1' ? 1 : ev[0] == '2' ? 2 : 0;
    return 0;
}

/* Whether a streamed plan on host threads skips the scan of the whole
 * table before its first day: from 2^22 events (SIMINF_SCAN_FREE=0/1
 * overrides).  Each planner thread then checks its own day (order, E1
 * events, planned failures, maxima), the launching thread buckets each
 * chunk's E1 events and grows E and N as the days reveal them, and the
 * run starts as soon as the first chunk is planned. */
enum { SCAN_FREE_FROM = 1 << 22 };
static bool scan_free_for(long long len)
{
    if (const char *ev = getenv("SIMINF_SCAN_FREE"))
        return len > 0 && ev[0] == '1';
    return len >= SCAN_FREE_FROM;
}

/* Threads used by the host planner (SIMINF_PLANNER_THREADS overrides the
 * hardware's count). */
static int planner_threads()
{
    if (const char *ev = getenv("SIMINF_PLANNER_THREADS")) {
        const int n = atoi(ev);
        if (n >= 1 && n <= 256)
            return n;
    }
    unsigned n = std::thread::hardware_concurrency();
    if (n < 1)
        n = 1;
    if (n > 64)
        n = 64;
    return (int) n;
}

/* Run f(t, n) on n = planner_threads() threads and join. */
template <class F>
static void parallel(F &&f)
{
    const unsigned n = (unsigned) planner_threads();
    std::vector<std::thread> th;
    for (unsigned t = 1; t < n; t++)
        th.emplace_back([&f, t, n] { f((int) t, (int) n); });
    f(0, (int) n);
    for (auto &x : th)
        x.join();
}

/* Pass over the schedule before any wave is planned: order check, planned
 * failures, the E1 records bucketed by node, and per day the number of
 * valid external transfers, their output offset and their input range. */
static int plan_scan(siminf_gpu_plan *p, const siminf_gpu_solver_args *a, int nsel,
                     std::vector<E1Rec> &e1, std::vector<int> &e1_ptr)
{
    const int Nn = a->Nn, ndays = p->ndays;
    const double tt0 = a->tspan[0];
    const long long len = a->len;

    /* Pass 1, parallel over chunks: order check, planned failures, E1
     * positions and E2 counts per day.  The order check compares each
     * event with its predecessor, so chunk borders are covered. */
    struct Chunk {
        long long bad = -1;
        int max_select = 0, max_shift = 0;
        std::vector<long long> e1;
        std::vector<long long> e2_per_day;
        std::vector<PlannedErr> planned;
    };
    std::vector<Chunk> chunks(planner_threads());
    const int E2 = SIMINF_GPU_EXTERNAL_TRANSFER_EVENT;
    parallel([&](int t, int n) {
        Chunk &c = chunks[t];
        c.e2_per_day.assign(ndays + 1, 0);
        const long long lo = len * t / n, hi = len * (t + 1) / n;
        const int *time = a->time, *event = a->event, *node_ = a->node, *dest_ = a->dest,
                  *select = a->select, *shift = a->shift;
        int msel = 0, mshift = 0;
        int pt = lo > 0 ? time[lo - 1] : INT_MIN, pk = lo > 0 ? event[lo - 1] : 0;
        /* times are sorted, so the day changes rarely: it is recomputed
         * when the time changes, and the day's count of valid transfers is
         * kept in a register until then */
        long long d = -1;
        int d_time = 0;
        long long run = 0;
        for (long long i = lo; i < hi; i++) {
            const int tm = time[i], kind = event[i];
            if (tm < pt || (tm == pt && pk == E2 && kind != E2)) {
                if (c.bad < 0)
                    c.bad = i;
            }
            pt = tm;
            pk = kind;
            msel = std::max(msel, select[i]);
            mshift = std::max(mshift, shift[i]);
            if (d < 0 || tm != d_time) {
                if (d >= 0 && d < ndays)
                    c.e2_per_day[d] += run;
                run = 0;
                d = event_day(tm, tt0);
                d_time = tm;
            }
            if (d >= ndays)
                continue;
            const unsigned node = (unsigned) (node_[i] - 1), dest = (unsigned) (dest_[i] - 1),
                           sel = (unsigned) (select[i] - 1);
            const bool ok = node < (unsigned) Nn && (unsigned) kind <= 3u && sel < (unsigned) nsel;
            if (ok && kind == E2 && dest < (unsigned) Nn) {
                run++;
                continue;
            }
            const int phase = kind == E2 ? PHASE_E2 : PHASE_E1;
            if (node >= (unsigned) Nn)
                c.planned.push_back({(int) d, SIMINF_GPU_ERR_NODE_OUT_OF_BOUNDS, (int) i, (int) node, phase});
            else if ((unsigned) kind > 3u)
                c.planned.push_back({(int) d, SIMINF_GPU_UNDEFINED_EVENT, (int) i, (int) node, phase});
            else if (sel >= (unsigned) nsel)
                c.planned.push_back({(int) d, SIMINF_GPU_ERR_SAMPLE_SELECT, (int) i, (int) node, phase});
            else if (kind == E2)
                c.planned.push_back({(int) d, SIMINF_GPU_ERR_DEST_OUT_OF_BOUNDS, (int) i, (int) node, phase});
            else
                c.e1.push_back(i);
        }
        if (d >= 0 && d < ndays)
            c.e2_per_day[d] += run;
        c.max_select = msel;
        c.max_shift = mshift;
    });
    long long bad = -1;
    p->max_select = p->max_shift = 0;
    for (auto &c : chunks) {
        if (c.bad >= 0 && (bad < 0 || c.bad < bad))
            bad = c.bad;
        p->max_select = std::max(p->max_select, c.max_select);
        p->max_shift = std::max(p->max_shift, c.max_shift);
        p->planned.insert(p->planned.end(), c.planned.begin(), c.planned.end());
    }
    if (bad >= 0) {
        char msg[200];
        snprintf(msg, sizeof(msg), "event %lld (time %d) breaks the (time, E1 before E2) order",
                 bad + 1, a->time[bad]);
        set_status(SIMINF_GPU_ERR_EVENTS_UNSORTED, -1, -1, (int) bad, a->time[bad], 0, msg);
        return SIMINF_GPU_ERR_EVENTS_UNSORTED;
    }

    /* E1: stable bucket by node (array order within a node is day order). */
    std::vector<int> e1_count(Nn + 1, 0);
    for (auto &c : chunks)
        for (long long i : c.e1)
            e1_count[a->node[i] - 1]++;
    e1_ptr.assign(Nn + 1, 0);
    for (int k = 0; k < Nn; k++)
        e1_ptr[k + 1] = e1_ptr[k] + e1_count[k];
    e1.resize(e1_ptr[Nn]);
    {
        std::vector<int> fill(e1_ptr.begin(), e1_ptr.end() - 1);
        for (auto &c : chunks)
            for (long long i : c.e1) {
                const int node = a->node[i] - 1;
                e1[fill[node]++] = E1Rec{(int) event_day(a->time[i], tt0), a->event[i], a->n[i],
                                         a->select[i] - 1, a->shift[i] - 1, (int) i,
                                         a->proportion[i]};
            }
    }

    /* E2 events of a day, in array order: the valid transfers inside the
     * day's time range (events are sorted, so a day is one contiguous
     * range of the input).  Day ranges by binary search on time. */
    std::vector<long long> day_cnt(ndays + 1, 0);
    for (auto &c : chunks)
        for (int d = 0; d < ndays; d++)
            day_cnt[d] += c.e2_per_day[d];
    std::vector<long long> &day_off = p->e2_day_off;
    day_off.assign(ndays + 1, 0);
    for (int d = 0; d < ndays; d++)
        day_off[d + 1] = day_off[d] + day_cnt[d];
    std::vector<long long> &range_lo = p->e2_lo, &range_hi = p->e2_hi;
    range_lo.assign(ndays, 0);
    range_hi.assign(ndays, 0);
    for (int d = 0; d < ndays; d++) {
        /* times of day d: (tt_{d-1}, tt_d]; day 0 takes every time <= tt0 */
        auto first_after = [&](double x) {
            long long lo = 0, hi = len;
            while (lo < hi) {
                const long long mid = (lo + hi) / 2;
                if ((double) a->time[mid] <= x)
                    lo = mid + 1;
                else
                    hi = mid;
            }
            return lo;
        };
        range_lo[d] = d == 0 ? 0 : first_after(p->days[d - 1].tt);
        range_hi[d] = first_after(p->days[d].tt);
    }
    p->e1_count = e1.size();
    p->e2_count = day_off[ndays];
    p->nsel = nsel;
    p->day_waves.assign(ndays, std::vector<long long>());
    return 0;
}

/* What a streamed run without the scan (p->scan_free) learns from one
 * day's input range on its planner thread, as plan_scan learns it for the
 * whole table: the first event out of order, the select and shift maxima,
 * the valid E1 events, the planned failures; and the day's valid external
 * transfers (their count, from the wave planner). */
struct DayScan {
    long long bad = -1;
    int max_select = 0, max_shift = 0;
    long long n2 = 0;
    std::vector<long long> e1;
    std::vector<PlannedErr> planned;
};

static void scan_day(const siminf_gpu_plan *p, const siminf_gpu_solver_args *a, int d, DayScan &r)
{
    const int Nn = a->Nn, nsel = p->nsel, E2 = SIMINF_GPU_EXTERNAL_TRANSFER_EVENT;
    const long long lo = p->e2_lo[d], hi = p->e2_hi[d];
    const int *time = a->time, *event = a->event, *node_ = a->node, *dest_ = a->dest,
              *select = a->select, *shift = a->shift;
    r.bad = -1;
    r.e1.clear();
    r.planned.clear();
    int msel = 0, mshift = 0;
    int pt = lo > 0 ? time[lo - 1] : INT_MIN, pk = lo > 0 ? event[lo - 1] : 0;
    for (long long i = lo; i < hi; i++) {
        const int tm = time[i], kind = event[i];
        if ((tm < pt || (tm == pt && pk == E2 && kind != E2)) && r.bad < 0)
            r.bad = i;
        pt = tm;
        pk = kind;
        msel = std::max(msel, select[i]);
        mshift = std::max(mshift, shift[i]);
        const unsigned node = (unsigned) (node_[i] - 1), dest = (unsigned) (dest_[i] - 1),
                       sel = (unsigned) (select[i] - 1);
        const bool ok = node < (unsigned) Nn && (unsigned) kind <= 3u && sel < (unsigned) nsel;
        if (ok && kind == E2 && dest < (unsigned) Nn)
            continue;
        const int phase = kind == E2 ? PHASE_E2 : PHASE_E1;
        if (node >= (unsigned) Nn)
            r.planned.push_back({d, SIMINF_GPU_ERR_NODE_OUT_OF_BOUNDS, (int) i, (int) node, phase});
        else if ((unsigned) kind > 3u)
            r.planned.push_back({d, SIMINF_GPU_UNDEFINED_EVENT, (int) i, (int) node, phase});
        else if (sel >= (unsigned) nsel)
            r.planned.push_back({d, SIMINF_GPU_ERR_SAMPLE_SELECT, (int) i, (int) node, phase});
        else if (kind == E2)
            r.planned.push_back({d, SIMINF_GPU_ERR_DEST_OUT_OF_BOUNDS, (int) i, (int) node, phase});
        else
            r.e1.push_back(i);
    }
    r.max_select = msel;
    r.max_shift = mshift;
}

/* The E1 records of the events at positions pos (lists in day order,
 * each in position order), bucketed by node: stable, so a node keeps day
 * and array order (plan_scan's E1 part).  ptr gets Nn + 1 offsets. */
static void bucket_e1(const siminf_gpu_solver_args *a,
                      const std::vector<const std::vector<long long> *> &pos, E1Rec *rec, int *ptr)
{
    const int Nn = a->Nn;
    const double tt0 = a->tspan[0];
    std::memset(ptr, 0, ((size_t) Nn + 1) * sizeof(int));
    for (const auto *v : pos)
        for (long long i : *v)
            ptr[a->node[i]]++;                  /* node i - 1, counted at i */
    for (int k = 0; k < Nn; k++)
        ptr[k + 1] += ptr[k];
    for (const auto *v : pos)
        for (long long i : *v) {
            const int node = a->node[i] - 1;
            rec[ptr[node]++] = E1Rec{(int) event_day(a->time[i], tt0), a->event[i], a->n[i],
                                     a->select[i] - 1, a->shift[i] - 1, (int) i, a->proportion[i]};
        }
    /* ptr[k] now ends node k's records: shift back to starts */
    for (int k = Nn; k > 0; k--)
        ptr[k] = ptr[k - 1];
    ptr[0] = 0;
}

/* Orders one day's E1 positions by node, then position (scan_day leaves
 * them in position order). */
static void sort_e1_by_node(const siminf_gpu_solver_args *a, std::vector<long long> &e1)
{
    const int *node = a->node;
    std::sort(e1.begin(), e1.end(), [node](long long x, long long y) {
        return node[x] != node[y] ? node[x] < node[y] : x < y;
    });
}

/* The E1 records of several days (each day's positions sorted by node,
 * then position; days in order) merged by node, then position -- stable by
 * node, so a node keeps day and array order (plan_scan's E1 part) -- into
 * rec, with each record's zero-based node in keys. */
static void merge_e1_days(const siminf_gpu_solver_args *a,
                          const std::vector<const std::vector<long long> *> &days, E1Rec *rec,
                          uint32_t *keys, std::vector<long long> &tmp, std::vector<long long> &out)
{
    const int *node = a->node;
    auto less = [node](long long x, long long y) {
        return node[x] != node[y] ? node[x] < node[y] : x < y;
    };
    out.clear();
    for (const auto *v : days) {
        tmp.swap(out);
        out.resize(tmp.size() + v->size());
        std::merge(tmp.begin(), tmp.end(), v->begin(), v->end(), out.begin(), less);
    }
    const double tt0 = a->tspan[0];
    for (size_t k = 0; k < out.size(); k++) {
        const long long i = out[k];
        rec[k] = E1Rec{(int) event_day(a->time[i], tt0), a->event[i], a->n[i], a->select[i] - 1,
                       a->shift[i] - 1, (int) i, a->proportion[i]};
        keys[k] = (uint32_t) (node[i] - 1);
    }
}

/* Per-thread scratch of the wave planner: per node, its two levels on
 * the day being planned (the last event with the node as source, `excl`,
 * and the last add into it, `add`), packed into one word so that an event
 * touches one cache line per node: 16 bits each, so the table of a
 * million nodes (4 MB) stays in cache.  Zero outside the day: after a day
 * that touches few nodes they are cleared one by one (listed in
 * `touched`), after a busy day the whole table at once.  A day whose wavefronts run
 * deeper than 2^16 - 1 is planned again with 32-bit levels. */
struct WaveTracker {
    std::vector<uint32_t> lv;
    std::vector<int> touched, level;
    std::vector<uint32_t> idx;          /* input positions, relative to the day's first */
    std::vector<long long> cnt, off;
    explicit WaveTracker(int Nn) : lv(Nn, 0) {}
};

/* Levels of day d's external transfers into w.level / w.idx; T is the
 * level type and P packs two of them (excl low, add high).  Returns false
 * if a level would not fit T. */
template <class T, class P>
static bool day_levels(const siminf_gpu_plan *p, const siminf_gpu_solver_args *a, int d,
                       WaveTracker &w, P *lv, int &maxl)
{
    constexpr int SH = 8 * sizeof(T);
    constexpr P LO = ((P) 1 << SH) - 1;
    constexpr long long PF = 16;            /* prefetch distance, in events */
    const unsigned Nn = (unsigned) a->Nn, nsel = (unsigned) p->nsel;
    const long long limit = (long long) std::numeric_limits<T>::max();
    const int *ev = a->event, *src = a->node, *dst = a->dest, *sel = a->select;
    const long long lo = p->e2_lo[d], hi = p->e2_hi[d];
    w.level.clear();
    w.idx.clear();
    w.touched.clear();
    maxl = 0;
    bool ok = true;
    /* a day that touches a fair part of the nodes clears the whole table
     * afterwards (one sequential pass) instead of listing the nodes it
     * touched and clearing them one by one (a random write each) */
    const bool sparse = 2 * (hi - lo) < (long long) Nn / 8;
    for (long long i = lo; i < hi; i++) {
        if (i + PF < hi) {
            const unsigned ps = (unsigned) (src[i + PF] - 1), pd = (unsigned) (dst[i + PF] - 1);
            __builtin_prefetch(lv + (ps < Nn ? ps : 0), 1);
            __builtin_prefetch(lv + (pd < Nn ? pd : 0), 1);
        }
        if (ev[i] != SIMINF_GPU_EXTERNAL_TRANSFER_EVENT)
            continue;
        const unsigned s = (unsigned) (src[i] - 1), t = (unsigned) (dst[i] - 1);
        if (s >= Nn || t >= Nn || (unsigned) (sel[i] - 1) >= nsel)
            continue;
        const P vs = lv[s], vt = lv[t];
        if (sparse && !vs)
            w.touched.push_back((int) s);
        if (sparse && !vt)
            w.touched.push_back((int) t);
        const long long es = (long long) (vs & LO), as = (long long) (vs >> SH),
                        et = (long long) (vt & LO);
        const long long L = 1 + std::max(std::max(es, as), et);
        if (L > limit) {
            ok = false;
            break;
        }
        lv[s] = (vs & ~LO) | (P) L;
        const P vt2 = lv[t];                /* re-read: s == t sees its own update */
        if ((long long) (vt2 >> SH) < L)
            lv[t] = (vt2 & LO) | ((P) L << SH);
        w.level.push_back((int) L);
        w.idx.push_back((uint32_t) (i - lo));
        maxl = std::max(maxl, (int) L);
    }
    if (sparse) {
        for (int n : w.touched)
            lv[n] = 0;
    } else {
        std::memset(lv, 0, (size_t) Nn * sizeof(P));
    }
    return ok;
}

/* Wave levels of day d: level = 1 + max(level of the last event with the
 * same source, of any add into the source, of the last event whose source
 * is our destination).  Then a stable counting sort of the day's events by
 * level into e2 (positions at ..), and the wave sizes into
 * p->day_waves[d].  Returns the day's transfer count. */
static long long plan_day_waves(siminf_gpu_plan *p, const siminf_gpu_solver_args *a, int d,
                                WaveTracker &w, E2Rec *e2, long long at)
{
    int maxl = 0;
    if (!day_levels<uint16_t>(p, a, d, w, w.lv.data(), maxl)) {
        std::vector<uint64_t> lv(a->Nn, 0);
        day_levels<uint32_t>(p, a, d, w, lv.data(), maxl);
    }
    const int *src = a->node, *dst = a->dest, *sel = a->select;
    const long long lo = p->e2_lo[d];
    std::vector<int> &level = w.level;
    std::vector<uint32_t> &idx = w.idx;
    std::vector<long long> &cnt = w.cnt, &off = w.off;
    cnt.assign(maxl + 2, 0);
    for (int L : level)
        cnt[L]++;
    off.assign(maxl + 2, at);
    for (int L = 1; L <= maxl; L++)
        off[L + 1] = off[L] + cnt[L];
    for (size_t k = 0; k < level.size(); k++) {
        const long long i = lo + idx[k];
        e2[off[level[k]]++] = E2Rec{src[i] - 1, dst[i] - 1, a->n[i], sel[i] - 1,
                                    a->shift[i] - 1, (int) i, a->proportion[i]};
    }
    p->day_waves[d].assign(cnt.begin() + 1, cnt.begin() + 1 + maxl);
    return (long long) level.size();
}

/* plan_day_waves for a streamed run: the day's transfers in wave order as
 * their positions relative to the input position rel (order[k], from
 * k = at), for the device to gather the records from the event columns it
 * receives by DMA (k_gather_e2).  Returns the day's transfer count. */
static long long plan_day_order(siminf_gpu_plan *p, const siminf_gpu_solver_args *a, int d,
                                WaveTracker &w, uint32_t *order, long long at, long long rel)
{
    int maxl = 0;
    if (!day_levels<uint16_t>(p, a, d, w, w.lv.data(), maxl)) {
        std::vector<uint64_t> lv(a->Nn, 0);
        day_levels<uint32_t>(p, a, d, w, lv.data(), maxl);
    }
    std::vector<int> &level = w.level;
    std::vector<uint32_t> &idx = w.idx;
    std::vector<long long> &cnt = w.cnt, &off = w.off;
    cnt.assign(maxl + 2, 0);
    for (int L : level)
        cnt[L]++;
    off.assign(maxl + 2, at);
    for (int L = 1; L <= maxl; L++)
        off[L + 1] = off[L] + cnt[L];
    const uint32_t shift = (uint32_t) (p->e2_lo[d] - rel);
    for (size_t k = 0; k < level.size(); k++)
        order[off[level[k]]++] = idx[k] + shift;
    p->day_waves[d].assign(cnt.begin() + 1, cnt.begin() + 1 + maxl);
    return (long long) level.size();
}

/* The levels of day d's transfers for the device planner (mode 2): pos[k]
 * for the day's input position e2_lo[d] + k is the transfer's 1-based
 * level, 0 for an event that is no valid transfer.  Returns the day's
 * deepest level. */
static int plan_day_pos_levels(const siminf_gpu_plan *p, const siminf_gpu_solver_args *a, int d,
                               WaveTracker &w, uint32_t *pos)
{
    int maxl = 0;
    if (!day_levels<uint16_t>(p, a, d, w, w.lv.data(), maxl)) {
        std::vector<uint64_t> lv(a->Nn, 0);
        day_levels<uint32_t>(p, a, d, w, lv.data(), maxl);
    }
    std::memset(pos, 0, (size_t) (p->e2_hi[d] - p->e2_lo[d]) * sizeof(uint32_t));
    for (size_t k = 0; k < w.level.size(); k++)
        pos[w.idx[k]] = (uint32_t) w.level[k];
    return maxl;
}

/* Levels of one day's transfers (input range [lo, hi)) by the host
 * planner, for the days the device planner leaves to it. */
long long siminf::host_day_waves(const int *event, const int *node, const int *dest, const int *n,
                                 const double *proportion, const int *select, const int *shift,
                                 long long lo, long long hi, int Nn, int nsel, E2Rec *out,
                                 std::vector<long long> &waves)
{
    siminf_gpu_plan p;
    p.nsel = nsel;
    p.e2_lo.assign(1, lo);
    p.e2_hi.assign(1, hi);
    p.e2_day_off.assign(2, 0);
    p.day_waves.assign(1, std::vector<long long>());
    siminf_gpu_solver_args a{};
    a.Nn = Nn;
    a.event = event;
    a.node = node;
    a.dest = dest;
    a.n = n;
    a.proportion = proportion;
    a.select = select;
    a.shift = shift;
    WaveTracker w(Nn);
    plan_day_waves(&p, &a, 0, w, out, 0);
    waves = p.day_waves[0];
    long long c = 0;
    for (long long x : waves)
        c += x;
    return c;
}

/* Wave offsets of every day, from day_waves. */
static void plan_wave_index(siminf_gpu_plan *p)
{
    p->day_wave.assign(p->ndays + 1, 0);
    p->wave_ptr.clear();
    p->wave_ptr.push_back(0);
    for (int d = 0; d < p->ndays; d++) {
        for (long long c : p->day_waves[d])
            p->wave_ptr.push_back(p->wave_ptr.back() + c);
        p->day_wave[d + 1] = (int) p->wave_ptr.size() - 1;
    }
}

/* The whole schedule: scan, then the waves of every day on the planner
 * threads.  e2 receives p->e2_count records (left unset otherwise). */
static int plan_events(siminf_gpu_plan *p, const siminf_gpu_solver_args *a, int nsel,
                       std::vector<E1Rec> &e1, std::vector<int> &e1_ptr,
                       std::unique_ptr<E2Rec[]> &e2)
{
    int rc = plan_scan(p, a, nsel, e1, e1_ptr);
    if (rc)
        return rc;
    e2.reset(new E2Rec[p->e2_count > 0 ? p->e2_count : 1]);
    std::atomic<int> next_day(0);
    E2Rec *dst = e2.get();
    parallel([&](int, int) {
        WaveTracker w(a->Nn);
        for (int d = next_day++; d < p->ndays; d = next_day++)
            plan_day_waves(p, a, d, w, dst, p->e2_day_off[d]);
    });
    plan_wave_index(p);
    return 0;
}

/* The day schedule (src/solvers/SimInf_solver_ssm.c:305-334): tt starts
 * at tspan[0], next = floor(tt) + 1, and after each day the columns k with
 * tt > tspan[k] are stored. */
static int make_days(siminf_gpu_plan *p, const siminf_gpu_solver_args *a)
{
    double tt = a->tspan[0], next = std::floor(tt) + 1.0;
    int it = 0;
    p->days.clear();
    while (it < a->tlen) {
        DayInfo di;
        di.tt = tt;
        di.next = next;
        tt = next;
        next += 1.0;
        di.c0 = it;
        while (it < a->tlen && tt > a->tspan[it])
            it++;
        di.c1 = it;
        p->days.push_back(di);
        if (p->days.size() > (size_t) 100000000) {
            set_status(SIMINF_GPU_ERR_INVALID_MODEL, -1, -1, -1, 0, 0, "tspan too long");
            return SIMINF_GPU_ERR_INVALID_MODEL;
        }
    }
    p->ndays = (int) p->days.size();
    return 0;
}

extern "C" {

int siminf_gpu_model_builtin(const char *name, siminf_gpu_model **out)
{
    if (!name || !out)
        return SIMINF_GPU_ERR_UNKNOWN_MODEL;
    const Launchers *L = launchers_for(name);
    if (!L) {
        set_status(SIMINF_GPU_ERR_UNKNOWN_MODEL, -1, -1, -1, 0, 0, name);
        return SIMINF_GPU_ERR_UNKNOWN_MODEL;
    }
    siminf_gpu_model *m = (siminf_gpu_model *) calloc(1, sizeof(siminf_gpu_model));
    if (!m)
        return SIMINF_GPU_ERR_ALLOC_MEMORY_BUFFER;
    snprintf(m->name, sizeof(m->name), "%s", name);
    m->L = L;
    *out = m;
    return 0;
}

int siminf_gpu_model_load(const char *path, siminf_gpu_model **out)
{
    if (!path || !out)
        return SIMINF_GPU_ERR_INVALID_MODEL;
    /* The library stays loaded for the life of the process: its kernels
     * may sit in plans, captured graphs and streams of any thread. */
    void *h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
    if (!h) {
        const char *why = dlerror();
        set_status(SIMINF_GPU_ERR_UNKNOWN_MODEL, -1, -1, -1, 0, 0, why ? why : path);
        return SIMINF_GPU_ERR_UNKNOWN_MODEL;
    }
    auto abi = (int (*)(void)) dlsym(h, "siminf_model_abi");
    auto table = (const Launchers *(*)(void)) dlsym(h, "siminf_model_launchers");
    if (!abi || !table || abi() != SIMINF_MODEL_ABI) {
        char msg[300];
        snprintf(msg, sizeof(msg), "%s: not a device model library of this build", path);
        set_status(SIMINF_GPU_ERR_UNKNOWN_MODEL, -1, -1, -1, 0, 0, msg);
        return SIMINF_GPU_ERR_UNKNOWN_MODEL;
    }
    siminf_gpu_model *m = (siminf_gpu_model *) calloc(1, sizeof(siminf_gpu_model));
    if (!m)
        return SIMINF_GPU_ERR_ALLOC_MEMORY_BUFFER;
    const char *base = strrchr(path, '/');
    snprintf(m->name, sizeof(m->name), "%s", base ? base + 1 : path);
    m->L = table();
    *out = m;
    return 0;
}

int siminf_gpu_model_dims(const siminf_gpu_model *model, int *Nc, int *Nt, int *Nd)
{
    if (!model)
        return SIMINF_GPU_ERR_INVALID_MODEL;
    if (Nc)
        *Nc = model->L->Nc;
    if (Nt)
        *Nt = model->L->Nt;
    if (Nd)
        *Nd = model->L->Nd;
    return 0;
}

void siminf_gpu_model_free(siminf_gpu_model *model)
{
    free(model);
}

int siminf_gpu_last_status(siminf_gpu_status *out)
{
    if (out)
        *out = g_status;
    return g_status.error;
}

int siminf_gpu_last_stats(siminf_gpu_stats *out)
{
    if (out)
        *out = g_stats;
    return 0;
}

void siminf_gpu_plan_free(siminf_gpu_plan *p)
{
    if (!p)
        return;
    if (p->run_graph)
        cudaGraphExecDestroy(p->run_graph);
    for (void *q : p->owned) {
        if (p->async_alloc)
            cudaFreeAsync(q, p->stream);
        else
            cudaFree(q);
    }
    if (p->async_alloc)
        cudaStreamSynchronize(p->stream);
    delete p;
}

static int plan_create_impl(const siminf_gpu_solver_args *a, const siminf_gpu_model *model,
                            const siminf_gpu_options *opt, siminf_gpu_plan **out, bool stream,
                            bool no_output = false);

int siminf_gpu_plan_create_ex(const siminf_gpu_solver_args *a, const siminf_gpu_model *model,
                              const siminf_gpu_options *opt, siminf_gpu_plan **out)
{
    return plan_create_impl(a, model, opt, out, opt && opt->streamed != 0);
}

int siminf_gpu_plan_create(const siminf_gpu_solver_args *a, const siminf_gpu_model *model,
                           siminf_gpu_plan **out)
{
    return siminf_gpu_plan_create_ex(a, model, nullptr, out);
}

static int plan_create_impl(const siminf_gpu_solver_args *a, const siminf_gpu_model *model,
                            const siminf_gpu_options *opt, siminf_gpu_plan **out, bool stream,
                            bool no_output)
{
    auto t0 = std::chrono::steady_clock::now();
    int rc;
    memset(&g_status, 0, sizeof(g_status));
    if (!out || !model)
        return SIMINF_GPU_ERR_INVALID_MODEL;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        set_status(SIMINF_GPU_ERR_NO_DEVICE, -1, -1, -1, 0, 0, "no CUDA device");
        return SIMINF_GPU_ERR_NO_DEVICE;
    }
    const Launchers *L = model->L;
    siminf_gpu_solver_args checked;
    if (no_output && a) {
        /* no U/V wanted: the output checks pass on a stand-in */
        static int stand_in;
        checked = *a;
        checked.U = &stand_in;
        a = &checked;
    }
    if ((rc = validate(a, L)))
        return rc;

    siminf_gpu_plan *p = new siminf_gpu_plan();
    p->L = L;
    DevState &s = p->s;
    const int Nn = a->Nn, Nc = a->Nc, Nt = a->Nt, Nd = a->Nd, Nrep = a->Nrep, tlen = a->tlen;
    const long long Ntot = (long long) Nn * Nrep;
    s.Nn = Nn;
    s.Nc = Nc;
    s.Nt = Nt;
    s.Nd = Nd;
    s.Nld = a->Nld;
    s.Nrep = Nrep;
    s.tlen = tlen;
    s.Ntot = Ntot;
    s.seed = (uint64_t) a->seed;
    s.cap = opt ? (opt->cap_transfers != 0) : 0;
    s.max_fired = (opt && opt->max_node_day_transitions > 0)
                      ? (unsigned) opt->max_node_day_transitions
                      : SIMINF_GPU_MAX_NODE_DAY_TRANSITIONS;
    s.ssa_variant = (opt && opt->ssa_variant == 1) ? 1 : 0;
    if (const char *ev = getenv("SIMINF_SSA_VARIANT"))
        s.ssa_variant = ev[0] == '1';
    s.wave_block = opt ? opt->wave_block : 0;
    s.heavy_lanes = opt ? std::max(0, std::min(32, opt->heavy_lanes)) : 0;
    if (const char *ev = getenv("SIMINF_HEAVY_LANES"))
        s.heavy_lanes = std::max(0, std::min(32, atoi(ev)));
    p->tt0 = a->tspan[0];

    if ((rc = make_days(p, a))) {
        delete p;
        return rc;
    }

    /* Dense S (Nt rows of Nc) and G column masks. */
    std::vector<int> Sd((size_t) Nt * Nc, 0);
    std::vector<uint32_t> Gm(Nt, 0);
    for (int j = 0; j < Nt; j++) {
        for (int k = a->jcS[j]; k < a->jcS[j + 1]; k++)
            Sd[(size_t) j * Nc + a->irS[k]] += a->prS[k];
        for (int k = a->jcG[j]; k < a->jcG[j + 1]; k++)
            Gm[j] |= 1u << a->irG[k];
    }

    const int nsel = (a->len > 0 && a->jcE) ? INT_MAX : 0;
    std::vector<E1Rec> e1;
    std::vector<int> e1_ptr;
    std::unique_ptr<E2Rec[]> e2;
    const int dev_mode = stream ? device_planner_for(a->len) : 0;
    const bool scan_free = stream && !dev_mode && scan_free_for(a->len);
    if ((dev_mode || scan_free) && event_day_ranges(a, p->days, p->e2_lo, p->e2_hi)) {
        /* the device plans the events during the first run: only the day
         * ranges now (E and N grow to the largest select and shift the
         * planner finds; E1 lists and waves come chunk by chunk) */
        p->dev_plan = dev_mode != 0;
        p->dev_levels = dev_mode == 2;
        p->scan_free = scan_free;
        p->nsel = nsel;
        p->max_select = p->max_shift = 0;
        p->e2_count = (uint64_t) a->len;        /* room for every event */
        p->e2_day_off.assign(p->ndays + 1, 0);
        p->day_waves.assign(p->ndays, std::vector<long long>());
        e1_ptr.assign((size_t) Nn + 1, 0);
        p->e2_pending = true;
        p->args = *a;
    } else {
        rc = stream ? plan_scan(p, a, nsel, e1, e1_ptr) : plan_events(p, a, nsel, e1, e1_ptr, e2);
        if (rc) {
            delete p;
            return rc;
        }
        if (stream && p->e2_count == 0)
            plan_wave_index(p);
        if (stream && p->e2_count > 0) {
            /* the waves are planned during the first run, beside the GPU */
            p->e2_pending = true;
            p->args = *a;
        }
    }
    p->stats.ms_plan = ms_since(t0);
    p->horizon = !p->dev_plan && !p->scan_free && (p->e2_count == 0) && L->pts_local &&
                 a->solver == 0;

    cudaStream_t st = g_plan_stream;
    p->stream = st;
    p->async_alloc = g_plan_async;
    auto &own = p->owned;
    int *dS;
    uint32_t *dG;
    double *dld, *dgd;
    const size_t nld = a->Nld > 0 ? (size_t) a->Nld * Nn : 1;
    rc = upload(&dS, Sd.data(), Sd.size(), own, st);
    if (!rc) rc = upload(&dG, Gm.data(), Gm.size(), own, st);
    if (!rc) rc = upload(&dld, a->ldata, a->ldata ? nld : 0, own, st);
    const int per_rep = opt && opt->gdata_per_replicate;
    s.gdata_stride = per_rep ? L->Ngd : 0;
    if (!rc) rc = upload(&dgd, a->gdata, a->gdata ? (size_t) L->Ngd * (per_rep ? Nrep : 1) : 0,
                         own, st);
    s.S = dS;
    s.Gmask = dG;
    s.ldata = dld;
    s.gdata = dgd;
    if (!rc && a->len > 0) {
        /* E and N have as many columns as the largest select and shift
         * the events use (the struct carries no column counts; the
         * schedule scan found both). */
        const int maxsel = p->max_select, maxshift = p->max_shift;
        const int ncolE = maxsel;
        const int nnzE = a->jcE[ncolE];
        int *dirE, *djcE;
        double *dprE;
        rc = upload(&djcE, a->jcE, (size_t) ncolE + 1, own, st);
        if (!rc) rc = upload(&dirE, a->irE, (size_t) nnzE, own, st);
        if (!rc) rc = upload(&dprE, (const double *) a->prE, (size_t) nnzE, own, st);
        s.jcE = djcE;
        s.irE = dirE;
        s.prE = dprE;
        /* N is "defined" whenever the caller passes it (src/SimInf.c:302-305),
         * even if no event shifts. */
        s.hasN = a->N != nullptr;
        if (!rc && a->N) {
            int *dN;
            rc = upload(&dN, maxshift > 0 ? a->N : nullptr, (size_t) std::max(maxshift, 1) * Nc,
                        own, st);
            s.Nshift = dN;
        } else {
            s.Nshift = nullptr;
        }
    }
    if (!rc) {
        int *de1p;
        E1Rec *de1;
        rc = upload(&de1p, e1_ptr.data(), e1_ptr.size(), own, st);
        if (!rc) rc = upload(&de1, e1.data(), e1.size(), own, st);
        s.e1_ptr = de1p;
        s.e1 = de1;
    }
    if (!rc) {
        if (p->e2_pending)
            rc = dalloc(&p->d_e2, (size_t) p->e2_count, own);
        else
            rc = upload(&p->d_e2, e2.get(), (size_t) p->e2_count, own, st);
    }
    if (!rc) rc = upload(&p->d_days, p->days.data(), p->days.size(), own, st);

    /* state */
    if (!rc) rc = dalloc(&s.u, (size_t) Ntot * Nc, own);
    if (!rc) rc = dalloc(&s.vA, (size_t) Ntot * Nd, own);
    if (!rc) rc = dalloc(&s.vB, (size_t) Ntot * Nd, own);
    if (!rc) rc = dalloc(&s.t_rate, (size_t) Ntot * Nt, own);
    if (!rc) rc = dalloc(&s.sum_rate, (size_t) Ntot, own);
    if (!rc) rc = dalloc(&s.t_time, (size_t) Ntot, own);
    if (!rc) rc = dalloc(&s.ctr, (size_t) Ntot, own);
    /* crn = 1 selects SimInf_run_solver_mssm_crn for replicated models
     * (src/SimInf.c:385-389): the SSA draws from a stream of its own */
    s.crn_ctr = nullptr;
    if (!rc && a->crn == 1 && Nrep > 1 && a->solver == 0)
        rc = dalloc(&s.crn_ctr, (size_t) Ntot, own);
    if (!rc) rc = dalloc(&s.update, (size_t) Ntot, own);
    if (!rc) rc = dalloc(&s.err, (size_t) MAX_ERR, own);
    if (!rc) rc = dalloc(&s.err_count, 3, own);
    if (!rc) rc = dalloc(&s.fired, 1, own);
    if (!rc) rc = dalloc(&s.heavy_list, (size_t) 2 * HEAVY_CLASSES * MAX_HEAVY, own);
    if (!rc) rc = dalloc(&s.heavy_count, (size_t) 2 * HEAVY_CLASSES, own);
    if (!rc) rc = dalloc(&s.queue_next, 6, own);
    if (!rc) rc = dalloc(&s.heavy_mark, (size_t) Ntot, own);
    /* heavy part of the work queue: threshold on the day-start rate sum
     * (options, else SIMINF_HEAVY_RATE in the environment, 0 = off;
     * default 8, the best of 2 to 128 on the 10^6-node SEIR workload) */
    s.heavy_rate = 8.0;
    if (const char *ev = getenv("SIMINF_HEAVY_RATE"))
        s.heavy_rate = atof(ev);
    if (opt && opt->heavy_rate > 0)
        s.heavy_rate = opt->heavy_rate;
    else if (opt && opt->heavy_rate < 0)
        s.heavy_rate = 0.0;
    s.aem = a->solver == 1;
    if (s.aem && !(opt && opt->heavy_rate > 0) && !getenv("SIMINF_HEAVY_RATE"))
        s.heavy_rate = 0.0;             /* aem: the heavy part is off unless asked for */
    if (s.aem) {
        if (!rc) rc = dalloc(&s.react_time, (size_t) Ntot * Nt, own);
        if (!rc) rc = dalloc(&s.react_inf, (size_t) Ntot * Nt, own);
        if (!rc) rc = dalloc(&s.react_ctr, (size_t) Ntot * Nt, own);
    }
    /* two-pass days (options, else SIMINF_TWO_PASS, else from 500,000
     * nodes: below that a day is short and the extra launch costs more
     * than the quiet nodes it takes out of the work queue) */
    s.two_pass = Ntot >= 500000;
    if (const char *ev = getenv("SIMINF_TWO_PASS"))
        s.two_pass = atoi(ev) > 0;
    if (opt && opt->two_pass)
        s.two_pass = opt->two_pass > 0;
    if (s.aem)
        s.two_pass = 0;                 /* the work queue is the direct method's */
    if (!rc) rc = dalloc(&s.active, (size_t) Ntot, own);
    if (!rc) {
        s.err_day = s.err_count + 1;
        s.err_day_pre_e2 = s.err_count + 2;
    }

    /* outputs */
    if (!rc && !no_output) {
        if (a->U) {
            p->U_len = (size_t) Nn * Nc * (size_t) Nrep * tlen;
            rc = dalloc(&s.U, p->U_len, own);
        } else {
            const size_t ncol = (size_t) Nrep * tlen;
            p->prU_len = (size_t) a->jcU[ncol];
            int *dir, *djc;
            rc = upload(&djc, a->jcU, ncol + 1, own, st);
            if (!rc) rc = upload(&dir, a->irU, p->prU_len, own, st);
            if (!rc) rc = dalloc(&s.prU, p->prU_len, own);
            s.jcU = djc;
            s.irU = dir;
        }
    }
    if (!rc && Nd > 0 && !no_output) {
        if (a->V) {
            p->V_len = (size_t) Nn * Nd * (size_t) Nrep * tlen;
            rc = dalloc(&s.V, p->V_len, own);
        } else if (a->jcV) {
            const size_t ncol = (size_t) Nrep * tlen;
            p->prV_len = (size_t) a->jcV[ncol];
            int *dir, *djc;
            rc = upload(&djc, a->jcV, ncol + 1, own, st);
            if (!rc) rc = upload(&dir, a->irV, p->prV_len, own, st);
            if (!rc) rc = dalloc(&s.prV, p->prV_len, own);
            s.jcV = djc;
            s.irV = dir;
        }
    }
    if (!rc) {
        /* initial state stays on the device so plan_run can restart */
        rc = upload(&p->d_u0, a->u0, (size_t) Ntot * Nc, own, st);
        if (!rc && Nd > 0)
            rc = upload(&p->d_v0, a->v0, (size_t) Ntot * Nd, own, st);
    }
    if (!rc) {
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess)
            rc = cuda_fail(e, "upload");
    }
    if (rc) {
        siminf_gpu_plan_free(p);
        return rc;
    }
    /* every replicate applies the whole schedule */
    p->stats.e1_events = p->e1_count * (uint64_t) Nrep;
    p->stats.e2_events = p->e2_count * (uint64_t) Nrep;
    p->stats.e2_waves = (int) p->wave_ptr.size() - 1;
    p->stats.days = p->ndays;
    p->stats.ms_upload = ms_since(t0);
    *out = p;
    return 0;
}

/* Pick the error the reference would report from the device candidates
 * and the planned ones. */
static int resolve_errors(siminf_gpu_plan *p, std::vector<ErrRec> &cands)
{
    for (const PlannedErr &pe : p->planned) {
        for (int r = 0; r < p->s.Nrep; r++) {
            ErrRec e{};
            e.code = pe.code;
            e.phase = pe.phase;
            e.day = pe.day;
            e.rep = r;
            e.node = pe.node;
            e.transition = -1;
            e.event_index = pe.index;
            e.time = p->days[pe.day].tt;
            cands.push_back(e);
        }
    }
    if (cands.empty())
        return 0;
    /* replicate first (mssm runs replicates one after another), then day */
    int rep = INT_MAX, day = INT_MAX;
    for (auto &e : cands)
        rep = std::min(rep, e.rep);
    for (auto &e : cands)
        if (e.rep == rep)
            day = std::min(day, e.day);
    std::vector<ErrRec> c;
    for (auto &e : cands)
        if (e.rep == rep && e.day == day)
            c.push_back(e);
    const ErrRec *best = nullptr;
    /* initialisation or SSA: lowest node */
    for (int ph : {(int) PHASE_INIT, (int) PHASE_SSA}) {
        for (auto &e : c)
            if (e.phase == ph && (!best || e.node < best->node))
                best = &e;
        if (best)
            break;
    }
    if (!best) {
        /* events: lowest position in the event arrays */
        for (auto &e : c)
            if ((e.phase == PHASE_E1 || e.phase == PHASE_E2) &&
                (!best || e.event_index < best->event_index))
                best = &e;
    }
    ErrRec res{};
    bool have = false;
    if (best) {
        res = *best;
        have = true;
    }
    if (!best || best->phase != PHASE_INIT) {
        /* the post-time-step loop runs in node order and overwrites */
        std::vector<ErrRec> pts;
        for (auto &e : c)
            if (e.phase == PHASE_PTS)
                pts.push_back(e);
        /* stable: one node's records stay in the order its thread wrote
         * them (transition order), so the last one wins as in the
         * reference's loop */
        std::stable_sort(pts.begin(), pts.end(), [](const ErrRec &x, const ErrRec &y) {
            return x.node < y.node;
        });
        for (auto &e : pts) {
            res = e;
            have = true;
            if (e.code != SIMINF_GPU_ERR_INVALID_RATE)
                break;
        }
    }
    if (!have)
        return 0;
    char msg[300];
    snprintf(msg, sizeof(msg),
             "error %d at time %g, replicate %d, node %d (one-based), transition %d, event %d, rate %g",
             res.code, res.time, res.rep + 1, res.node + 1,
             res.transition >= 0 ? res.transition + 1 : 0,
             res.event_index >= 0 ? res.event_index + 1 : 0, res.rate);
    set_status(res.code, res.node, res.transition, res.event_index, res.time, res.rate, msg);
    return res.code;
}

/* Per-kernel-kind device time of one run: [0] init, [1] ssa_e1, [2] e2_wave,
 * [3] pts_store, [4] horizon, [5] quick. */
struct KernelProfile {
    cudaEvent_t a, b;
    double ms[8];
    long long n[8];
};

}  /* extern "C" */

template <class F>
static cudaError_t timed(KernelProfile *kp, int kind, cudaStream_t st, F &&launch)
{
    if (!kp)
        return launch();
    cudaEventRecord(kp->a, st);
    cudaError_t e = launch();
    cudaEventRecord(kp->b, st);
    if (e == cudaSuccess)
        e = cudaEventSynchronize(kp->b);
    float ms = 0;
    cudaEventElapsedTime(&ms, kp->a, kp->b);
    kp->ms[kind] += ms;
    kp->n[kind]++;
    return e;
}

/* Copies of columns [c_lo, c_hi) of every replicate's U and V (dense or
 * sparse, column k of replicate r at k + r * tlen) to a's host arrays,
 * queued on st. */
static cudaError_t download_columns(const siminf_gpu_plan *p, const siminf_gpu_solver_args *a,
                                    int c_lo, int c_hi, cudaStream_t st)
{
    const DevState &s = p->s;
    const size_t col_u = (size_t) s.Nn * s.Nc, col_v = (size_t) s.Nn * s.Nd;
    const auto d2h = cudaMemcpyDeviceToHost;
    cudaError_t e = cudaSuccess;
    for (int r = 0; r < s.Nrep && c_hi > c_lo && e == cudaSuccess; r++) {
        const size_t k0 = (size_t) r * s.tlen + c_lo, k1 = (size_t) r * s.tlen + c_hi;
        if (a->U && s.U) {
            e = cudaMemcpyAsync(a->U + k0 * col_u, s.U + k0 * col_u,
                                (k1 - k0) * col_u * sizeof(int), d2h, st);
        } else if (a->prU && s.prU) {
            const size_t j0 = (size_t) a->jcU[k0], j1 = (size_t) a->jcU[k1];
            if (j1 > j0)
                e = cudaMemcpyAsync(a->prU + j0, s.prU + j0, (j1 - j0) * sizeof(double), d2h, st);
        }
        if (e != cudaSuccess)
            break;
        if (a->V && s.V && col_v) {
            e = cudaMemcpyAsync(a->V + k0 * col_v, s.V + k0 * col_v,
                                (k1 - k0) * col_v * sizeof(double), d2h, st);
        } else if (a->prV && s.prV) {
            const size_t j0 = (size_t) a->jcV[k0], j1 = (size_t) a->jcV[k1];
            if (j1 > j0)
                e = cudaMemcpyAsync(a->prV + j0, s.prV + j0, (j1 - j0) * sizeof(double), d2h, st);
        }
    }
    return e;
}

/* The wavefronts of one day: offsets into d_e2 and event counts.  The
 * last ones, while each holds at most E2_TAIL_ITEMS events x replicates,
 * run together in one block (k_e2_tail), up to E2_TAIL_WAVES per launch;
 * the others, one launch each. */
static cudaError_t launch_day_waves(const siminf_gpu_plan *p, const DevState &s,
                                    const long long *off, const long long *cnt, int nw, int d,
                                    double tt, cudaStream_t st, KernelProfile *kp)
{
    const Launchers *L = p->L;
    int t = nw;
    while (t > 0 && cnt[t - 1] * (long long) s.Nrep <= E2_TAIL_ITEMS)
        t--;
    if (nw - t < 2)
        t = nw;                         /* a single small wave: its own launch */
    cudaError_t e = cudaSuccess;
    for (int w = 0; w < t && e == cudaSuccess; w++)
        e = timed(kp, 2, st, [&] { return L->e2_wave(s, p->d_e2 + off[w], (int) cnt[w], d, tt, st); });
    for (int w = t; w < nw && e == cudaSuccess; w += E2_TAIL_WAVES) {
        E2Tail tail;
        tail.n = std::min((int) E2_TAIL_WAVES, nw - w);
        for (int k = 0; k < tail.n; k++) {
            tail.off[k] = off[w + k];
            tail.count[k] = (int) cnt[w + k];
        }
        e = timed(kp, 2, st, [&] { return L->e2_tail(s, p->d_e2, tail, d, tt, st); });
    }
    return e;
}

static cudaError_t launch_all(siminf_gpu_plan *p, DevState s, cudaStream_t st, KernelProfile *kp)
{
    const Launchers *L = p->L;
    const int ndays = p->max_days > 0 ? std::min(p->max_days, p->ndays) : p->ndays;
    cudaError_t e = timed(kp, 0, st, [&] {
        return s.aem ? L->aem_init(s, p->tt0, st) : L->init(s, p->tt0, st);
    });
    if (e != cudaSuccess)
        return e;
    if (p->horizon)
        return timed(kp, 4, st, [&] { return L->horizon(s, p->d_days, ndays, st); });
    for (int d = 0; d < ndays && e == cudaSuccess; d++) {
        const DayInfo &di = p->days[d];
        if (s.two_pass && !s.aem)
            e = timed(kp, 5, st, [&] { return L->quick(s, d, di.tt, di.next, st); });
        if (e == cudaSuccess)
            e = timed(kp, 1, st, [&] {
                return s.aem ? L->aem_day(s, d, di.tt, di.next, st)
                             : L->ssa_e1(s, d, di.tt, di.next, st);
            });
        if (e == cudaSuccess) {
            const int w0 = p->day_wave[d], nw = p->day_wave[d + 1] - w0;
            std::vector<long long> cnt((size_t) nw);
            for (int w = 0; w < nw; w++)
                cnt[w] = p->wave_ptr[w0 + w + 1] - p->wave_ptr[w0 + w];
            e = launch_day_waves(p, s, p->wave_ptr.data() + w0, cnt.data(), nw, d, di.tt, st, kp);
        }
        if (e == cudaSuccess)
            e = timed(kp, 3, st, [&] {
                return s.aem ? L->aem_pts(s, d, di.tt, di.c0, di.c1, s.vA, s.vB, st)
                             : L->pts_store(s, d, di.tt, di.c0, di.c1, s.vA, s.vB, st);
            });
        std::swap(s.vA, s.vB);
    }
    return e;
}

/* Records of n external transfers in wave order, from the event columns
 * of one chunk's input range (staged on the device, position 0 = input
 * position rel) and the order the host planned (positions within it). */
struct StagedCols {
    int *node, *dest, *n, *select, *shift;
    double *proportion;
};

__global__ void k_gather_e2(StagedCols c, const uint32_t *order, long long n, long long rel,
                            E2Rec *out)
{
    const long long k = blockIdx.x * (long long) blockDim.x + threadIdx.x;
    if (k >= n)
        return;
    const uint32_t j = order[k];
    E2Rec e;
    e.src = c.node[j] - 1;
    e.dst = c.dest[j] - 1;
    e.n = c.n[j];
    e.select = c.select[j] - 1;
    e.shift = c.shift[j] - 1;
    e.index = (int) (rel + j);
    e.proportion = c.proportion[j];
    out[k] = e;
}

/* The first run of a streamed plan: host threads plan the external
 * transfers' waves day by day while this thread copies each chunk of
 * finished days to the device on a copy stream and queues the chunk's
 * kernels behind it, so planning and copying overlap the GPU's work on
 * earlier days.  The planners write each chunk straight into one slot of a
 * ring of pinned host buffers, from which the copy runs as DMA without
 * holding this thread; a slot is reused once its previous copy is done.
 * With pinned output arrays (p->out_args) the columns of U/V each chunk
 * finishes are copied back on a third stream while later days run.
 * The kernels and their order are those of launch_all. */
static cudaError_t launch_streamed(siminf_gpu_plan *p, DevState s, cudaStream_t st)
{
    const Launchers *L = p->L;
    const siminf_gpu_solver_args *a = &p->args;
    const int ndays = p->ndays;
    enum { CHUNK_DAYS = 8, RING = 8 };
    cudaError_t e = s.aem ? L->aem_init(s, p->tt0, st) : L->init(s, p->tt0, st);
    if (e != cudaSuccess)
        return e;

    const int nchunks = (ndays + CHUNK_DAYS - 1) / CHUNK_DAYS;
    /* without the scan (p->scan_free) a day's transfers go to its chunk's
     * slot at the day's input offset in the chunk, and the day offsets in
     * d_e2 come from the planners' counts chunk by chunk */
    const bool sf = p->scan_free;
    long long slot_len = 1, in_len = 1;
    for (int c = 0; c < nchunks; c++) {
        const int d0 = c * CHUNK_DAYS, d1 = std::min(ndays, d0 + (int) CHUNK_DAYS);
        if (!sf)
            slot_len = std::max(slot_len, p->e2_day_off[d1] - p->e2_day_off[d0]);
        in_len = std::max(in_len, p->e2_hi[d1 - 1] - p->e2_lo[d0]);
    }
    if (sf)
        slot_len = in_len;
    std::vector<DayScan> scans(sf ? ndays : 0);
    /* With the transfer columns in pinned host memory, the planners write
     * each day's order (4 B a transfer) and the device gathers the records
     * from the columns it receives by DMA (28 B an event); otherwise they
     * write the records (32 B a transfer) into the ring, as the copy then
     * needs */
    const bool gather = host_pinned(a->node) && host_pinned(a->dest) && host_pinned(a->n) &&
                        host_pinned(a->select) && host_pinned(a->shift) &&
                        host_pinned(a->proportion);
    const size_t elem = gather ? sizeof(uint32_t) : sizeof(E2Rec);
    char *ring = nullptr;
    size_t ring_bytes = 0;
    e = pinned_acquire((size_t) RING * slot_len * elem, (void **) &ring, &ring_bytes);
    if (e != cudaSuccess)
        return e;
    /* two sets of staged event columns and orders on the device */
    StagedCols stg[2] = {};
    uint32_t *dorder[2] = {};
    std::vector<void *> dbufs;
    for (int k = 0; k < 2 && gather && e == cudaSuccess; k++) {
        int **cols[5] = {&stg[k].node, &stg[k].dest, &stg[k].n, &stg[k].select, &stg[k].shift};
        for (int j = 0; j < 5 && e == cudaSuccess; j++) {
            e = cudaMalloc((void **) cols[j], (size_t) in_len * sizeof(int));
            if (e == cudaSuccess)
                dbufs.push_back(*cols[j]);
        }
        if (e == cudaSuccess) e = cudaMalloc((void **) &stg[k].proportion, (size_t) in_len * sizeof(double));
        if (e == cudaSuccess) dbufs.push_back(stg[k].proportion);
        if (e == cudaSuccess) e = cudaMalloc((void **) &dorder[k], (size_t) slot_len * sizeof(uint32_t));
        if (e == cudaSuccess) dbufs.push_back(dorder[k]);
    }
    /* without the scan: each chunk's E1 lists by node go up through one of
     * E1_RING pinned slots into one of E1_RING device buffers, which the
     * chunk's kernels read (a buffer is rewritten once the kernels of the
     * chunk E1_RING earlier are done) */
    enum { E1_RING = 4 };
    const int Nn = a->Nn;
    int *d_e1p[E1_RING] = {};
    E1Rec *d_e1r[E1_RING] = {};
    uint32_t *d_e1k[E1_RING] = {};
    long long d_e1r_cap[E1_RING] = {};
    std::vector<long long> e1_tmp, e1_merged;
    char *h_e1[E1_RING] = {};
    size_t h_e1_bytes[E1_RING] = {};
    std::vector<cudaEvent_t> e1_used(sf ? nchunks : 0, nullptr);
    for (int r = 0; r < E1_RING && sf && e == cudaSuccess; r++) {
        e = cudaMalloc((void **) &d_e1p[r], ((size_t) Nn + 1) * sizeof(int));
        if (e == cudaSuccess)
            dbufs.push_back(d_e1p[r]);
    }
    if (e != cudaSuccess) {
        for (void *q : dbufs)
            cudaFree(q);
        pinned_release(ring, ring_bytes);
        return e;
    }

    std::unique_ptr<std::atomic<int>[]> done(new std::atomic<int>[ndays]);
    std::unique_ptr<std::atomic<int>[]> issued(new std::atomic<int>[nchunks]);
    std::vector<cudaEvent_t> copied(nchunks, nullptr);
    for (int d = 0; d < ndays; d++)
        done[d].store(0);
    for (int c = 0; c < nchunks; c++)
        issued[c].store(0);
    std::atomic<int> next_day(0), failed(0), abort(0);
    std::vector<std::thread> workers;
    const int nthreads = std::max(1, planner_threads() - 1);
    for (int t = 0; t < nthreads; t++)
        workers.emplace_back([&]() {
            try {
                WaveTracker w(a->Nn);
                for (int d = next_day++; d < ndays && !abort.load(); d = next_day++) {
                    const int c = d / CHUNK_DAYS;
                    if (c >= RING) {
                        /* the slot's previous chunk must have left it;
                         * planners that wait sleep (blocking-sync events,
                         * short naps), so the launching thread keeps a
                         * core */
                        while (!issued[c - RING].load(std::memory_order_acquire) &&
                               !abort.load())
                            std::this_thread::sleep_for(std::chrono::microseconds(50));
                        if (abort.load())
                            break;
                        cudaEventSynchronize(copied[c - RING]);
                    }
                    char *slot = ring + (size_t) (c % RING) * slot_len * elem;
                    const int d0 = c * CHUNK_DAYS;
                    if (sf) {
                        scan_day(p, a, d, scans[d]);
                        sort_e1_by_node(a, scans[d].e1);
                    }
                    const long long at = sf ? p->e2_lo[d] - p->e2_lo[d0]
                                            : p->e2_day_off[d] - p->e2_day_off[d0];
                    const long long n2 =
                        gather ? plan_day_order(p, a, d, w, (uint32_t *) slot, at, p->e2_lo[d0])
                               : plan_day_waves(p, a, d, w, (E2Rec *) slot, at);
                    if (sf)
                        scans[d].n2 = n2;
                    done[d].store(1, std::memory_order_release);
                }
            } catch (...) {
                failed.store(1);
            }
        });

    cudaStream_t cs = nullptr, ds = nullptr;
    std::vector<cudaEvent_t> stored;
    e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (e == cudaSuccess && p->out_args)
        e = cudaStreamCreateWithFlags(&ds, cudaStreamNonBlocking);
    static const bool prof = getenv("SIMINF_SCHED_PROFILE") && getenv("SIMINF_SCHED_PROFILE")[0] == '1';
    double waited = 0;
    long long e1_total = 0;
    int issued_chunks = 0;
    for (int c = 0; c < nchunks && e == cudaSuccess; c++) {
        const int d0 = c * CHUNK_DAYS, d1 = std::min(ndays, d0 + (int) CHUNK_DAYS);
        auto w0 = std::chrono::steady_clock::now();
        for (int d = d0; d < d1 && !failed.load(); d++)
            while (!done[d].load(std::memory_order_acquire) && !failed.load())
                std::this_thread::yield();
        waited += ms_since(w0);
        if (failed.load()) {
            e = cudaErrorMemoryAllocation;
            break;
        }
        if (sf) {
            /* what plan_scan would have found in these days */
            long long bad = -1;
            for (int d = d0; d < d1 && bad < 0; d++)
                bad = scans[d].bad;
            if (bad >= 0) {
                p->dev_bad = bad;       /* out of order: the run stops here */
                break;
            }
            int msel = p->max_select, mshift = p->max_shift;
            long long n1 = 0;
            std::vector<const std::vector<long long> *> pos;
            for (int d = d0; d < d1; d++) {
                p->e2_day_off[d + 1] = p->e2_day_off[d] + scans[d].n2;
                p->planned.insert(p->planned.end(), scans[d].planned.begin(),
                                  scans[d].planned.end());
                msel = std::max(msel, scans[d].max_select);
                mshift = std::max(mshift, scans[d].max_shift);
                n1 += (long long) scans[d].e1.size();
                pos.push_back(&scans[d].e1);
            }
            /* E and N up to the largest select and shift seen so far */
            if (msel > p->max_select && a->jcE) {
                int *djcE, *dirE;
                double *dprE;
                const int nnz = a->jcE[msel];
                int rc = upload(&djcE, a->jcE, (size_t) msel + 1, p->owned, st);
                if (!rc) rc = upload(&dirE, a->irE, (size_t) nnz, p->owned, st);
                if (!rc) rc = upload(&dprE, (const double *) a->prE, (size_t) nnz, p->owned, st);
                if (rc) {
                    e = cudaErrorMemoryAllocation;
                    break;
                }
                s.jcE = p->s.jcE = djcE;
                s.irE = p->s.irE = dirE;
                s.prE = p->s.prE = dprE;
                p->max_select = msel;
            }
            if (mshift > p->max_shift && a->N) {
                int *dN;
                if (upload(&dN, a->N, (size_t) mshift * a->Nc, p->owned, st)) {
                    e = cudaErrorMemoryAllocation;
                    break;
                }
                s.Nshift = p->s.Nshift = dN;
                p->max_shift = mshift;
            }
            /* the chunk's E1 lists by node: records and their nodes go up,
             * the per-node offsets are found on the device */
            const int r = c % E1_RING;
            if (c >= E1_RING) {
                e = cudaEventSynchronize(copied[c - E1_RING]);     /* the slot's last copy */
                if (e == cudaSuccess)
                    e = cudaStreamWaitEvent(cs, e1_used[c - E1_RING], 0);
            }
            const size_t need = (size_t) std::max(1LL, n1) * (sizeof(E1Rec) + sizeof(uint32_t));
            if (e == cudaSuccess && need > h_e1_bytes[r]) {
                pinned_release(h_e1[r], h_e1_bytes[r]);
                h_e1[r] = nullptr;
                h_e1_bytes[r] = 0;
                e = pinned_acquire(need, (void **) &h_e1[r], &h_e1_bytes[r]);
            }
            if (e == cudaSuccess && std::max(1LL, n1) > d_e1r_cap[r]) {
                const long long cap1 = std::max(1LL, n1);
                E1Rec *nb = nullptr;
                uint32_t *nk = nullptr;
                e = cudaMalloc((void **) &nb, (size_t) cap1 * sizeof(E1Rec));
                if (e == cudaSuccess)
                    dbufs.push_back(nb);        /* the old ones are freed at the end */
                if (e == cudaSuccess)
                    e = cudaMalloc((void **) &nk, (size_t) cap1 * sizeof(uint32_t));
                if (e == cudaSuccess) {
                    dbufs.push_back(nk);
                    d_e1r[r] = nb;
                    d_e1k[r] = nk;
                    d_e1r_cap[r] = cap1;
                }
            }
            if (e != cudaSuccess)
                break;
            E1Rec *hr = (E1Rec *) h_e1[r];
            uint32_t *hk = (uint32_t *) (h_e1[r] + (size_t) std::max(1LL, n1) * sizeof(E1Rec));
            merge_e1_days(a, pos, hr, hk, e1_tmp, e1_merged);
            if (n1 > 0)
                e = cudaMemcpyAsync(d_e1r[r], hr, (size_t) n1 * sizeof(E1Rec),
                                    cudaMemcpyHostToDevice, cs);
            if (e == cudaSuccess && n1 > 0)
                e = cudaMemcpyAsync(d_e1k[r], hk, (size_t) n1 * sizeof(uint32_t),
                                    cudaMemcpyHostToDevice, cs);
            if (e == cudaSuccess)
                e = e1_ptr_from_keys(d_e1k[r], n1, Nn, d_e1p[r], cs);
            if (e != cudaSuccess)
                break;
            s.e1 = d_e1r[r];
            s.e1_ptr = d_e1p[r];
            e1_total += n1;
        }
        const long long lo = p->e2_day_off[d0], hi = p->e2_day_off[d1];
        /* the chunk's event columns and the planned order go up, and the
         * records are gathered on the device (the copy stream runs chunks
         * in order, so a staging set is free again two chunks later) */
        const long long in_lo = p->e2_lo[d0], in_n = p->e2_hi[d1 - 1] - in_lo;
        StagedCols &sc = stg[c % 2];
        e = cudaEventCreateWithFlags(&copied[c], cudaEventDisableTiming | cudaEventBlockingSync);
        if (e == cudaSuccess && hi > lo && !gather && sf) {
            /* each day's records from its place in the slot */
            for (int d = d0; d < d1 && e == cudaSuccess; d++)
                if (scans[d].n2 > 0)
                    e = cudaMemcpyAsync(p->d_e2 + p->e2_day_off[d],
                                        ring + ((size_t) (c % RING) * slot_len +
                                                (size_t) (p->e2_lo[d] - in_lo)) * elem,
                                        (size_t) scans[d].n2 * sizeof(E2Rec),
                                        cudaMemcpyHostToDevice, cs);
        } else if (e == cudaSuccess && hi > lo && !gather) {
            e = cudaMemcpyAsync(p->d_e2 + lo, ring + (size_t) (c % RING) * slot_len * elem,
                                (size_t) (hi - lo) * sizeof(E2Rec), cudaMemcpyHostToDevice, cs);
        } else if (e == cudaSuccess && hi > lo) {
            const int *src_i[5] = {a->node, a->dest, a->n, a->select, a->shift};
            int *dst_i[5] = {sc.node, sc.dest, sc.n, sc.select, sc.shift};
            for (int k = 0; k < 5 && e == cudaSuccess; k++)
                e = cudaMemcpyAsync(dst_i[k], src_i[k] + in_lo, (size_t) in_n * sizeof(int),
                                    cudaMemcpyHostToDevice, cs);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(sc.proportion, a->proportion + in_lo,
                                    (size_t) in_n * sizeof(double), cudaMemcpyHostToDevice, cs);
            /* the order: one run of hi - lo entries, or with the days at
             * their input offsets (gaps where other events sit) */
            const long long ord_n = sf ? in_n : hi - lo;
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(dorder[c % 2], ring + (size_t) (c % RING) * slot_len * elem,
                                    (size_t) ord_n * sizeof(uint32_t), cudaMemcpyHostToDevice, cs);
            if (e == cudaSuccess && !sf) {
                k_gather_e2<<<(unsigned) ((hi - lo + 255) / 256), 256, 0, cs>>>(
                    sc, dorder[c % 2], hi - lo, in_lo, p->d_e2 + lo);
                e = cudaGetLastError();
            }
            for (int d = d0; sf && d < d1 && e == cudaSuccess; d++) {
                const long long n2 = scans[d].n2;
                if (n2 <= 0)
                    continue;
                k_gather_e2<<<(unsigned) ((n2 + 255) / 256), 256, 0, cs>>>(
                    sc, dorder[c % 2] + (p->e2_lo[d] - in_lo), n2, in_lo,
                    p->d_e2 + p->e2_day_off[d]);
                e = cudaGetLastError();
            }
        }
        if (e == cudaSuccess)
            e = cudaEventRecord(copied[c], cs);
        if (e != cudaSuccess)
            break;
        issued[c].store(1, std::memory_order_release);
        e = cudaStreamWaitEvent(st, copied[c], 0);
        for (int d = d0; d < d1 && e == cudaSuccess; d++) {
            const DayInfo &di = p->days[d];
            if (s.two_pass && !s.aem)
                e = L->quick(s, d, di.tt, di.next, st);
            if (e == cudaSuccess)
                e = s.aem ? L->aem_day(s, d, di.tt, di.next, st)
                          : L->ssa_e1(s, d, di.tt, di.next, st);
            if (e == cudaSuccess) {
                const std::vector<long long> &cnt = p->day_waves[d];
                std::vector<long long> off(cnt.size());
                long long o = p->e2_day_off[d];
                for (size_t w = 0; w < cnt.size(); w++) {
                    off[w] = o;
                    o += cnt[w];
                }
                e = launch_day_waves(p, s, off.data(), cnt.data(), (int) cnt.size(), d, di.tt,
                                     st, nullptr);
            }
            if (e == cudaSuccess)
                e = s.aem ? L->aem_pts(s, d, di.tt, di.c0, di.c1, s.vA, s.vB, st)
                          : L->pts_store(s, d, di.tt, di.c0, di.c1, s.vA, s.vB, st);
            std::swap(s.vA, s.vB);
        }
        if (sf && e == cudaSuccess) {
            /* the chunk's E1 buffers are free once its days have run */
            e = cudaEventCreateWithFlags(&e1_used[c], cudaEventDisableTiming);
            if (e == cudaSuccess)
                e = cudaEventRecord(e1_used[c], st);
        }
        if (e == cudaSuccess)
            issued_chunks = c + 1;
        /* the columns this chunk finished go back while later days run */
        const int c_hi = p->days[d1 - 1].c1;
        if (ds && e == cudaSuccess && c_hi > p->cols_sent) {
            cudaEvent_t ev = nullptr;
            e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
            if (e == cudaSuccess) {
                stored.push_back(ev);
                e = cudaEventRecord(ev, st);
            }
            if (e == cudaSuccess)
                e = cudaStreamWaitEvent(ds, ev, 0);
            if (e == cudaSuccess)
                e = download_columns(p, p->out_args, p->cols_sent, c_hi, ds);
            if (e == cudaSuccess)
                p->cols_sent = c_hi;
        }
    }
    /* planners waiting for a slot give up once the copies stop */
    abort.store(1);
    for (auto &t : workers)
        t.join();
    if (sf && e == cudaSuccess && p->dev_bad < 0 && issued_chunks == nchunks) {
        /* events past the last day: the order check */
        const long long len = a->len, tail_lo = p->e2_hi[ndays - 1];
        for (long long i = std::max(1LL, tail_lo); i < len; i++) {
            const int tm = a->time[i], pt = a->time[i - 1];
            const int kind = a->event[i], pk = a->event[i - 1];
            if (tm < pt || (tm == pt && pk == SIMINF_GPU_EXTERNAL_TRANSFER_EVENT &&
                            kind != SIMINF_GPU_EXTERNAL_TRANSFER_EVENT)) {
                p->dev_bad = i;
                break;
            }
        }
        /* the E1 lists of the whole run by node, for later runs */
        std::vector<const std::vector<long long> *> pos;
        for (int d = 0; d < ndays; d++)
            pos.push_back(&scans[d].e1);
        std::vector<int> ptr((size_t) Nn + 1);
        std::vector<E1Rec> rec((size_t) std::max(1LL, e1_total));
        bucket_e1(a, pos, rec.data(), ptr.data());
        int *dptr = nullptr;
        E1Rec *drec = nullptr;
        if (upload(&dptr, ptr.data(), ptr.size(), p->owned, cs) ||
            upload(&drec, rec.data(), rec.size(), p->owned, cs)) {
            e = cudaErrorMemoryAllocation;
        } else {
            e = cudaStreamSynchronize(cs);
            p->s.e1 = drec;
            p->s.e1_ptr = dptr;
            p->e1_count = (uint64_t) e1_total;
            p->e2_count = (uint64_t) p->e2_day_off[ndays];
        }
    }
    if (prof)
        fprintf(stderr, "streamed run (host waves): %.2f ms waiting for plans\n", waited);
    if (cs) {
        const cudaError_t e2 = cudaStreamSynchronize(cs);
        if (e == cudaSuccess)
            e = e2;
        cudaStreamDestroy(cs);
    }
    if (ds) {
        const cudaError_t e2 = cudaStreamSynchronize(ds);
        if (e == cudaSuccess)
            e = e2;
        cudaStreamDestroy(ds);
    }
    for (cudaEvent_t ev : copied)
        if (ev)
            cudaEventDestroy(ev);
    for (cudaEvent_t ev : stored)
        cudaEventDestroy(ev);
    for (cudaEvent_t ev : e1_used)
        if (ev)
            cudaEventDestroy(ev);
    if (!dbufs.empty())
        cudaStreamSynchronize(st);      /* the chunk buffers' last readers */
    for (void *q : dbufs)
        cudaFree(q);
    for (int r = 0; r < E1_RING; r++)
        pinned_release(h_e1[r], h_e1_bytes[r]);
    pinned_release(ring, ring_bytes);
    return e;
}

/* The first run of a streamed plan whose events the device plans
 * (siminf_schedule.cu).  A planner thread copies each chunk of days'
 * event columns to the device and plans them on its own stream -- the
 * chunk's external transfers in wave order go to d_e2 after the previous
 * chunks', its E1 records by node to e1_all after the previous chunks',
 * its per-node offsets to one of E1_RING buffers -- while this thread
 * queues each planned chunk's kernels, so planning overlaps the GPU's work
 * on earlier days.  After the run, the planner's status gives the order
 * check and the planned failures, and the E1 records of all chunks merge
 * into the per-node CSR later runs read. */
static cudaError_t launch_streamed_dev(siminf_gpu_plan *p, DevState s, cudaStream_t st)
{
    const Launchers *L = p->L;
    const siminf_gpu_solver_args *a = &p->args;
    const int ndays = p->ndays, Nn = a->Nn;
    enum { CHUNK_DAYS = 8, E1_RING = 3 };
    const int nchunks = (ndays + CHUNK_DAYS - 1) / CHUNK_DAYS;
    const long long len = a->len, tail_lo = p->e2_hi[ndays - 1];
    long long cap = 1;
    for (int c = 0; c < nchunks; c++) {
        const int d0 = c * CHUNK_DAYS, d1 = std::min(ndays, d0 + (int) CHUNK_DAYS);
        cap = std::max(cap, p->e2_hi[d1 - 1] - p->e2_lo[d0]);
    }
    /* the day kernels go to their own stream, which starts after and ends
     * before the caller's.  When the device plans the levels (its rounds
     * are most of its work), that stream has the highest priority, so that
     * the planner's kernels fill the SMs the day kernels leave idle instead
     * of delaying them; when the host plans them, the planner's few kernels
     * a chunk go first, each between two of the day kernels, instead of
     * waiting for a gap in them */
    cudaStream_t caller = st;
    int lo_pri = 0, hi_pri = 0;
    cudaDeviceGetStreamPriorityRange(&lo_pri, &hi_pri);
    const int day_pri = p->dev_levels ? lo_pri : hi_pri;
    const int plan_pri = p->dev_levels ? hi_pri : lo_pri;
    cudaStream_t hs = nullptr;
    cudaEvent_t hs_start = nullptr, hs_end = nullptr;
    cudaError_t e = cudaStreamCreateWithPriority(&hs, cudaStreamNonBlocking, day_pri);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&hs_start, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&hs_end, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventRecord(hs_start, caller);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(hs, hs_start, 0);
    if (e != cudaSuccess)
        return e;
    st = hs;
    e = s.aem ? L->aem_init(s, p->tt0, st) : L->init(s, p->tt0, st);
    if (e != cudaSuccess)
        return e;

    cudaStream_t ps = nullptr, ds = nullptr;
    e = cudaStreamCreateWithPriority(&ps, cudaStreamNonBlocking, plan_pri);
    if (e == cudaSuccess && p->out_args)
        e = cudaStreamCreateWithFlags(&ds, cudaStreamNonBlocking);
    int dev = 0;
    cudaGetDevice(&dev);
    DevScheduler sch;
    if (e == cudaSuccess)
        e = sch.init(std::min(cap, std::max(len - tail_lo, cap)), Nn, p->nsel, ps);
    /* E1 records of every chunk, their nodes, and a ring of offsets */
    long long e1_cap = std::max(1LL, len / 64);
    E1Rec *e1_all = nullptr;
    uint32_t *e1_nodes = nullptr;
    std::vector<void *> old_e1;
    int *ring[E1_RING] = {};
    if (e == cudaSuccess) e = cudaMalloc((void **) &e1_all, (size_t) e1_cap * sizeof(E1Rec));
    if (e == cudaSuccess) e = cudaMalloc((void **) &e1_nodes, (size_t) e1_cap * sizeof(uint32_t));
    for (int r = 0; r < E1_RING && e == cudaSuccess; r++)
        e = cudaMalloc((void **) &ring[r], ((size_t) Nn + 1) * sizeof(int));
    /* levels from host threads (p->dev_levels): each chunk's transfers'
     * levels by input position in one of LRING pinned slots, copied up
     * before the device plans the chunk */
    enum { LRING = 4 };
    const bool hl = p->dev_levels;
    uint32_t *lslot = nullptr, *d_lslot = nullptr;
    size_t lslot_bytes = 0;
    if (hl && e == cudaSuccess)
        e = pinned_acquire((size_t) LRING * cap * sizeof(uint32_t), (void **) &lslot, &lslot_bytes);
    if (hl && e == cudaSuccess)
        e = cudaMalloc((void **) &d_lslot, (size_t) cap * sizeof(uint32_t));
    if (e != cudaSuccess) {
        for (int r = 0; r < E1_RING; r++)
            cudaFree(ring[r]);
        cudaFree(e1_all);
        cudaFree(e1_nodes);
        cudaFree(d_lslot);
        pinned_release(lslot, lslot_bytes);
        for (cudaStream_t x : {ps, ds})
            if (x)
                cudaStreamDestroy(x);
        return e;
    }

    struct Planned {
        SchedChunk ch;
        long long base2 = 0;
        E1Rec *e1 = nullptr;
        cudaError_t err = cudaSuccess;
    };
    std::vector<Planned> plans(nchunks);
    std::unique_ptr<std::atomic<int>[]> ready(new std::atomic<int>[nchunks]);
    std::unique_ptr<std::atomic<int>[]> queued(new std::atomic<int>[nchunks]);
    std::vector<cudaEvent_t> done(nchunks, nullptr);
    for (int c = 0; c < nchunks; c++) {
        ready[c].store(0);
        queued[c].store(0);
    }
    std::atomic<int> abort(0);
    long long e1_total = 0, e2_total = 0;
    unsigned long long bad = ~0ULL;

    /* the host's level planners: days in order, each into its chunk's
     * slot; a slot is reused once the device planner has copied it up */
    std::unique_ptr<std::atomic<int>[]> lday(new std::atomic<int>[hl ? ndays : 1]);
    std::unique_ptr<std::atomic<int>[]> lfree(new std::atomic<int>[hl ? nchunks : 1]);
    std::unique_ptr<std::atomic<int>[]> ldeep(new std::atomic<int>[hl ? nchunks : 1]);
    /* the first dev_first chunks the device plans whole (levels too):
     * early in a run the day kernels leave the GPU idle more than the host
     * threads can plan for it, and those threads start further ahead */
    int dev_first = 0;
    if (const char *ev = getenv("SIMINF_DEVICE_FIRST_CHUNKS"))
        dev_first = std::max(0, std::min(nchunks, atoi(ev)));
    if (!hl)
        dev_first = 0;
    std::atomic<int> lnext(std::min(ndays, dev_first * (int) CHUNK_DAYS)), lfail(0);
    std::vector<std::thread> lworkers;
    if (hl) {
        for (int d = 0; d < ndays; d++)
            lday[d].store(0);
        for (int c = 0; c < nchunks; c++) {
            lfree[c].store(0);
            ldeep[c].store(0);
        }
        const int nthreads = std::max(1, planner_threads() - 2);
        for (int t = 0; t < nthreads; t++)
            lworkers.emplace_back([&]() {
                try {
                    WaveTracker w(Nn);
                    for (int d = lnext++; d < ndays && !abort.load(); d = lnext++) {
                        const int c = d / CHUNK_DAYS;
                        if (c >= LRING) {
                            while (!lfree[c - LRING].load(std::memory_order_acquire) &&
                                   !abort.load())
                                std::this_thread::sleep_for(std::chrono::microseconds(50));
                            if (abort.load())
                                break;
                        }
                        const long long l0 = p->e2_lo[c * CHUNK_DAYS];
                        uint32_t *slot = lslot + (size_t) (c % LRING) * cap;
                        const int maxl = plan_day_pos_levels(p, a, d, w, slot + (p->e2_lo[d] - l0));
                        if (maxl > DevScheduler::max_host_level())
                            ldeep[c].store(1);
                        lday[d].store(1, std::memory_order_release);
                    }
                } catch (...) {
                    lfail.store(1);
                }
            });
    }

    std::thread planner([&]() {
        cudaSetDevice(dev);
        long long base1 = 0, base2 = 0;
        for (int c = 0; c < nchunks && !abort.load(); c++) {
            Planned &pl = plans[c];
            const int d0 = c * CHUNK_DAYS, d1 = std::min(ndays, d0 + (int) CHUNK_DAYS),
                      nd = d1 - d0;
            const long long l0 = p->e2_lo[d0], m = p->e2_hi[d1 - 1] - l0;
            cudaError_t pe = cudaSuccess;
            if (c >= E1_RING) {
                /* the offsets buffer is free once that chunk's days ran */
                while (!queued[c - E1_RING].load(std::memory_order_acquire) && !abort.load())
                    std::this_thread::sleep_for(std::chrono::microseconds(20));
                if (abort.load())
                    break;
                pe = cudaStreamWaitEvent(ps, done[c - E1_RING], 0);
            }
            /* room for the chunk's E1 records (earlier buffers stay until
             * the run ends: their chunks' kernels may still read them) */
            if (pe == cudaSuccess && base1 + m > e1_cap) {
                const long long ncap = std::max(2 * e1_cap, base1 + m);
                E1Rec *n_all = nullptr;
                uint32_t *n_nodes = nullptr;
                pe = cudaMalloc((void **) &n_all, (size_t) ncap * sizeof(E1Rec));
                if (pe == cudaSuccess)
                    pe = cudaMalloc((void **) &n_nodes, (size_t) ncap * sizeof(uint32_t));
                if (pe == cudaSuccess && base1 > 0)
                    pe = cudaMemcpyAsync(n_all, e1_all, base1 * sizeof(E1Rec),
                                         cudaMemcpyDeviceToDevice, ps);
                if (pe == cudaSuccess && base1 > 0)
                    pe = cudaMemcpyAsync(n_nodes, e1_nodes, base1 * sizeof(uint32_t),
                                         cudaMemcpyDeviceToDevice, ps);
                old_e1.push_back(e1_all);
                old_e1.push_back(e1_nodes);
                e1_all = n_all;
                e1_nodes = n_nodes;
                e1_cap = ncap;
            }
            long long bounds[DevScheduler::MAX_CHUNK_DAYS + 1];
            for (int j = 0; j < nd; j++)
                bounds[j] = p->e2_lo[d0 + j] - l0;
            bounds[nd] = m;
            const int *cols_i[7] = {a->time, a->event, a->node, a->dest, a->n, a->select, a->shift};
            int *dst_i[7] = {sch.time, sch.event, sch.node, sch.dest, sch.n, sch.select, sch.shift};
            for (int k = 0; k < 7 && pe == cudaSuccess && m > 0; k++)
                pe = cudaMemcpyAsync(dst_i[k], cols_i[k] + l0, (size_t) m * sizeof(int),
                                     cudaMemcpyHostToDevice, ps);
            if (pe == cudaSuccess && m > 0)
                pe = cudaMemcpyAsync(sch.proportion, a->proportion + l0, (size_t) m * sizeof(double),
                                     cudaMemcpyHostToDevice, ps);
            /* the host's levels of the chunk, once its days are planned */
            const uint32_t *pos_level = nullptr;
            if (hl && pe == cudaSuccess && c >= dev_first) {
                for (int d = d0; d < d1 && !abort.load() && !lfail.load(); d++)
                    while (!lday[d].load(std::memory_order_acquire) && !abort.load() &&
                           !lfail.load())
                        std::this_thread::sleep_for(std::chrono::microseconds(20));
                if (lfail.load())
                    pe = cudaErrorMemoryAllocation;
                else if (abort.load())
                    break;
                if (pe == cudaSuccess && m > 0 && !ldeep[c].load()) {
                    pe = cudaMemcpyAsync(d_lslot, lslot + (size_t) (c % LRING) * cap,
                                         (size_t) m * sizeof(uint32_t), cudaMemcpyHostToDevice, ps);
                    pos_level = d_lslot;
                }
            }
            if (pe == cudaSuccess)
                pe = sch.plan_chunk(l0, m, d0, nd, bounds, l0 > 0 ? a->time[l0 - 1] : 0,
                                    l0 > 0 ? a->event[l0 - 1] : 0, l0 > 0, p->d_e2 + base2,
                                    e1_all + base1, ring[c % E1_RING], nullptr, pl.ch,
                                    e1_nodes + base1, pos_level);
            /* plan_chunk returns with its stream idle: the slot is free */
            if (hl && pe == cudaSuccess)
                lfree[c].store(1, std::memory_order_release);
            /* days too deep for the rounds: the host planner's waves */
            for (size_t k = 0; pe == cudaSuccess && k < pl.ch.deep.size(); k++) {
                const int j = pl.ch.deep[k];
                std::vector<E2Rec> recs((size_t) (p->e2_hi[d0 + j] - p->e2_lo[d0 + j]) + 1);
                host_day_waves(a->event, a->node, a->dest, a->n, a->proportion, a->select,
                               a->shift, p->e2_lo[d0 + j], p->e2_hi[d0 + j], Nn, p->nsel,
                               recs.data(), pl.ch.waves[j]);
                const long long cnt = pl.ch.off[j + 1] - pl.ch.off[j];
                if (cnt > 0)
                    pe = cudaMemcpyAsync(p->d_e2 + base2 + pl.ch.off[j], recs.data(),
                                         (size_t) cnt * sizeof(E2Rec), cudaMemcpyHostToDevice, ps);
                if (pe == cudaSuccess)
                    pe = cudaStreamSynchronize(ps);
            }
            pl.base2 = base2;
            pl.e1 = e1_all + base1;
            pl.err = pe;
            base1 += pl.ch.n1;
            base2 += pl.ch.n2;
            e1_total = base1;
            e2_total = base2;
            ready[c].store(1, std::memory_order_release);
            if (pe != cudaSuccess || pl.ch.bad != ~0ULL)
                break;
        }
    });

    static const bool prof = getenv("SIMINF_SCHED_PROFILE") && getenv("SIMINF_SCHED_PROFILE")[0] == '1';
    double waited = 0;
    for (int c = 0; c < nchunks && e == cudaSuccess; c++) {
        auto w0 = std::chrono::steady_clock::now();
        while (!ready[c].load(std::memory_order_acquire))
            std::this_thread::yield();
        waited += ms_since(w0);
        const Planned &pl = plans[c];
        if (pl.err != cudaSuccess) {
            e = pl.err;
            break;
        }
        if (pl.ch.bad != ~0ULL) {
            bad = pl.ch.bad;            /* out of order: the run stops here */
            break;
        }
        /* E and N up to the largest select and shift seen so far */
        if (pl.ch.max_select > p->max_select && a->jcE) {
            int *djcE, *dirE;
            double *dprE;
            const int nnz = a->jcE[pl.ch.max_select];
            int rc = upload(&djcE, a->jcE, (size_t) pl.ch.max_select + 1, p->owned, st);
            if (!rc) rc = upload(&dirE, a->irE, (size_t) nnz, p->owned, st);
            if (!rc) rc = upload(&dprE, (const double *) a->prE, (size_t) nnz, p->owned, st);
            if (rc) {
                e = cudaErrorMemoryAllocation;
                break;
            }
            s.jcE = p->s.jcE = djcE;
            s.irE = p->s.irE = dirE;
            s.prE = p->s.prE = dprE;
            p->max_select = pl.ch.max_select;
        }
        if (pl.ch.max_shift > p->max_shift && a->N) {
            int *dN;
            if (upload(&dN, a->N, (size_t) pl.ch.max_shift * a->Nc, p->owned, st)) {
                e = cudaErrorMemoryAllocation;
                break;
            }
            s.Nshift = p->s.Nshift = dN;
            p->max_shift = pl.ch.max_shift;
        }
        s.e1 = pl.e1;
        s.e1_ptr = ring[c % E1_RING];
        const int d0 = c * CHUNK_DAYS, d1 = std::min(ndays, d0 + (int) CHUNK_DAYS);
        for (int d = d0; d < d1 && e == cudaSuccess; d++) {
            const int j = d - d0;
            const DayInfo &di = p->days[d];
            p->e2_day_off[d] = pl.base2 + pl.ch.off[j];
            p->e2_day_off[d + 1] = pl.base2 + pl.ch.off[j + 1];
            p->day_waves[d] = pl.ch.waves[j];
            if (s.two_pass && !s.aem)
                e = L->quick(s, d, di.tt, di.next, st);
            if (e == cudaSuccess)
                e = s.aem ? L->aem_day(s, d, di.tt, di.next, st)
                          : L->ssa_e1(s, d, di.tt, di.next, st);
            if (e == cudaSuccess) {
                const std::vector<long long> &cnt = p->day_waves[d];
                std::vector<long long> off(cnt.size());
                long long o = p->e2_day_off[d];
                for (size_t w = 0; w < cnt.size(); w++) {
                    off[w] = o;
                    o += cnt[w];
                }
                e = launch_day_waves(p, s, off.data(), cnt.data(), (int) cnt.size(), d, di.tt,
                                     st, nullptr);
            }
            if (e == cudaSuccess)
                e = s.aem ? L->aem_pts(s, d, di.tt, di.c0, di.c1, s.vA, s.vB, st)
                          : L->pts_store(s, d, di.tt, di.c0, di.c1, s.vA, s.vB, st);
            std::swap(s.vA, s.vB);
        }
        if (e == cudaSuccess)
            e = cudaEventCreateWithFlags(&done[c], cudaEventDisableTiming);
        if (e == cudaSuccess)
            e = cudaEventRecord(done[c], st);
        queued[c].store(1, std::memory_order_release);
        /* the columns this chunk finished go back while later days run */
        const int c_hi = p->days[d1 - 1].c1;
        if (ds && e == cudaSuccess && c_hi > p->cols_sent) {
            e = cudaStreamWaitEvent(ds, done[c], 0);
            if (e == cudaSuccess)
                e = download_columns(p, p->out_args, p->cols_sent, c_hi, ds);
            if (e == cudaSuccess)
                p->cols_sent = c_hi;
        }
    }
    abort.store(1);
    planner.join();
    for (auto &t : lworkers)
        t.join();
    if (prof)
        fprintf(stderr, "streamed run (%s levels): %.2f ms waiting for plans\n",
                hl ? "host" : "device", waited);

    /* events past the last day: the order check and the maxima */
    for (long long l0 = tail_lo; e == cudaSuccess && bad == ~0ULL && l0 < len; ) {
        const long long m = std::min(len - l0, cap);
        const int *cols_i[4] = {a->time, a->event, a->select, a->shift};
        int *dst_i[4] = {sch.time, sch.event, sch.select, sch.shift};
        for (int k = 0; k < 4 && e == cudaSuccess; k++)
            e = cudaMemcpyAsync(dst_i[k], cols_i[k] + l0, (size_t) m * sizeof(int),
                                cudaMemcpyHostToDevice, ps);
        if (e == cudaSuccess)
            e = sch.check_tail(l0, m, l0 > 0 ? a->time[l0 - 1] : 0, l0 > 0 ? a->event[l0 - 1] : 0,
                               l0 > 0);
        l0 += m;
    }
    std::vector<SchedPlanned> planned;
    int msel = 0, mshift = 0;
    if (e == cudaSuccess) {
        unsigned long long b2 = ~0ULL;
        e = sch.status(b2, msel, mshift, planned);
        bad = std::min(bad, b2);
    }
    p->dev_bad = (long long) (bad == ~0ULL ? -1 : (long long) bad);
    if (e == cudaSuccess && bad == ~0ULL) {
        for (const SchedPlanned &x : planned)
            p->planned.push_back({x.day, x.code, x.index, x.node, x.phase});
        p->e1_count = (uint64_t) e1_total;
        p->e2_count = (uint64_t) e2_total;
        /* the E1 records of all chunks as one per-node CSR for later runs
         * (after every chunk's kernels: they read the chunk buffers) */
        E1Rec *de1 = nullptr;
        int *de1p = nullptr;
        e = cudaStreamSynchronize(st);
        if (e == cudaSuccess && !dalloc(&de1, (size_t) std::max(1LL, e1_total), p->owned) &&
            !dalloc(&de1p, (size_t) Nn + 1, p->owned))
            e = sch.merge_e1(e1_all, e1_nodes, e1_total, de1, de1p);
        else if (e == cudaSuccess)
            e = cudaErrorMemoryAllocation;
        if (e == cudaSuccess) {
            p->s.e1 = de1;
            p->s.e1_ptr = de1p;
        }
    }
    if (ds) {
        const cudaError_t e2 = cudaStreamSynchronize(ds);
        if (e == cudaSuccess)
            e = e2;
        cudaStreamDestroy(ds);
    }
    cudaStreamSynchronize(ps);
    /* the caller's stream continues after the day kernels */
    if (cudaEventRecord(hs_end, hs) == cudaSuccess)
        cudaStreamWaitEvent(caller, hs_end, 0);
    cudaStreamSynchronize(hs);
    for (cudaEvent_t ev : done)
        if (ev)
            cudaEventDestroy(ev);
    cudaEventDestroy(hs_start);
    cudaEventDestroy(hs_end);
    cudaStreamDestroy(hs);
    for (int r = 0; r < E1_RING; r++)
        cudaFree(ring[r]);
    cudaFree(e1_all);
    cudaFree(e1_nodes);
    for (void *q : old_e1)
        cudaFree(q);
    cudaFree(d_lslot);
    pinned_release(lslot, lslot_bytes);
    cudaStreamDestroy(ps);
    return e;
}

/* The reset at the start of every run: error counters, transition counter,
 * work queues, the state from u0/v0. */
static cudaError_t reset_run(siminf_gpu_plan *p, const DevState &s, cudaStream_t st,
                             bool from_device)
{
    static const int init_flags[3] = {0, INT_MAX, INT_MAX};
    cudaError_t e = from_device
                        ? cudaMemcpyAsync(s.err_count, p->d_init_flags, sizeof(init_flags),
                                          cudaMemcpyDeviceToDevice, st)
                        : cudaMemcpyAsync(s.err_count, init_flags, sizeof(init_flags),
                                          cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(s.fired, 0, sizeof(unsigned long long), st);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(s.heavy_count, 0, 2 * HEAVY_CLASSES * sizeof(int), st);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(s.queue_next, 0, 6 * sizeof(unsigned long long), st);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(s.heavy_mark, 0, (size_t) s.Ntot * sizeof(int), st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(s.u, p->d_u0, (size_t) s.Ntot * s.Nc * sizeof(int),
                            cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess && s.Nd > 0) {
        e = cudaMemcpyAsync(s.vA, p->d_v0, (size_t) s.Ntot * s.Nd * sizeof(double),
                            cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(s.vB, p->d_v0, (size_t) s.Ntot * s.Nd * sizeof(double),
                                cudaMemcpyDeviceToDevice, st);
    }
    return e;
}

/* A graph of one whole run (reset + launch_all), captured on a side stream;
 * false when it cannot be built (the run then goes launch by launch). */
static bool build_run_graph(siminf_gpu_plan *p, const DevState &s)
{
    if (p->run_graph) {
        cudaGraphExecDestroy(p->run_graph);
        p->run_graph = nullptr;
    }
    if (!p->d_init_flags) {
        static const int init_flags[3] = {0, INT_MAX, INT_MAX};
        if (upload(&p->d_init_flags, init_flags, 3, p->owned, p->stream) ||
            cudaStreamSynchronize(p->stream) != cudaSuccess)
            return false;
    }
    cudaStream_t cs = nullptr;
    if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess)
        return false;
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cudaError_t c = reset_run(p, s, cs, true);
        if (c == cudaSuccess)
            c = launch_all(p, s, cs, nullptr);
        e = cudaStreamEndCapture(cs, &graph);
        if (e == cudaSuccess)
            e = c;
    }
    if (e == cudaSuccess)
        e = cudaGraphInstantiate(&p->run_graph, graph, 0);
    if (graph)
        cudaGraphDestroy(graph);
    cudaStreamDestroy(cs);
    if (e != cudaSuccess) {
        cudaGetLastError();             /* clear the sticky-free capture error */
        p->run_graph = nullptr;
        return false;
    }
    return true;
}

extern "C" {

static int plan_run_impl(siminf_gpu_plan *p, cudaStream_t st, KernelProfile *kp)
{
    if (!p)
        return SIMINF_GPU_ERR_INVALID_MODEL;
    memset(&g_status, 0, sizeof(g_status));
    DevState s = p->s;
    cudaError_t e;
    /* the run's two timing events, destroyed on every return path */
    struct EventPair {
        cudaEvent_t a = nullptr, b = nullptr;
        ~EventPair()
        {
            if (a)
                cudaEventDestroy(a);
            if (b)
                cudaEventDestroy(b);
        }
    } ev;
    e = cudaEventCreate(&ev.a);
    if (e == cudaSuccess)
        e = cudaEventCreate(&ev.b);
    if (e == cudaSuccess)
        e = cudaEventRecord(ev.a, st);
    if (e != cudaSuccess)
        return cuda_fail(e, "plan_run events");

    /* a run that repeats the previous one unchanged replays its graph */
    const char *g_env = getenv("SIMINF_RUN_GRAPH");
    const bool graphs = !(g_env && g_env[0] == '0');
    const bool replay = graphs && !kp && !p->e2_pending && p->runs_unchanged >= 1 &&
                        (p->run_graph || build_run_graph(p, s));
    p->runs_unchanged++;
    if (replay) {
        e = cudaGraphLaunch(p->run_graph, st);
    } else {
        e = reset_run(p, s, st, false);
        if (e != cudaSuccess)
            return cuda_fail(e, "plan_run reset");
    }

    if (replay) {
        /* the graph holds the whole run */
    } else if (p->e2_pending) {
        e = p->dev_plan ? launch_streamed_dev(p, s, st) : launch_streamed(p, s, st);
        p->scan_free = false;
        p->e2_pending = false;
        p->h_e2.reset();
        plan_wave_index(p);
        p->stats.e2_waves = (int) p->wave_ptr.size() - 1;
        p->stats.e1_events = p->e1_count * (uint64_t) s.Nrep;
        p->stats.e2_events = p->e2_count * (uint64_t) s.Nrep;
        if (e == cudaSuccess && p->dev_bad >= 0) {
            /* the device planner found the table out of order */
            const long long bad = p->dev_bad;
            char msg[200];
            snprintf(msg, sizeof(msg), "event %lld (time %d) breaks the (time, E1 before E2) order",
                     bad + 1, p->args.time[bad]);
            cudaStreamSynchronize(st);
            set_status(SIMINF_GPU_ERR_EVENTS_UNSORTED, -1, -1, (int) bad, p->args.time[bad], 0, msg);
            return SIMINF_GPU_ERR_EVENTS_UNSORTED;
        }
    } else {
        e = launch_all(p, s, st, kp);
    }
    if (e != cudaSuccess)
        return cuda_fail(e, "kernel launch");
    e = cudaEventRecord(ev.b, st);
    if (e == cudaSuccess)
        e = cudaEventSynchronize(ev.b);
    if (e != cudaSuccess)
        return cuda_fail(e, "solver kernels");
    float ms = 0;
    e = cudaEventElapsedTime(&ms, ev.a, ev.b);
    if (e != cudaSuccess)
        return cuda_fail(e, "solver time");

    int counts[3];
    unsigned long long fired = 0;
    e = cudaMemcpyAsync(counts, s.err_count, sizeof(counts), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&fired, s.fired, sizeof(fired), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
        return cuda_fail(e, "read counters");
    p->stats.transitions = fired;
    p->stats.node_days = (uint64_t) p->ndays * (uint64_t) s.Ntot;
    p->stats.ms_solve = ms;
    p->ran = true;

    std::vector<ErrRec> cands;
    if (counts[0] > 0) {
        cands.resize(std::min(counts[0], (int) MAX_ERR));
        e = cudaMemcpyAsync(cands.data(), s.err, cands.size() * sizeof(ErrRec),
                            cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(st);
        if (e != cudaSuccess)
            return cuda_fail(e, "read errors");
    }
    return resolve_errors(p, cands);
}

int siminf_gpu_plan_run(siminf_gpu_plan *p, void *cuda_stream)
{
    return plan_run_impl(p, (cudaStream_t) cuda_stream, nullptr);
}

/* The autotuner's choices, kept per device model and size class. */
struct TuneKey {
    const Launchers *L;
    int nodes_class, days_class, transfers, aem, probe_days;
    bool operator<(const TuneKey &o) const
    {
        return std::tie(L, nodes_class, days_class, transfers, aem, probe_days) <
               std::tie(o.L, o.nodes_class, o.days_class, o.transfers, o.aem, o.probe_days);
    }
};
static std::mutex g_tune_mu;
static std::map<TuneKey, siminf_gpu_tune_result> g_tune_cache;

static int log2_class(long long n)
{
    int c = 0;
    while (n > 1) {
        n >>= 1;
        c++;
    }
    return c;
}

int siminf_gpu_plan_tune(siminf_gpu_plan *p, void *cuda_stream, int probe_days,
                         siminf_gpu_tune_result *out)
{
    if (!p || p->e2_pending)
        return SIMINF_GPU_ERR_INVALID_MODEL;
    const bool force = probe_days < 0;
    const int want_days = probe_days < 0 ? -probe_days : probe_days;
    const int pdays = std::min(want_days > 0 ? want_days : 16, p->ndays);
    const TuneKey key{p->L, log2_class(p->s.Ntot), log2_class(p->ndays), p->e2_count > 0,
                      p->s.aem, pdays};
    auto apply = [&](const siminf_gpu_tune_result &r, int k) {
        p->s.heavy_rate = r.heavy_rate[k];
        p->s.two_pass = r.two_pass[k];
        p->s.ssa_variant = r.ssa_variant[k];
        p->s.wave_block = r.wave_block[k];
        p->s.heavy_lanes = r.heavy_lanes[k];
        plan_changed(p);
    };
    if (!force) {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end() && it->second.chosen >= 0) {
            siminf_gpu_tune_result r = it->second;
            r.cached = 1;
            apply(r, r.chosen);
            if (out)
                *out = r;
            return 0;
        }
    }
    static const double cand[4] = {0.0, 2.0, 8.0, 32.0};
    const cudaStream_t st = (cudaStream_t) cuda_stream;
    const double saved = p->s.heavy_rate;
    const int saved_tp = p->s.two_pass, saved_v = p->s.ssa_variant, saved_w = p->s.wave_block,
              saved_hl = p->s.heavy_lanes;
    p->max_days = pdays;
    plan_changed(p);
    siminf_gpu_tune_result r{};
    int best = -1, rc = plan_run_impl(p, st, nullptr);     /* warm-up */
    auto probe = [&](double hr, int tp, int var, int wb, int hl) {
        const int k = r.n_candidates++;
        r.heavy_rate[k] = hr;
        r.two_pass[k] = p->s.aem ? 0 : tp;      /* two-pass days are the direct method's */
        r.ssa_variant[k] = var;
        r.wave_block[k] = wb;
        r.heavy_lanes[k] = hl;
        apply(r, k);
        rc = plan_run_impl(p, st, nullptr);
        r.ms[k] = p->stats.ms_solve;
        if (!rc && (best < 0 || r.ms[k] < r.ms[best]))
            best = k;
    };
    /* stage 1: the work queue's layout */
    for (int k = 0; k < 8 && !rc; k++)
        probe(cand[k % 4], k / 4, 0, 256, 0);
    /* stage 2: the SSA kernel's other register budget, then, for one
     * model run once, fewer lanes a warp for the heaviest nodes (a warp
     * holding the day's longest chains shares its issue slots and FP64 pipe
     * with fewer lanes; with replicates or a batch of models the heavy
     * class is large, the run is bound by throughput, and idle lanes only
     * cost: 16 replicates of the headline took 3.13 s a year with 8 lanes
     * against 2.76 s with 32) */
    if (!rc && best >= 0 && !p->s.aem)
        probe(r.heavy_rate[best], r.two_pass[best], 1, 256, 0);
    if (!rc && best >= 0 && !p->s.aem && r.heavy_rate[best] > 0.0 && p->L->time_invariant &&
        p->s.Nrep == 1 && !p->s.job_of)
        probe(r.heavy_rate[best], r.two_pass[best], r.ssa_variant[best], 256, 8);
    /* stage 3: the wavefront block */
    if (!rc && best >= 0 && p->e2_count > 0) {
        const siminf_gpu_tune_result b = r;
        const int kb = best;
        for (int wb : {128, 512})
            if (!rc)
                probe(b.heavy_rate[kb], b.two_pass[kb], b.ssa_variant[kb], wb, b.heavy_lanes[kb]);
    }
    /* final: the three fastest again, as repeated runs execute them (a
     * run after an unchanged one replays the run's graph, which takes the
     * launch overhead off the layouts with more launches): the third run
     * of each is timed and replaces its probe time */
    if (!rc && r.n_candidates > 1) {
        int order[SIMINF_GPU_TUNE_CANDIDATES];
        for (int k = 0; k < r.n_candidates; k++)
            order[k] = k;
        std::sort(order, order + r.n_candidates,
                  [&](int x, int y) { return r.ms[x] < r.ms[y]; });
        best = -1;
        for (int i = 0; i < std::min(3, r.n_candidates) && !rc; i++) {
            const int k = order[i];
            apply(r, k);
            for (int rep = 0; rep < 3 && !rc; rep++)
                rc = plan_run_impl(p, st, nullptr);
            r.ms[k] = p->stats.ms_solve;
            if (!rc && (best < 0 || r.ms[k] < r.ms[best]))
                best = k;
        }
    }
    p->max_days = 0;
    if (best >= 0) {
        apply(r, best);
    } else {
        p->s.heavy_rate = saved;
        p->s.two_pass = saved_tp;
        p->s.ssa_variant = saved_v;
        p->s.wave_block = saved_w;
        p->s.heavy_lanes = saved_hl;
        plan_changed(p);
    }
    r.chosen = best;
    r.probe_days = pdays;
    if (!rc && best >= 0) {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_cache[key] = r;
    }
    if (out)
        *out = r;
    return rc;
}

int siminf_gpu_plan_day_max(siminf_gpu_plan *p, void *cuda_stream, unsigned *day_max)
{
    if (!p || !day_max || p->e2_pending)
        return SIMINF_GPU_ERR_INVALID_MODEL;
    const cudaStream_t st = (cudaStream_t) cuda_stream;
    unsigned *d = nullptr;
    cudaError_t e = cudaMalloc((void **) &d, (size_t) p->ndays * sizeof(unsigned));
    if (e == cudaSuccess)
        e = cudaMemsetAsync(d, 0, (size_t) p->ndays * sizeof(unsigned), st);
    if (e != cudaSuccess) {
        if (d)
            cudaFree(d);
        return cuda_fail(e, "day_max buffer");
    }
    p->s.day_max = d;
    plan_changed(p);                    /* launch by launch, not from a graph */
    int rc = plan_run_impl(p, st, nullptr);
    p->s.day_max = nullptr;
    plan_changed(p);
    if (!rc) {
        e = cudaMemcpy(day_max, d, (size_t) p->ndays * sizeof(unsigned), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess)
            rc = cuda_fail(e, "day_max copy");
    }
    cudaFree(d);
    return rc;
}

int siminf_gpu_plan_profile(siminf_gpu_plan *p, void *cuda_stream, double ms[8],
                            long long launches[8])
{
    KernelProfile kp{};
    cudaEventCreate(&kp.a);
    cudaEventCreate(&kp.b);
    const int rc = plan_run_impl(p, (cudaStream_t) cuda_stream, &kp);
    cudaEventDestroy(kp.a);
    cudaEventDestroy(kp.b);
    for (int i = 0; i < 8; i++) {
        if (ms)
            ms[i] = kp.ms[i];
        if (launches)
            launches[i] = kp.n[i];
    }
    return rc;
}

int siminf_gpu_plan_download(siminf_gpu_plan *p, siminf_gpu_solver_args *a)
{
    if (!p || !a)
        return SIMINF_GPU_ERR_INVALID_MODEL;
    auto t0 = std::chrono::steady_clock::now();
    cudaError_t e = cudaSuccess;
    const cudaStream_t st = p->stream;
    const auto d2h = cudaMemcpyDeviceToHost;
    if (a->U && p->s.U)
        e = cudaMemcpyAsync(a->U, p->s.U, p->U_len * sizeof(int), d2h, st);
    else if (a->prU && p->s.prU)
        e = cudaMemcpyAsync(a->prU, p->s.prU, p->prU_len * sizeof(double), d2h, st);
    if (e == cudaSuccess && a->V && p->s.V)
        e = cudaMemcpyAsync(a->V, p->s.V, p->V_len * sizeof(double), d2h, st);
    else if (e == cudaSuccess && a->prV && p->s.prV)
        e = cudaMemcpyAsync(a->prV, p->s.prV, p->prV_len * sizeof(double), d2h, st);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
        return cuda_fail(e, "download");
    p->stats.ms_download = ms_since(t0);
    return 0;
}

int siminf_gpu_plan_stats(const siminf_gpu_plan *p, siminf_gpu_stats *out)
{
    if (!p || !out)
        return SIMINF_GPU_ERR_INVALID_MODEL;
    *out = p->stats;
    return 0;
}

int siminf_gpu_schedule(const siminf_gpu_solver_args *a, int *days, int *waves,
                        long long *e1_events, long long *e2_events, int *wave)
{
    memset(&g_status, 0, sizeof(g_status));
    if (!a || !a->tspan || a->tlen < 1 || a->Nn < 1)
        return SIMINF_GPU_ERR_INVALID_MODEL;
    if (a->len > 0 && (!a->event || !a->time || !a->node || !a->dest || !a->n ||
                       !a->proportion || !a->select || !a->shift))
        return SIMINF_GPU_ERR_INVALID_MODEL;
    siminf_gpu_plan p;
    int rc = make_days(&p, a);
    if (rc)
        return rc;
    std::vector<E1Rec> e1;
    std::vector<int> e1_ptr;
    std::unique_ptr<E2Rec[]> e2;
    rc = plan_events(&p, a, a->len > 0 ? INT_MAX : 0, e1, e1_ptr, e2);
    if (rc)
        return rc;
    if (days)
        *days = p.ndays;
    if (waves)
        *waves = (int) p.wave_ptr.size() - 1;
    if (e1_events)
        *e1_events = (long long) p.e1_count;
    if (e2_events)
        *e2_events = (long long) p.e2_count;
    if (wave) {
        for (int i = 0; i < a->len; i++)
            wave[i] = -1;
        for (int d = 0; d < p.ndays; d++)
            for (int w = p.day_wave[d]; w < p.day_wave[d + 1]; w++)
                for (long long k = p.wave_ptr[w]; k < p.wave_ptr[w + 1]; k++)
                    wave[e2[k].index] = w - p.day_wave[d];
    }
    return 0;
}

/* Re-point a plan without events at another tspan (at most 2 points here):
 * new day schedule, uploaded; U/V columns per replicate = tlen. */
static int plan_set_tspan(siminf_gpu_plan *p, const double *tspan, int tlen)
{
    siminf_gpu_solver_args a{};
    a.tspan = tspan;
    a.tlen = tlen;
    int rc = make_days(p, &a);
    if (rc)
        return rc;
    p->s.tlen = tlen;
    p->tt0 = tspan[0];
    plan_changed(p);
    if (p->days_cap < p->ndays) {
        DayInfo *d = nullptr;
        if ((rc = dalloc(&d, (size_t) p->ndays, p->owned)))
            return rc;
        p->d_days = d;
        p->days_cap = p->ndays;
    }
    cudaError_t e = cudaMemcpyAsync(p->d_days, p->days.data(), p->days.size() * sizeof(DayInfo),
                                    cudaMemcpyHostToDevice, p->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(p->stream);
    return e == cudaSuccess ? 0 : cuda_fail(e, "days upload");
}

/* A particle filter's plan, buffers and interval graph, resident across
 * filter passes over the same model, observations and particle count.
 * siminf_gpu_pfilter is one pass of a session made for it; a PMCMC chain
 * keeps one session for all its iterations. */
struct PfSession {
    siminf_gpu_plan *p = nullptr;
    int Np = 0, Nn = 0, Nc = 0, Nd = 0, n_obs = 0, obs_c = 0, per_particle = 0, Ngd = 0;
    size_t nu = 0, nv = 0;
    int tablen = 1;
    double logp = 0, logq = 0, log_np = 0;
    double *d_lfact = nullptr, *d_w = nullptr, *d_loglik = nullptr, *d_ess = nullptr;
    int *d_anc = nullptr, *d_anc_out = nullptr, *d_obs = nullptr;
    int *d_u0_start = nullptr;          /* the particles' initial state (p->d_u0 takes the */
    double *d_v0_start = nullptr;       /* gathered ancestors interval by interval) */
    std::vector<std::array<double, 2>> tsps;
    std::vector<int> tlens, ndays_i;
    int g0 = 0;                         /* intervals g0 .. replay one graph */
    /* the replayed intervals: day schedules, seeds, interval counter, graph */
    int nd = 0;
    DayInfo *d_alldays = nullptr;
    uint64_t *d_seeds = nullptr;
    int *d_interval = nullptr;
    cudaStream_t gs = nullptr;
    cudaGraphExec_t exec = nullptr;
};

static void pf_session_free(PfSession *ss)
{
    if (!ss)
        return;
    if (ss->exec)
        cudaGraphExecDestroy(ss->exec);
    if (ss->gs)
        cudaStreamDestroy(ss->gs);
    siminf_gpu_plan_free(ss->p);
    delete ss;
}

/* Seed of particle-filter interval i. */
static inline uint64_t pf_interval_seed(uint64_t seed, int i)
{
    return seed + ((uint64_t) i + 1) * 0x9E3779B97F4A7C15ULL;
}

static int pf_session_create(const siminf_gpu_solver_args *a1, const siminf_gpu_model *model,
                             const siminf_gpu_pfilter_args *pf, PfSession **out)
{
    memset(&g_status, 0, sizeof(g_status));
    *out = nullptr;
    if (!a1 || !model || !pf || pf->n_particles < 1 || pf->n_obs < 1 || !pf->obs ||
        !pf->obs_time || a1->len > 0 || a1->solver != 0 || pf->obs_compartment < 0 ||
        pf->obs_compartment >= a1->Nc || !(pf->detect_p > 0.0 && pf->detect_p < 1.0)) {
        set_status(SIMINF_GPU_ERR_INVALID_MODEL, -1, -1, -1, 0, 0,
                   "invalid particle filter arguments (events and the aem solver are not supported)");
        return SIMINF_GPU_ERR_INVALID_MODEL;
    }
    for (int i = 0; i < pf->n_obs; i++) {
        if ((i == 0 && pf->obs_time[0] < a1->tspan[0]) ||
            (i > 0 && pf->obs_time[i] <= pf->obs_time[i - 1])) {
            set_status(SIMINF_GPU_ERR_INVALID_MODEL, -1, -1, -1, 0, 0,
                       "observation times must increase from tspan[0]");
            return SIMINF_GPU_ERR_INVALID_MODEL;
        }
    }
    PfSession *ss = new PfSession();
    const int Np = pf->n_particles, Nn = a1->Nn, Nc = a1->Nc, Nd = a1->Nd;
    ss->Np = Np;
    ss->Nn = Nn;
    ss->Nc = Nc;
    ss->Nd = Nd;
    ss->n_obs = pf->n_obs;
    ss->obs_c = pf->obs_compartment;
    ss->per_particle = pf->gdata_per_particle;
    ss->Ngd = model->L->Ngd;
    const size_t nu = (size_t) Nn * Nc, nv = (size_t) Nn * Nd;
    ss->nu = nu;
    ss->nv = nv;
    /* particles = replicates of one plan */
    std::vector<int> u0((size_t) Np * nu);
    std::vector<double> v0((size_t) Np * nv + 1);
    for (int q = 0; q < Np; q++) {
        memcpy(&u0[q * nu], a1->u0, nu * sizeof(int));
        if (nv)
            memcpy(&v0[q * nv], a1->v0, nv * sizeof(double));
    }
    for (int node = 0; node < Nn; node++) {
        long long tot = 0;
        for (int c = 0; c < Nc; c++)
            tot += a1->u0[(size_t) node * Nc + c];
        ss->tablen = (int) std::max<long long>(ss->tablen, tot + 1);
    }
    std::vector<double> lfact(ss->tablen);
    si_lfact_fill(lfact.data(), ss->tablen);
    double tsp0[2] = {a1->tspan[0], a1->tspan[0] + 1.0};
    int dummyU = 0;
    double dummyV = 0;
    siminf_gpu_solver_args a = *a1;
    a.u0 = u0.data();
    a.v0 = v0.data();
    a.Nrep = Np;
    a.tspan = tsp0;
    a.tlen = 2;
    a.U = &dummyU;
    a.V = Nd > 0 ? &dummyV : nullptr;
    a.len = 0;
    siminf_gpu_options opt{};
    opt.gdata_per_replicate = pf->gdata_per_particle;
    int rc = siminf_gpu_plan_create_ex(&a, model, &opt, &ss->p);
    if (rc) {
        delete ss;
        return rc;
    }
    siminf_gpu_plan *p = ss->p;
    p->days_cap = p->ndays;
    const cudaStream_t pst = p->stream;
    rc = upload(&ss->d_lfact, lfact.data(), lfact.size(), p->owned, pst);
    if (!rc) rc = dalloc(&ss->d_w, (size_t) Np, p->owned);
    if (!rc) rc = dalloc(&ss->d_anc, (size_t) Np, p->owned);
    if (!rc) rc = dalloc(&ss->d_anc_out, (size_t) Np * pf->n_obs, p->owned);
    if (!rc) rc = upload(&ss->d_obs, pf->obs, (size_t) pf->n_obs * Nn, p->owned, pst);
    if (!rc) rc = dalloc(&ss->d_loglik, 1, p->owned);
    if (!rc) rc = dalloc(&ss->d_ess, (size_t) pf->n_obs, p->owned);
    if (!rc) rc = upload(&ss->d_u0_start, u0.data(), u0.size(), p->owned, pst);
    if (!rc && nv) rc = upload(&ss->d_v0_start, v0.data(), (size_t) Np * nv, p->owned, pst);
    ss->logp = si_log(pf->detect_p);
    ss->logq = si_log(1.0 - pf->detect_p);
    ss->log_np = si_log((double) Np);
    /* interval i runs tspan tsps[i] (R/pfilter.R:177-193) */
    ss->tsps.resize(pf->n_obs);
    ss->tlens.resize(pf->n_obs);
    ss->ndays_i.resize(pf->n_obs);
    for (int i = 0; i < pf->n_obs; i++) {
        const double prev = (i == 0) ? a1->tspan[0] : (double) pf->obs_time[i - 1];
        if ((i == 0 && prev < pf->obs_time[0]) ||
            (i > 0 && pf->obs_time[i] - pf->obs_time[i - 1] > 1)) {
            ss->tsps[i] = {prev, (double) pf->obs_time[i]};
            ss->tlens[i] = 2;
        } else {
            ss->tsps[i] = {(double) pf->obs_time[i], 0.0};
            ss->tlens[i] = 1;
        }
        std::vector<DayInfo> dd;
        plan_days(ss->tsps[i].data(), ss->tlens[i], dd);
        ss->ndays_i[i] = (int) dd.size();
    }
    /* Intervals 1.. with one shape (tspan length and day count) replay one
     * CUDA graph; the rest run launch by launch. */
    ss->g0 = pf->n_obs;
    if (p->horizon && pf->n_obs > 2) {
        ss->g0 = 1;
        for (int i = 2; i < pf->n_obs; i++)
            if (ss->tlens[i] != ss->tlens[1] || ss->ndays_i[i] != ss->ndays_i[1])
                ss->g0 = pf->n_obs;
    }
    if (!rc && ss->g0 < ss->n_obs) {
        ss->nd = ss->ndays_i[ss->g0];
        std::vector<DayInfo> alldays((size_t) ss->n_obs * ss->nd);
        for (int i = ss->g0; i < ss->n_obs; i++) {
            std::vector<DayInfo> dd;
            plan_days(ss->tsps[i].data(), ss->tlens[i], dd);
            std::copy(dd.begin(), dd.end(), alldays.begin() + (size_t) i * ss->nd);
        }
        rc = upload(&ss->d_alldays, alldays.data(), alldays.size(), p->owned, pst);
        if (!rc) rc = dalloc(&ss->d_seeds, (size_t) ss->n_obs + 1, p->owned);
        if (!rc) rc = dalloc(&ss->d_interval, 1, p->owned);
    }
    if (rc) {
        pf_session_free(ss);
        return rc;
    }
    *out = ss;
    return 0;
}

/* Intervals g0 .. n_obs - 1 as replays of one CUDA graph, captured on the
 * session's first pass: the interval's seed, day schedule and observation
 * row are read from the device, and the finalize kernel moves the
 * interval counter on.  One replay: reset the state from the gathered
 * ancestors, k_init, k_horizon, weights, finalize (normalise, ESS,
 * resample), gather for the next interval.  Errors are read once, after
 * the last replay. */
static int pf_session_graph(PfSession *ss, uint64_t seed, int prev_tlen)
{
    siminf_gpu_plan *p = ss->p;
    const int g0 = ss->g0, n_obs = ss->n_obs, Np = ss->Np, tl = ss->tlens[g0];
    const cudaStream_t pst = p->stream;
    /* the intervals' seeds, then the pass's own (resampling) seed */
    std::vector<uint64_t> seeds(n_obs + 1);
    for (int i = 0; i < n_obs; i++)
        seeds[i] = pf_interval_seed(seed, i);
    seeds[n_obs] = seed;
    cudaError_t e = cudaMemcpyAsync(ss->d_seeds, seeds.data(), (n_obs + 1) * sizeof(uint64_t),
                                    cudaMemcpyHostToDevice, pst);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ss->d_interval, &g0, sizeof(int), cudaMemcpyHostToDevice, pst);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(pst);
    if (e != cudaSuccess)
        return cuda_fail(e, "pfilter graph set-up");
    int rc = plan_set_tspan(p, ss->tsps[g0].data(), tl);
    if (rc)
        return rc;
    DevState s = p->s;
    s.pf_interval = ss->d_interval;
    s.pf_seeds = ss->d_seeds;
    s.pf_days = ss->d_alldays;
    s.pf_days_stride = ss->nd;
    const Launchers *L = p->L;
    const int Nn = s.Nn, Nc = s.Nc;

    /* the state of interval g0 from its ancestors, then the error flags */
    e = pf_gather(s.U, s.V, prev_tlen, (long long) ss->nu, (long long) ss->nv, ss->d_anc, Np,
                  p->d_u0, p->d_v0, pst);
    const int init_flags[3] = {0, INT_MAX, INT_MAX};
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(s.err_count, init_flags, sizeof(init_flags), cudaMemcpyHostToDevice,
                            pst);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(pst);
    if (e != cudaSuccess)
        return cuda_fail(e, "pfilter graph set-up");

    if (!ss->exec) {
        cudaGraph_t graph = nullptr;
        e = cudaStreamCreateWithFlags(&ss->gs, cudaStreamNonBlocking);
        if (e == cudaSuccess)
            e = cudaStreamBeginCapture(ss->gs, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            cudaStream_t gs = ss->gs;
            cudaError_t c = cudaMemcpyAsync(s.u, p->d_u0, (size_t) s.Ntot * Nc * sizeof(int),
                                            cudaMemcpyDeviceToDevice, gs);
            if (c == cudaSuccess && s.Nd > 0)
                c = cudaMemcpyAsync(s.vA, p->d_v0, (size_t) s.Ntot * s.Nd * sizeof(double),
                                    cudaMemcpyDeviceToDevice, gs);
            if (c == cudaSuccess && s.Nd > 0)
                c = cudaMemcpyAsync(s.vB, p->d_v0, (size_t) s.Ntot * s.Nd * sizeof(double),
                                    cudaMemcpyDeviceToDevice, gs);
            if (c == cudaSuccess)
                c = L->init(s, 0.0, gs);
            if (c == cudaSuccess)
                c = L->horizon(s, ss->d_alldays, ss->nd, gs);
            if (c == cudaSuccess)
                c = pf_weights(s.U, tl, Nn, Nc, Np, ss->d_obs, ss->obs_c, ss->d_lfact,
                               ss->tablen, ss->logp, ss->logq, ss->d_w, gs, ss->d_interval);
            if (c == cudaSuccess)
                c = pf_finalize(ss->d_w, Np, ss->log_np, ss->d_loglik, ss->d_ess, 0, seed,
                                ((uint64_t) 1) << 62, ss->d_anc, ss->d_anc_out, gs,
                                ss->d_interval, ss->d_seeds + n_obs);
            if (c == cudaSuccess)
                c = pf_gather(s.U, s.V, tl, (long long) ss->nu, (long long) ss->nv, ss->d_anc,
                              Np, p->d_u0, p->d_v0, gs);
            e = cudaStreamEndCapture(gs, &graph);
            if (e == cudaSuccess)
                e = c;
        }
        if (e == cudaSuccess)
            e = cudaGraphInstantiate(&ss->exec, graph, 0);
        if (graph)
            cudaGraphDestroy(graph);
        if (e != cudaSuccess)
            return cuda_fail(e, "pfilter graph");
    }
    for (int i = g0; i < n_obs && e == cudaSuccess; i++)
        e = cudaGraphLaunch(ss->exec, ss->gs);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(ss->gs);
    if (e != cudaSuccess)
        return cuda_fail(e, "pfilter graph");

    /* errors of all replayed intervals */
    int counts[3];
    e = cudaMemcpy(counts, s.err_count, sizeof(counts), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess)
        return cuda_fail(e, "read counters");
    std::vector<ErrRec> cands;
    if (counts[0] > 0) {
        cands.resize(std::min(counts[0], (int) MAX_ERR));
        e = cudaMemcpy(cands.data(), s.err, cands.size() * sizeof(ErrRec), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess)
            return cuda_fail(e, "read errors");
    }
    return resolve_errors(p, cands);
}

/* One filter pass from the particles' initial state.  gdata, if not
 * NULL, replaces the plan's gdata first (Ngd values, or Np rows of them
 * for a session with one row per particle).  Outputs as in
 * siminf_gpu_pfilter_args (ess, ancestors may be NULL). */
static int pf_session_run(PfSession *ss, const double *gdata, uint64_t seed, double *loglik,
                          double *ess, int *ancestors)
{
    siminf_gpu_plan *p = ss->p;
    const cudaStream_t pst = p->stream;
    const int Np = ss->Np, Nn = ss->Nn, Nc = ss->Nc, n_obs = ss->n_obs;
    cudaError_t e = cudaMemsetAsync(ss->d_loglik, 0, sizeof(double), pst);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(p->d_u0, ss->d_u0_start, (size_t) Np * ss->nu * sizeof(int),
                            cudaMemcpyDeviceToDevice, pst);
    if (e == cudaSuccess && ss->nv)
        e = cudaMemcpyAsync(p->d_v0, ss->d_v0_start, (size_t) Np * ss->nv * sizeof(double),
                            cudaMemcpyDeviceToDevice, pst);
    if (e == cudaSuccess && gdata && ss->Ngd > 0)
        e = cudaMemcpyAsync((void *) p->s.gdata, gdata,
                            (size_t) ss->Ngd * (ss->per_particle ? Np : 1) * sizeof(double),
                            cudaMemcpyHostToDevice, pst);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(pst);
    if (e != cudaSuccess)
        return cuda_fail(e, "pfilter reset");
    plan_changed(p);
    int rc = 0, prev_tlen = 2;
    for (int i = 0; i < ss->g0 && !rc; i++) {
        const double *tsp = ss->tsps[i].data();
        const int tlen = ss->tlens[i];
        if (i > 0) {
            e = pf_gather(p->s.U, p->s.V, prev_tlen, (long long) ss->nu, (long long) ss->nv,
                          ss->d_anc, Np, p->d_u0, p->d_v0, pst);
            if (e != cudaSuccess) {
                rc = cuda_fail(e, "pf_gather");
                break;
            }
        }
        if ((rc = plan_set_tspan(p, tsp, tlen)))
            break;
        p->s.seed = pf_interval_seed(seed, i);
        if ((rc = plan_run_impl(p, pst, nullptr)))
            break;
        e = pf_weights(p->s.U, tlen, Nn, Nc, Np, ss->d_obs + (size_t) i * Nn, ss->obs_c,
                       ss->d_lfact, ss->tablen, ss->logp, ss->logq, ss->d_w, pst);
        if (e == cudaSuccess)
            e = pf_finalize(ss->d_w, Np, ss->log_np, ss->d_loglik, ss->d_ess, i, seed,
                            (((uint64_t) 1) << 62) + (uint64_t) i, ss->d_anc,
                            ss->d_anc_out + (size_t) i * Np, pst);
        if (e != cudaSuccess) {
            rc = cuda_fail(e, "pf kernels");
            break;
        }
        prev_tlen = tlen;
    }
    if (!rc && ss->g0 < n_obs)
        rc = pf_session_graph(ss, seed, prev_tlen);
    if (!rc) {
        e = cudaMemcpyAsync(loglik, ss->d_loglik, sizeof(double), cudaMemcpyDeviceToHost, pst);
        if (e == cudaSuccess && ess)
            e = cudaMemcpyAsync(ess, ss->d_ess, (size_t) n_obs * sizeof(double),
                                cudaMemcpyDeviceToHost, pst);
        if (e == cudaSuccess && ancestors)
            e = cudaMemcpyAsync(ancestors, ss->d_anc_out, (size_t) n_obs * Np * sizeof(int),
                                cudaMemcpyDeviceToHost, pst);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(pst);
        if (e != cudaSuccess)
            rc = cuda_fail(e, "pf results");
    }
    return rc;
}

int siminf_gpu_pfilter(const siminf_gpu_solver_args *a1, const siminf_gpu_model *model,
                       siminf_gpu_pfilter_args *pf)
{
    auto t0 = std::chrono::steady_clock::now();
    if (!pf || !pf->loglik || !pf->ess) {
        set_status(SIMINF_GPU_ERR_INVALID_MODEL, -1, -1, -1, 0, 0,
                   "invalid particle filter arguments");
        return SIMINF_GPU_ERR_INVALID_MODEL;
    }
    PfSession *ss = nullptr;
    int rc = pf_session_create(a1, model, pf, &ss);
    if (!rc)
        rc = pf_session_run(ss, nullptr, (uint64_t) pf->seed, pf->loglik, pf->ess,
                            pf->ancestors);
    pf_session_free(ss);
    pf->ms_total = ms_since(t0);
    return rc;
}

/* ------------------------------------------------------------------ */
/* Particle-marginal Metropolis-Hastings (R/pmcmc.R:470-600): a chain    */
/* resident across calls, whose particle filter session stays on the     */
/* device from iteration to iteration and from call to call.             */
/* ------------------------------------------------------------------ */
#define PMCMC_SID (5ULL << 60)

struct siminf_gpu_pmcmc {
    std::mutex mu;                      /* one call at a time on a chain */
    PfSession *ss = nullptr;
    int n_pars = 0;
    std::vector<int> idx;
    std::vector<double> lo, hi, chol, gdata, theta;
    uint64_t seed = 0;
    long long length = 0;               /* iterations so far */
    double logLik = 0, logPrior = 0, logPost = 0;
};

/* log of the uniform priors' density at th (R/pmcmc.R dpriors for
 * U(lo, hi)): -sum log(hi - lo) inside the box, -Inf outside. */
static double pmcmc_log_prior(const siminf_gpu_pmcmc *c, const std::vector<double> &th)
{
    double lp = 0.0;
    for (int k = 0; k < c->n_pars; k++) {
        if (!(th[k] >= c->lo[k] && th[k] <= c->hi[k]))
            return -INFINITY;
        lp -= std::log(c->hi[k] - c->lo[k]);
    }
    return lp;
}

/* One filter pass at th: the chain's gdata with th at its parameters. */
static int pmcmc_loglik(siminf_gpu_pmcmc *c, const std::vector<double> &th, long long it,
                        double *ll)
{
    for (int k = 0; k < c->n_pars; k++)
        c->gdata[c->idx[k]] = th[k];
    const uint64_t seed = c->seed ^ ((uint64_t) it * 0xD1B54A32D192ED03ULL);
    return pf_session_run(c->ss, c->gdata.data(), seed, ll, nullptr, nullptr);
}

int siminf_gpu_pmcmc_create(const siminf_gpu_solver_args *args, const siminf_gpu_model *model,
                            const siminf_gpu_pfilter_args *pf, const siminf_gpu_pmcmc_args *pm,
                            siminf_gpu_pmcmc **out)
{
    memset(&g_status, 0, sizeof(g_status));
    if (!out || !pm || !args || !model || pm->n_pars < 1 || !pm->gdata_index || !pm->theta ||
        !pm->prior_lo || !pm->prior_hi || !pm->chol || !args->gdata ||
        (pf && pf->gdata_per_particle)) {
        set_status(SIMINF_GPU_ERR_INVALID_MODEL, -1, -1, -1, 0, 0, "invalid pmcmc arguments");
        return SIMINF_GPU_ERR_INVALID_MODEL;
    }
    *out = nullptr;
    const int Ngd = model->L->Ngd;
    for (int k = 0; k < pm->n_pars; k++) {
        if (pm->gdata_index[k] < 0 || pm->gdata_index[k] >= Ngd ||
            !(pm->prior_lo[k] < pm->prior_hi[k])) {
            set_status(SIMINF_GPU_ERR_INVALID_MODEL, -1, -1, -1, 0, 0,
                       "pmcmc parameter outside gdata or with an empty prior");
            return SIMINF_GPU_ERR_INVALID_MODEL;
        }
    }
    siminf_gpu_pmcmc *c = new siminf_gpu_pmcmc();
    int rc = pf_session_create(args, model, pf, &c->ss);
    if (rc) {
        delete c;
        return rc;
    }
    c->n_pars = pm->n_pars;
    c->idx.assign(pm->gdata_index, pm->gdata_index + pm->n_pars);
    c->lo.assign(pm->prior_lo, pm->prior_lo + pm->n_pars);
    c->hi.assign(pm->prior_hi, pm->prior_hi + pm->n_pars);
    c->chol.assign(pm->chol, pm->chol + (size_t) pm->n_pars * pm->n_pars);
    c->gdata.assign(args->gdata, args->gdata + Ngd);
    c->theta.assign(pm->theta, pm->theta + pm->n_pars);
    c->seed = (uint64_t) pm->seed;
    *out = c;
    return 0;
}

int siminf_gpu_pmcmc_run(siminf_gpu_pmcmc *c, int n_iterations, double *rows)
{
    if (!c || n_iterations < 0)
        return SIMINF_GPU_ERR_INVALID_MODEL;
    std::lock_guard<std::mutex> lock(c->mu);
    memset(&g_status, 0, sizeof(g_status));
    const int np = c->n_pars, width = 4 + np;
    for (int r = 0; r < n_iterations; r++) {
        const long long it = ++c->length;         /* one-based, as the chain's rows */
        double accept = 0.0;
        int rc = 0;
        if (it == 1) {
            /* the first row: the initial theta (R/pmcmc.R:519-545) */
            rc = pmcmc_loglik(c, c->theta, it, &c->logLik);
            c->logPrior = pmcmc_log_prior(c, c->theta);
            c->logPost = c->logLik + c->logPrior;
        } else {
            /* random-walk proposal theta + z Q, Q the upper Cholesky
             * factor (R/pmcmc.R:423-437); z by Box-Muller (Box & Muller,
             * 1958) from the chain's stream, then one uniform to accept */
            si_rng rng;
            si_rng_init(&rng, c->seed, PMCMC_SID + (uint64_t) it, 0);
            std::vector<double> z(np), prop(np);
            for (int k = 0; k < np; k++) {
                const double u1 = si_uniform_pos(&rng), u2 = si_uniform_pos(&rng);
                z[k] = std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
            }
            for (int j = 0; j < np; j++) {
                double acc = c->theta[j];
                for (int k = 0; k <= j; k++)
                    acc += z[k] * c->chol[(size_t) k * np + j];
                prop[j] = acc;
            }
            const double u = si_uniform_pos(&rng);
            const double lp_prop = pmcmc_log_prior(c, prop);
            if (std::isfinite(lp_prop)) {
                double ll_prop = 0.0;
                rc = pmcmc_loglik(c, prop, it, &ll_prop);
                const double alpha = std::exp(ll_prop + lp_prop - c->logLik - c->logPrior);
                if (!rc && std::isfinite(alpha) && u < alpha) {
                    c->logLik = ll_prop;
                    c->logPrior = lp_prop;
                    c->logPost = c->logLik + c->logPrior;
                    c->theta = prop;
                    accept = 1.0;
                }
            }
        }
        if (rc) {
            c->length--;
            return rc;
        }
        if (rows) {
            double *row = rows + (size_t) r * width;
            row[0] = c->logPost;
            row[1] = c->logLik;
            row[2] = c->logPrior;
            row[3] = accept;
            for (int k = 0; k < np; k++)
                row[4 + k] = c->theta[k];
        }
    }
    return 0;
}

long long siminf_gpu_pmcmc_length(const siminf_gpu_pmcmc *c)
{
    return c ? c->length : 0;
}

void siminf_gpu_pmcmc_free(siminf_gpu_pmcmc *c)
{
    if (!c)
        return;
    pf_session_free(c->ss);
    delete c;
}

static int run_solver(siminf_gpu_solver_args *args, const siminf_gpu_model *model,
                      const siminf_gpu_options *opt)
{
    siminf_gpu_plan *p = nullptr;
    /* streamed: the external transfers' waves are planned and copied
     * while the GPU runs the earlier days */
    int rc = plan_create_impl(args, model, opt, &p, true);
    if (rc)
        return rc;
    /* pinned outputs come back chunk by chunk during the run */
    if (p->e2_pending && host_pinned(args->U ? (const void *) args->U : args->prU) &&
        (p->s.Nd == 0 || host_pinned(args->V ? (const void *) args->V : args->prV)))
        p->out_args = args;
    rc = plan_run_impl(p, p->stream, nullptr);
    if (!rc && p->out_args) {
        auto t0 = std::chrono::steady_clock::now();
        cudaError_t e = download_columns(p, args, p->cols_sent, p->s.tlen, p->stream);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(p->stream);
        if (e != cudaSuccess)
            rc = cuda_fail(e, "download");
        p->stats.ms_download = ms_since(t0);
    } else if (!rc) {
        rc = siminf_gpu_plan_download(p, args);
    }
    g_stats = p->stats;
    siminf_gpu_plan_free(p);
    return rc;
}

int siminf_gpu_run_solver_ssm(siminf_gpu_solver_args *args, const siminf_gpu_model *model)
{
    return run_solver(args, model, nullptr);
}

int siminf_gpu_run_solver_mssm(siminf_gpu_solver_args *args, const siminf_gpu_model *model)
{
    return run_solver(args, model, nullptr);
}

int siminf_gpu_run_solver_ex(siminf_gpu_solver_args *args, const siminf_gpu_model *model,
                             const siminf_gpu_options *options)
{
    return run_solver(args, model, options);
}

void siminf_gpu_release_cached(void)
{
    PinnedCache &c = pinned_cache();
    std::vector<std::pair<void *, size_t>> drop;
    {
        std::lock_guard<std::mutex> lk(c.mu);
        drop.swap(c.free_list);
    }
    for (auto &b : drop)
        cudaFreeHost(b.first);
}

}  /* extern "C" */
