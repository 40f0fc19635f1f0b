/*
 * siminf_noalloc.cu -- siminf_gpu_run_solver_ssm_noalloc: the ssm solver
 * for a model without scheduled events, run in a fixed device array that
 * this file declares, so that a call allocates no memory at all.
 *
 * Who needs it: callers that must not allocate at the moment they run a
 * trajectory.  A process whose device memory is held by another allocator
 * (a caching allocator that has reserved the free memory of the GPU) sees
 * cudaMalloc fail or fragment that pool; a loop that runs trajectories
 * between kernels of its own on other streams (a particle filter, an ABC
 * sampler, a serving loop) cannot afford cudaFree, which waits for the whole
 * device.  siminf_gpu_run_solver_ssm allocates and frees its buffers on
 * every call; this entry point takes the same arguments and does neither.
 *
 * What it runs: the kernels of siminf_gpu_run_solver_ssm for a schedule
 * without external transfers -- k_init, then k_horizon (every day of a node
 * in one thread) -- with every buffer they use (model matrices, node state,
 * day schedule, error log, U and V) carved out of g_noalloc_scratch.  The
 * results are those of siminf_gpu_run_solver_ssm on the same arguments.
 *
 * Limits: one replicate (Nrep = 1), no scheduled events (len = 0), a dense
 * U (and a dense V or none), and everything in SIMINF_GPU_NOALLOC_SCRATCH_BYTES
 * (16 MiB).  Larger runs are rejected with SIMINF_GPU_ERR_SCRATCH_LIMIT.
 *
 * Sharing: every call on a device uses the same array, which keeps the last
 * call's contents; each call clears what must start at zero (error counters,
 * the event index, U and V) and overwrites the rest.  Calls that overlap on
 * the GPU (from two host threads, or on two streams without an ordering
 * between them) race on the array.
 *
 * Set-up: the first call on a device, with that device current, looks up
 * the array's device address (cudaGetSymbolAddress) and keeps it; make that
 * first call before any stream capture on the device.
 */
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include <cuda_runtime.h>

#include "../../include/siminf_gb300.h"
#include "siminf_capi_internal.h"
#include "siminf_launch.h"
#include "siminf_plan.h"

using namespace siminf;

/* The scratch of every call on a device (one copy per device). */
static __device__ __align__(256) unsigned char g_noalloc_scratch[SIMINF_GPU_NOALLOC_SCRATCH_BYTES];

namespace {

enum { NOALLOC_MAX_DEVICES = 64, DAY_CHUNK = 128 };

/* Control block at the start of the scratch: the error counters k_init and
 * k_horizon update (err_count, err_day, err_day_pre_e2 contiguous, as the
 * kernels expect), the transition counter and the error chosen for the
 * caller. */
struct NoallocCtl {
    int err_count, err_day, err_day_pre_e2, have;
    unsigned long long fired;
    ErrRec pick;
};

/* Byte offsets of the buffers inside the scratch, each 256-aligned. */
struct Layout {
    size_t ctl, S, G, e1_ptr, u, vA, vB, t_rate, sum_rate, t_time, ctr, update, err, days,
        ldata, gdata, U, V, total;
};

size_t carve(size_t &off, size_t bytes)
{
    const size_t at = off;
    off += (bytes + 255) & ~(size_t) 255;
    return at;
}

std::mutex g_setup_mutex;
void *g_scratch_addr[NOALLOC_MAX_DEVICES];

/* Device address of g_noalloc_scratch on the current device, looked up on
 * the first call on that device. */
int scratch_address(void **out)
{
    int ndev = 0, dev = -1;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        capi_set_status(SIMINF_GPU_ERR_NO_DEVICE, -1, -1, -1, 0, 0, "no CUDA device");
        return SIMINF_GPU_ERR_NO_DEVICE;
    }
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return capi_cuda_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) {
        capi_set_status(SIMINF_GPU_ERR_NO_DEVICE, -1, -1, -1, 0, 0,
                        "device ordinal beyond the 64 the scratch table covers");
        return SIMINF_GPU_ERR_NO_DEVICE;
    }
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess)
            return capi_cuda_fail(e, "cudaGetSymbolAddress of the solver scratch");
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return 0;
}

/* Days of the schedule: tt starts at tspan[0] and moves to the next whole
 * unit of time; the run ends at the first day past tspan[tlen - 1]
 * (src/solvers/SimInf_solver_ssm.c:305-334).  Returns -1 past max_days. */
long long count_days(const double *tspan, int tlen, long long max_days)
{
    double tt = tspan[0], next = floor(tt) + 1.0;
    int it = 0;
    long long n = 0;
    while (it < tlen) {
        tt = next;
        next += 1.0;
        while (it < tlen && tt > tspan[it])
            it++;
        if (++n > max_days)
            return -1;
    }
    return n;
}

/* Initial values of the control block and the empty per-node event index. */
__global__ void k_noalloc_reset(NoallocCtl *ctl, int *e1_ptr, int nn1)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) {
        ctl->err_count = 0;
        ctl->err_day = INT_MAX;
        ctl->err_day_pre_e2 = INT_MAX;
        ctl->have = 0;
        ctl->fired = 0ULL;
    }
    if (i < nn1)
        e1_ptr[i] = 0;
}

/* The error siminf_gpu_run_solver_ssm reports from the same log: the
 * earliest day; on it the lowest node of the initialisation, else of the
 * SSA; unless that is an initialisation error, the post-time-step errors
 * override it in node order, the first that is not an invalid rate, else
 * the last. */
__global__ void k_noalloc_pick(const ErrRec *err, NoallocCtl *ctl)
{
    const int n = ctl->err_count < (int) MAX_ERR ? ctl->err_count : (int) MAX_ERR;
    if (n <= 0)
        return;
    int day = INT_MAX;
    for (int i = 0; i < n; i++)
        day = err[i].day < day ? err[i].day : day;
    int best = -1;
    for (int ph = PHASE_INIT; ph <= PHASE_SSA && best < 0; ph++)
        for (int i = 0; i < n; i++)
            if (err[i].day == day && err[i].phase == ph && (best < 0 || err[i].node < err[best].node))
                best = i;
    if (best < 0 || err[best].phase != PHASE_INIT) {
        int other = -1, last_rate = -1;
        for (int i = 0; i < n; i++) {
            if (err[i].day != day || err[i].phase != PHASE_PTS)
                continue;
            if (err[i].code != SIMINF_GPU_ERR_INVALID_RATE) {
                if (other < 0 || err[i].node < err[other].node)
                    other = i;
            } else if (last_rate < 0 || err[i].node >= err[last_rate].node) {
                last_rate = i;
            }
        }
        /* in node order, the first error that is not an invalid rate,
         * else the last invalid rate: of the highest node, its last record
         * (one thread records a node's rates in transition order) */
        if (other >= 0) {
            best = other;
        } else if (last_rate >= 0) {
            best = last_rate;
        }
    }
    if (best >= 0) {
        ctl->pick = err[best];
        ctl->have = 1;
    }
}

int fail(int code, const char *msg)
{
    capi_set_status(code, -1, -1, -1, 0, 0, msg);
    return code;
}

}  // namespace

extern "C" int siminf_gpu_run_solver_ssm_noalloc(siminf_gpu_solver_args *a,
                                                 const siminf_gpu_model *model,
                                                 void *cuda_stream)
{
    capi_clear_status();
    if (!model || !model->L)
        return fail(SIMINF_GPU_ERR_UNKNOWN_MODEL, "no device model");
    const Launchers *L = model->L;
    int rc = capi_validate(a, L);
    if (rc)
        return rc;
    if (a->solver != 0)
        return fail(SIMINF_GPU_ERR_UNKNOWN_SOLVER,
                    "the allocation-free solver runs the ssm solver");
    if (a->Nrep != 1 || a->len > 0 || !a->U || !L->pts_local)
        return fail(SIMINF_GPU_ERR_INVALID_MODEL,
                    "the allocation-free solver runs one replicate without scheduled "
                    "events into a dense U");
    const int Nn = a->Nn, Nc = a->Nc, Nt = a->Nt, Nd = a->Nd, tlen = a->tlen;
    const bool want_V = Nd > 0 && a->V;

    /* Size check before anything touches the device. */
    const long long ndays = count_days(a->tspan, tlen, (long long) SIMINF_GPU_NOALLOC_SCRATCH_BYTES);
    Layout lo{};
    size_t off = 0;
    if (ndays >= 0) {
        const size_t nn = (size_t) Nn;
        lo.ctl = carve(off, sizeof(NoallocCtl));
        lo.S = carve(off, (size_t) Nt * Nc * sizeof(int));
        lo.G = carve(off, (size_t) Nt * sizeof(uint32_t));
        lo.e1_ptr = carve(off, (nn + 1) * sizeof(int));
        lo.u = carve(off, nn * Nc * sizeof(int));
        lo.vA = carve(off, nn * Nd * sizeof(double));
        lo.vB = carve(off, nn * Nd * sizeof(double));
        lo.t_rate = carve(off, nn * Nt * sizeof(double));
        lo.sum_rate = carve(off, nn * sizeof(double));
        lo.t_time = carve(off, nn * sizeof(double));
        lo.ctr = carve(off, nn * sizeof(uint64_t));
        lo.update = carve(off, nn * sizeof(uint8_t));
        lo.err = carve(off, (size_t) MAX_ERR * sizeof(ErrRec));
        lo.days = carve(off, (size_t) ndays * sizeof(DayInfo));
        lo.ldata = carve(off, (a->Nld > 0 ? nn * a->Nld : 1) * sizeof(double));
        lo.gdata = carve(off, (size_t) (L->Ngd > 0 ? L->Ngd : 1) * sizeof(double));
        lo.U = carve(off, (size_t) tlen * nn * Nc * sizeof(int));
        lo.V = carve(off, want_V ? (size_t) tlen * nn * Nd * sizeof(double) : 0);
        lo.total = off;
    }
    if (ndays < 0 || lo.total > (size_t) SIMINF_GPU_NOALLOC_SCRATCH_BYTES) {
        char msg[256];
        snprintf(msg, sizeof(msg),
                 "Nn=%d, tlen=%d needs %zu bytes of solver scratch; the allocation-free "
                 "solver has %u",
                 Nn, tlen, ndays < 0 ? (size_t) -1 : lo.total,
                 (unsigned) SIMINF_GPU_NOALLOC_SCRATCH_BYTES);
        return fail(SIMINF_GPU_ERR_SCRATCH_LIMIT, msg);
    }

    void *base_ptr = nullptr;
    if ((rc = scratch_address(&base_ptr)))
        return rc;
    unsigned char *base = (unsigned char *) base_ptr;
    cudaStream_t st = (cudaStream_t) cuda_stream;

    DevState s{};
    s.Nn = Nn;
    s.Nc = Nc;
    s.Nt = Nt;
    s.Nd = Nd;
    s.Nld = a->Nld;
    s.Nrep = 1;
    s.tlen = tlen;
    s.Ntot = Nn;
    s.seed = (uint64_t) a->seed;
    s.cap = 0;
    s.max_fired = SIMINF_GPU_MAX_NODE_DAY_TRANSITIONS;
    s.S = (const int *) (base + lo.S);
    s.Gmask = (const uint32_t *) (base + lo.G);
    s.hasN = 0;
    s.ldata = (const double *) (base + lo.ldata);
    s.gdata = (const double *) (base + lo.gdata);
    s.gdata_stride = 0;
    s.u = (int *) (base + lo.u);
    s.vA = (double *) (base + lo.vA);
    s.vB = (double *) (base + lo.vB);
    s.t_rate = (double *) (base + lo.t_rate);
    s.sum_rate = (double *) (base + lo.sum_rate);
    s.t_time = (double *) (base + lo.t_time);
    s.ctr = (uint64_t *) (base + lo.ctr);
    s.update = (uint8_t *) (base + lo.update);
    s.e1_ptr = (const int *) (base + lo.e1_ptr);
    s.e1 = nullptr;
    s.U = (int *) (base + lo.U);
    s.V = want_V ? (double *) (base + lo.V) : nullptr;
    NoallocCtl *ctl = (NoallocCtl *) (base + lo.ctl);
    s.err = (ErrRec *) (base + lo.err);
    s.err_count = &ctl->err_count;
    s.err_day = &ctl->err_day;
    s.err_day_pre_e2 = &ctl->err_day_pre_e2;
    s.fired = &ctl->fired;
    s.heavy_rate = 0.0;          /* the horizon kernel has no work queue */
    DayInfo *d_days = (DayInfo *) (base + lo.days);

    /* Dense S (Nt rows of Nc) and the G column masks, built on the stack. */
    int Sd[MAX_NT * MAX_NC];
    uint32_t Gm[MAX_NT];
    if (Nt > MAX_NT || Nc > MAX_NC)
        return fail(SIMINF_GPU_ERR_INVALID_MODEL, "model larger than the device limits");
    memset(Sd, 0, sizeof(Sd));
    memset(Gm, 0, sizeof(Gm));
    for (int j = 0; j < Nt; j++) {
        for (int k = a->jcS[j]; k < a->jcS[j + 1]; k++)
            Sd[j * Nc + a->irS[k]] += a->prS[k];
        for (int k = a->jcG[j]; k < a->jcG[j + 1]; k++)
            Gm[j] |= 1u << a->irG[k];
    }

    /* Inputs.  Copies from pageable host memory return once the source has
     * been read, so the stack buffers may be reused right away. */
    cudaError_t e = cudaSuccess;
    const char *what = "copy inputs into the solver scratch";
    auto h2d = [&](size_t at, const void *src, size_t bytes) {
        if (e == cudaSuccess && bytes)
            e = cudaMemcpyAsync(base + at, src, bytes, cudaMemcpyHostToDevice, st);
    };
    h2d(lo.S, Sd, (size_t) Nt * Nc * sizeof(int));
    h2d(lo.G, Gm, (size_t) Nt * sizeof(uint32_t));
    h2d(lo.u, a->u0, (size_t) Nn * Nc * sizeof(int));
    if (Nd > 0) {
        h2d(lo.vA, a->v0, (size_t) Nn * Nd * sizeof(double));
        h2d(lo.vB, a->v0, (size_t) Nn * Nd * sizeof(double));
    }
    if (a->Nld > 0)
        h2d(lo.ldata, a->ldata, (size_t) Nn * a->Nld * sizeof(double));
    if (a->gdata && L->Ngd > 0)
        h2d(lo.gdata, a->gdata, (size_t) L->Ngd * sizeof(double));
    {
        DayInfo chunk[DAY_CHUNK];
        double tt = a->tspan[0], next = floor(tt) + 1.0;
        int it = 0;
        long long d = 0;
        while (it < tlen && e == cudaSuccess) {
            int k = 0;
            for (; k < DAY_CHUNK && it < tlen; k++) {
                DayInfo di;
                di.tt = tt;
                di.next = next;
                tt = next;
                next += 1.0;
                di.c0 = it;
                while (it < tlen && tt > a->tspan[it])
                    it++;
                di.c1 = it;
                chunk[k] = di;
            }
            h2d(lo.days + (size_t) d * sizeof(DayInfo), chunk, (size_t) k * sizeof(DayInfo));
            d += k;
        }
    }
    /* What must start at zero: the counters, the (empty) event index and
     * the outputs. */
    if (e == cudaSuccess) {
        what = "reset the solver scratch";
        k_noalloc_reset<<<(unsigned) ((Nn + 1 + 255) / 256), 256, 0, st>>>(ctl, (int *) (base + lo.e1_ptr), Nn + 1);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemsetAsync(base + lo.U, 0, (size_t) tlen * Nn * Nc * sizeof(int), st);
    if (e == cudaSuccess && want_V)
        e = cudaMemsetAsync(base + lo.V, 0, (size_t) tlen * Nn * Nd * sizeof(double), st);

    if (e == cudaSuccess) {
        what = "solver kernels";
        e = L->init(s, a->tspan[0], st);
    }
    if (e == cudaSuccess)
        e = L->horizon(s, d_days, (int) ndays, st);
    if (e == cudaSuccess) {
        k_noalloc_pick<<<1, 1, 0, st>>>(s.err, ctl);
        e = cudaGetLastError();
    }
    NoallocCtl hc;
    if (e == cudaSuccess) {
        what = "read the solver status";
        e = cudaMemcpyAsync(&hc, ctl, sizeof(hc), cudaMemcpyDeviceToHost, st);
    }
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
        return capi_cuda_fail(e, what);

    if (hc.have) {
        const ErrRec &r = hc.pick;
        char msg[300];
        snprintf(msg, sizeof(msg),
                 "error %d at time %g, replicate %d, node %d (one-based), transition %d, event %d, rate %g",
                 r.code, r.time, r.rep + 1, r.node + 1, r.transition >= 0 ? r.transition + 1 : 0,
                 r.event_index >= 0 ? r.event_index + 1 : 0, r.rate);
        capi_set_status(r.code, r.node, r.transition, r.event_index, r.time, r.rate, msg);
        return r.code;
    }

    /* Outputs: the reference's column-major U (and V). */
    e = cudaMemcpyAsync(a->U, base + lo.U, (size_t) tlen * Nn * Nc * sizeof(int),
                        cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && want_V)
        e = cudaMemcpyAsync(a->V, base + lo.V, (size_t) tlen * Nn * Nd * sizeof(double),
                            cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
        return capi_cuda_fail(e, "copy U and V out of the solver scratch");
    return 0;
}
