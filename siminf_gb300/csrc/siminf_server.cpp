/*
 * siminf_server.cpp -- a request loop over the solver for serving:
 * simulation runs, particle filters and re-runs of device-resident plans
 * arrive as they come, are admitted while their device memory fits an HBM
 * budget, and run side by side on the GPU, one per slot.
 *
 * The reference has no server: R runs one simulation per run() call on the
 * calling thread (R/run.R:178-283).  Here a slot is a host thread with its
 * own non-blocking CUDA stream; the plans it creates put every copy and
 * kernel on that stream and take their buffers from the stream-ordered
 * allocator, so a request that starts or ends never waits for the others'
 * work (cudaFree would wait for the whole device).  Admission is by
 * estimated device bytes against the budget, oldest request first, and a
 * younger request that fits is admitted while an older one waits for
 * memory, so small requests keep flowing past large ones.  Every request's
 * results are those of the same call made alone: the kernels draw from
 * streams keyed only by the request's own seed and node indices.
 *
 * A plan request re-runs a plan the caller created and keeps on the device
 * (siminf_gpu_plan_create): the continuation path, with no upload.
 */
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/siminf_gb300.h"
#include "siminf_capi_internal.h"

using namespace siminf;

struct siminf_gpu_server {
    std::mutex mu;
    std::condition_variable work, done;
    std::deque<siminf_gpu_request *> pending;
    long long budget = 0, in_use = 0;
    int running = 0;
    bool stop = false;
    int device = 0;
    std::vector<std::thread> slots;
};

namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b)
{
    return std::chrono::duration<double, std::milli>(b - a).count();
}

/* Device bytes a run of args needs: state, events, outputs, with a
 * quarter of headroom for the planner's buffers. */
long long run_bytes(const siminf_gpu_solver_args *a)
{
    const long long Ntot = (long long) a->Nn * std::max(1, a->Nrep);
    long long b = Ntot * (4LL * a->Nc + 8LL * a->Nt + 8 * 4 + 16LL * a->Nd);
    b += 32LL * a->len;
    if (a->U)
        b += Ntot * a->Nc * 4LL * a->tlen;
    if (a->V)
        b += Ntot * a->Nd * 8LL * a->tlen;
    b += (long long) a->Nn * 8LL * std::max(0, a->Nld);
    return b + b / 4 + (1 << 20);
}

long long request_bytes(const siminf_gpu_request *r)
{
    if (r->bytes > 0)
        return r->bytes;
    switch (r->kind) {
    case SIMINF_GPU_REQUEST_RUN:
        return r->args ? run_bytes(r->args) : 0;
    case SIMINF_GPU_REQUEST_PFILTER: {
        if (!r->args || !r->pfilter)
            return 0;
        siminf_gpu_solver_args a = *r->args;
        a.Nrep = r->pfilter->n_particles;
        a.tlen = 2;
        a.U = nullptr;
        a.V = nullptr;
        const long long per = (long long) a.Nn * a.Nrep;
        return run_bytes(&a) + per * (a.Nc * 4LL * 2 + a.Nd * 8LL * 2);
    }
    default:
        return 0;                       /* a resident plan holds its memory already */
    }
}

void copy_status(siminf_gpu_request *r)
{
    siminf_gpu_status st;
    siminf_gpu_last_status(&st);
    snprintf(r->message, sizeof(r->message), "%.199s", st.message);
}

int execute(siminf_gpu_request *r, cudaStream_t stream)
{
    switch (r->kind) {
    case SIMINF_GPU_REQUEST_RUN: {
        siminf_gpu_plan *p = nullptr;
        int rc = plan_create_internal(r->args, r->model, &r->options, &p, false, false);
        if (!rc)
            rc = plan_run_internal(p, stream);
        if (!rc)
            rc = siminf_gpu_plan_download(p, r->args);
        if (p)
            siminf_gpu_plan_stats(p, &r->stats);
        siminf_gpu_plan_free(p);
        return rc;
    }
    case SIMINF_GPU_REQUEST_PFILTER:
        return siminf_gpu_pfilter(r->args, r->model, r->pfilter);
    case SIMINF_GPU_REQUEST_PLAN: {
        const int rc = plan_run_internal(r->plan, stream);
        siminf_gpu_plan_stats(r->plan, &r->stats);
        return rc;
    }
    case SIMINF_GPU_REQUEST_PMCMC:
        /* the chain's filter session is resident: only its iterations run */
        return siminf_gpu_pmcmc_run(r->pmcmc, r->pmcmc_iterations, r->pmcmc_rows);
    default:
        capi_set_status(SIMINF_GPU_ERR_INVALID_MODEL, -1, -1, -1, 0, 0, "unknown request kind");
        return SIMINF_GPU_ERR_INVALID_MODEL;
    }
}

void slot_main(siminf_gpu_server *sv)
{
    cudaSetDevice(sv->device);
    cudaStream_t stream = nullptr;
    if (cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking) != cudaSuccess)
        stream = nullptr;
    plan_thread_stream(stream, stream != nullptr);
    std::unique_lock<std::mutex> lk(sv->mu);
    for (;;) {
        siminf_gpu_request *r = nullptr;
        long long bytes = 0;
        for (;;) {
            /* the oldest request that fits; one that alone exceeds the
             * budget runs when nothing else does */
            for (auto it = sv->pending.begin(); it != sv->pending.end(); ++it) {
                const long long b = request_bytes(*it);
                if (sv->in_use + b <= sv->budget || sv->running == 0) {
                    r = *it;
                    bytes = b;
                    sv->pending.erase(it);
                    break;
                }
            }
            if (r || (sv->stop && sv->pending.empty()))
                break;
            sv->work.wait(lk);
        }
        if (!r)
            break;
        sv->in_use += bytes;
        sv->running++;
        lk.unlock();

        const auto t0 = Clock::now();
        r->ms_wait = ms_between(Clock::time_point(std::chrono::nanoseconds(r->submit_ns)), t0);
        capi_clear_status();
        const int rc = execute(r, stream);
        if (rc)
            copy_status(r);
        r->ms_run = ms_between(t0, Clock::now());

        lk.lock();
        sv->in_use -= bytes;
        sv->running--;
        r->status = rc;
        r->finished = 1;
        sv->done.notify_all();
        sv->work.notify_all();
    }
    lk.unlock();
    plan_thread_stream(nullptr, false);
    if (stream)
        cudaStreamDestroy(stream);
}

}  // namespace

extern "C" {

int siminf_gpu_server_create(const siminf_gpu_server_options *opt, siminf_gpu_server **out)
{
    capi_clear_status();
    if (!out)
        return SIMINF_GPU_ERR_INVALID_MODEL;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        capi_set_status(SIMINF_GPU_ERR_NO_DEVICE, -1, -1, -1, 0, 0, "no CUDA device");
        return SIMINF_GPU_ERR_NO_DEVICE;
    }
    siminf_gpu_server *sv = new siminf_gpu_server();
    cudaGetDevice(&sv->device);
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    sv->budget = (opt && opt->hbm_budget_bytes > 0) ? opt->hbm_budget_bytes
                                                    : (long long) (0.9 * (double) free_b);
    /* keep freed blocks in the stream-ordered pool between requests */
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, sv->device) == cudaSuccess) {
        uint64_t keep = (uint64_t) sv->budget;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    const int n = (opt && opt->slots > 0) ? opt->slots : 8;
    for (int i = 0; i < n; i++)
        sv->slots.emplace_back(slot_main, sv);
    *out = sv;
    return 0;
}

int siminf_gpu_server_submit(siminf_gpu_server *sv, siminf_gpu_request *r)
{
    if (!sv || !r)
        return SIMINF_GPU_ERR_INVALID_MODEL;
    /* a plan or a pmcmc chain is resident and carries its own model */
    const bool resident = r->kind == SIMINF_GPU_REQUEST_PLAN ||
                          r->kind == SIMINF_GPU_REQUEST_PMCMC;
    if ((r->kind == SIMINF_GPU_REQUEST_PLAN && !r->plan) ||
        (r->kind == SIMINF_GPU_REQUEST_PMCMC && (!r->pmcmc || r->pmcmc_iterations < 0)) ||
        (!resident && (!r->args || !r->model)) ||
        (r->kind == SIMINF_GPU_REQUEST_PFILTER && !r->pfilter))
        return SIMINF_GPU_ERR_INVALID_MODEL;
    r->status = 0;
    r->finished = 0;
    r->ms_wait = r->ms_run = 0;
    r->message[0] = 0;
    r->submit_ns = (long long) std::chrono::duration_cast<std::chrono::nanoseconds>(
                       Clock::now().time_since_epoch())
                       .count();
    std::lock_guard<std::mutex> lk(sv->mu);
    if (sv->stop)
        return SIMINF_GPU_ERR_INVALID_MODEL;
    sv->pending.push_back(r);
    sv->work.notify_one();
    return 0;
}

int siminf_gpu_server_wait(siminf_gpu_server *sv, siminf_gpu_request *r, double timeout_ms)
{
    if (!sv || !r)
        return SIMINF_GPU_ERR_INVALID_MODEL;
    std::unique_lock<std::mutex> lk(sv->mu);
    auto ready = [r] { return r->finished != 0; };
    if (timeout_ms < 0)
        sv->done.wait(lk, ready);
    else
        sv->done.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms), ready);
    return r->finished ? 1 : 0;
}

int siminf_gpu_server_load(siminf_gpu_server *sv, int *pending, int *running,
                           long long *bytes_in_use)
{
    if (!sv)
        return SIMINF_GPU_ERR_INVALID_MODEL;
    std::lock_guard<std::mutex> lk(sv->mu);
    if (pending)
        *pending = (int) sv->pending.size();
    if (running)
        *running = sv->running;
    if (bytes_in_use)
        *bytes_in_use = sv->in_use;
    return 0;
}

void siminf_gpu_server_free(siminf_gpu_server *sv)
{
    if (!sv)
        return;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->stop = true;
        sv->work.notify_all();
    }
    for (auto &t : sv->slots)
        t.join();
    delete sv;
}

}  /* extern "C" */
