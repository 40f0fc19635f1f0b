/*
 * siminf_individual.cu -- cleaning of individual-based event data on the
 * device: SimInf_individual_events (src/misc/SimInf_individual_events.c:
 * 167-249) keeps, for every individual, the events on its longest
 * consistent path (enter -> external transfers -> exit) and drops the rest.
 * It is the step that turns livestock registers of 10^7-10^8 individual
 * events into the node-level schedules the solver runs.
 *
 * Input, as R/SimInf_individual_events.R:397-410 hands it over: events
 * sorted by (id, time, event, node, dest) with exact duplicates removed,
 * event 0 (exit), 1 (enter) or 3 (external transfer), dest NA (INT_MIN)
 * except for transfers.  Output: keep[i] = 1 or 0.
 *
 * Two launches on one stream, no host round trip between them:
 *  1. k_indiv_starts, eight events per thread: zeroes keep, checks the
 *     event type (the smallest invalid index by atomicMin), and appends
 *     the event to the list of individuals' first events when its id
 *     differs from the previous one (warp ballots, one atomic per block of
 *     2,048 events; the list is unordered, which no result depends on).
 *  2. k_indiv_paths, a grid-stride loop over that list, one thread per
 *     individual: finds the individual's last event and runs its
 *     depth-first search over its own slice of the columns, with a path
 *     scratch of the same slice.  Nothing runs when an event type was
 *     invalid; the host then reports the reference's error.
 *
 * The search keeps the reference's order (roots, then branches, in array
 * order; a path replaces the best only when strictly longer; a root stops
 * once its path cannot grow), which decides which of several equally long
 * paths survives: see ie_longest_path.
 *
 * Bytes per event: the five columns read once and keep written once (24
 * B) are compulsory; id and event are read by both launches, and keep and
 * the path scratch are written per individual inside L2.
 */
#include <chrono>
#include <climits>
#include <cstdint>
#include <cstdio>

#include <cuda_runtime.h>

#include "../../include/siminf_gb300.h"
#include "siminf_capi_internal.h"

using namespace siminf;

namespace {

enum { IE_EXIT = 0, IE_ENTER = 1, IE_EXTERNAL_TRANSFER = 3 };
enum { IE_BLOCK = 256, IE_ITEMS = 8, IE_TILE = IE_BLOCK * IE_ITEMS, IE_BLOCKS_PER_SM = 8 };
constexpr unsigned long long IE_NONE = ~0ULL;

/* May event j of an individual follow its event i on a path?  The
 * individual is at node[i] after an enter and at dest[i] after a transfer;
 * j must happen later, start there, not lead back there, and be an exit or
 * a transfer (SimInf_individual_events.c:111-115). */
__host__ __device__ __forceinline__ bool ie_follows(const int *event, const int *time,
                                                    const int *node, const int *dest, int i,
                                                    int j)
{
    const int at = event[i] == IE_ENTER ? node[i] : dest[i];
    const int ej = event[j];
    return time[j] > time[i] && node[j] == at && dest[j] != at &&
           (ej == IE_EXIT || ej == IE_EXTERNAL_TRANSFER);
}

/* The longest path of one individual's n events (SimInf_find_longest_path,
 * SimInf_individual_events.c:50-147).  keep (zero on entry) gets 1 on the
 * kept events; path is scratch of n ints holding one-based event positions
 * of the current path, 0 for an empty level.
 *
 * With any enter present a path must start with one; with any exit present
 * a kept path must end with one.  Each admissible root starts a depth-first
 * search: at each level the next branch is the first later event that may
 * follow the previous level's event; the search backs up when none is
 * left or the branch is an exit.  A lone root is kept when no path exists
 * yet: an exit if exits are present, else an enter or a transfer.
 *
 * The search can take time exponential in n (branches that rejoin, exits
 * that no path reaches, so nothing prunes it); the reference runs it on a
 * CPU, here it would hold a GPU thread.  budget bounds the candidate
 * events examined; the function returns false when it runs out, with keep
 * cleared. */
__host__ __device__ inline bool ie_longest_path(const int *event, const int *time,
                                                const int *node, const int *dest, int n,
                                                int *path, int *keep, long long budget)
{
    bool any_enter = false, any_exit = false;
    for (int i = 0; i < n; i++) {
        any_enter |= event[i] == IE_ENTER;
        any_exit |= event[i] == IE_EXIT;
    }
    int best = 0;
    for (int root = 0; root < n; root++) {
        const int er = event[root];
        if (any_enter && er != IE_ENTER)
            continue;
        if (best == 0 && (any_exit ? er == IE_EXIT
                                   : (er == IE_ENTER || er == IE_EXTERNAL_TRANSFER))) {
            best = 1;
            keep[root] = 1;
        }
        for (int k = 0; k < n; k++)
            path[k] = 0;
        path[0] = root + 1;
        const int room = n - root;
        int depth = 1;
        while (depth > 0 && depth < room && best < room) {
            const int prev = path[depth - 1] - 1;
            int j = path[depth] > 0 ? path[depth] : prev + 1;
            path[depth] = 0;
            for (; j < n; j++) {
                if (--budget < 0) {
                    for (int k = 0; k < n; k++)
                        keep[k] = 0;
                    return false;
                }
                if (!ie_follows(event, time, node, dest, prev, j))
                    continue;
                path[depth] = j + 1;
                if (!(any_exit && event[j] == IE_EXTERNAL_TRANSFER) && depth + 1 > best) {
                    best = depth + 1;
                    for (int k = 0; k < n; k++)
                        keep[k] = 0;
                    for (int k = 0; k < best; k++)
                        keep[path[k] - 1] = 1;
                }
                break;
            }
            if (path[depth] == 0) {
                depth--;
            } else if (event[path[depth] - 1] == IE_EXIT) {
                path[depth] = 0;
                depth--;
            } else {
                depth++;
            }
        }
    }
    return true;
}

/* counts[0]: individuals listed so far; counts[1]: smallest index of an
 * invalid event type (IE_NONE when none); counts[2]: smallest first event
 * of an individual whose search ran out of steps (IE_NONE when none).  A
 * block takes IE_TILE events, IE_ITEMS per thread in strides of the block,
 * and appends its first events with one atomic: a counter shared by every
 * warp of the grid was the kernel's bottleneck. */
__global__ void __launch_bounds__(IE_BLOCK) k_indiv_starts(const int *__restrict__ id,
                                                           const int *__restrict__ event,
                                                           long long len, int *starts,
                                                           unsigned long long *counts,
                                                           int *keep)
{
    __shared__ unsigned warp_offset[IE_BLOCK / 32];
    __shared__ unsigned long long block_base;
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long tile = blockIdx.x * (long long) IE_TILE;
    unsigned mask[IE_ITEMS];
    unsigned listed = 0;
#pragma unroll
    for (int r = 0; r < IE_ITEMS; r++) {
        const long long i = tile + r * IE_BLOCK + threadIdx.x;
        bool first = false;
        if (i < len) {
            const int e = event[i];
            if (e != IE_EXIT && e != IE_ENTER && e != IE_EXTERNAL_TRANSFER)
                atomicMin(&counts[1], (unsigned long long) i);
            first = i == 0 || id[i] != id[i - 1];
            keep[i] = 0;
        }
        mask[r] = __ballot_sync(0xFFFFFFFFu, first);
        listed += __popc(mask[r]);
    }
    if (lane == 0)
        warp_offset[warp] = listed;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned sum = 0;
        for (int w = 0; w < IE_BLOCK / 32; w++) {
            const unsigned c = warp_offset[w];
            warp_offset[w] = sum;
            sum += c;
        }
        block_base = sum ? atomicAdd(&counts[0], (unsigned long long) sum) : 0;
    }
    __syncthreads();
    unsigned long long at = block_base + warp_offset[warp];
    const unsigned below = (1u << lane) - 1u;
#pragma unroll
    for (int r = 0; r < IE_ITEMS; r++) {
        if ((mask[r] >> lane) & 1u)
            starts[at + __popc(mask[r] & below)] = (int) (tile + r * IE_BLOCK + threadIdx.x);
        at += __popc(mask[r]);
    }
}

__global__ void __launch_bounds__(IE_BLOCK) k_indiv_paths(const int *__restrict__ id,
                                                          const int *__restrict__ event,
                                                          const int *__restrict__ time,
                                                          const int *__restrict__ node,
                                                          const int *__restrict__ dest,
                                                          long long len,
                                                          const int *__restrict__ starts,
                                                          unsigned long long *counts,
                                                          int *path, int *keep,
                                                          long long budget)
{
    if (counts[1] != IE_NONE)
        return;
    const long long ngroups = (long long) counts[0];
    for (long long g = blockIdx.x * (long long) IE_BLOCK + threadIdx.x; g < ngroups;
         g += (long long) gridDim.x * IE_BLOCK) {
        const long long b = starts[g];
        const int who = id[b];
        long long e = b + 1;
        while (e < len && id[e] == who)
            e++;
        if (!ie_longest_path(event + b, time + b, node + b, dest + b, (int) (e - b), path + b,
                             keep + b, budget))
            atomicMin(&counts[2], (unsigned long long) b);  /* the search gave up */
    }
}

int fail(int code, long long index, const char *msg)
{
    capi_set_status(code, -1, -1, index >= 0 && index <= INT_MAX ? (int) index : -1, 0, 0, msg);
    return code;
}

}  // namespace

extern "C" int siminf_gpu_individual_events(long long len, const int *id, const int *event,
                                            const int *time, const int *node, const int *dest,
                                            int *keep, void *cuda_stream,
                                            siminf_gpu_reduce_stats *stats)
{
    return siminf_gpu_individual_events_ex(len, id, event, time, node, dest, keep,
                                           SIMINF_GPU_INDIVIDUAL_MAX_STEPS, cuda_stream, stats);
}

extern "C" int siminf_gpu_individual_events_ex(long long len, const int *id, const int *event,
                                               const int *time, const int *node,
                                               const int *dest, int *keep, long long max_steps,
                                               void *cuda_stream,
                                               siminf_gpu_reduce_stats *stats)
{
    capi_clear_status();
    const cudaStream_t st = (cudaStream_t) cuda_stream;
    if (len < 0 || len > (long long) INT_MAX ||
        (len > 0 && (!id || !event || !time || !node || !dest || !keep)))
        return fail(SIMINF_GPU_ERR_INVALID_MODEL, -1, "invalid individual event table");
    if (len == 0)
        return 0;
    auto t0 = std::chrono::steady_clock::now();
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const size_t ib = (size_t) len * sizeof(int);
    /* five input columns, then keep, the path scratch and the start list */
    int *d_cols = nullptr;
    unsigned long long *d_counts = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (e == cudaSuccess) e = cudaMallocAsync((void **) &d_cols, 8 * ib, st);
    if (e == cudaSuccess) e = cudaMallocAsync((void **) &d_counts, 3 * sizeof(unsigned long long), st);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    int *d_id = d_cols, *d_event = d_cols + len, *d_time = d_cols + 2 * len,
        *d_node = d_cols + 3 * len, *d_dest = d_cols + 4 * len, *d_keep = d_cols + 5 * len,
        *d_path = d_cols + 6 * len, *d_starts = d_cols + 7 * len;
    const int *host[5] = {id, event, time, node, dest};
    int *dev_col[5] = {d_id, d_event, d_time, d_node, d_dest};
    for (int c = 0; c < 5 && e == cudaSuccess; c++)
        e = cudaMemcpyAsync(dev_col[c], host[c], ib, cudaMemcpyHostToDevice, st);
    unsigned long long counts[3] = {0, IE_NONE, IE_NONE};
    if (max_steps <= 0)
        max_steps = SIMINF_GPU_INDIVIDUAL_MAX_STEPS;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_counts, counts, sizeof(counts), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        const long long tiles = (len + IE_TILE - 1) / IE_TILE;
        const long long blocks = (len + IE_BLOCK - 1) / IE_BLOCK;
        const long long grid = blocks < (long long) sms * IE_BLOCKS_PER_SM
                                   ? blocks : (long long) sms * IE_BLOCKS_PER_SM;
        cudaEventRecord(e0, st);
        k_indiv_starts<<<(unsigned) tiles, IE_BLOCK, 0, st>>>(d_id, d_event, len, d_starts,
                                                              d_counts, d_keep);
        k_indiv_paths<<<(unsigned) grid, IE_BLOCK, 0, st>>>(d_id, d_event, d_time, d_node,
                                                            d_dest, len, d_starts, d_counts,
                                                            d_path, d_keep, max_steps);
        cudaEventRecord(e1, st);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(keep, d_keep, ib, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(counts, d_counts, sizeof(counts), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess && stats) {
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        stats->ms_kernel = ms;
        stats->ms_total = std::chrono::duration<double, std::milli>(
                              std::chrono::steady_clock::now() - t0).count();
        stats->bytes_read = len * 20;
        stats->bytes_written = len * 4;
    }
    if (e0)
        cudaEventDestroy(e0);
    if (e1)
        cudaEventDestroy(e1);
    if (d_cols)
        cudaFreeAsync(d_cols, st);
    if (d_counts)
        cudaFreeAsync(d_counts, st);
    const cudaError_t e2 = cudaStreamSynchronize(st);
    if (e == cudaSuccess)
        e = e2;
    if (e != cudaSuccess)
        return capi_cuda_fail(e, "individual events");
    if (counts[1] != IE_NONE) {
        char msg[96];
        snprintf(msg, sizeof(msg), "'event[%lld]' is invalid.", (long long) counts[1] + 1);
        return fail(SIMINF_GPU_UNDEFINED_EVENT, (long long) counts[1], msg);
    }
    if (counts[2] != IE_NONE) {
        char msg[160];
        snprintf(msg, sizeof(msg),
                 "the search of the individual whose events start at 'event[%lld]' "
                 "gave up after %lld steps.", (long long) counts[2] + 1, max_steps);
        return fail(SIMINF_GPU_ERR_TIMEOUT, (long long) counts[2], msg);
    }
    return 0;
}
