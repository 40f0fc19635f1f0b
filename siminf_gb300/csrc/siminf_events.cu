/*
 * siminf_events.cu -- the ordering of a scheduled-event table on the
 * device: SimInf_events sorts the events by (time, event, select), keeping
 * the input order among equal keys (R/SimInf_events.R:396, `order` is a
 * stable radix sort), before the solver may see them.  For the 1.8e8-event
 * schedules of the headline workload that sort dominates building the
 * model on the host; here it is an LSD radix sort in HBM.
 *
 * Steps, on one stream:
 *  1. time, event and select go to the device; one pass finds their
 *     ranges, so the composite key (time - tmin, event - emin, select -
 *     smin) packs into 32 or 64 bits with no wasted digits;
 *  2. key and input position are sorted by 8-bit digits, least significant
 *     first: per digit, a histogram per tile of 2,048 keys, one exclusive
 *     scan over (digit, tile), and a stable scatter in which each key's
 *     rank within its tile follows input order (rounds of 256 keys, ranks
 *     within a warp from __match_any_sync, across warps from shared
 *     counts);
 *  3. every column of the table is gathered through the sorted positions
 *     and copied back in place.
 *
 * Bytes per pass: read key + position, write key + position (16 B per
 * event for 32-bit keys); the gathers read and write each column once.
 */
#include <chrono>
#include <climits>
#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/siminf_gb300.h"
#include "siminf_capi_internal.h"
#include "siminf_sort.cuh"

using namespace siminf;
using namespace siminf::sortk;

namespace {

/* Minimum and maximum of three int columns; out = {min, max} x 3, set to
 * {INT_MAX, INT_MIN} beforehand. */
__global__ void k_ranges(const int *a, const int *b, const int *c, long long n, int *out)
{
    int mn[3] = {INT_MAX, INT_MAX, INT_MAX}, mx[3] = {INT_MIN, INT_MIN, INT_MIN};
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n;
         i += (long long) gridDim.x * blockDim.x) {
        const int v[3] = {a[i], b[i], c[i]};
#pragma unroll
        for (int k = 0; k < 3; k++) {
            mn[k] = min(mn[k], v[k]);
            mx[k] = max(mx[k], v[k]);
        }
    }
#pragma unroll
    for (int k = 0; k < 3; k++) {
        for (int o = 16; o > 0; o >>= 1) {
            mn[k] = min(mn[k], __shfl_down_sync(0xFFFFFFFFu, mn[k], o));
            mx[k] = max(mx[k], __shfl_down_sync(0xFFFFFFFFu, mx[k], o));
        }
        if ((threadIdx.x & 31) == 0) {
            atomicMin(&out[2 * k], mn[k]);
            atomicMax(&out[2 * k + 1], mx[k]);
        }
    }
}

/* x << b, 0 when b is the key's width (the field then holds only 0). */
template <class K>
__device__ __forceinline__ K shl(K x, int b)
{
    return b >= (int) (8 * sizeof(K)) ? (K) 0 : (K) (x << b);
}

/* Composite keys and input positions. */
template <class K>
__global__ void k_make_keys(const int *time, const int *event, const int *select, long long n,
                            int tmin, int emin, int smin, int be, int bs, K *key,
                            uint32_t *pos)
{
    const long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const K t = (K) ((uint32_t) time[i] - (uint32_t) tmin),
            e = (K) ((uint32_t) event[i] - (uint32_t) emin),
            s = (K) ((uint32_t) select[i] - (uint32_t) smin);
    key[i] = shl<K>(t, be + bs) | shl<K>(e, bs) | s;
    pos[i] = (uint32_t) i;
}

int fail(int code, const char *msg)
{
    capi_set_status(code, -1, -1, -1, 0, 0, msg);
    return code;
}

int bits_of(long long range)
{
    int b = 0;
    while (b < 63 && (1LL << b) <= range)
        b++;
    return b;
}

/* Gather one host column through the sorted positions, in place. */
template <class T>
cudaError_t gather_column(T *host, const uint32_t *pos, long long n, void *a, void *b,
                          cudaStream_t st)
{
    cudaError_t e = cudaMemcpyAsync(a, host, n * sizeof(T), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        k_gather<T><<<(unsigned) ((n + 255) / 256), 256, 0, st>>>((const T *) a, pos, n, (T *) b);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(host, b, n * sizeof(T), cudaMemcpyDeviceToHost, st);
    return e;
}

}  // namespace

extern "C" int siminf_gpu_sort_events(long long len, int *event, int *time, int *node, int *dest,
                                      int *n, double *proportion, int *select, int *shift,
                                      void *cuda_stream, siminf_gpu_reduce_stats *stats)
{
    capi_clear_status();
    const cudaStream_t st = (cudaStream_t) cuda_stream;
    if (len < 0 || len > (long long) UINT32_MAX || (len > 0 && (!event || !time || !node ||
        !dest || !n || !proportion || !select || !shift)))
        return fail(SIMINF_GPU_ERR_INVALID_MODEL, "invalid event table");
    if (len < 2)
        return 0;
    auto t0 = std::chrono::steady_clock::now();
    const long long ntiles = (len + SORT_TILE - 1) / SORT_TILE;
    const long long hn = ntiles * RADIX, hblocks = (hn + SORT_TILE - 1) / SORT_TILE;
    /* buffers: three key columns, keys and positions twice, histogram,
     * block totals, ranges; the column gathers reuse the key buffers */
    int *d_t = nullptr, *d_e = nullptr, *d_s = nullptr, *d_rng = nullptr;
    void *d_k = nullptr, *d_k2 = nullptr;
    uint32_t *d_p = nullptr, *d_p2 = nullptr, *d_hist = nullptr;
    unsigned long long *d_tot = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    const size_t ib = (size_t) len * sizeof(int);
    cudaError_t e = cudaMallocAsync((void **) &d_t, ib, st);
    if (e == cudaSuccess) e = cudaMallocAsync((void **) &d_e, ib, st);
    if (e == cudaSuccess) e = cudaMallocAsync((void **) &d_s, ib, st);
    if (e == cudaSuccess) e = cudaMallocAsync((void **) &d_rng, 6 * sizeof(int), st);
    if (e == cudaSuccess) e = cudaMallocAsync(&d_k, (size_t) len * 8, st);
    if (e == cudaSuccess) e = cudaMallocAsync(&d_k2, (size_t) len * 8, st);
    if (e == cudaSuccess) e = cudaMallocAsync((void **) &d_p, (size_t) len * 4, st);
    if (e == cudaSuccess) e = cudaMallocAsync((void **) &d_p2, (size_t) len * 4, st);
    if (e == cudaSuccess) e = cudaMallocAsync((void **) &d_hist, (size_t) hn * 4, st);
    if (e == cudaSuccess) e = cudaMallocAsync((void **) &d_tot, (size_t) hblocks * 8, st);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_t, time, ib, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_e, event, ib, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_s, select, ib, cudaMemcpyHostToDevice, st);
    int rng[6] = {INT_MAX, INT_MIN, INT_MAX, INT_MIN, INT_MAX, INT_MIN};
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_rng, rng, sizeof(rng), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        cudaEventRecord(e0, st);
        k_ranges<<<152 * 4, 256, 0, st>>>(d_t, d_e, d_s, len, d_rng);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(rng, d_rng, sizeof(rng), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    int bits = 0;
    if (e == cudaSuccess) {
        const int bt = bits_of((long long) rng[1] - rng[0]), be = bits_of((long long) rng[3] - rng[2]),
                  bs = bits_of((long long) rng[5] - rng[4]);
        bits = bt + be + bs;
        if (bits > 64) {
            e = cudaErrorInvalidValue;
        } else if (bits <= 32) {
            k_make_keys<uint32_t><<<(unsigned) ((len + 255) / 256), 256, 0, st>>>(
                d_t, d_e, d_s, len, rng[0], rng[2], rng[4], be, bs, (uint32_t *) d_k, d_p);
            uint32_t *k1 = (uint32_t *) d_k, *k2 = (uint32_t *) d_k2;
            e = radix_sort<uint32_t>(k1, d_p, k2, d_p2, len, bits, d_hist, d_tot, st);
        } else {
            k_make_keys<unsigned long long><<<(unsigned) ((len + 255) / 256), 256, 0, st>>>(
                d_t, d_e, d_s, len, rng[0], rng[2], rng[4], be, bs, (unsigned long long *) d_k,
                d_p);
            unsigned long long *k1 = (unsigned long long *) d_k, *k2 = (unsigned long long *) d_k2;
            e = radix_sort<unsigned long long>(k1, d_p, k2, d_p2, len, bits, d_hist, d_tot, st);
        }
        cudaEventRecord(e1, st);
    }
    /* d_p holds the sorted positions after an even or odd number of
     * passes: radix_sort swapped the pointers it was given */
    if (e == cudaSuccess) e = gather_column<int>(time, d_p, len, d_t, d_k, st);
    if (e == cudaSuccess) e = gather_column<int>(event, d_p, len, d_e, d_k, st);
    if (e == cudaSuccess) e = gather_column<int>(select, d_p, len, d_s, d_k, st);
    if (e == cudaSuccess) e = gather_column<int>(node, d_p, len, d_t, d_k, st);
    if (e == cudaSuccess) e = gather_column<int>(dest, d_p, len, d_e, d_k, st);
    if (e == cudaSuccess) e = gather_column<int>(n, d_p, len, d_s, d_k, st);
    if (e == cudaSuccess) e = gather_column<int>(shift, d_p, len, d_t, d_k, st);
    if (e == cudaSuccess) e = gather_column<double>(proportion, d_p, len, d_k2, d_k, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess && stats) {
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        stats->ms_kernel = ms;
        stats->ms_total = std::chrono::duration<double, std::milli>(
                              std::chrono::steady_clock::now() - t0).count();
        /* ranges and keys read the three columns twice; a pass reads the
         * keys for its histogram, then keys and positions to scatter them */
        const long long kb = bits <= 32 ? 4 : 8, passes = (bits + 7) / 8;
        stats->bytes_read = len * 24 + passes * len * (2 * kb + 4);
        stats->bytes_written = len * (kb + 4) + passes * len * (kb + 4);
    }
    if (e0)
        cudaEventDestroy(e0);
    if (e1)
        cudaEventDestroy(e1);
    for (void *q : {(void *) d_t, (void *) d_e, (void *) d_s, (void *) d_rng, d_k, d_k2,
                    (void *) d_p, (void *) d_p2, (void *) d_hist, (void *) d_tot})
        if (q)
            cudaFreeAsync(q, st);
    const cudaError_t e2 = cudaStreamSynchronize(st);
    if (e == cudaSuccess)
        e = e2;
    if (e == cudaErrorInvalidValue && bits > 64)
        return fail(SIMINF_GPU_ERR_INVALID_MODEL, "event keys span more than 64 bits");
    return e == cudaSuccess ? 0 : capi_cuda_fail(e, "sort events");
}
