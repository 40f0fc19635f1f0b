/*
 * siminf_sort.cuh -- device building blocks shared by the event-table sort
 * (siminf_events.cu) and the device event planner (siminf_schedule.cu):
 * an exclusive scan of 32-bit counts in three kernels and a stable LSD
 * radix sort of (key, position) pairs by 8-bit digits.
 *
 * Radix pass: a histogram per tile of SORT_TILE keys, one exclusive scan
 * over (digit, tile), and a stable scatter in which each key's rank within
 * its tile follows input order (rounds of 256 keys, ranks within a warp
 * from __match_any_sync, across warps from shared counts).
 */
#ifndef SIMINF_SORT_CUH
#define SIMINF_SORT_CUH

#include <cstdint>
#include <utility>

#include <cuda_runtime.h>

namespace siminf {
namespace sortk {

enum { SORT_BLOCK = 256, SORT_ITEMS = 8, SORT_TILE = SORT_BLOCK * SORT_ITEMS, RADIX = 256 };

/* Digit counts of each tile: hist[digit * ntiles + tile]. */
template <class K>
__global__ void __launch_bounds__(SORT_BLOCK) k_radix_hist(const K *key, long long n, int shift,
                                                           uint32_t *hist, long long ntiles)
{
    __shared__ uint32_t cnt[RADIX];
    cnt[threadIdx.x] = 0;
    __syncthreads();
    const long long base = blockIdx.x * (long long) SORT_TILE;
#pragma unroll
    for (int r = 0; r < SORT_ITEMS; r++) {
        const long long i = base + r * SORT_BLOCK + threadIdx.x;
        if (i < n)
            atomicAdd(&cnt[(uint32_t) (key[i] >> shift) & (RADIX - 1)], 1u);
    }
    __syncthreads();
    hist[(long long) threadIdx.x * ntiles + blockIdx.x] = cnt[threadIdx.x];
}

/* Exclusive scan of x[0 .. n) in three kernels: per-block totals, a scan of
 * the totals in one block, and the per-block scans with their bases. */
static __global__ void __launch_bounds__(SORT_BLOCK) k_scan_totals(const uint32_t *x, long long n,
                                                            unsigned long long *tot)
{
    __shared__ unsigned long long sh[SORT_BLOCK / 32];
    const long long base = blockIdx.x * (long long) SORT_TILE;
    unsigned long long s = 0;
#pragma unroll
    for (int r = 0; r < SORT_ITEMS; r++) {
        const long long i = base + r * SORT_BLOCK + threadIdx.x;
        if (i < n)
            s += x[i];
    }
    for (int o = 16; o > 0; o >>= 1)
        s += __shfl_down_sync(0xFFFFFFFFu, s, o);
    if ((threadIdx.x & 31) == 0)
        sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
        for (int w = 0; w < SORT_BLOCK / 32; w++)
            t += sh[w];
        tot[blockIdx.x] = t;
    }
}

/* Exclusive scan of tot[0 .. m) in place, one block. */
static __global__ void __launch_bounds__(1024) k_scan_one_block(unsigned long long *tot, long long m)
{
    __shared__ unsigned long long sh[1024];
    const long long per = (m + 1023) / 1024;
    const long long lo = threadIdx.x * per, hi = min(m, lo + per);
    unsigned long long s = 0;
    for (long long i = lo; i < hi; i++)
        s += tot[i];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const unsigned long long v = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
        __syncthreads();
        sh[threadIdx.x] += v;
        __syncthreads();
    }
    unsigned long long run = sh[threadIdx.x] - s;      /* exclusive base of this thread */
    for (long long i = lo; i < hi; i++) {
        const unsigned long long v = tot[i];
        tot[i] = run;
        run += v;
    }
}

/* The per-block exclusive scans, in the order of the blocked layout (each
 * thread's SORT_ITEMS consecutive entries). */
static __global__ void __launch_bounds__(SORT_BLOCK) k_scan_apply(uint32_t *x, long long n,
                                                           const unsigned long long *tot)
{
    __shared__ unsigned long long sh[SORT_BLOCK];
    const long long base = blockIdx.x * (long long) SORT_TILE + threadIdx.x * SORT_ITEMS;
    uint32_t v[SORT_ITEMS];
    unsigned long long s = 0;
#pragma unroll
    for (int r = 0; r < SORT_ITEMS; r++) {
        v[r] = base + r < n ? x[base + r] : 0;
        s += v[r];
    }
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = 1; o < SORT_BLOCK; o <<= 1) {
        const unsigned long long a = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
        __syncthreads();
        sh[threadIdx.x] += a;
        __syncthreads();
    }
    unsigned long long run = tot[blockIdx.x] + sh[threadIdx.x] - s;
#pragma unroll
    for (int r = 0; r < SORT_ITEMS; r++) {
        if (base + r < n)
            x[base + r] = (uint32_t) run;
        run += v[r];
    }
}

/* Stable scatter of one digit: key i goes to off[digit * ntiles + tile] +
 * (its rank among the tile's keys with that digit, in input order). */
template <class K>
__global__ void __launch_bounds__(SORT_BLOCK) k_radix_scatter(const K *key, const uint32_t *pos,
                                                              long long n, int shift,
                                                              const uint32_t *off,
                                                              long long ntiles, K *key_out,
                                                              uint32_t *pos_out)
{
    __shared__ uint32_t before[RADIX];                    /* keys of earlier rounds */
    __shared__ uint32_t wcnt[SORT_BLOCK / 32][RADIX];     /* the current 256 keys, per warp */
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    before[threadIdx.x] = 0;
    const long long base = blockIdx.x * (long long) SORT_TILE;
    for (int r = 0; r < SORT_ITEMS; r++) {
#pragma unroll
        for (int k = 0; k < SORT_BLOCK / 32; k++)
            wcnt[k][threadIdx.x] = 0;
        __syncthreads();
        const long long i = base + r * SORT_BLOCK + threadIdx.x;
        const bool live = i < n;
        K k = 0;
        uint32_t d = RADIX;                               /* no digit for a lane past n */
        if (live) {
            k = key[i];
            d = (uint32_t) (k >> shift) & (RADIX - 1);
        }
        const unsigned peers = __match_any_sync(0xFFFFFFFFu, d);
        const unsigned lt = peers & ((1u << lane) - 1u);
        if (live && lt == 0)
            wcnt[w][d] = __popc(peers);
        __syncthreads();
        if (live) {
            uint32_t rank = before[d] + __popc(lt);
            for (int k2 = 0; k2 < w; k2++)
                rank += wcnt[k2][d];
            const uint32_t dst = off[(long long) d * ntiles + blockIdx.x] + rank;
            key_out[dst] = k;
            pos_out[dst] = pos[i];
        }
        __syncthreads();
        uint32_t add = 0;
#pragma unroll
        for (int k2 = 0; k2 < SORT_BLOCK / 32; k2++)
            add += wcnt[k2][threadIdx.x];
        before[threadIdx.x] += add;
        __syncthreads();
    }
}

template <class T>
__global__ void k_gather(const T *in, const uint32_t *pos, long long n, T *out)
{
    const long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x;
    if (i < n)
        out[i] = in[pos[i]];
}

/* Exclusive scan of x[0 .. n) in place; tot holds scan_blocks(n) entries. */
inline long long scan_blocks(long long n)
{
    return (n + SORT_TILE - 1) / SORT_TILE;
}

inline cudaError_t exclusive_scan(uint32_t *x, long long n, unsigned long long *tot,
                                  cudaStream_t st)
{
    const long long nb = scan_blocks(n);
    if (nb == 0)
        return cudaSuccess;
    k_scan_totals<<<(unsigned) nb, SORT_BLOCK, 0, st>>>(x, n, tot);
    k_scan_one_block<<<1, 1024, 0, st>>>(tot, nb);
    k_scan_apply<<<(unsigned) nb, SORT_BLOCK, 0, st>>>(x, n, tot);
    return cudaGetLastError();
}

/* Histogram entries and scan totals a radix sort of n keys needs. */
inline long long radix_hist_len(long long n)
{
    return ((n + SORT_TILE - 1) / SORT_TILE) * RADIX;
}

inline long long radix_tot_len(long long n)
{
    return scan_blocks(radix_hist_len(n));
}

/* Stable sort of (key, pos) by the low `bits` bits of key.  The pointers
 * are swapped with the second buffers once per pass: on return key and
 * pos name the sorted arrays. */
template <class K>
cudaError_t radix_sort(K *&key, uint32_t *&pos, K *&key2, uint32_t *&pos2, long long n,
                       int bits, uint32_t *hist, unsigned long long *tot, cudaStream_t st)
{
    const long long ntiles = (n + SORT_TILE - 1) / SORT_TILE;
    const long long hn = ntiles * RADIX, hblocks = (hn + SORT_TILE - 1) / SORT_TILE;
    cudaError_t e = cudaSuccess;
    for (int shift = 0; shift < bits && e == cudaSuccess; shift += 8) {
        k_radix_hist<K><<<(unsigned) ntiles, SORT_BLOCK, 0, st>>>(key, n, shift, hist, ntiles);
        k_scan_totals<<<(unsigned) hblocks, SORT_BLOCK, 0, st>>>(hist, hn, tot);
        k_scan_one_block<<<1, 1024, 0, st>>>(tot, hblocks);
        k_scan_apply<<<(unsigned) hblocks, SORT_BLOCK, 0, st>>>(hist, hn, tot);
        k_radix_scatter<K><<<(unsigned) ntiles, SORT_BLOCK, 0, st>>>(key, pos, n, shift, hist,
                                                                    ntiles, key2, pos2);
        e = cudaGetLastError();
        std::swap(key, key2);
        std::swap(pos, pos2);
    }
    return e;
}

}  // namespace sortk
}  // namespace siminf

#endif
