/*
 * siminf_schedule.cu -- the scheduled events planned on the device, a
 * chunk of days at a time: what the host planner of siminf_capi.cpp
 * (plan_scan, day_levels) does for SimInf_scheduled_events_create
 * (src/solvers/SimInf_solver.c:443-510) and SimInf_split_events
 * (:353-385), with the same results.
 *
 * For the events [lo, lo + m) of days d0 .. d0 + nd - 1 (their columns in
 * staging buffers on the device):
 *  1. classify: order check against the predecessor (time non-decreasing,
 *     E1 before E2 at equal time), largest select and shift, and each
 *     event an E1 event, an external transfer (E2) or a planned failure;
 *  2. compact E1 and E2 in array order (exclusive scans of the flags);
 *  3. E2 levels.  The serial rule -- a transfer goes one wavefront after
 *     every earlier transfer of its day that touched its source and after
 *     every earlier transfer whose source is its destination -- is, with
 *     zero-based levels, the fixed point of Lz[k] = max(Lz[p1] + 1,
 *     Lz[p3] + 1, A[k] + 1, 0): p1 the previous transfer with the same
 *     source, p3 the last earlier transfer whose source is k's destination,
 *     A[k] the largest level of the transfers into k's source since p1
 *     (those before p1 are below Lz[p1] already).  So each transfer feeds
 *     only A of the first later transfer whose source is its destination
 *     ("attach").  A stable radix sort by (day, source) gives p1, p3 and
 *     attach by binary search; then rounds over the whole chunk update
 *     every transfer in place, feeding A by atomic maximum, until nothing
 *     changes.  Iterating from below reaches that fixed point in at most
 *     (deepest level + 1) rounds; a day still changing after MAX_ROUNDS is
 *     left to the host planner;
 *  4. a stable sort by (day, level) puts the transfers in wave order, and
 *     their records are written out with the per-day wave sizes;
 *  5. E1: a stable sort by node gives the chunk's per-node CSR, in the
 *     layout of the whole-run CSR that node_e1 reads.
 */
#include <algorithm>
#include <climits>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/siminf_gb300.h"
#include "siminf_capi_internal.h"
#include "siminf_schedule.h"
#include "siminf_sort.cuh"

namespace siminf {

using namespace sortk;

namespace {

enum { SCHED_BLOCK = 256, LEVEL_BITS = 11, WOUT_CAP = 1 << 16, ROUND_BATCH = 8 };
static_assert((1 << LEVEL_BITS) >= DevScheduler::MAX_ROUNDS, "levels fit the key");
static_assert(2048 == 256 * 8, "tile size of the buffers");

const int E2KIND = SIMINF_GPU_EXTERNAL_TRANSFER_EVENT;

/* The fewest bits that hold values 0 .. n - 1 (at least 1). */
int bits_for(long long n)
{
    int b = 1;
    while (b < 62 && (1LL << b) < n)
        b++;
    return b;
}

unsigned blocks_of(long long n, int threads)
{
    return (unsigned) ((n + threads - 1) / threads);
}

/* Day bounds of a chunk, relative to its first event: day j of the chunk
 * holds events [b[j], b[j + 1]). */
struct DayBounds {
    long long b[DevScheduler::MAX_CHUNK_DAYS + 1];
};

/* 1. Classify.  With classify == false (events past the last day) only the
 * order check and the select / shift maxima run. */
__global__ void __launch_bounds__(SCHED_BLOCK) k_classify(SchedCols c, long long lo, long long m,
                                                          DayBounds db, int nd, int d0, int Nn,
                                                          int nsel, int prev_time,
                                                          int prev_event, int has_prev,
                                                          bool classify, uint8_t *cls,
                                                          uint8_t *jday, uint32_t *f1,
                                                          uint32_t *f2, SchedStatus *st)
{
    const long long t = blockIdx.x * (long long) blockDim.x + threadIdx.x;
    int msel = 0, mshift = 0;
    if (t < m) {
        const int tm = c.time[t], kind = c.event[t];
        int pt = prev_time, pk = prev_event, hp = has_prev;
        if (t > 0) {
            pt = c.time[t - 1];
            pk = c.event[t - 1];
            hp = 1;
        }
        if (hp && (tm < pt || (tm == pt && pk == E2KIND && kind != E2KIND)))
            atomicMin(&st->bad, (unsigned long long) (lo + t));
        msel = c.select[t];
        mshift = c.shift[t];
        if (classify) {
            int j = 0;
            while (j + 1 < nd && t >= db.b[j + 1])
                j++;
            const unsigned node = (unsigned) (c.node[t] - 1), dest = (unsigned) (c.dest[t] - 1),
                           sel = (unsigned) (c.select[t] - 1);
            const bool ok = node < (unsigned) Nn && (unsigned) kind <= 3u && sel < (unsigned) nsel;
            uint8_t k = 0;
            if (ok && kind == E2KIND && dest < (unsigned) Nn) {
                k = 2;
            } else if (ok && kind != E2KIND) {
                k = 1;
            } else {
                int code;
                if (node >= (unsigned) Nn)
                    code = SIMINF_GPU_ERR_NODE_OUT_OF_BOUNDS;
                else if ((unsigned) kind > 3u)
                    code = SIMINF_GPU_UNDEFINED_EVENT;
                else if (sel >= (unsigned) nsel)
                    code = SIMINF_GPU_ERR_SAMPLE_SELECT;
                else
                    code = SIMINF_GPU_ERR_DEST_OUT_OF_BOUNDS;
                const unsigned slot = atomicAdd(&st->n_planned, 1u);
                if (slot < (unsigned) DevScheduler::MAX_PLANNED) {
                    SchedPlanned e;
                    e.day = d0 + j;
                    e.code = code;
                    e.index = (int) (lo + t);
                    e.node = (int) node;
                    e.phase = kind == E2KIND ? (int) PHASE_E2 : (int) PHASE_E1;
                    st->planned[slot] = e;
                }
            }
            cls[t] = k;
            jday[t] = (uint8_t) j;
            f1[t] = k == 1;
            f2[t] = k == 2;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        msel = max(msel, __shfl_down_sync(0xFFFFFFFFu, msel, o));
        mshift = max(mshift, __shfl_down_sync(0xFFFFFFFFu, mshift, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(&st->max_select, msel);
        atomicMax(&st->max_shift, mshift);
    }
}

/* 2. Compaction through the exclusive scans s1, s2 of the flags: per
 * transfer q its (day, source) and (day, destination) keys in compacted
 * order (ks0, kd0), its (day, source) key again with its position for the
 * sort (ka, pa), and its event; per E1 event its node key and position. */
__global__ void __launch_bounds__(SCHED_BLOCK) k_compact(SchedCols c, long long m,
                                                         const uint8_t *cls, const uint8_t *jday,
                                                         const uint32_t *s1, const uint32_t *s2,
                                                         int nb, uint32_t *ks0, uint32_t *kd0,
                                                         uint32_t *idx2, uint32_t *ka,
                                                         uint32_t *pa, uint32_t *ke, uint32_t *pe,
                                                         uint32_t *idx1)
{
    const long long t = blockIdx.x * (long long) blockDim.x + threadIdx.x;
    if (t >= m)
        return;
    const uint8_t k = cls[t];
    if (k == 2) {
        const uint32_t q = s2[t], j = jday[t];
        const uint32_t ks = (j << nb) | (uint32_t) (c.node[t] - 1);
        const uint32_t kd = (j << nb) | (uint32_t) (c.dest[t] - 1);
        ks0[q] = ks;
        kd0[q] = kd;
        ka[q] = ks;
        pa[q] = q;
        idx2[q] = (uint32_t) t;
    } else if (k == 1) {
        const uint32_t q = s1[t];
        ke[q] = (uint32_t) (c.node[t] - 1);
        pe[q] = q;
        idx1[q] = (uint32_t) t;
    }
}

/* Counts and the E2 offset of each day's first transfer:
 * info = {n1, n2, off[0 .. nd]}. */
__global__ void k_totals(long long m, const uint8_t *cls, const uint32_t *s1, const uint32_t *s2,
                         DayBounds db, int nd, long long *info)
{
    if (threadIdx.x != 0 || blockIdx.x != 0)
        return;
    const long long n1 = m > 0 ? (long long) s1[m - 1] + (cls[m - 1] == 1) : 0;
    const long long n2 = m > 0 ? (long long) s2[m - 1] + (cls[m - 1] == 2) : 0;
    info[0] = n1;
    info[1] = n2;
    for (int j = 0; j < nd; j++)
        info[2 + j] = db.b[j] < m ? (long long) s2[db.b[j]] : n2;
    info[2 + nd] = n2;
}

/* First position in a[lo, hi) whose value is not below x. */
__device__ __forceinline__ long long lower_bound_u32(const uint32_t *a, long long lo, long long hi,
                                                     uint32_t x)
{
    while (lo < hi) {
        const long long mid = (lo + hi) >> 1;
        if (a[mid] < x)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

/* First position in a[lo, hi) whose value is above x. */
__device__ __forceinline__ long long upper_bound_u32(const uint32_t *a, long long lo, long long hi,
                                                     uint32_t x)
{
    while (lo < hi) {
        const long long mid = (lo + hi) >> 1;
        if (a[mid] <= x)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

__global__ void __launch_bounds__(SCHED_BLOCK) k_inverse(const uint32_t *perm, long long n,
                                                         uint32_t *inv)
{
    const long long j = blockIdx.x * (long long) blockDim.x + threadIdx.x;
    if (j < n)
        inv[perm[j]] = (uint32_t) j;
}

/* 3a. Links of transfer k.  ks/ps: keys and compacted indices in (day,
 * source) order, inv_s the position of each transfer there.  Within a key
 * the compacted indices increase (a stable sort), so "the last earlier"
 * and "the first later" are binary searches. */
__global__ void __launch_bounds__(SCHED_BLOCK) k_links(long long n, const uint32_t *ks0,
                                                       const uint32_t *kd0, const uint32_t *ks,
                                                       const uint32_t *ps, const uint32_t *inv_s,
                                                       int *p1, int *p3, int *attach)
{
    const long long k = blockIdx.x * (long long) blockDim.x + threadIdx.x;
    if (k >= n)
        return;
    const long long j = inv_s[k];
    const uint32_t my_src = ks0[k], my_dst = kd0[k];
    p1[k] = (j > 0 && ks[j - 1] == my_src) ? (int) ps[j - 1] : -1;
    /* the transfers whose source is k's destination */
    const long long a = lower_bound_u32(ks, 0, n, my_dst);
    const long long b = upper_bound_u32(ks, a, n, my_dst);
    /* the last one before k, and the first one after k */
    const long long r = lower_bound_u32(ps, a, b, (uint32_t) k);
    p3[k] = r > a ? (int) ps[r - 1] : -1;
    const long long r2 = upper_bound_u32(ps, r, b, (uint32_t) k);
    attach[k] = r2 < b ? (int) ps[r2] : -1;
}

/* Every transfer starts at level 0, so each attach target starts at 0. */
__global__ void __launch_bounds__(SCHED_BLOCK) k_attach_init(long long n, const int *attach,
                                                             int *A)
{
    const long long k = blockIdx.x * (long long) blockDim.x + threadIdx.x;
    if (k < n && attach[k] >= 0)
        A[attach[k]] = 0;
}

/* 3b. One round: every transfer's level from its links, in place; a
 * change feeds A of the transfer it attaches to (atomic maximum), sets
 * flags[r] and records r as its day's last changing round.  Every value
 * read is at most the final level, so the in-place rounds still rise to
 * the fixed point, and a round that changes nothing has reached it (A
 * changes only when a level does).  A round returns at once when round
 * r - 1 changed nothing, so rounds queued past convergence cost only their
 * launches. */
__global__ void __launch_bounds__(SCHED_BLOCK) k_round(int r, int *flags, long long n, int nb,
                                                       const uint32_t *ks0, const int *p1,
                                                       const int *p3, const int *attach, int *Lz,
                                                       int *A, int *lastchg)
{
    if (r > 0 && flags[r - 1] == 0)
        return;
    const long long k = blockIdx.x * (long long) blockDim.x + threadIdx.x;
    if (k >= n)
        return;
    const int x1 = p1[k], x3 = p3[k];
    int v = A[k] + 1;                   /* A = -1: nothing attached */
    if (x1 >= 0)
        v = max(v, Lz[x1] + 1);
    if (x3 >= 0)
        v = max(v, Lz[x3] + 1);
    if (v != Lz[k]) {
        Lz[k] = v;
        const int t = attach[k];
        if (t >= 0)
            atomicMax(&A[t], v);
        flags[r] = 1;
        atomicMax(&lastchg[ks0[k] >> nb], r);
    }
}

/* 3'. The levels the host planned, by the transfers' chunk positions
 * (1-based there, zero-based here); flag[0] is set when a transfer has no
 * host level or one deeper than the wave keys hold. */
__global__ void __launch_bounds__(SCHED_BLOCK) k_host_levels(long long n, const uint32_t *idx2,
                                                             const uint32_t *pos_level, int *Lz,
                                                             int *flag)
{
    const long long k = blockIdx.x * (long long) blockDim.x + threadIdx.x;
    if (k >= n)
        return;
    const uint32_t v = pos_level[idx2[k]];
    if (v == 0u || v > (1u << LEVEL_BITS)) {
        flag[0] = 1;
        Lz[k] = 0;
    } else {
        Lz[k] = (int) v - 1;
    }
}

/* Each day's wave sizes (cnt[off[day] + level]) and wave count.  Most
 * transfers share a few low levels, so the lanes of a warp that count
 * into one wave add their number with one atomic, and those of one day
 * their deepest level with one. */
__global__ void __launch_bounds__(SCHED_BLOCK) k_level_counts(long long n, int nb,
                                                              const uint32_t *ks0, const int *Lz,
                                                              const long long *off, int *cnt,
                                                              int *dmax)
{
    const long long k = blockIdx.x * (long long) blockDim.x + threadIdx.x;
    const bool act = k < n;
    const int day = act ? (int) (ks0[k] >> nb) : -1, l = act ? Lz[k] : 0;
    const long long slot = act ? off[day] + l : -1;    /* 0 <= l < the day's transfers */
    const int lane = threadIdx.x & 31;
    const unsigned same_slot = __match_any_sync(0xFFFFFFFFu, (unsigned long long) slot);
    if (act && lane == __ffs(same_slot) - 1)
        atomicAdd(&cnt[slot], __popc(same_slot));
    const unsigned same_day = __match_any_sync(0xFFFFFFFFu, day);
    const int deepest = (int) __reduce_max_sync(same_day, (unsigned) (l + 1));
    if (act && lane == __ffs(same_day) - 1)
        atomicMax(&dmax[day], deepest);
}

/* Days whose levels still changed in the last round allowed: 1 (left to
 * the host planner), others 0; in place over lastchg. */
__global__ void k_deep_days(int nd, int *lastchg, int last_round)
{
    const int j = threadIdx.x;
    if (j < nd)
        lastchg[j] = lastchg[j] >= last_round ? 1 : 0;
}

/* 4. Keys of the wave order: (day, zero-based level). */
__global__ void __launch_bounds__(SCHED_BLOCK) k_level_keys(long long n, int nb,
                                                            const uint32_t *ks0, const int *L,
                                                            uint32_t *key, uint32_t *pos)
{
    const long long k = blockIdx.x * (long long) blockDim.x + threadIdx.x;
    if (k >= n)
        return;
    key[k] = ((ks0[k] >> nb) << LEVEL_BITS) | ((uint32_t) L[k] & ((1u << LEVEL_BITS) - 1u));
    pos[k] = (uint32_t) k;
}

/* The transfers' records in wave order (and their waves by event). */
__global__ void __launch_bounds__(SCHED_BLOCK) k_e2_records(long long n, SchedCols c, long long lo,
                                                            const uint32_t *pw,
                                                            const uint32_t *idx2, const int *L,
                                                            E2Rec *out, int *wave_out)
{
    const long long w = blockIdx.x * (long long) blockDim.x + threadIdx.x;
    if (w >= n)
        return;
    const uint32_t k = pw[w], t = idx2[k];
    E2Rec e;
    e.src = c.node[t] - 1;
    e.dst = c.dest[t] - 1;
    e.n = c.n[t];
    e.select = c.select[t] - 1;
    e.shift = c.shift[t] - 1;
    e.index = (int) (lo + t);
    e.proportion = c.proportion[t];
    out[w] = e;
    if (wave_out)
        wave_out[lo + t] = L[k];
}

/* The per-day wave sizes, packed for the host: out = {dmax[0 .. nd),
 * deep[0 .. nd), then each day's dmax sizes}; out[2 nd] .. are the sizes,
 * or out holds -1 at index 2 nd when they do not fit. */
__global__ void k_wave_sizes(int nd, const long long *off, const int *dmax, const int *deep,
                             const int *cnt, int *out)
{
    if (blockIdx.x != 0)
        return;
    long long total = 0;
    for (int j = 0; j < nd; j++)
        total += dmax[j];
    const bool fits = 2 * nd + total <= WOUT_CAP;
    if (threadIdx.x == 0) {
        for (int j = 0; j < nd; j++) {
            out[j] = dmax[j];
            out[nd + j] = deep[j];
        }
        if (!fits)
            out[2 * nd] = -1;
    }
    if (!fits)
        return;
    long long base = 2 * nd;
    for (int j = 0; j < nd; j++) {
        for (int l = threadIdx.x; l < dmax[j]; l += blockDim.x)
            out[base + l] = cnt[off[j] + l];
        base += dmax[j];
    }
}

/* 5. E1 records in node order and the per-node offsets. */
__global__ void __launch_bounds__(SCHED_BLOCK) k_e1_records(long long n, SchedCols c, long long lo,
                                                            int d0, const uint8_t *jday,
                                                            const uint32_t *pe,
                                                            const uint32_t *idx1, E1Rec *out)
{
    const long long p = blockIdx.x * (long long) blockDim.x + threadIdx.x;
    if (p >= n)
        return;
    const uint32_t t = idx1[pe[p]];
    E1Rec e;
    e.day = d0 + jday[t];
    e.kind = c.event[t];
    e.n = c.n[t];
    e.select = c.select[t] - 1;
    e.shift = c.shift[t] - 1;
    e.index = (int) (lo + t);
    e.proportion = c.proportion[t];
    out[p] = e;
}

__global__ void __launch_bounds__(SCHED_BLOCK) k_e1_ptr(long long n1, const uint32_t *ke, int Nn,
                                                        int *ptr)
{
    const long long x = blockIdx.x * (long long) blockDim.x + threadIdx.x;
    if (x <= Nn)
        ptr[x] = (int) lower_bound_u32(ke, 0, n1, (uint32_t) x);
}

__global__ void __launch_bounds__(SCHED_BLOCK) k_iota(uint32_t *p, long long n)
{
    const long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x;
    if (i < n)
        p[i] = (uint32_t) i;
}

__global__ void __launch_bounds__(SCHED_BLOCK) k_gather_e1(const E1Rec *in, const uint32_t *pos,
                                                           long long n, E1Rec *out)
{
    const long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x;
    if (i < n)
        out[i] = in[pos[i]];
}

}  // namespace

DevScheduler::~DevScheduler()
{
    if (h_info_)
        cudaFreeHost(h_info_);
    if (h_wout_)
        cudaFreeHost(h_wout_);
    if (h_status_)
        cudaFreeHost(h_status_);
    if (h_flag_)
        cudaFreeHost(h_flag_);
    for (void *p : bufs_)
        cudaFree(p);
}

template <class T>
cudaError_t DevScheduler::alloc(T **p, size_t n)
{
    *p = nullptr;
    const cudaError_t e = cudaMalloc((void **) p, (n ? n : 1) * sizeof(T));
    if (e == cudaSuccess)
        bufs_.push_back(*p);
    return e;
}

cudaError_t DevScheduler::init(long long max_events, int Nn, int nsel, cudaStream_t st)
{
    st_ = st;
    cap_ = std::max(1LL, max_events);
    Nn_ = Nn;
    nsel_ = nsel;
    nb_ = bits_for(Nn);
    /* keys: day (4 bits for 16 days) and node, or day and level, in 32 bits */
    if (nb_ + 4 > 32 || cap_ >= (1LL << 32))
        return cudaErrorInvalidValue;
    const size_t m = (size_t) cap_;
    cudaError_t e = cudaSuccess;
#define SCHED_ALLOC(p, n) \
    if (e == cudaSuccess) \
        e = alloc(&(p), (n))
    SCHED_ALLOC(time, m);
    SCHED_ALLOC(event, m);
    SCHED_ALLOC(node, m);
    SCHED_ALLOC(dest, m);
    SCHED_ALLOC(n, m);
    SCHED_ALLOC(select, m);
    SCHED_ALLOC(shift, m);
    SCHED_ALLOC(proportion, m);
    SCHED_ALLOC(cls_, m);
    SCHED_ALLOC(jday_, m);
    SCHED_ALLOC(s1_, m);
    SCHED_ALLOC(s2_, m);
    SCHED_ALLOC(ks0_, m);
    SCHED_ALLOC(kd0_, m);
    SCHED_ALLOC(idx2_, m);
    SCHED_ALLOC(idx1_, m);
    SCHED_ALLOC(ka_, m);
    SCHED_ALLOC(pa_, m);
    SCHED_ALLOC(kb_, m);
    SCHED_ALLOC(pb_, m);
    SCHED_ALLOC(ke_, m);
    SCHED_ALLOC(pe_, m);
    SCHED_ALLOC(ke2_, m);
    SCHED_ALLOC(pe2_, m);
    SCHED_ALLOC(inv_, m);
    SCHED_ALLOC(p1_, m);
    SCHED_ALLOC(p3_, m);
    SCHED_ALLOC(attach_, m);
    SCHED_ALLOC(L_, m);
    SCHED_ALLOC(A_, m);
    SCHED_ALLOC(cnt_, m);
    SCHED_ALLOC(hist_, (size_t) std::max(radix_hist_len(cap_), scan_blocks(cap_) + 1));
    SCHED_ALLOC(tot_, (size_t) std::max(radix_tot_len(cap_), scan_blocks(cap_)) + 1);
    SCHED_ALLOC(flags_, (size_t) MAX_ROUNDS);
    SCHED_ALLOC(dmax_, (size_t) MAX_CHUNK_DAYS);
    SCHED_ALLOC(deep_, (size_t) MAX_CHUNK_DAYS);
    SCHED_ALLOC(info_, (size_t) MAX_CHUNK_DAYS + 3);
    SCHED_ALLOC(wout_, (size_t) WOUT_CAP);
#undef SCHED_ALLOC
    if (e == cudaSuccess)
        e = cudaMalloc((void **) &status_,
                       sizeof(SchedStatus) + (MAX_PLANNED - 1) * sizeof(SchedPlanned));
    if (e == cudaSuccess)
        bufs_.push_back(status_);
    if (e == cudaSuccess)
        e = cudaMallocHost((void **) &h_info_, (MAX_CHUNK_DAYS + 3) * sizeof(long long));
    if (e == cudaSuccess)
        e = cudaMallocHost((void **) &h_wout_, WOUT_CAP * sizeof(int));
    if (e == cudaSuccess)
        e = cudaMallocHost((void **) &h_status_, sizeof(SchedStatus));
    if (e == cudaSuccess)
        e = cudaMallocHost((void **) &h_flag_, sizeof(int));
    if (e == cudaSuccess) {
        SchedStatus s0{};
        s0.bad = ~0ULL;
        e = cudaMemcpyAsync(status_, &s0, sizeof(SchedStatus), cudaMemcpyHostToDevice, st_);
    }
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(st_);
    return e;
}

cudaError_t DevScheduler::check_tail(long long lo, long long m, int prev_time, int prev_event,
                                     bool has_prev)
{
    if (m <= 0)
        return cudaSuccess;
    if (m > cap_)
        return cudaErrorInvalidValue;
    SchedCols c{time, event, node, dest, n, select, shift, proportion};
    DayBounds db{};
    k_classify<<<blocks_of(m, SCHED_BLOCK), SCHED_BLOCK, 0, st_>>>(
        c, lo, m, db, 1, 0, Nn_, nsel_, prev_time, prev_event, has_prev ? 1 : 0, false, cls_,
        jday_, s1_, s2_, status_);
    return cudaGetLastError();
}

int DevScheduler::max_host_level()
{
    return 1 << LEVEL_BITS;
}

cudaError_t DevScheduler::plan_chunk(long long lo, long long m, int d0, int nd,
                                     const long long *bounds, int prev_time, int prev_event,
                                     bool has_prev, E2Rec *e2_out, E1Rec *e1_out, int *e1_ptr,
                                     int *wave_out, SchedChunk &out, uint32_t *e1_node_out,
                                     const uint32_t *pos_level)
{
    if (m > cap_ || m < 0 || nd < 1 || nd > MAX_CHUNK_DAYS)
        return cudaErrorInvalidValue;
    DayBounds db{};
    for (int j = 0; j <= nd; j++) {
        db.b[j] = bounds[j];
        if (bounds[j] < 0 || bounds[j] > m || (j > 0 && bounds[j] < bounds[j - 1]))
            return cudaErrorInvalidValue;
    }
    if (bounds[nd] != m)
        return cudaErrorInvalidValue;
    SchedCols c{time, event, node, dest, n, select, shift, proportion};
    cudaError_t e = cudaSuccess;
    const unsigned gm = blocks_of(m, SCHED_BLOCK);
    /* SIMINF_SCHED_PROFILE=1: each phase's device time on stderr */
    static const bool prof = getenv("SIMINF_SCHED_PROFILE") && getenv("SIMINF_SCHED_PROFILE")[0] == '1';
    cudaEvent_t pev[8] = {};
    int npev = 0;
    auto mark = [&]() {
        if (prof && npev < 8 && cudaEventCreate(&pev[npev]) == cudaSuccess)
            cudaEventRecord(pev[npev++], st_);
    };
    mark();
    if (m > 0) {
        k_classify<<<gm, SCHED_BLOCK, 0, st_>>>(c, lo, m, db, nd, d0, Nn_, nsel_, prev_time,
                                                prev_event, has_prev ? 1 : 0, true, cls_, jday_,
                                                s1_, s2_, status_);
        e = cudaGetLastError();
        if (e == cudaSuccess)
            e = exclusive_scan(s1_, m, tot_, st_);
        if (e == cudaSuccess)
            e = exclusive_scan(s2_, m, tot_, st_);
        if (e == cudaSuccess) {
            k_compact<<<gm, SCHED_BLOCK, 0, st_>>>(c, m, cls_, jday_, s1_, s2_, nb_, ks0_, kd0_,
                                                   idx2_, ka_, pa_, ke_, pe_, idx1_);
            e = cudaGetLastError();
        }
    }
    if (e == cudaSuccess) {
        k_totals<<<1, 32, 0, st_>>>(m, cls_, s1_, s2_, db, nd, info_);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(h_info_, info_, (nd + 3) * sizeof(long long), cudaMemcpyDeviceToHost,
                            st_);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess)
        return e;
    out.n1 = h_info_[0];
    out.n2 = h_info_[1];
    out.off.assign(h_info_ + 2, h_info_ + 3 + nd);
    out.waves.assign(nd, std::vector<long long>());
    out.deep.clear();
    const long long n1 = out.n1, n2 = out.n2;
    const int jb = bits_for(nd);

    mark();
    /* the host's levels, if it planned them: no links, no rounds */
    bool host = pos_level != nullptr && n2 > 0;
    if (host) {
        const unsigned g2 = blocks_of(n2, SCHED_BLOCK);
        e = cudaMemsetAsync(flags_, 0, sizeof(int), st_);
        if (e == cudaSuccess) {
            k_host_levels<<<g2, SCHED_BLOCK, 0, st_>>>(n2, idx2_, pos_level, L_, flags_);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(h_flag_, flags_, sizeof(int), cudaMemcpyDeviceToHost, st_);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(st_);
        if (e != cudaSuccess)
            return e;
        host = *h_flag_ == 0;
    }
    if (n2 > 0 && host) {
        /* every day within the rounds' depth: none left to the host */
        const unsigned g2 = blocks_of(n2, SCHED_BLOCK);
        e = cudaMemsetAsync(cnt_, 0, n2 * sizeof(int), st_);
        if (e == cudaSuccess)
            e = cudaMemsetAsync(dmax_, 0, MAX_CHUNK_DAYS * sizeof(int), st_);
        if (e == cudaSuccess)
            e = cudaMemsetAsync(deep_, 0, MAX_CHUNK_DAYS * sizeof(int), st_);
        if (e == cudaSuccess) {
            k_level_counts<<<g2, SCHED_BLOCK, 0, st_>>>(n2, nb_, ks0_, L_, info_ + 2, cnt_, dmax_);
            e = cudaGetLastError();
        }
    }
    if (n2 > 0) {
        uint32_t *ks = ka_, *ps = pa_, *ks2 = kb_, *ps2 = pb_;
        if (n2 > 1 && !host)
            e = radix_sort<uint32_t>(ks, ps, ks2, ps2, n2, jb + nb_, hist_, tot_, st_);
        const unsigned g2 = blocks_of(n2, SCHED_BLOCK);
        mark();
        if (!host) {
            if (e == cudaSuccess) {
                k_inverse<<<g2, SCHED_BLOCK, 0, st_>>>(ps, n2, inv_);
                k_links<<<g2, SCHED_BLOCK, 0, st_>>>(n2, ks0_, kd0_, ks, ps, inv_, p1_, p3_, attach_);
                e = cudaGetLastError();
            }
            if (e == cudaSuccess)
                e = cudaMemsetAsync(cnt_, 0, n2 * sizeof(int), st_);
            if (e == cudaSuccess)
                e = cudaMemsetAsync(dmax_, 0, MAX_CHUNK_DAYS * sizeof(int), st_);
            if (e == cudaSuccess)
                e = cudaMemsetAsync(deep_, 0xFF, MAX_CHUNK_DAYS * sizeof(int), st_);  /* lastchg = -1 */
            if (e == cudaSuccess)
                e = cudaMemsetAsync(L_, 0, n2 * sizeof(int), st_);
            if (e == cudaSuccess)
                e = cudaMemsetAsync(A_, 0xFF, n2 * sizeof(int), st_);                 /* A = -1 */
            if (e == cudaSuccess)
                e = cudaMemsetAsync(flags_, 0, MAX_ROUNDS * sizeof(int), st_);
            if (e == cudaSuccess) {
                k_attach_init<<<g2, SCHED_BLOCK, 0, st_>>>(n2, attach_, A_);
                e = cudaGetLastError();
            }
            mark();
            /* rounds in batches; the host looks at the last round's flag after
             * each batch */
            int r = 0;
            while (e == cudaSuccess && r < MAX_ROUNDS) {
                for (int b = 0; b < ROUND_BATCH && r < MAX_ROUNDS && e == cudaSuccess; b++, r++) {
                    k_round<<<g2, SCHED_BLOCK, 0, st_>>>(r, flags_, n2, nb_, ks0_, p1_, p3_, attach_, L_,
                                                         A_, deep_);
                    e = cudaGetLastError();
                }
                if (e == cudaSuccess)
                    e = cudaMemcpyAsync(h_flag_, flags_ + r - 1, sizeof(int), cudaMemcpyDeviceToHost,
                                        st_);
                if (e == cudaSuccess)
                    e = cudaStreamSynchronize(st_);
                if (e != cudaSuccess || !*h_flag_)
                    break;
            }
            if (e == cudaSuccess) {
                k_level_counts<<<g2, SCHED_BLOCK, 0, st_>>>(n2, nb_, ks0_, L_, info_ + 2, cnt_, dmax_);
                k_deep_days<<<1, 32, 0, st_>>>(nd, deep_, MAX_ROUNDS - 1);
                e = cudaGetLastError();
            }
        }
        mark();
        /* the wave order: the (day, source) sort's buffers are free now */
        uint32_t *kw = ks == ka_ ? kb_ : ka_, *pw = ps == pa_ ? pb_ : pa_;
        uint32_t *kw2 = ks, *pw2 = ps;
        if (e == cudaSuccess) {
            k_level_keys<<<g2, SCHED_BLOCK, 0, st_>>>(n2, nb_, ks0_, L_, kw, pw);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess && n2 > 1)
            e = radix_sort<uint32_t>(kw, pw, kw2, pw2, n2, jb + LEVEL_BITS, hist_, tot_, st_);
        if (e == cudaSuccess) {
            k_e2_records<<<g2, SCHED_BLOCK, 0, st_>>>(n2, c, lo, pw, idx2_, L_, e2_out, wave_out);
            k_wave_sizes<<<1, 256, 0, st_>>>(nd, info_ + 2, dmax_, deep_, cnt_, wout_);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(h_wout_, wout_, WOUT_CAP * sizeof(int), cudaMemcpyDeviceToHost,
                                st_);
    }
    mark();
    if (e == cudaSuccess && n1 > 0) {
        uint32_t *ke = ke_, *pe = pe_, *ke2 = ke2_, *pe2 = pe2_;
        if (n1 > 1)
            e = radix_sort<uint32_t>(ke, pe, ke2, pe2, n1, nb_, hist_, tot_, st_);
        if (e == cudaSuccess) {
            k_e1_records<<<blocks_of(n1, SCHED_BLOCK), SCHED_BLOCK, 0, st_>>>(n1, c, lo, d0, jday_,
                                                                             pe, idx1_, e1_out);
            k_e1_ptr<<<blocks_of((long long) Nn_ + 1, SCHED_BLOCK), SCHED_BLOCK, 0, st_>>>(
                n1, ke, Nn_, e1_ptr);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess && e1_node_out)
            e = cudaMemcpyAsync(e1_node_out, ke, n1 * sizeof(uint32_t), cudaMemcpyDeviceToDevice,
                                st_);
    } else if (e == cudaSuccess) {
        e = cudaMemsetAsync(e1_ptr, 0, ((size_t) Nn_ + 1) * sizeof(int), st_);
    }
    mark();
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(h_status_, status_, sizeof(SchedStatus), cudaMemcpyDeviceToHost, st_);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(st_);
    if (prof) {
        fprintf(stderr, "sched chunk d0=%d m=%lld n2=%lld ms:", d0, m, out.n2);
        for (int k = 1; k < npev; k++) {
            float ms = 0;
            cudaEventElapsedTime(&ms, pev[k - 1], pev[k]);
            fprintf(stderr, " %.3f", ms);
        }
        fprintf(stderr, "\n");
    }
    for (int k = 0; k < npev; k++)
        cudaEventDestroy(pev[k]);
    if (e != cudaSuccess)
        return e;
    out.bad = h_status_->bad;
    out.max_select = h_status_->max_select;
    out.max_shift = h_status_->max_shift;
    if (n2 == 0)
        return cudaSuccess;

    /* the per-day wave sizes */
    std::vector<int> sizes;
    const int *w = h_wout_;
    if (w[2 * nd] == -1) {
        /* more sizes than the packed buffer holds: copy the whole counts */
        sizes.resize((size_t) n2);
        e = cudaMemcpy(sizes.data(), cnt_, n2 * sizeof(int), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess)
            return e;
    }
    long long base = 2 * nd;
    for (int j = 0; j < nd; j++) {
        const int dm = w[j];
        if (w[nd + j]) {
            out.deep.push_back(j);
        } else {
            std::vector<long long> &v = out.waves[j];
            v.resize(dm);
            for (int l = 0; l < dm; l++)
                v[l] = sizes.empty() ? w[base + l] : sizes[out.off[j] - out.off[0] + l];
        }
        base += dm;
    }
    return cudaSuccess;
}

cudaError_t e1_ptr_from_keys(const uint32_t *keys, long long n, int Nn, int *ptr,
                             cudaStream_t st)
{
    k_e1_ptr<<<blocks_of((long long) Nn + 1, SCHED_BLOCK), SCHED_BLOCK, 0, st>>>(n, keys, Nn, ptr);
    return cudaGetLastError();
}

cudaError_t DevScheduler::merge_e1(const E1Rec *in, const uint32_t *nodes, long long n,
                                   E1Rec *out, int *ptr)
{
    if (n <= 0)
        return cudaMemsetAsync(ptr, 0, ((size_t) Nn_ + 1) * sizeof(int), st_);
    uint32_t *k = nullptr, *p = nullptr, *k2 = nullptr, *p2 = nullptr, *hist = nullptr;
    unsigned long long *tot = nullptr;
    cudaError_t e = cudaMallocAsync((void **) &k, n * sizeof(uint32_t), st_);
    if (e == cudaSuccess) e = cudaMallocAsync((void **) &p, n * sizeof(uint32_t), st_);
    if (e == cudaSuccess) e = cudaMallocAsync((void **) &k2, n * sizeof(uint32_t), st_);
    if (e == cudaSuccess) e = cudaMallocAsync((void **) &p2, n * sizeof(uint32_t), st_);
    if (e == cudaSuccess)
        e = cudaMallocAsync((void **) &hist, radix_hist_len(n) * sizeof(uint32_t), st_);
    if (e == cudaSuccess)
        e = cudaMallocAsync((void **) &tot, (radix_tot_len(n) + 1) * sizeof(unsigned long long),
                            st_);
    uint32_t *kk = k, *pp = p, *kk2 = k2, *pp2 = p2;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(k, nodes, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st_);
    if (e == cudaSuccess) {
        k_iota<<<blocks_of(n, SCHED_BLOCK), SCHED_BLOCK, 0, st_>>>(p, n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && n > 1)
        e = radix_sort<uint32_t>(kk, pp, kk2, pp2, n, nb_, hist, tot, st_);
    if (e == cudaSuccess) {
        k_gather_e1<<<blocks_of(n, SCHED_BLOCK), SCHED_BLOCK, 0, st_>>>(in, pp, n, out);
        k_e1_ptr<<<blocks_of((long long) Nn_ + 1, SCHED_BLOCK), SCHED_BLOCK, 0, st_>>>(n, kk, Nn_,
                                                                                    ptr);
        e = cudaGetLastError();
    }
    for (void *q : {(void *) k, (void *) p, (void *) k2, (void *) p2, (void *) hist, (void *) tot})
        if (q)
            cudaFreeAsync(q, st_);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(st_);
    return e;
}

cudaError_t DevScheduler::status(unsigned long long &bad, int &max_select, int &max_shift,
                                 std::vector<SchedPlanned> &planned)
{
    SchedStatus s;
    cudaError_t e = cudaMemcpyAsync(&s, status_, sizeof(SchedStatus), cudaMemcpyDeviceToHost, st_);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess)
        return e;
    bad = s.bad;
    max_select = s.max_select;
    max_shift = s.max_shift;
    const unsigned np = std::min(s.n_planned, (unsigned) MAX_PLANNED);
    planned.resize(np);
    if (np)
        e = cudaMemcpy(planned.data(), (const char *) status_ + offsetof(SchedStatus, planned),
                       np * sizeof(SchedPlanned), cudaMemcpyDeviceToHost);
    return e;
}

}  // namespace siminf

namespace siminf {

/* Input range of each day's events, [lo[d], hi[d]): the times after the
 * previous day's start up to this day's (day 0: every time up to its
 * start).  Returns false when the ranges do not tile the table in order,
 * which only an unsorted table can make happen. */
bool event_day_ranges(const siminf_gpu_solver_args *a, const std::vector<DayInfo> &days,
                      std::vector<long long> &lo, std::vector<long long> &hi)
{
    const long long len = a->len;
    const int nd = (int) days.size();
    auto first_after = [&](double x) {
        long long l = 0, h = len;
        while (l < h) {
            const long long mid = (l + h) / 2;
            if ((double) a->time[mid] <= x)
                l = mid + 1;
            else
                h = mid;
        }
        return l;
    };
    lo.assign(nd, 0);
    hi.assign(nd, 0);
    for (int d = 0; d < nd; d++) {
        lo[d] = d == 0 ? 0 : hi[d - 1];
        hi[d] = first_after(days[d].tt);
        if (hi[d] < lo[d])
            return false;
    }
    return true;
}

}  // namespace siminf

using namespace siminf;

namespace {

template <class T>
cudaError_t stage(T *dst, const T *src, long long lo, long long m, cudaStream_t st)
{
    if (m <= 0)
        return cudaSuccess;
    return cudaMemcpyAsync(dst, src + lo, (size_t) m * sizeof(T), cudaMemcpyHostToDevice, st);
}

/* Copy the columns of events [lo, lo + m) into the scheduler's staging
 * buffers (only time, event, select and shift for the order check). */
cudaError_t stage_chunk(DevScheduler &s, const siminf_gpu_solver_args *a, long long lo,
                        long long m, bool all, cudaStream_t st)
{
    cudaError_t e = stage(s.time, a->time, lo, m, st);
    if (e == cudaSuccess) e = stage(s.event, a->event, lo, m, st);
    if (e == cudaSuccess) e = stage(s.select, a->select, lo, m, st);
    if (e == cudaSuccess) e = stage(s.shift, a->shift, lo, m, st);
    if (all) {
        if (e == cudaSuccess) e = stage(s.node, a->node, lo, m, st);
        if (e == cudaSuccess) e = stage(s.dest, a->dest, lo, m, st);
        if (e == cudaSuccess) e = stage(s.n, a->n, lo, m, st);
        if (e == cudaSuccess) e = stage(s.proportion, a->proportion, lo, m, st);
    }
    return e;
}

}  // namespace

extern "C" int siminf_gpu_schedule_device(const siminf_gpu_solver_args *a, int *days, int *waves,
                                          long long *e1_events, long long *e2_events, int *wave)
{
    capi_clear_status();
    if (!a || !a->tspan || a->tlen < 1 || a->Nn < 1 || a->len < 0)
        return SIMINF_GPU_ERR_INVALID_MODEL;
    if (a->len > 0 && (!a->event || !a->time || !a->node || !a->dest || !a->n ||
                       !a->proportion || !a->select || !a->shift))
        return SIMINF_GPU_ERR_INVALID_MODEL;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        capi_set_status(SIMINF_GPU_ERR_NO_DEVICE, -1, -1, -1, 0, 0, "no CUDA device");
        return SIMINF_GPU_ERR_NO_DEVICE;
    }
    std::vector<DayInfo> dv;
    int rc = plan_days(a->tspan, a->tlen, dv);
    if (rc)
        return rc;
    const int ndays = (int) dv.size();
    std::vector<long long> lo, hi;
    if (!event_day_ranges(a, dv, lo, hi))
        /* out of order: the host planner finds and reports the first
         * offending event */
        return siminf_gpu_schedule(a, days, waves, e1_events, e2_events, wave);
    const long long len = a->len, tail_lo = ndays > 0 ? hi[ndays - 1] : 0;
    const int CH = 8;
    long long cap = std::max(1LL, len - tail_lo);
    for (int d0 = 0; d0 < ndays; d0 += CH) {
        const int d1 = std::min(ndays, d0 + CH);
        cap = std::max(cap, hi[d1 - 1] - lo[d0]);
    }
    const int nsel = (a->len > 0 && a->jcE) ? INT_MAX : 0;
    cudaStream_t st = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    E2Rec *d_e2 = nullptr;
    E1Rec *d_e1 = nullptr;
    int *d_ptr = nullptr, *d_wave = nullptr;
    long long n1 = 0, n2 = 0, nwaves = 0;
    std::vector<std::pair<long long, long long>> deep;     /* input ranges of deep days */
    {
        DevScheduler sch;
        if (e == cudaSuccess) e = sch.init(cap, a->Nn, nsel, st);
        if (e == cudaSuccess) e = cudaMalloc((void **) &d_e2, (size_t) cap * sizeof(E2Rec));
        if (e == cudaSuccess) e = cudaMalloc((void **) &d_e1, (size_t) cap * sizeof(E1Rec));
        if (e == cudaSuccess) e = cudaMalloc((void **) &d_ptr, ((size_t) a->Nn + 1) * sizeof(int));
        if (e == cudaSuccess) e = cudaMalloc((void **) &d_wave, (size_t) std::max(1LL, len) * sizeof(int));
        if (e == cudaSuccess) e = cudaMemsetAsync(d_wave, 0xFF, (size_t) std::max(1LL, len) * sizeof(int), st);
        for (int d0 = 0; d0 < ndays && e == cudaSuccess; d0 += CH) {
            const int d1 = std::min(ndays, d0 + CH), nd = d1 - d0;
            const long long l0 = lo[d0], m = hi[d1 - 1] - l0;
            long long bounds[DevScheduler::MAX_CHUNK_DAYS + 1];
            for (int j = 0; j < nd; j++)
                bounds[j] = lo[d0 + j] - l0;
            bounds[nd] = m;
            e = stage_chunk(sch, a, l0, m, true, st);
            SchedChunk out;
            if (e == cudaSuccess)
                e = sch.plan_chunk(l0, m, d0, nd, bounds, l0 > 0 ? a->time[l0 - 1] : 0,
                                   l0 > 0 ? a->event[l0 - 1] : 0, l0 > 0, d_e2, d_e1, d_ptr,
                                   d_wave, out);
            if (e != cudaSuccess)
                break;
            n1 += out.n1;
            n2 += out.n2;
            for (int j = 0; j < nd; j++)
                nwaves += (long long) out.waves[j].size();
            for (int j : out.deep)
                deep.push_back({lo[d0 + j], hi[d0 + j]});
        }
        if (e == cudaSuccess && len > tail_lo) {
            e = stage_chunk(sch, a, tail_lo, len - tail_lo, false, st);
            if (e == cudaSuccess)
                e = sch.check_tail(tail_lo, len - tail_lo, tail_lo > 0 ? a->time[tail_lo - 1] : 0,
                                   tail_lo > 0 ? a->event[tail_lo - 1] : 0, tail_lo > 0);
        }
        unsigned long long bad = ~0ULL;
        int msel = 0, mshift = 0;
        std::vector<SchedPlanned> planned;
        if (e == cudaSuccess)
            e = sch.status(bad, msel, mshift, planned);
        if (e == cudaSuccess && bad != ~0ULL) {
            char msg[200];
            snprintf(msg, sizeof(msg), "event %lld (time %d) breaks the (time, E1 before E2) order",
                     (long long) bad + 1, a->time[bad]);
            capi_set_status(SIMINF_GPU_ERR_EVENTS_UNSORTED, -1, -1, (int) bad, a->time[bad], 0, msg);
            rc = SIMINF_GPU_ERR_EVENTS_UNSORTED;
        }
        if (e == cudaSuccess && !rc && wave)
            e = cudaMemcpyAsync(wave, d_wave, (size_t) len * sizeof(int), cudaMemcpyDeviceToHost,
                                st);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(st);
    }
    if (e == cudaSuccess && !rc) {
        /* days too deep for the rounds: the host planner's levels */
        for (auto &r : deep) {
            std::vector<E2Rec> recs((size_t) (r.second - r.first) + 1);
            std::vector<long long> wv;
            host_day_waves(a->event, a->node, a->dest, a->n, a->proportion, a->select, a->shift,
                           r.first, r.second, a->Nn, nsel, recs.data(), wv);
            nwaves += (long long) wv.size();
            long long k = 0;
            for (size_t w = 0; w < wv.size(); w++)
                for (long long c = 0; c < wv[w]; c++, k++)
                    if (wave)
                        wave[recs[k].index] = (int) w;
        }
    }
    for (void *q : {(void *) d_e2, (void *) d_e1, (void *) d_ptr, (void *) d_wave})
        if (q)
            cudaFree(q);
    if (st)
        cudaStreamDestroy(st);
    if (e != cudaSuccess)
        return capi_cuda_fail(e, "device schedule");
    if (rc)
        return rc;
    if (days)
        *days = ndays;
    if (waves)
        *waves = (int) nwaves;
    if (e1_events)
        *e1_events = n1;
    if (e2_events)
        *e2_events = n2;
    return 0;
}
