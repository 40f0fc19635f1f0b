/*
 * siminf_kernels.cuh -- the GB300 kernels of the ssm/mssm solver, as
 * templates over the device model, and their launchers.  siminf_kernels.cu
 * instantiates them for the models the library ships; a model compiled
 * from generated C code (siminf_gb300/devmodel.py) instantiates them in a
 * library of its own, with the same launcher table.
 *
 * One thread owns one (replicate, node) pair g for the node phases:
 *   k_init       rate initialisation      src/solvers/SimInf_solver_ssm.c:96-117
 *   k_ssa_e1     direct-method SSA up to the next unit of time
 *                                          src/solvers/SimInf_solver_ssm.c:144-235
 *                followed by the node's E1 events of the day
 *                                          src/solvers/SimInf_solver.c:658-822
 *   k_e2_wave    one conflict-free wavefront of external transfers
 *                                          src/solvers/SimInf_solver.c:824-902
 *   k_pts_store  post time step, rate refresh, U/V store
 *                                          src/solvers/SimInf_solver_ssm.c:262-334
 *   k_horizon    all days of one node in one thread, for schedules without
 *                external transfers (nodes never interact)
 *
 * Node state lives in registers for the whole day (u as int[NC], rates as
 * double[NT]); S and the G column masks sit in shared memory so the
 * transition index can stay dynamic without spilling the register arrays.
 * Random draws come from the node's Philox stream (siminf_stream.h), and
 * the waiting-time logarithm is the integer fixed-point si_neglog_u32 (a
 * 32-bit-input -log(u) with two table reductions): on GB300 the FP64 pipe
 * retires one warp instruction per 64 cycles per SM sub-partition, while the
 * integer pipes are ~40x faster, so the SSA chain keeps only the FP64
 * operations the reference's arithmetic requires.
 *
 * Compiled with -fmad=false: every double operation rounds as in the
 * reference's C, which is what makes trajectories bit-identical.
 */
#ifndef SIMINF_KERNELS_CUH
#define SIMINF_KERNELS_CUH

#include <cfloat>
#include <climits>
#include <cstdint>
#include <cuda_runtime.h>

#include "siminf_stream.h"
#include "siminf_models.cuh"
#include "siminf_plan.h"
#include "siminf_launch.h"

namespace siminf {

enum { ERR_NEGATIVE_STATE = -1, ERR_UNDEFINED_EVENT = -3, ERR_SAMPLE_SELECT = -8,
       ERR_INVALID_RATE = -11, ERR_EVENTS_N = -15, ERR_EVENT_SHIFT = -16,
       ERR_SHIFT_OUT_OF_BOUNDS = -17, ERR_INVALID_PROPORTION = -18, ERR_TIMEOUT = -33 };


enum { EV_EXIT = 0, EV_ENTER = 1, EV_INTERNAL = 2, EV_EXTERNAL = 3 };

/* Out of line: errors are rare, and every kernel calls this. */
static __device__ __noinline__ void record_error(const DevState &s, int code, int phase,
                                                int day, long long g, int tr, int evi,
                                                double time, double rate)
{
    const int slot = atomicAdd(s.err_count, 1);
    atomicMin(s.err_day, day);
    if (phase <= PHASE_E1)
        atomicMin(s.err_day_pre_e2, day);
    if (slot < MAX_ERR) {
        ErrRec e;
        e.code = code;
        e.phase = phase;
        e.day = day;
        e.rep = (int) (g / s.Nn);
        e.node = (int) (g % s.Nn);
        e.transition = tr;
        e.event_index = evi;
        e.pad = 0;
        e.time = time;
        e.rate = rate;
        s.err[slot] = e;
    }
}

__device__ __forceinline__ const double *gdata_of(const DevState &s, long long g)
{
    if (s.job_of)
        return s.gdata + (size_t) s.job_of[g] * s.gdata_stride;
    return s.gdata + (size_t) (g / s.Nn) * s.gdata_stride;
}

/* Key of node g's stream: (seed, replicate * Nn + node) for one model, the
 * job's own seed and local node index in a batch. */
__device__ __forceinline__ void stream_key(const DevState &s, long long g, uint64_t &seed,
                                           uint64_t &sid)
{
    if (s.job_of) {
        const int j = s.job_of[g];
        seed = s.job_seed[j];
        sid = (uint64_t) (g - s.job_node0[j]);
    } else {
        seed = s.pf_seeds ? s.pf_seeds[*s.pf_interval] : s.seed;
        sid = (uint64_t) g;
    }
}

/* Node g's model has run all its days (batches only). */
__device__ __forceinline__ bool job_over(const DevState &s, long long g, int day)
{
    return s.job_of && day >= s.job_ndays[s.job_of[g]];
}

__device__ __forceinline__ int load_flag(const int *p)
{
    return *(volatile const int *) p;
}

/* Sum the per-thread transition counts of a warp into the global counter. */
__device__ __forceinline__ void add_fired(const DevState &s, unsigned long long n)
{
    for (int o = 16; o > 0; o >>= 1)
        n += __shfl_down_sync(0xFFFFFFFFu, n, o);
    if ((threadIdx.x & 31) == 0 && n)
        atomicAdd(s.fired, n);
}

/* ------------------------------------------------------------------ */
/* Direct-method SSA of one node up to `next`                           */
/* (src/solvers/SimInf_solver_ssm.c:144-235), arranged for latency: the */
/* heaviest node of a day sets the day's critical path, and one node's  */
/* transitions form a chain of dependent operations, so everything that */
/* does not depend on the running sum leaves the chain:                 */
/*  - the two draws of the next transition (Philox block, -log(u) by    */
/*    si_neglog_u32, the selection uniform) are computed while the      */
/*    current transition updates the state, from the draw index alone;  */
/*  - the prefix sums of the rates, used by the inversion, are formed   */
/*    once per rate update, so choosing the transition is NT-1          */
/*    independent comparisons instead of a dependent add/compare chain; */
/*  - divisions, comparisons and int->double conversions run on the     */
/*    integer pipes (si_div, si_dge/si_dgt, si_i2d): same bits, and a   */
/*    rate's division by a population count reuses its prepared         */
/*    reciprocal (si_div_cached).                                       */
/* Draw i of the node's stream is word i & 3 of Philox block i >> 2; a  */
/* transition uses draws c (waiting time) and c + 1 (selection), so the */
/* next transition's pair lies in block (c + 3) >> 2, except the first  */
/* draw when (c + 2) & 3 == 3, which lies in the block this transition  */
/* fetched.                                                             */
/* ------------------------------------------------------------------ */
template <class M>
__device__ __forceinline__ void prefix_sums(const double (&rate)[M::NT], double (&cum)[M::NT])
{
    cum[0] = rate[0];
#pragma unroll
    for (int k = 1; k < M::NT; k++)
        cum[k] = cum[k - 1] + rate[k];
}

/* The transition the inversion picks (ssm.c:165-169): the first k with
 * !(rnd > rate[0] + ... + rate[k]), else NT - 1.  The prefix sums are
 * formed from the rates at each selection -- they depend on the rates
 * alone, so they run beside the rate sum's update -- instead of being
 * carried from step to step in registers. */
template <class M>
__device__ __forceinline__ int select_transition(const double (&rate)[M::NT], double rnd)
{
    double cum[M::NT];
    prefix_sums<M>(rate, cum);
    int tr = M::NT - 1;
#pragma unroll
    for (int k = M::NT - 2; k >= 0; k--)
        if (!(rnd > cum[k]))
            tr = k;
    return tr;
}

__device__ __forceinline__ uint32_t word_of(uint32_t b0, uint32_t b1, uint32_t b2, uint32_t b3,
                                            uint32_t i)
{
    const uint32_t lo = (i & 1) ? b1 : b0, hi = (i & 1) ? b3 : b2;
    return (i & 2) ? hi : lo;
}

/* x <= 0.0 for the double with bits b (false for NaN), on the integer pipes. */
__device__ __forceinline__ bool le_zero(uint64_t b)
{
    return (int64_t) b <= 0 && !si_isnan_bits(b);
}

/* Philox block `blk` of the stream held in r (key and stream id only). */
__device__ __forceinline__ void philox_block(const si_rng &r, uint64_t blk, uint32_t &b0,
                                             uint32_t &b1, uint32_t &b2, uint32_t &b3)
{
    b0 = (uint32_t) blk;
    b1 = (uint32_t) (blk >> 32);
    b2 = r.s0;
    b3 = r.s1;
    si_philox4x32_10(&b0, &b1, &b2, &b3, r.k0, r.k1);
}

/* The SSA state of one node during its day, held by one thread. */
template <class M>
struct SsaLane {
    int u[M::NC];
    double rate[M::NT];
    double sum, t, L, U, tau;
    uint64_t c;                       /* draw index of the next waiting time */
    uint32_t q0, q1, q2, q3;          /* Philox block (c + 1) >> 2 */
    unsigned fired;
    int err, err_tr;
    double err_t, err_rate;
    si_recip dc;
};

/* Start the day of a node whose u, rate, sum and t are loaded and whose
 * next draw is `c`; key holds the stream's key.  Returns true when nothing
 * fires today (rate sum <= 0, or not finite after a recorded invalid rate,
 * which would never reach `next`). */
template <class M>
__device__ __forceinline__ bool ssa_begin(SsaLane<M> &ln, const si_rng &key, uint64_t c,
                                          double next)
{
    ln.fired = 0;
    ln.c = c;
    if (!si_finite_pos(ln.sum)) {
        /* sum <= 0: nothing fires (ssm.c:148-151) */
        if (!le_zero(si_double_bits(ln.sum)) && !ln.err) {
            ln.err = ERR_INVALID_RATE;
            ln.err_tr = -1;
            ln.err_t = ln.t;
            ln.err_rate = ln.sum;
        }
        ln.t = next;
        return true;
    }
    /* the pair of the first transition */
    uint32_t p0, p1, p2, p3;
    philox_block(key, c >> 2, p0, p1, p2, p3);
    philox_block(key, (c + 1) >> 2, ln.q0, ln.q1, ln.q2, ln.q3);
    ln.L = si_neglog_u32(word_of(p0, p1, p2, p3, (uint32_t) c & 3u));
    ln.U = si_u32_to_uniform_pos(word_of(ln.q0, ln.q1, ln.q2, ln.q3, (uint32_t) (c + 1) & 3u));
    if (!M::RATES_TIME_INVARIANT)
        ln.tau = si_div(ln.L, ln.sum);  /* ssa_step_ahead divides at each step */
    return false;
}

/* One step of the direct method for models whose rates do not read t:
 * the same operations as ssa_step_in_order, arranged so that the waiting
 * time's division (~550 cycles) does not hold up the next transition.
 * The transition the step would fire is selected and applied to copies of
 * the state while the division runs -- its rates need no time -- and the
 * copies replace the state only once the waiting time shows that it fires
 * before the day ends.  Returns true when the node's day is over.  It is
 * the exact path behind ssa_step_spec, taken only for that step's rare
 * cases, so it stays out of line: inlined, it doubled the code of the SSA
 * loop that every warp keeps in its instruction cache (3% of the headline
 * run's time). */
template <class M>
__device__ __noinline__ bool ssa_step_ahead(SsaLane<M> &ln, const si_rng &key, double next,
                                               const double *v, const double *ld,
                                               const double *gd, const int *sS,
                                               const uint32_t *sG, unsigned max_fired)
{
    constexpr int NC = M::NC, NT = M::NT;
    const double tau = si_div(ln.L, ln.sum);
    const double rnd = ln.U * ln.sum;

    int tr = select_transition<M>(ln.rate, rnd);
    double rtr = ln.rate[0];
#pragma unroll
    for (int k = 1; k < NT; k++)
        if (tr == k)
            rtr = ln.rate[k];
    bool nil = false;
    if (si_is_zero(rtr)) {
        /* Back-scan to the first non-zero rate (ssm.c:171-189). */
#pragma unroll
        for (int k = NT - 1; k >= 1; k--)
            if (tr == k && si_is_zero(ln.rate[k]))
                tr = k - 1;
        double r2 = ln.rate[0];
#pragma unroll
        for (int k = 1; k < NT; k++)
            if (tr == k)
                r2 = ln.rate[k];
        nil = si_is_zero(r2);
    }

    /* The state after that transition, in copies. */
    int u2[NC];
    int neg = 0;
#pragma unroll
    for (int cc = 0; cc < NC; cc++) {
        const int d = sS[tr * NC + cc];
        u2[cc] = ln.u[cc] + d;
        neg |= (d != 0) & (u2[cc] < 0);
    }
    double rate2[NT];
    double delta = 0.0;
    const uint32_t gm = sG[tr];
    int bad = -1;
    double bad_rate = 0.0;
#pragma unroll
    for (int k = 0; k < NT; k++) {
        rate2[k] = ln.rate[k];
        if (gm & (1u << k)) {
            const double nr = M::rate(k, u2, v, ld, gd, ln.t, ln.dc);
            rate2[k] = nr;
            delta += nr - ln.rate[k];
            if (si_bad_rate(nr)) {
                bad = k;
                bad_rate = nr;
            }
        }
    }
    const double sum2 = ln.sum + delta;

    /* Draws of the transition after it. */
    const uint64_t c2 = ln.c + 2;
    uint32_t n0, n1, n2, n3;
    philox_block(key, (c2 + 1) >> 2, n0, n1, n2, n3);
    const uint32_t ci = (uint32_t) c2 & 3u;
    const uint32_t wl = (ci == 3u) ? ln.q3 : word_of(n0, n1, n2, n3, ci);
    const uint32_t wu = word_of(n0, n1, n2, n3, (ci + 1u) & 3u);

    /* The waiting time decides: the day ends first, or the transition fires. */
    const double tn = tau + ln.t;
    if (tn >= next) {
        ln.t = next;
        ln.c += 1;                            /* the waiting time's draw was used */
        return true;
    }
    ln.t = tn;
    ln.c = c2;
    if (nil) {
        ln.sum = 0.0;
        return true;
    }
    if (++ln.fired > max_fired) {
        ln.err = ERR_TIMEOUT;
        ln.err_tr = tr;
        ln.err_t = ln.t;
        ln.t = next;
        return true;
    }
#pragma unroll
    for (int cc = 0; cc < NC; cc++)
        ln.u[cc] = u2[cc];
#pragma unroll
    for (int k = 0; k < NT; k++)
        ln.rate[k] = rate2[k];
    ln.sum = sum2;
    ln.q0 = n0;
    ln.q1 = n1;
    ln.q2 = n2;
    ln.q3 = n3;
    ln.L = si_neglog_u32(wl);
    ln.U = si_u32_to_uniform_pos(wu);
    if (neg) {
        ln.err = ERR_NEGATIVE_STATE;
        ln.err_tr = tr;
        ln.err_t = ln.t;
        ln.err_rate = 0.0;
    }
    if (bad >= 0) {
        ln.err = ERR_INVALID_RATE;
        ln.err_tr = bad;
        ln.err_t = ln.t;
        ln.err_rate = bad_rate;
    }
    if (!si_finite_pos(ln.sum)) {
        if (!le_zero(si_double_bits(ln.sum)) && !ln.err) {
            ln.err = ERR_INVALID_RATE;
            ln.err_tr = -1;
            ln.err_t = ln.t;
            ln.err_rate = ln.sum;
        }
        ln.t = next;
        return true;
    }
    return false;
}

/* The step of ssa_step_ahead as one block of straight-line code, for
 * the common case: no zero rate selected, no negative state, no invalid
 * or non-positive rate sum, no division off the integer path, a prepared
 * divisor that every rate's division finds in the cache, a waiting time
 * on the table path of -log(u), and the transition count within
 * max_fired.  Every rate is evaluated (and kept where its G bit is set),
 * so that no branch splits the block.  L and U are the step's -log(u) and
 * selection uniform; with NEXT, the step also computes the next step's
 * pair into ln.L and ln.U (the way ssa_step_ahead does), without it the
 * caller supplies every step's pair.  Returns SSA_FIRED or SSA_DAY_OVER
 * with the state updated exactly as ssa_step_ahead updates it, or
 * SSA_REDO with the state untouched when any of those conditions fails;
 * the caller then runs ssa_step_ahead on the same state and draws. */
enum { SSA_FIRED = 0, SSA_DAY_OVER = 1, SSA_REDO = 2 };

template <class M, bool NEXT>
__device__ __forceinline__ int ssa_step_spec(SsaLane<M> &ln, const si_rng &key, double L,
                                             double U, double next, const double *v,
                                             const double *ld, const double *gd, const int *sS,
                                             const uint32_t *sG, unsigned max_fired)
{
    constexpr int NC = M::NC, NT = M::NT;
    int tau_special = 0;
    const double tau = si_div_spec(L, ln.sum, &tau_special);
    const double rnd = U * ln.sum;

    int tr = select_transition<M>(ln.rate, rnd);
    double rtr = ln.rate[0];
#pragma unroll
    for (int k = 1; k < NT; k++)
        if (tr == k)
            rtr = ln.rate[k];
    int redo = si_is_zero(rtr);             /* the back-scan of ssm.c:171-189 */

    /* The state after that transition. */
    int u2[NC];
#pragma unroll
    for (int cc = 0; cc < NC; cc++) {
        const int d = sS[tr * NC + cc];
        u2[cc] = ln.u[cc] + d;
        redo |= (d != 0) & (u2[cc] < 0);
    }
    /* Every rate at that state; those flagged in column tr of G replace
     * the old ones and enter the delta in row order. */
    const uint32_t gm = sG[tr];
    si_recip_spec dcs;
    dcs.c = &ln.dc;
    dcs.flag = 0;
    double rate2[NT];
    double delta = 0.0;
#pragma unroll
    for (int k = 0; k < NT; k++) {
        const int f0 = dcs.flag;            /* a rate that is not kept flags nothing */
        const double nr = M::rate(k, u2, v, ld, gd, ln.t, dcs);
        const bool g = (gm >> k) & 1u;
        dcs.flag = g ? dcs.flag : f0;
        rate2[k] = g ? nr : ln.rate[k];
        const double dk = delta + (nr - ln.rate[k]);
        delta = g ? dk : delta;
        redo |= g & si_bad_rate(nr);
    }
    const double sum2 = ln.sum + delta;
    redo |= dcs.flag | !si_finite_pos(sum2);
    redo |= ln.fired + 1u > max_fired;

    /* Draws of the transition after it. */
    const uint64_t c2 = ln.c + 2;
    uint32_t n0 = 0, n1 = 0, n2 = 0, n3 = 0;
    double L2 = 0.0, U2 = 0.0;
    if constexpr (NEXT) {
        philox_block(key, (c2 + 1) >> 2, n0, n1, n2, n3);
        const uint32_t ci = (uint32_t) c2 & 3u;
        const uint32_t wl = (ci == 3u) ? ln.q3 : word_of(n0, n1, n2, n3, ci);
        const uint32_t wu = word_of(n0, n1, n2, n3, (ci + 1u) & 3u);
        L2 = si_neglog_u32_spec(wl, &redo);
        U2 = si_u32_to_uniform_pos(wu);
    }

    if (tau_special)
        return SSA_REDO;
    const double tn = tau + ln.t;
    if (tn >= next) {
        ln.t = next;
        ln.c += 1;                            /* the waiting time's draw was used */
        return SSA_DAY_OVER;
    }
    if (redo)
        return SSA_REDO;
    ln.t = tn;
    ln.c = c2;
    ln.fired++;
#pragma unroll
    for (int cc = 0; cc < NC; cc++)
        ln.u[cc] = u2[cc];
#pragma unroll
    for (int k = 0; k < NT; k++)
        ln.rate[k] = rate2[k];
    ln.sum = sum2;
    if constexpr (NEXT) {
        ln.q0 = n0;
        ln.q1 = n1;
        ln.q2 = n2;
        ln.q3 = n3;
        ln.L = L2;
        ln.U = U2;
    }
    return SSA_FIRED;
}

/* Draws of four transitions of a node whose next waiting-time draw is c:
 * words c .. c + 7 of its stream (waiting time, selection, four times),
 * from the three Philox blocks that can hold them, as -log(u) and
 * uniform values.  The four -log(u) are independent chains of integer
 * operations that the compiler interleaves. */
__device__ __forceinline__ void draw_four(const si_rng &key, uint64_t c, double (&L)[4],
                                          double (&U)[4])
{
    uint32_t w[12];
    const uint64_t b = c >> 2;
#pragma unroll
    for (int k = 0; k < 3; k++)
        philox_block(key, b + k, w[4 * k], w[4 * k + 1], w[4 * k + 2], w[4 * k + 3]);
    const uint32_t o = (uint32_t) c & 3u;
    uint32_t x[8];
#pragma unroll
    for (int i = 0; i < 8; i++)
        x[i] = o == 0 ? w[i] : o == 1 ? w[i + 1] : o == 2 ? w[i + 2] : w[i + 3];
    int slow = 0;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        L[j] = si_neglog_u32_spec(x[2 * j], &slow);
        U[j] = si_u32_to_uniform_pos(x[2 * j + 1]);
    }
    if (slow) {
#pragma unroll
        for (int j = 0; j < 4; j++)
            L[j] = si_neglog_u32(x[2 * j]);
    }
}

/* The rest of a node's day after ssa_begin, for models whose rates do not
 * read t: straight-line steps in batches of four, their draws computed
 * together ahead of them (draw_four); a step that meets a rare case is
 * redone by ssa_step_ahead with the same draws, and the next batch starts
 * at the draw index it leaves.  The draws, and so the trajectory, are
 * those of ssa_step. */
template <class M>
__device__ __forceinline__ void ssa_run_day(SsaLane<M> &ln, const si_rng &key, double next,
                                            const double *v, const double *ld, const double *gd,
                                            const int *sS, const uint32_t *sG,
                                            unsigned max_fired)
{
    for (;;) {
        double L[4], U[4];
        draw_four(key, ln.c, L, U);
        int j = 0, st;
        double Lj, Uj;
        do {
            Lj = j == 0 ? L[0] : j == 1 ? L[1] : j == 2 ? L[2] : L[3];
            Uj = j == 0 ? U[0] : j == 1 ? U[1] : j == 2 ? U[2] : U[3];
            st = ssa_step_spec<M, false>(ln, key, Lj, Uj, next, v, ld, gd, sS, sG, max_fired);
        } while (st == SSA_FIRED && ++j < 4);
        if (st == SSA_DAY_OVER)
            return;
        if (st == SSA_REDO) {
            /* the exact step, with this step's draws and the Philox block
             * of its selection draw, as ssa_step_ahead expects them */
            ln.L = Lj;
            ln.U = Uj;
            philox_block(key, (ln.c + 1) >> 2, ln.q0, ln.q1, ln.q2, ln.q3);
            if (ssa_step_ahead<M>(ln, key, next, v, ld, gd, sS, sG, max_fired))
                return;
        }
    }
}

/* One step of the direct method in the reference's order: the waiting
 * time ends the day, or one transition fires.  Returns true when the
 * node's day is over. */
template <class M>
__device__ __forceinline__ bool ssa_step_in_order(SsaLane<M> &ln, const si_rng &key,
                                                  double next, const double *v,
                                                  const double *ld, const double *gd,
                                                  const int *sS, const uint32_t *sG,
                                                  unsigned max_fired)
{
    constexpr int NC = M::NC, NT = M::NT;
    const double tn = ln.tau + ln.t;
    /* the hardware FP64 comparisons of the chain (IEEE, false on NaN, as
     * si_dge/si_dgt): one instruction each, ~3% off a transition's latency */
    if (tn >= next) {
        ln.t = next;
        ln.c += 1;                            /* the waiting time's draw was used */
        return true;
    }
    ln.t = tn;
    const double rnd = ln.U * ln.sum;
    ln.c += 2;

    /* Draws of the next transition, off the chain. */
    {
        uint32_t n0, n1, n2, n3;
        philox_block(key, (ln.c + 1) >> 2, n0, n1, n2, n3);
        const uint32_t ci = (uint32_t) ln.c & 3u;
        const uint32_t wl = (ci == 3u) ? ln.q3 : word_of(n0, n1, n2, n3, ci);
        const uint32_t wu = word_of(n0, n1, n2, n3, (ci + 1u) & 3u);
        ln.q0 = n0;
        ln.q1 = n1;
        ln.q2 = n2;
        ln.q3 = n3;
        ln.L = si_neglog_u32(wl);
        ln.U = si_u32_to_uniform_pos(wu);
    }

    int tr = select_transition<M>(ln.rate, rnd);
    double rtr = ln.rate[0];
#pragma unroll
    for (int k = 1; k < NT; k++)
        if (tr == k)
            rtr = ln.rate[k];
    if (si_is_zero(rtr)) {
        /* Back-scan to the first non-zero rate (ssm.c:171-189). */
#pragma unroll
        for (int k = NT - 1; k >= 1; k--)
            if (tr == k && si_is_zero(ln.rate[k]))
                tr = k - 1;
        double r2 = ln.rate[0];
#pragma unroll
        for (int k = 1; k < NT; k++)
            if (tr == k)
                r2 = ln.rate[k];
        if (si_is_zero(r2)) {
            ln.sum = 0.0;
            return true;
        }
    }

    if (++ln.fired > max_fired) {
        /* Bounded work per node-day: a time step that stopped advancing t
         * (a rate sum near the overflow threshold) ends the run with an
         * error instead of spinning. */
        ln.err = ERR_TIMEOUT;
        ln.err_tr = tr;
        ln.err_t = ln.t;
        ln.t = next;
        return true;
    }
    int neg = 0;
#pragma unroll
    for (int cc = 0; cc < NC; cc++) {
        const int d = sS[tr * NC + cc];
        ln.u[cc] += d;
        neg |= (d != 0) & (ln.u[cc] < 0);
    }
    if (neg) {
        ln.err = ERR_NEGATIVE_STATE;
        ln.err_tr = tr;
        ln.err_t = ln.t;
        ln.err_rate = 0.0;
    }

    /* Refresh the rates flagged in column tr of G, in row order. */
    double delta = 0.0;
    const uint32_t gm = sG[tr];
    int bad = -1;
    double bad_rate = 0.0;
#pragma unroll
    for (int k = 0; k < NT; k++) {
        if (gm & (1u << k)) {
            const double old = ln.rate[k];
            const double nr = M::rate(k, ln.u, v, ld, gd, ln.t, ln.dc);
            ln.rate[k] = nr;
            delta += nr - old;
            if (si_bad_rate(nr)) {
                bad = k;
                bad_rate = nr;
            }
        }
    }
    if (bad >= 0) {
        ln.err = ERR_INVALID_RATE;
        ln.err_tr = bad;
        ln.err_t = ln.t;
        ln.err_rate = bad_rate;
    }
    ln.sum += delta;

    if (!si_finite_pos(ln.sum)) {
        if (!le_zero(si_double_bits(ln.sum)) && !ln.err) {
            ln.err = ERR_INVALID_RATE;
            ln.err_tr = -1;
            ln.err_t = ln.t;
            ln.err_rate = ln.sum;
        }
        ln.t = next;
        return true;
    }
    ln.tau = si_div(ln.L, ln.sum);
    return false;
}

/* One step of the direct method (src/solvers/SimInf_solver_ssm.c:
 * 144-235): where the rates do not read t, the straight-line speculative
 * step, redone ahead of the waiting time on the exact path when it meets
 * a rare case. */
template <class M>
__device__ __forceinline__ bool ssa_step(SsaLane<M> &ln, const si_rng &key, double next,
                                         const double *v, const double *ld, const double *gd,
                                         const int *sS, const uint32_t *sG, unsigned max_fired)
{
    if constexpr (M::RATES_TIME_INVARIANT) {
        const int st = ssa_step_spec<M, true>(ln, key, ln.L, ln.U, next, v, ld, gd, sS, sG,
                                              max_fired);
        if (st != SSA_REDO)
            return st == SSA_DAY_OVER;
        return ssa_step_ahead<M>(ln, key, next, v, ld, gd, sS, sG, max_fired);
    } else {
        return ssa_step_in_order<M>(ln, key, next, v, ld, gd, sS, sG, max_fired);
    }
}

/* A node's whole SSA day in one call (used where one thread keeps one
 * node for the whole run). */
template <class M>
__device__ __forceinline__ unsigned ssa_day(SsaLane<M> &ln, si_rng &r, double next,
                                            const double *v, const double *ld, const double *gd,
                                            const int *sS, const uint32_t *sG, unsigned max_fired)
{
    if (!ssa_begin<M>(ln, r, r.ctr, next)) {
        /* two steps one at a time, then, for a node that is still going,
         * batches of four (a node with one transition or none in the day
         * computes no draws it does not use) */
        for (int n = 0;; n++) {
            if (M::RATES_TIME_INVARIANT && n == 2) {
                ssa_run_day<M>(ln, r, next, v, ld, gd, sS, sG, max_fired);
                break;
            }
            if (ssa_step<M>(ln, r, next, v, ld, gd, sS, sG, max_fired))
                break;
        }
    }
    r.ctr = ln.c;
    r.have = 0;
    return ln.fired;
}

/* ------------------------------------------------------------------ */
/* Event sampling on a node's compartments uu (src/solvers/             */
/* SimInf_solver.c:62-324), drawing from the node's stream.             */
/* ------------------------------------------------------------------ */
template <int NC>
__device__ int sample_select(const DevState &s, const int *uu, int select, int n,
                             double proportion, int *ind, si_rng *r)
{
    const int *irE = s.irE, *jcE = s.jcE;
    const double *prE = s.prE;
    int i, Nstates, Nindividuals = 0, Nkinds = 0;

    for (int c = 0; c < NC; c++)
        ind[c] = 0;
    for (i = jcE[select]; i < jcE[select + 1]; i++) {
        const int nk = uu[irE[i]];
        if (nk > 0)
            Nkinds++;
        Nindividuals += nk;
    }
    Nstates = jcE[select + 1] - jcE[select];
    if (n == 0) {
        if (proportion < 0 || proportion > 1)
            return ERR_INVALID_PROPORTION;
        n = si_binomial(r, proportion, Nindividuals);
    }
    if (s.cap && n > Nindividuals)
        n = Nindividuals;
    if (Nstates <= 0 || n > Nindividuals || n < 0)
        return ERR_SAMPLE_SELECT;
    if (n == 0)
        return 0;
    if (Nindividuals == n) {
        for (i = jcE[select]; i < jcE[select + 1]; i++)
            ind[irE[i]] = uu[irE[i]];
        return 0;
    }
    if (Nstates == 1) {
        ind[irE[jcE[select]]] = n;
        return 0;
    }
    if (Nkinds == 1) {
        for (i = jcE[select]; i < jcE[select + 1]; i++) {
            if (uu[irE[i]] > 0) {
                ind[irE[i]] = n;
                break;
            }
        }
        return 0;
    }
    bool equal = true;
    for (i = jcE[select] + 1; i < jcE[select + 1]; i++)
        if (prE[i] != prE[i - 1])
            equal = false;
    if (equal) {
        /* Sequential multivariate hypergeometric. */
        for (i = jcE[select]; i < jcE[select + 1] - 1; i++) {
            if (n == 0)
                break;
            const int nk = uu[irE[i]];
            ind[irE[i]] = si_hypergeometric(r, nk, Nindividuals - nk, n);
            Nindividuals -= nk;
            n -= ind[irE[i]];
        }
        ind[irE[i]] = n;
        return 0;
    }
    /* Wallenius' noncentral hypergeometric by a biased urn. */
    while (n > 0) {
        double rand, cum = 0;
        for (i = jcE[select]; i < jcE[select + 1]; i++)
            cum += prE[i] * (uu[irE[i]] - ind[irE[i]]);
        rand = si_uniform_pos(r) * cum;
        i = jcE[select];
        cum = prE[i] * (uu[irE[i]] - ind[irE[i]]);
        while (i < jcE[select + 1] && rand > cum) {
            i++;
            if (i < jcE[select + 1])
                cum += prE[i] * (uu[irE[i]] - ind[irE[i]]);
        }
        if (i >= jcE[select + 1])
            i = jcE[select + 1] - 1;
        if ((prE[i] * (uu[irE[i]] - ind[irE[i]])) == 0.0) {
            for (; i > jcE[select] && (prE[i] * (uu[irE[i]] - ind[irE[i]])) == 0.0; i--);
            if ((prE[i] * (uu[irE[i]] - ind[irE[i]])) == 0.0)
                return ERR_SAMPLE_SELECT;
        }
        ind[irE[i]] += 1;
        n--;
    }
    return 0;
}

template <int NC>
__device__ int sample_select_enter(const DevState &s, const int *uu, int select, int n,
                                   double proportion, int *ind, si_rng *r)
{
    const int *irE = s.irE, *jcE = s.jcE;
    const double *prE = s.prE;
    int i, Nstates = jcE[select + 1] - jcE[select];
    double w_cum = 0;

    for (int c = 0; c < NC; c++)
        ind[c] = 0;
    if (n == 0) {
        if (proportion < 0 || proportion > 1)
            return ERR_INVALID_PROPORTION;
        for (i = jcE[select]; i < jcE[select + 1]; i++)
            n += uu[irE[i]];
        n = si_binomial(r, proportion, n);
    }
    if (Nstates <= 0 || n < 0)
        return ERR_SAMPLE_SELECT;
    if (n == 0)
        return 0;
    if (Nstates == 1) {
        ind[irE[jcE[select]]] = n;
        return 0;
    }
    for (i = jcE[select]; i < jcE[select + 1]; i++)
        w_cum += prE[i];
    while (n > 0) {
        double cum, rand = si_uniform_pos(r) * w_cum;
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
                return ERR_SAMPLE_SELECT;
        }
        ind[irE[i]] += 1;
        n--;
    }
    return 0;
}

/* Apply one E1 event to the node's compartments uu
 * (src/solvers/SimInf_solver.c:680-822).  Returns 0 or an error code. */
template <int NC>
__device__ int apply_e1(const DevState &s, int *uu, const E1Rec &e, si_rng *r)
{
    int ind[NC];
    int err;
    const int *irE = s.irE, *jcE = s.jcE;

    switch (e.kind) {
    case EV_EXIT:
        err = sample_select<NC>(s, uu, e.select, e.n, e.proportion, ind, r);
        if (err)
            return err;
        for (int i = jcE[e.select]; i < jcE[e.select + 1]; i++) {
            const int jj = irE[i];
            uu[jj] -= ind[jj];
            if (uu[jj] < 0)
                return ERR_NEGATIVE_STATE;
        }
        return 0;
    case EV_ENTER:
        err = sample_select_enter<NC>(s, uu, e.select, e.n, e.proportion, ind, r);
        if (err)
            return err;
        for (int i = jcE[e.select]; i < jcE[e.select + 1]; i++) {
            const int jj = irE[i];
            if (e.shift < 0) {
                uu[jj] += ind[jj];
                if (uu[jj] < 0)
                    return ERR_NEGATIVE_STATE;
            } else if (!s.hasN) {
                return ERR_EVENTS_N;
            } else {
                const int ll = s.Nshift[e.shift * NC + jj];
                if (jj + ll < 0 || jj + ll >= NC)
                    return ERR_SHIFT_OUT_OF_BOUNDS;
                uu[jj + ll] += ind[jj];
                if (uu[jj + ll] < 0)
                    return ERR_NEGATIVE_STATE;
            }
        }
        return 0;
    case EV_INTERNAL:
        if (!s.hasN)
            return ERR_EVENTS_N;
        if (e.shift < 0)
            return ERR_EVENT_SHIFT;
        err = sample_select<NC>(s, uu, e.select, e.n, e.proportion, ind, r);
        if (err)
            return err;
        for (int i = jcE[e.select]; i < jcE[e.select + 1]; i++) {
            const int jj = irE[i];
            const int ll = s.Nshift[e.shift * NC + jj];
            if (jj + ll < 0 || jj + ll >= NC)
                return ERR_SHIFT_OUT_OF_BOUNDS;
            uu[jj + ll] += ind[jj];
            if (uu[jj + ll] < 0)
                return ERR_NEGATIVE_STATE;
            uu[jj] -= ind[jj];
            if (uu[jj] < 0)
                return ERR_NEGATIVE_STATE;
        }
        return 0;
    default:
        return ERR_UNDEFINED_EVENT;
    }
}

/* The E1 events of one node-day.  Inlined: a call would make the SSA
 * kernels save the registers live across it to local memory (spills),
 * while the samplers' code, after the SSA loop, runs only on the one
 * node-day in about 250 that has events.  State and stream counter go in
 * and out by value, so the caller's copies stay in registers. */
template <int NC>
struct E1Out {
    int u[NC];
    uint64_t ctr;
    int err_code, err_event;
    bool any;
};

template <int NC>
__device__ __forceinline__ E1Out<NC> node_e1_apply(const DevState &s, E1Out<NC> o, si_rng r, int lo,
                                                int end, int day)
{
    for (int k = lo; k < end; k++) {
        const E1Rec e = s.e1[k];
        if (e.day != day)
            break;
        const int err = apply_e1<NC>(s, o.u, e, &r);
        o.any = true;
        if (err) {
            o.err_code = err;
            o.err_event = e.index;
            break;
        }
    }
    o.ctr = r.ctr;
    return o;
}

/* The node's E1 events of `day` (src/solvers/SimInf_solver.c:658-822), in
 * array order, applied to u with draws from r.  Returns true when an event
 * was applied (the node is then flagged for a rate refresh).  A node's
 * events are stored in day order: the day's first is found by bisection. */
template <int NC>
__device__ __forceinline__ bool node_e1(const DevState &s, int (&u)[NC], int node, int day,
                                        si_rng &r, long long g, double tt, int &err_code,
                                        int &err_event)
{
    int lo = s.e1_ptr[node], hi = s.e1_ptr[node + 1];
    if (lo == hi)
        return false;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (s.e1[mid].day < day)
            lo = mid + 1;
        else
            hi = mid;
    }
    const int end = s.e1_ptr[node + 1];
    if (lo >= end || s.e1[lo].day != day)
        return false;
    E1Out<NC> o;
#pragma unroll
    for (int c = 0; c < NC; c++)
        o.u[c] = u[c];
    o.ctr = r.ctr;
    o.err_code = 0;
    o.err_event = -1;
    o.any = false;
    o = node_e1_apply<NC>(s, o, r, lo, end, day);
#pragma unroll
    for (int c = 0; c < NC; c++)
        u[c] = o.u[c];
    r.ctr = o.ctr;
    r.have = 0;
    if (o.err_code) {
        err_code = o.err_code;
        err_event = o.err_event;
    }
    return o.any;
}

/* node_e1 as a call, for k_horizon with models of at most two
 * compartments: inlined, its samplers take the registers the one-node-a-
 * thread loop keeps live and 12 bytes spill; called, they do not (and the
 * call is made only for a node that has E1 events at all). */
template <int NC>
__device__ __noinline__ bool node_e1_call(const DevState &s, int (&u)[NC], int node, int day,
                                          si_rng &r, long long g, double tt, int &err_code,
                                          int &err_event)
{
    return node_e1<NC>(s, u, node, day, r, g, tt, err_code, err_event);
}

/* The NC compartments of one node, loaded or stored with 16-byte (NC a
 * multiple of 4) or 8-byte (NC even) accesses: a node's block of u or of a
 * U column starts at a multiple of NC ints from a 256-byte aligned base. */
template <int NC>
__device__ __forceinline__ void load_u(const int *p, int (&u)[NC])
{
    if constexpr (NC % 4 == 0) {
#pragma unroll
        for (int c = 0; c < NC; c += 4) {
            const int4 w = *reinterpret_cast<const int4 *>(p + c);
            u[c] = w.x;
            u[c + 1] = w.y;
            u[c + 2] = w.z;
            u[c + 3] = w.w;
        }
    } else if constexpr (NC % 2 == 0) {
#pragma unroll
        for (int c = 0; c < NC; c += 2) {
            const int2 w = *reinterpret_cast<const int2 *>(p + c);
            u[c] = w.x;
            u[c + 1] = w.y;
        }
    } else {
#pragma unroll
        for (int c = 0; c < NC; c++)
            u[c] = p[c];
    }
}

template <int NC>
__device__ __forceinline__ void store_u(int *p, const int (&u)[NC])
{
    if constexpr (NC % 4 == 0) {
#pragma unroll
        for (int c = 0; c < NC; c += 4)
            *reinterpret_cast<int4 *>(p + c) = make_int4(u[c], u[c + 1], u[c + 2], u[c + 3]);
    } else if constexpr (NC % 2 == 0) {
#pragma unroll
        for (int c = 0; c < NC; c += 2)
            *reinterpret_cast<int2 *>(p + c) = make_int2(u[c], u[c + 1]);
    } else {
#pragma unroll
        for (int c = 0; c < NC; c++)
            p[c] = u[c];
    }
}

/* Store the node's U/V entries for columns [c0, c1) of its replicate. */
template <int NC, int ND>
__device__ __forceinline__ void store_columns(const DevState &s, int rep, int node,
                                              const int (&u)[NC], const double *vnew,
                                              int c0, int c1)
{
    for (int col = c0; col < c1; col++) {
        const size_t ccol = (size_t) rep * s.tlen + col;
        if (s.U) {
            store_u<NC>(s.U + ccol * (size_t) s.Nn * NC + (size_t) node * NC, u);
        } else if (s.jcU) {
            /* rows of this node in the sorted CSC column */
            int lo = s.jcU[ccol], hi = s.jcU[ccol + 1];
            const int row0 = node * NC;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (s.irU[mid] < row0)
                    lo = mid + 1;
                else
                    hi = mid;
            }
            for (int k = lo; k < s.jcU[ccol + 1] && s.irU[k] < row0 + NC; k++) {
                const int c = s.irU[k] - row0;
                int val = u[0];
#pragma unroll
                for (int q = 1; q < NC; q++)
                    if (c == q)
                        val = u[q];
                s.prU[k] = (double) val;
            }
        }
        if (ND > 0) {
            if (s.V) {
                double *dst = s.V + ccol * (size_t) s.Nn * ND + (size_t) node * ND;
#pragma unroll
                for (int d = 0; d < ND; d++)
                    dst[d] = vnew[d];
            } else if (s.jcV) {
                int lo = s.jcV[ccol], hi = s.jcV[ccol + 1];
                const int row0 = node * ND;
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (s.irV[mid] < row0)
                        lo = mid + 1;
                    else
                        hi = mid;
                }
                for (int k = lo; k < s.jcV[ccol + 1] && s.irV[k] < row0 + ND; k++)
                    s.prV[k] = vnew[s.irV[k] - row0];
            }
        }
    }
}

template <class M>
__device__ __forceinline__ void load_model_smem(const DevState &s, int *sS, uint32_t *sG)
{
    for (int i = threadIdx.x; i < M::NT * M::NC; i += blockDim.x)
        sS[i] = s.S[i];
    for (int i = threadIdx.x; i < M::NT; i += blockDim.x)
        sG[i] = s.Gmask[i];
    __syncthreads();
}

/* ------------------------------------------------------------------ */
/* Kernels.                                                              */
/* ------------------------------------------------------------------ */

/* List g as heavy for `day` when its rate sum promises many transitions
 * in one unit of time (only for models whose rates ignore t). */
/* The heavy class of a node whose rate sum at the start of a day is
 * `sum`: 0 for sum >= 16 h, 1 for >= 4 h, 2 for >= h (h = heavy_rate),
 * -1 for a node that is not heavy or a model whose rates depend on time. */
template <class M>
__device__ __forceinline__ int heavy_class(const DevState &s, double sum)
{
    if (!M::RATES_TIME_INVARIANT || !(s.heavy_rate > 0.0))
        return -1;
    if (!si_dge(sum, s.heavy_rate) || !si_finite_pos(sum))
        return -1;
    return si_dge(sum, 16.0 * s.heavy_rate) ? 0 : si_dge(sum, 4.0 * s.heavy_rate) ? 1 : 2;
}

/* Warp-wide (every lane of the warp calls it): lanes with cls >= 0 append
 * their node to heavy list cls of `day`, with one atomic per class present
 * in the warp; a list that is full takes nothing more. */
__device__ __forceinline__ void push_heavy_warp(const DevState &s, long long g, int cls, int day)
{
    const unsigned FULL = 0xFFFFFFFFu;
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int c = 0; c < HEAVY_CLASSES; c++) {
        const unsigned m = __ballot_sync(FULL, cls == c);
        if (!m)
            continue;
        const int q = (day & 1) * HEAVY_CLASSES + c;
        const int leader = __ffs(m) - 1;
        int base = MAX_HEAVY;
        if (lane == leader && load_flag(&s.heavy_count[q]) < MAX_HEAVY)
            base = atomicAdd(&s.heavy_count[q], __popc(m));
        base = __shfl_sync(FULL, base, leader);
        if (cls == c) {
            const int slot = base + __popc(m & ((1u << lane) - 1u));
            if (slot < MAX_HEAVY) {
                s.heavy_list[q * MAX_HEAVY + slot] = (int) g;
                s.heavy_mark[g] = day + 1;
            }
        }
    }
}

/* k_init for one (replicate, node); returns its heavy class on day 0. */
template <class M>
__device__ __forceinline__ int init_node(const DevState &s, long long g, double tt0)
{
    constexpr int NC = M::NC, NT = M::NT, ND = M::ND;
    if (s.pf_days)
        tt0 = s.pf_days[(size_t) *s.pf_interval * s.pf_days_stride].tt;
    const int node = (int) (g % s.Nn);
    int u[NC];
    load_u<NC>(s.u + g * NC, u);
    const double *v = s.vA + g * ND;
    const double *ld = s.ldata + (size_t) node * s.Nld;
    si_recip dc = si_recip_none();
    double sum = 0.0;
#pragma unroll
    for (int j = 0; j < NT; j++) {
        const double rate = M::rate(j, u, v, ld, gdata_of(s, g), tt0, dc);
        s.t_rate[(size_t) j * s.Ntot + g] = rate;
        sum += rate;
        if (!isfinite(rate) || rate < 0.0)
            record_error(s, ERR_INVALID_RATE, PHASE_INIT, 0, g, j, -1, tt0, rate);
    }
    s.sum_rate[g] = sum;
    s.t_time[g] = tt0;
    s.ctr[g] = 0;
    if (s.crn_ctr)
        s.crn_ctr[g] = 0;
    s.update[g] = 0;
    return heavy_class<M>(s, sum);
}

template <class M>
__global__ void k_init(DevState s, double tt0)
{
    const long long g = blockIdx.x * (long long) blockDim.x + threadIdx.x;
    int cls = -1;
    if (g < s.Ntot)
        cls = init_node<M>(s, g, tt0);
    push_heavy_warp(s, g, cls, 0);
}

/* The end of a node's day: its E1 events (or its SSA error) and the state
 * written back. */
template <class M>
__device__ __forceinline__ void node_finish(const DevState &s, SsaLane<M> &ln, si_rng &r,
                                            long long g, int day, double tt,
                                            unsigned long long &fired)
{
    constexpr int NC = M::NC, NT = M::NT;
    if (s.crn_ctr) {
        /* common random numbers: the day's SSA draws came from the SSA's
         * own stream; the events draw from the node's */
        s.crn_ctr[g] = ln.c;
        r.s1 &= ~SI_CRN_S1;
        r.ctr = s.ctr[g];
    } else {
        r.ctr = ln.c;
    }
    r.have = 0;
    fired += ln.fired;
    if (s.day_max && ln.fired > *(volatile unsigned *) (s.day_max + day))
        atomicMax(s.day_max + day, ln.fired);       /* profiling: the day's busiest node */
    if (ln.err) {
        record_error(s, ln.err, PHASE_SSA, day, g, ln.err_tr, -1, ln.err_t, ln.err_rate);
    } else {
        int e_code = 0, e_idx = -1;
        const bool upd = node_e1<NC>(s, ln.u, (int) (g % s.Nn), day, r, g, tt, e_code, e_idx);
        if (upd)
            s.update[g] = 1;
        if (e_code)
            record_error(s, e_code, PHASE_E1, day, g, -1, e_idx, tt, 0);
    }
    store_u<NC>(s.u + g * NC, ln.u);
#pragma unroll
    for (int k = 0; k < NT; k++)
        s.t_rate[(size_t) k * s.Ntot + g] = ln.rate[k];
    s.sum_rate[g] = ln.sum;
    s.t_time[g] = ln.t;
    s.ctr[g] = r.ctr;
}

/* The first pass of a two-pass day, one ordinary node (not in the day's
 * heavy lists) per thread: a node whose day has no transition -- rate sum
 * 0, or a first waiting time that passes the end of the day -- finishes
 * here (its E1 events, state written back), with the warp's lanes in step;
 * a node with a transition is listed in s.active for k_ssa_e1, which draws
 * the same first waiting time again (same draw index) and steps it.  The
 * draws and comparisons are those of ssa_begin and ssa_step. */
template <class M>
__global__ void __launch_bounds__(256) k_quick(DevState s, int day, double tt, double next)
{
    constexpr int NC = M::NC;
    const long long g = blockIdx.x * (long long) blockDim.x + threadIdx.x;
    bool listed = false;
    if (g < s.Ntot && load_flag(s.err_day) >= day && s.heavy_mark[g] != day + 1 &&
        !job_over(s, g, day)) {
        const double sum = s.sum_rate[g], t = s.t_time[g];
        uint64_t c = s.crn_ctr ? s.crn_ctr[g] : s.ctr[g];
        si_rng r;
        {
            uint64_t seed, sid;
            stream_key(s, g, seed, sid);
            si_rng_init(&r, seed, sid, 0);
            if (s.crn_ctr)
                r.s1 |= SI_CRN_S1;      /* the SSA's own stream */
        }
        int err = 0;
        if (!si_finite_pos(sum)) {
            /* nothing fires (src/solvers/SimInf_solver_ssm.c:148-151) */
            if (!le_zero(si_double_bits(sum)))
                err = ERR_INVALID_RATE;
        } else {
            uint32_t p0, p1, p2, p3;
            philox_block(r, c >> 2, p0, p1, p2, p3);
            const double tau = si_div(si_neglog_u32(word_of(p0, p1, p2, p3, (uint32_t) c & 3u)), sum);
            if (tau + t >= next)
                c += 1;                         /* the waiting time's draw was used */
            else
                listed = true;
        }
        if (!listed) {
            if (s.crn_ctr) {
                /* the SSA stream's counter is done for the day; c becomes
                 * the node stream's, which the events draw from */
                s.crn_ctr[g] = c;
                c = s.ctr[g];
                r.s1 &= ~SI_CRN_S1;
            }
            if (err) {
                record_error(s, err, PHASE_SSA, day, g, -1, -1, t, sum);
            } else {
                const int node = (int) (g % s.Nn);
                if (s.e1_ptr[node] != s.e1_ptr[node + 1]) {
                    int u[NC];
                    load_u<NC>(s.u + g * NC, u);
                    r.ctr = c;
                    r.have = 0;
                    int e_code = 0, e_idx = -1;
                    if (node_e1<NC>(s, u, node, day, r, g, tt, e_code, e_idx)) {
                        s.update[g] = 1;
                        store_u<NC>(s.u + g * NC, u);
                    }
                    if (e_code)
                        record_error(s, e_code, PHASE_E1, day, g, -1, e_idx, tt, 0);
                    c = r.ctr;
                }
            }
            s.t_time[g] = next;
            s.ctr[g] = c;
        }
    }
    /* list the nodes with a transition, one atomic per warp */
    const unsigned FULL = 0xFFFFFFFFu;
    const unsigned m = __ballot_sync(FULL, listed);
    if (m) {
        const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
        unsigned long long base = 0;
        if (lane == leader)
            base = atomicAdd(&s.queue_next[4 + (day & 1)], (unsigned long long) __popc(m));
        base = __shfl_sync(FULL, base, leader);
        if (listed)
            s.active[base + __popc(m & ((1u << lane) - 1u))] = (int) g;
    }
}

/* One day of SSA and E1 events for every (replicate, node): a persistent
 * grid whose threads take nodes from the day's work queue, one node per
 * thread at a time.  The queue has two parts: the heavy nodes (rate sum >=
 * heavy_rate at the start of the day, heaviest class first) and then every
 * other node in index order.  Heavy nodes go out 32 to a warp, and a warp
 * that holds one takes nothing more until they are all done: the day lasts
 * as long as its longest chain, and work started beside it in the same
 * warp would stretch that chain.  Ordinary nodes go out lane by lane: a
 * thread whose node's day is over takes the next entry at once, so the
 * lanes of a warp keep stepping transitions instead of waiting for the
 * warp's busiest node.  One atomic per warp hands out the entries. */
template <class M, int MINB>
__global__ void __launch_bounds__(SSA_BLOCK, MINB) k_ssa_e1(DevState s, int day, double tt,
                                                         double next)
{
    constexpr int NC = M::NC, NT = M::NT, ND = M::ND;
    __shared__ int sS[NT * NC];
    __shared__ uint32_t sG[NT];
    load_model_smem<M>(s, sS, sG);
    const int par = day & 1, npar = (day + 1) & 1;
    if (blockIdx.x == 0 && threadIdx.x < HEAVY_CLASSES)
        s.heavy_count[npar * HEAVY_CLASSES + threadIdx.x] = 0;  /* filled by this day's pts */
    if (blockIdx.x == 0 && threadIdx.x < 2)
        s.queue_next[npar * 2 + threadIdx.x] = 0;
    if (blockIdx.x == 0 && threadIdx.x == 2)
        s.queue_next[4 + npar] = 0;                     /* filled by the next k_quick */
    unsigned long long fired = 0;
    if (load_flag(s.err_day) < day) {
        add_fired(s, fired);
        return;
    }
    int n[HEAVY_CLASSES];
    unsigned long long H = 0;
#pragma unroll
    for (int c = 0; c < HEAVY_CLASSES; c++) {
        n[c] = min(s.heavy_count[par * HEAVY_CLASSES + c], (int) MAX_HEAVY);
        H += (unsigned long long) n[c];
    }
    /* the ordinary part: every node in index order, or on two-pass days
     * the nodes k_quick listed */
    const unsigned long long Ntot = s.two_pass ? s.queue_next[4 + par]
                                               : (unsigned long long) s.Ntot;
    const int lane = threadIdx.x & 31;
    const unsigned FULL = 0xFFFFFFFFu;

    SsaLane<M> ln;
    si_rng r;
    long long g = -1;
    bool alive = true, need = true, done = false, heavy = false;
    bool heavy_left = H > 0;         /* warp-uniform: the heavy part may have entries */
    const double *v = nullptr, *ld = nullptr, *gd = nullptr;
    for (;;) {
        /* hand queue entries to the lanes without a node; while the
         * heaviest class lasts, only the first heavy_lanes lanes take them */
        unsigned want = __ballot_sync(FULL, alive && need);
        const bool holds_heavy = __any_sync(FULL, alive && !need && heavy);
        const bool from_heavy = heavy_left;
        if (from_heavy && s.heavy_lanes > 0 && s.heavy_lanes < 32 && want && !holds_heavy) {
            unsigned long long at = 0;
            if (lane == 0)
                at = *(volatile const unsigned long long *) &s.queue_next[par * 2];
            at = __shfl_sync(FULL, at, 0);
            if (at < (unsigned long long) n[0])
                want &= (1u << s.heavy_lanes) - 1u;
        }
        if (want && !holds_heavy) {
            const int leader = __ffs(want) - 1;
            unsigned long long base = 0;
            if (lane == leader)
                base = atomicAdd(&s.queue_next[par * 2 + (from_heavy ? 0 : 1)],
                                 (unsigned long long) __popc(want));
            base = __shfl_sync(FULL, base, leader);
            long long cand = -1;
            bool empty = false;
            if ((want >> lane) & 1u) {
                const unsigned long long pos = base + __popc(want & ((1u << lane) - 1u));
                if (from_heavy) {
                    if (pos < H) {
                        int idx = (int) pos, c = 0;
                        while (c < HEAVY_CLASSES - 1 && idx >= n[c]) {
                            idx -= n[c];
                            c++;
                        }
                        cand = s.heavy_list[(par * HEAVY_CLASSES + c) * MAX_HEAVY + idx];
                    } else {
                        empty = true;
                    }
                } else if (pos >= Ntot) {
                    alive = false;
                } else if (s.two_pass) {
                    cand = s.active[pos];
                } else if (s.heavy_mark[pos] != day + 1) {
                    cand = (long long) pos;     /* heavy ones come from the heavy part */
                }
                if (cand >= 0 && job_over(s, cand, day))
                    cand = -1;                  /* its model has run all its days */
            }
            if (from_heavy && __any_sync(FULL, empty))
                heavy_left = false;
            if (cand >= 0) {
                g = cand;
                heavy = from_heavy;
                const int node = (int) (g % s.Nn);
                load_u<NC>(s.u + g * NC, ln.u);
#pragma unroll
                for (int k = 0; k < NT; k++)
                    ln.rate[k] = s.t_rate[(size_t) k * s.Ntot + g];
                ln.sum = s.sum_rate[g];
                ln.t = s.t_time[g];
                ln.err = 0;
                ln.err_tr = -1;
                ln.err_t = 0.0;
                ln.err_rate = 0.0;
                ln.dc = si_recip_none();
                {
                    uint64_t seed, sid;
                    stream_key(s, g, seed, sid);
                    si_rng_init(&r, seed, sid, 0);
                    if (s.crn_ctr)
                        r.s1 |= SI_CRN_S1;      /* the SSA's own stream */
                }
                v = s.vA + g * ND;
                ld = s.ldata + (size_t) node * s.Nld;
                gd = gdata_of(s, g);
                done = ssa_begin<M>(ln, r, s.crn_ctr ? s.crn_ctr[g] : s.ctr[g], next);
                need = false;
            }
        }
        if (!__any_sync(FULL, alive))
            break;
        if (alive && !need) {
            if (done) {
                node_finish<M>(s, ln, r, g, day, tt, fired);
                need = true;
                heavy = false;
            } else {
                /* one step; a heavy warp has nothing else to do and runs
                 * its whole day, in batches of four steps where the rates
                 * do not read t */
                if constexpr (M::RATES_TIME_INVARIANT) {
                    if (heavy) {
                        ssa_run_day<M>(ln, r, next, v, ld, gd, sS, sG, s.max_fired);
                        done = true;
                    } else {
                        done = ssa_step<M>(ln, r, next, v, ld, gd, sS, sG, s.max_fired);
                    }
                } else {
                    do
                        done = ssa_step<M>(ln, r, next, v, ld, gd, sS, sG, s.max_fired);
                    while (heavy && !done);
                }
            }
        }
    }
    add_fired(s, fired);
}

/* One external transfer of one replicate (src/solvers/SimInf_solver.c:
 * 824-902): sample from the source, add to the destination (atomics: adds
 * into one destination commute within a wavefront), subtract from the
 * source (exclusive to this event within its wavefront). */
template <class M>
__device__ __forceinline__ void e2_apply(const DevState &s, const E2Rec &e, int rep, int day,
                                         double tt)
{
    constexpr int NC = M::NC;
    const long long gs = (long long) rep * s.Nn + e.src;
    const long long gd = (long long) rep * s.Nn + e.dst;
    int uu[NC], ind[NC];
    for (int c = 0; c < NC; c++)
        uu[c] = s.u[gs * NC + c];
    si_rng r;
    {
        uint64_t seed, sid;
        stream_key(s, gs, seed, sid);
        si_rng_init(&r, seed, sid, s.ctr[gs]);
    }
    int err = sample_select<NC>(s, uu, e.select, e.n, e.proportion, ind, &r);
    s.ctr[gs] = r.ctr;
    if (err) {
        record_error(s, err, PHASE_E2, day, gs, -1, e.index, tt, 0);
        return;
    }
    for (int k = s.jcE[e.select]; k < s.jcE[e.select + 1]; k++) {
        const int jj = s.irE[k];
        int dj = jj;
        if (e.shift >= 0) {
            if (!s.hasN) {
                record_error(s, ERR_EVENTS_N, PHASE_E2, day, gs, -1, e.index, tt, 0);
                return;
            }
            const int ll = s.Nshift[e.shift * NC + jj];
            if (jj + ll < 0 || jj + ll >= NC) {
                record_error(s, ERR_SHIFT_OUT_OF_BOUNDS, PHASE_E2, day, gs, -1, e.index, tt, 0);
                return;
            }
            dj = jj + ll;
        }
        if (ind[jj]) {
            const int old = atomicAdd(&s.u[gd * NC + dj], ind[jj]);
            if (old + ind[jj] < 0) {
                record_error(s, ERR_NEGATIVE_STATE, PHASE_E2, day, gs, -1, e.index, tt, 0);
                return;
            }
            /* The source is exclusive to this event within the wave; a
             * self-transfer reads back its own atomic add. */
            const int nv = s.u[gs * NC + jj] - ind[jj];
            s.u[gs * NC + jj] = nv;
            if (nv < 0) {
                record_error(s, ERR_NEGATIVE_STATE, PHASE_E2, day, gs, -1, e.index, tt, 0);
                return;
            }
        }
    }
    s.update[gd] = 1;
    s.update[gs] = 1;
}

template <class M>
__global__ void __launch_bounds__(512) k_e2_wave(DevState s, const E2Rec *ev, int count, int day,
                                                 double tt)
{
    const long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x;
    if (i >= (long long) count * s.Nrep)
        return;
    if (load_flag(s.err_day) < day || load_flag(s.err_day_pre_e2) <= day)
        return;
    const int rep = (int) (i / count);
    e2_apply<M>(s, ev[i - (long long) rep * count], rep, day, tt);
}

/* A day's last, small wavefronts in one block, in order, a barrier between
 * two (the block's writes before it are visible to the block after it):
 * one launch instead of one per wavefront.  Each holds at most
 * E2_TAIL_ITEMS = 1024 events x replicates, one per thread. */
template <class M>
__global__ void __launch_bounds__(1024) k_e2_tail(DevState s, const E2Rec *ev, E2Tail tail,
                                                  int day, double tt)
{
    if (load_flag(s.err_day) < day || load_flag(s.err_day_pre_e2) <= day)
        return;                                     /* the same for every thread */
    for (int w = 0; w < tail.n; w++) {
        const int count = tail.count[w];
        const E2Rec *wev = ev + tail.off[w];
        const long long items = (long long) count * s.Nrep;
        for (long long i = threadIdx.x; i < items; i += blockDim.x) {
            const int rep = (int) (i / count);
            e2_apply<M>(s, wev[i - (long long) rep * count], rep, day, tt);
        }
        __syncthreads();
    }
}

/* Batches: node g's share of its job's prevalence sums at columns c0 ..
 * c1 - 1 (integer sums, so the order of the additions does not matter). */
template <int NC>
__device__ __forceinline__ void add_prevalence(const DevState &s, long long g, const int (&u)[NC],
                                               int c0, int c1)
{
    const int j = s.job_of[g];
    unsigned long long num = 0, den = 0;
#pragma unroll
    for (int c = 0; c < NC; c++) {
        const unsigned long long x = (unsigned long long) (long long) u[c];
        if (s.prev_num_mask & (1u << c))
            num += x;
        if (s.prev_den_mask & (1u << c))
            den += x;
    }
    const int tl = s.job_tlen[j];
    for (int col = c0; col < c1 && col < tl; col++) {
        unsigned long long *p = s.prev + 2 * (s.job_col0[j] + col);
        atomicAdd(p, num);
        atomicAdd(p + 1, den);
    }
}

enum { NEEDS_REFRESH = -2 };

/* k_pts_store for one (replicate, node): post-time-step function, U/V
 * columns, prevalence.  Returns NEEDS_REFRESH when its rates must be
 * recomputed (an event touched it, or the post-time-step function changed
 * v), else its heavy class on the next day. */
template <class M>
__device__ __forceinline__ int pts_node(const DevState &s, long long g, int day, double tt,
                                        int c0, int c1, const double *v_in, double *v_out)
{
    constexpr int NC = M::NC, ND = M::ND;
    const int rep = (int) (g / s.Nn), node = (int) (g % s.Nn);
    int u[NC];
    load_u<NC>(s.u + g * NC, u);
    const double *vi = v_in + g * ND;
    double *vo = v_out + g * ND;
    const double *ld = s.ldata + (size_t) node * s.Nld;
    const double *gd = gdata_of(s, g);
    /* a post-time-step function that reads other nodes (by offsets from
     * its node, src/models/SISe_sp.c:127-134) gets the node's place in the
     * replicate's arrays; every node's external transfers are done */
    const int rc = M::PTS_LOCAL ? M::pts(vo, u, vi, ld, gd, node, tt)
                                : M::pts(vo, s.u + g * NC, vi, ld, gd, node, tt);
    store_columns<NC, ND>(s, rep, node, u, vo, c0, c1);
    if (s.prev && c1 > c0)
        add_prevalence<NC>(s, g, u, c0, c1);
    if (rc < 0)
        record_error(s, rc, PHASE_PTS, day, g, -1, -1, tt, 0);
    else if (rc > 0 || s.update[g])
        return NEEDS_REFRESH;
    return job_over(s, g, day + 1) ? -1 : heavy_class<M>(s, s.sum_rate[g]);
}

/* The rate refresh of the day's end (src/solvers/SimInf_solver_ssm.c:
 * 285-306): every rate recomputed with v_new at tt, their changes added to
 * the rate sum in transition order.  Returns the heavy class on the next
 * day. */
template <class M>
__device__ __forceinline__ int refresh_node(const DevState &s, long long g, int day, double tt,
                                            const double *v_out)
{
    constexpr int NC = M::NC, NT = M::NT, ND = M::ND;
    const int node = (int) (g % s.Nn);
    int u[NC];
    load_u<NC>(s.u + g * NC, u);
    const double *vo = v_out + g * ND;
    const double *ld = s.ldata + (size_t) node * s.Nld;
    const double *gd = gdata_of(s, g);
    si_recip dc = si_recip_none();
    double delta = 0.0;
#pragma unroll
    for (int k = 0; k < NT; k++) {
        const double old = s.t_rate[(size_t) k * s.Ntot + g];
        const double nr = M::rate(k, u, vo, ld, gd, tt, dc);
        s.t_rate[(size_t) k * s.Ntot + g] = nr;
        delta += nr - old;
        if (si_bad_rate(nr))
            record_error(s, ERR_INVALID_RATE, PHASE_PTS, day, g, k, -1, tt, nr);
    }
    s.sum_rate[g] += delta;
    s.update[g] = 0;
    return job_over(s, g, day + 1) ? -1 : heavy_class<M>(s, s.sum_rate[g]);
}

template <class M>
__global__ void __launch_bounds__(256) k_pts_store(DevState s, int day, double tt, int c0, int c1,
                                                   const double *v_in, double *v_out)
{
    /* The block's nodes whose rates need a refresh are gathered first and
     * refreshed by the block's first threads: the refresh is FP64 work,
     * and the FP64 pipe issues a warp instruction at the same cost however
     * few of its lanes are active. */
    __shared__ int listed[256];
    __shared__ int nlisted;
    if (threadIdx.x == 0)
        nlisted = 0;
    __syncthreads();
    const long long g0 = blockIdx.x * (long long) blockDim.x;
    const long long g = g0 + threadIdx.x;
    int cls = -1;
    if (g < s.Ntot && load_flag(s.err_day) >= day && !job_over(s, g, day)) {
        cls = pts_node<M>(s, g, day, tt, c0, c1, v_in, v_out);
        if (cls == NEEDS_REFRESH) {
            listed[atomicAdd(&nlisted, 1)] = threadIdx.x;
            cls = -1;
        }
    }
    push_heavy_warp(s, g, cls, day + 1);
    __syncthreads();
    long long gr = -1;
    int cls2 = -1;
    if (threadIdx.x < nlisted) {
        gr = g0 + listed[threadIdx.x];
        cls2 = refresh_node<M>(s, gr, day, tt, v_out);
    }
    push_heavy_warp(s, gr, cls2, day + 1);
}

/* ------------------------------------------------------------------ */
/* All-events method (src/solvers/SimInf_solver_aem.c), one thread per   */
/* node.  Transition j of node g draws from its own stream, keyed (seed, */
/* AEM_SID | (g * Nt + j)); the next event is the smallest event time,   */
/* the lowest transition among equal times.                              */
/* ------------------------------------------------------------------ */
#define AEM_SID (1ULL << 63)

__device__ __forceinline__ double aem_neglog(uint64_t seed, long long g, int Nt, int j,
                                             uint64_t &ctr)
{
    si_rng r;
    si_rng_init(&r, seed, AEM_SID | ((uint64_t) g * (uint64_t) Nt + (uint64_t) j), ctr);
    const double x = si_neglog_u32(si_next_u32(&r));
    ctr = r.ctr;
    return x;
}

/* calcTimes (src/solvers/SimInf_solver_aem.c:52-75), with its three
 * quotients -- a new waiting time -log(u) / new_rate, a sleeping time
 * inf / new_rate, a rescaling old_rate / new_rate -- formed by one division
 * (one copy of the division's code in the kernel).  Addition commutes
 * exactly, so tt + q and q + tt are the same double. */
__device__ __forceinline__ void aem_calc_times(double &time, double &inf, double tt,
                                               double old_rate, double new_rate, uint64_t seed,
                                               long long g, int Nt, int j, uint64_t &ctr)
{
    const double oldtime = time;
    int kind;                           /* 0: q + tt, 1: q * (oldtime - tt) + tt, 2: none */
    bool draw = false;
    double num = 0.0;
    if (isinf(oldtime)) {
        if (inf == 0.0) {
            draw = true;
            kind = 0;
        } else if (new_rate > 0.0) {
            num = inf;
            kind = 0;
        } else {
            kind = 2;
        }
    } else if (new_rate >= DBL_MIN) {
        if (oldtime == tt) {
            draw = true;
            kind = 0;
        } else {
            num = old_rate;
            kind = 1;
        }
    } else {
        inf = (oldtime - tt) * old_rate;
        time = si_bits_double(0x7FF0000000000000ULL);
        return;
    }
    if (kind == 2)
        return;
    if (draw)
        num = aem_neglog(seed, g, Nt, j, ctr);
    const double q = si_div(num, new_rate);
    time = kind == 0 ? q + tt : (q * (oldtime - tt)) + tt;
}

/* Initial rates and event times (src/solvers/SimInf_solver_aem.c:113-158). */
template <class M>
__device__ __forceinline__ int aem_init_node(const DevState &s, long long g, double tt0);

template <class M>
__global__ void k_aem_init(DevState s, double tt0)
{
    const long long g = blockIdx.x * (long long) blockDim.x + threadIdx.x;
    int cls = -1;
    if (g < s.Ntot)
        cls = aem_init_node<M>(s, g, tt0);
    push_heavy_warp(s, g, cls, 0);
}

/* k_aem_init for one node; returns its heavy class on day 0 (from the sum
 * of its rates, for the order of the work queue only). */
template <class M>
__device__ __forceinline__ int aem_init_node(const DevState &s, long long g, double tt0)
{
    constexpr int NC = M::NC, NT = M::NT, ND = M::ND;
    const int node = (int) (g % s.Nn);
    int u[NC];
    load_u<NC>(s.u + g * NC, u);
    const double *v = s.vA + g * ND;
    const double *ld = s.ldata + (size_t) node * s.Nld;
    si_recip dc = si_recip_none();
    double sum = 0.0;
#pragma unroll
    for (int j = 0; j < NT; j++) {
        const double rate = M::rate(j, u, v, ld, gdata_of(s, g), tt0, dc);
        const size_t k = (size_t) j * s.Ntot + g;
        s.t_rate[k] = rate;
        if (!isfinite(rate) || rate < 0.0)
            record_error(s, ERR_INVALID_RATE, PHASE_INIT, 0, g, j, -1, tt0, rate);
        uint64_t c = 0;
        double t = si_div(aem_neglog(s.seed, g, NT, j, c), rate) + tt0;
        if (t <= 0.0)
            t = si_bits_double(0x7FF0000000000000ULL);
        s.react_time[k] = t;
        s.react_inf[k] = 0.0;
        s.react_ctr[k] = c;
        sum += rate;
    }
    s.t_time[g] = tt0;
    s.ctr[g] = 0;
    s.update[g] = 0;
    return heavy_class<M>(s, sum);
}

/* The state of one node's aem day, held by one thread. */
template <class M>
struct AemNode {
    int u[M::NC];
    double rate[M::NT], time[M::NT], inf[M::NT];
    uint64_t ctr[M::NT];
    int err, err_tr;
    double err_t, err_rate;
};

/* Rate j refreshed at time t (rate functions) and its event time at tc
 * (calcTimes), recording an invalid rate. */
template <class M>
__device__ __forceinline__ void aem_refresh(const DevState &s, AemNode<M> &a, long long g, int j,
                                            const double *v, const double *ld, const double *gd,
                                            double t, double tc, si_recip &dc)
{
    const double old = a.rate[j];
    const double nr = M::rate(j, a.u, v, ld, gd, t, dc);
    a.rate[j] = nr;
    if (si_bad_rate(nr)) {
        a.err = ERR_INVALID_RATE;
        a.err_tr = j;
        a.err_t = t;
        a.err_rate = nr;
    }
    aem_calc_times(a.time[j], a.inf[j], tc, old, nr, s.seed, g, M::NT, j, a.ctr[j]);
}

/* One aem step of a node at its day (src/solvers/SimInf_solver_aem.c:
 * 179-307): the transition with the smallest event time fires, then its
 * dependents in G's column (row order) and itself get new rates and event
 * times.  Returns true when the next event falls past the day's end. */
template <class M>
__device__ __forceinline__ bool aem_step(const DevState &s, AemNode<M> &a, long long g,
                                         double next, const double *v, const double *ld,
                                         const double *gd, const int *sS, const uint32_t *sG,
                                         unsigned &fired, si_recip &dc)
{
    constexpr int NC = M::NC, NT = M::NT;
    int tr = 0;
    double t = a.time[0];
#pragma unroll
    for (int j = 1; j < NT; j++)
        if (a.time[j] < t) {
            t = a.time[j];
            tr = j;
        }
    if (isinf(t) || t >= next)
        return true;
    if (++fired > s.max_fired) {
        a.err = ERR_TIMEOUT;
        a.err_tr = tr;
        a.err_t = t;
        return true;
    }
    int neg = 0;
#pragma unroll
    for (int c = 0; c < NC; c++) {
        const int d = sS[tr * NC + c];
        a.u[c] += d;
        neg |= (d != 0) & (a.u[c] < 0);
    }
    if (neg) {
        a.err = ERR_NEGATIVE_STATE;
        a.err_tr = tr;
        a.err_t = t;
        a.err_rate = 0.0;
    }
    const uint32_t gm = sG[tr];
#pragma unroll
    for (int j = 0; j < NT; j++)
        if (j != tr && (gm & (1u << j)))
            aem_refresh<M>(s, a, g, j, v, ld, gd, t, t, dc);
#pragma unroll
    for (int j = 0; j < NT; j++)
        if (j == tr)
            aem_refresh<M>(s, a, g, j, v, ld, gd, t, t, dc);
    return false;
}

/* The end of a node's aem day: its error, or its E1 events; the state
 * written back with t = next. */
template <class M>
__device__ __forceinline__ void aem_finish(const DevState &s, AemNode<M> &a, long long g, int day,
                                           double tt, double next)
{
    constexpr int NC = M::NC, NT = M::NT;
    si_rng r;
    {
        uint64_t seed, sid;
        stream_key(s, g, seed, sid);
        si_rng_init(&r, seed, sid, s.ctr[g]);
    }
    if (a.err) {
        record_error(s, a.err, PHASE_SSA, day, g, a.err_tr, -1, a.err_t, a.err_rate);
    } else {
        int e_code = 0, e_idx = -1;
        if (node_e1<NC>(s, a.u, (int) (g % s.Nn), day, r, g, tt, e_code, e_idx))
            s.update[g] = 1;
        if (e_code)
            record_error(s, e_code, PHASE_E1, day, g, -1, e_idx, tt, 0);
    }
    store_u<NC>(s.u + g * NC, a.u);
#pragma unroll
    for (int j = 0; j < NT; j++) {
        const size_t k = (size_t) j * s.Ntot + g;
        s.t_rate[k] = a.rate[j];
        s.react_time[k] = a.time[j];
        s.react_inf[k] = a.inf[j];
        s.react_ctr[k] = a.ctr[j];
    }
    s.t_time[g] = next;
    s.ctr[g] = r.ctr;
}

/* One day of every node under the all-events method, then its E1 events:
 * a persistent grid fed by the day's work queue, as k_ssa_e1 -- first the
 * heavy nodes (rate sum >= heavy_rate at the start of the day, listed by
 * the previous day's end, heaviest class first), 32 to a warp that runs
 * them to the day's end in a tight loop, then every other node in index
 * order, lane by lane, a lane whose node's day is over taking the next
 * node at once.  One atomic per warp hands out the entries. */
template <class M>
__global__ void __launch_bounds__(SSA_BLOCK, M::NT <= 4 ? 4 : 3) k_aem_day(DevState s, int day,
                                                                          double tt, double next)
{
    constexpr int NC = M::NC, NT = M::NT, ND = M::ND;
    __shared__ int sS[NT * NC];
    __shared__ uint32_t sG[NT];
    load_model_smem<M>(s, sS, sG);
    const int par = day & 1, npar = (day + 1) & 1;
    if (blockIdx.x == 0 && threadIdx.x < HEAVY_CLASSES)
        s.heavy_count[npar * HEAVY_CLASSES + threadIdx.x] = 0;  /* filled by this day's end */
    if (blockIdx.x == 0 && threadIdx.x < 2)
        s.queue_next[npar * 2 + threadIdx.x] = 0;
    unsigned long long fired = 0;
    if (load_flag(s.err_day) < day) {
        add_fired(s, fired);
        return;
    }
    int n[HEAVY_CLASSES];
    unsigned long long H = 0;
#pragma unroll
    for (int c = 0; c < HEAVY_CLASSES; c++) {
        n[c] = min(s.heavy_count[par * HEAVY_CLASSES + c], (int) MAX_HEAVY);
        H += (unsigned long long) n[c];
    }
    const unsigned long long Ntot = (unsigned long long) s.Ntot;
    const int lane = threadIdx.x & 31;
    const unsigned FULL = 0xFFFFFFFFu;
    AemNode<M> a;
    long long g = -1;
    bool alive = true, need = true, heavy = false;
    bool heavy_left = H > 0;            /* warp-uniform: the heavy part may have entries */
    unsigned nfired = 0;
    const double *v = nullptr, *ld = nullptr, *gd = nullptr;
    si_recip dc = si_recip_none();
    for (;;) {
        const unsigned want = __ballot_sync(FULL, alive && need);
        const bool holds_heavy = __any_sync(FULL, alive && !need && heavy);
        const bool from_heavy = heavy_left;
        if (want && !holds_heavy) {
            const int leader = __ffs(want) - 1;
            unsigned long long base = 0;
            if (lane == leader)
                base = atomicAdd(&s.queue_next[par * 2 + (from_heavy ? 0 : 1)],
                                 (unsigned long long) __popc(want));
            base = __shfl_sync(FULL, base, leader);
            long long cand = -1;
            bool empty = false;
            if (alive && need) {
                const unsigned long long pos = base + __popc(want & ((1u << lane) - 1u));
                if (from_heavy) {
                    if (pos < H) {
                        int idx = (int) pos, c = 0;
                        while (c < HEAVY_CLASSES - 1 && idx >= n[c]) {
                            idx -= n[c];
                            c++;
                        }
                        cand = s.heavy_list[(par * HEAVY_CLASSES + c) * MAX_HEAVY + idx];
                    } else {
                        empty = true;
                    }
                } else if (pos >= Ntot) {
                    alive = false;
                } else if (s.heavy_mark[pos] != day + 1) {
                    cand = (long long) pos;     /* heavy ones come from the heavy part */
                }
            }
            if (from_heavy && __any_sync(FULL, empty))
                heavy_left = false;
            if (cand >= 0) {
                g = cand;
                heavy = from_heavy;
                const int node = (int) (g % s.Nn);
                load_u<NC>(s.u + g * NC, a.u);
#pragma unroll
                for (int j = 0; j < NT; j++) {
                    const size_t k = (size_t) j * s.Ntot + g;
                    a.rate[j] = s.t_rate[k];
                    a.time[j] = s.react_time[k];
                    a.inf[j] = s.react_inf[k];
                    a.ctr[j] = s.react_ctr[k];
                }
                a.err = 0;
                a.err_tr = -1;
                a.err_t = 0.0;
                a.err_rate = 0.0;
                v = s.vA + g * ND;
                ld = s.ldata + (size_t) node * s.Nld;
                gd = gdata_of(s, g);
                dc = si_recip_none();
                nfired = 0;
                need = false;
            }
        }
        if (!__any_sync(FULL, alive))
            break;
        if (alive && !need) {
            /* one event; a heavy warp has nothing else to do and runs its
             * nodes' whole days in this loop */
            bool done;
            do
                done = aem_step<M>(s, a, g, next, v, ld, gd, sS, sG, nfired, dc);
            while (heavy && !done);
            if (done) {
                aem_finish<M>(s, a, g, day, tt, next);
                fired += nfired;
                need = true;
                heavy = false;
            }
        }
    }
    add_fired(s, fired);
}

/* The day's end (src/solvers/SimInf_solver_aem.c:329-381): post-time-step
 * function, U/V columns, and for a node an event touched or whose v
 * changed, every rate recomputed with v_new at tt and its event time
 * rescaled at the node's time (the end of the day). */
template <class M>
__device__ __forceinline__ int aem_pts_node(const DevState &s, long long g, int day, double tt,
                                            int c0, int c1, const double *v_in, double *v_out);

template <class M>
__global__ void __launch_bounds__(256) k_aem_pts(DevState s, int day, double tt, int c0, int c1,
                                                 const double *v_in, double *v_out)
{
    const long long g = blockIdx.x * (long long) blockDim.x + threadIdx.x;
    int cls = -1;
    if (g < s.Ntot && load_flag(s.err_day) >= day)
        cls = aem_pts_node<M>(s, g, day, tt, c0, c1, v_in, v_out);
    push_heavy_warp(s, g, cls, day + 1);
}

/* k_aem_pts for one node; returns its heavy class on the next day. */
template <class M>
__device__ __forceinline__ int aem_pts_node(const DevState &s, long long g, int day, double tt,
                                            int c0, int c1, const double *v_in, double *v_out)
{
    constexpr int NC = M::NC, NT = M::NT, ND = M::ND;
    const int rep = (int) (g / s.Nn), node = (int) (g % s.Nn);
    AemNode<M> a;
    load_u<NC>(s.u + g * NC, a.u);
    const double *vi = v_in + g * ND;
    double *vo = v_out + g * ND;
    const double *ld = s.ldata + (size_t) node * s.Nld;
    const double *gd = gdata_of(s, g);
    const int rc = M::PTS_LOCAL ? M::pts(vo, a.u, vi, ld, gd, node, tt)
                                : M::pts(vo, s.u + g * NC, vi, ld, gd, node, tt);
    store_columns<NC, ND>(s, rep, node, a.u, vo, c0, c1);
    if (rc < 0) {
        record_error(s, rc, PHASE_PTS, day, g, -1, -1, tt, 0);
        return -1;
    }
    double sum = 0.0;
    if (rc == 0 && !s.update[g]) {
#pragma unroll
        for (int j = 0; j < NT; j++)
            sum += s.t_rate[(size_t) j * s.Ntot + g];
        return heavy_class<M>(s, sum);
    }
    const double tc = s.t_time[g];
#pragma unroll
    for (int j = 0; j < NT; j++) {
        const size_t k = (size_t) j * s.Ntot + g;
        a.rate[j] = s.t_rate[k];
        a.time[j] = s.react_time[k];
        a.inf[j] = s.react_inf[k];
        a.ctr[j] = s.react_ctr[k];
    }
    a.err = 0;
    si_recip dc = si_recip_none();
#pragma unroll
    for (int j = 0; j < NT; j++) {
        aem_refresh<M>(s, a, g, j, vo, ld, gd, tt, tc, dc);
        if (a.err) {
            record_error(s, ERR_INVALID_RATE, PHASE_PTS, day, g, j, -1, tt, a.err_rate);
            a.err = 0;
        }
    }
#pragma unroll
    for (int j = 0; j < NT; j++) {
        const size_t k = (size_t) j * s.Ntot + g;
        s.t_rate[k] = a.rate[j];
        s.react_time[k] = a.time[j];
        s.react_inf[k] = a.inf[j];
        s.react_ctr[k] = a.ctr[j];
        sum += a.rate[j];
    }
    s.update[g] = 0;
    return heavy_class<M>(s, sum);
}

/* Whole horizon of one (replicate, node) in one thread: valid when no
 * external transfer couples nodes and the post-time-step function reads
 * only its own node. */
template <class M>
__global__ void __launch_bounds__(256, M::NT <= 4 ? 2 : 1) k_horizon(DevState s, const DayInfo *days, int ndays)
{
    if (s.pf_days)
        days = s.pf_days + (size_t) *s.pf_interval * s.pf_days_stride;
    constexpr int NC = M::NC, NT = M::NT, ND = M::ND;
    __shared__ int sS[NT * NC];
    __shared__ uint32_t sG[NT];
    load_model_smem<M>(s, sS, sG);
    const long long g = blockIdx.x * (long long) blockDim.x + threadIdx.x;
    unsigned long long fired = 0;
    if (g < s.Ntot) {
        const int rep = (int) (g / s.Nn), node = (int) (g % s.Nn);
        SsaLane<M> ln;
        load_u<NC>(s.u + g * NC, ln.u);
#pragma unroll
        for (int k = 0; k < NT; k++)
            ln.rate[k] = s.t_rate[(size_t) k * s.Ntot + g];
        ln.sum = s.sum_rate[g];
        ln.t = s.t_time[g];
        ln.dc = si_recip_none();
        si_rng r;
        uint64_t c_other = 0;       /* common random numbers: the other stream's counter */
        {
            uint64_t seed, sid;
            stream_key(s, g, seed, sid);
            if (s.crn_ctr) {
                /* r holds the SSA's own stream; the events switch to the node's */
                si_rng_init(&r, seed, sid, s.crn_ctr[g]);
                r.s1 |= SI_CRN_S1;
                c_other = s.ctr[g];
            } else {
                si_rng_init(&r, seed, sid, s.ctr[g]);
            }
        }
        double *v = s.vA + g * ND, *vn = s.vB + g * ND;
        const double *ld = s.ldata + (size_t) node * s.Nld;
        const double *gd = gdata_of(s, g);
        for (int d = 0; d < ndays; d++) {
            if (load_flag(s.err_day) < d)
                break;
            const DayInfo di = days[d];
            ln.err = 0;
            ln.err_tr = -1;
            ln.err_t = 0.0;
            ln.err_rate = 0.0;
            fired += ssa_day<M>(ln, r, di.next, v, ld, gd, sS, sG, s.max_fired);
            if (ln.err) {
                record_error(s, ln.err, PHASE_SSA, d, g, ln.err_tr, -1, ln.err_t, ln.err_rate);
                break;
            }
            int e_code = 0, e_idx = -1;
            if (s.crn_ctr) {
                const uint64_t t = r.ctr;   /* to the node's stream */
                r.ctr = c_other;
                c_other = t;
                r.s1 ^= SI_CRN_S1;
                r.have = 0;
            }
            bool upd = false;
            if constexpr (NC <= 2) {
                if (s.e1_ptr[node] != s.e1_ptr[node + 1])
                    upd = node_e1_call<NC>(s, ln.u, node, d, r, g, di.tt, e_code, e_idx);
            } else {
                upd = node_e1<NC>(s, ln.u, node, d, r, g, di.tt, e_code, e_idx);
            }
            if (s.crn_ctr) {
                const uint64_t t = r.ctr;   /* back to the SSA's */
                r.ctr = c_other;
                c_other = t;
                r.s1 ^= SI_CRN_S1;
                r.have = 0;
            }
            if (e_code) {
                record_error(s, e_code, PHASE_E1, d, g, -1, e_idx, di.tt, 0);
                break;
            }
            const int rc = M::pts(vn, ln.u, v, ld, gd, node, di.tt);
            if (rc < 0) {
                record_error(s, rc, PHASE_PTS, d, g, -1, -1, di.tt, 0);
                break;
            }
            if (rc > 0 || upd) {
                double delta = 0.0;
                bool bad = false;
#pragma unroll
                for (int k = 0; k < NT; k++) {
                    const double old = ln.rate[k];
                    const double nr = M::rate(k, ln.u, vn, ld, gd, di.tt, ln.dc);
                    ln.rate[k] = nr;
                    delta += nr - old;
                    if (!isfinite(nr) || nr < 0.0) {
                        record_error(s, ERR_INVALID_RATE, PHASE_PTS, d, g, k, -1, di.tt, nr);
                        bad = true;
                    }
                }
                ln.sum += delta;
                if (bad)
                    break;
            }
            store_columns<NC, ND>(s, rep, node, ln.u, vn, di.c0, di.c1);
            double *tmp = v;
            v = vn;
            vn = tmp;
        }
        store_u<NC>(s.u + g * NC, ln.u);
#pragma unroll
        for (int k = 0; k < NT; k++)
            s.t_rate[(size_t) k * s.Ntot + g] = ln.rate[k];
        s.sum_rate[g] = ln.sum;
        s.t_time[g] = ln.t;
        if (s.crn_ctr) {
            s.crn_ctr[g] = r.ctr;
            s.ctr[g] = c_other;
        } else {
            s.ctr[g] = r.ctr;
        }
    }
    add_fired(s, fired);
}

/* ------------------------------------------------------------------ */
/* Launchers, one table per model.                                      */
/* ------------------------------------------------------------------ */

static inline unsigned blocks_for(long long n, int threads)
{
    return (unsigned) ((n + threads - 1) / threads);
}

template <class M>
struct Launch {
    static cudaError_t init(const DevState &s, double tt0, cudaStream_t st)
    {
        k_init<M><<<blocks_for(s.Ntot, 256), 256, 0, st>>>(s, tt0);
        return cudaGetLastError();
    }
    static cudaError_t horizon(const DevState &s, const DayInfo *days, int ndays, cudaStream_t st)
    {
        k_horizon<M><<<blocks_for(s.Ntot, 256), 256, 0, st>>>(s, days, ndays);
        return cudaGetLastError();
    }
    /* k_ssa_e1 is persistent: as many blocks as can be resident at once
     * (looked up once per model), fewer for small models. */
    /* The SSA kernel's two register budgets: blocks of SSA_BLOCK threads
     * resident per SM that __launch_bounds__ asks for (the default keeps
     * larger models within their registers; the other trades warps for
     * registers). */
    static constexpr int SSA_MINB0 = M::NT <= 4 ? 4 : 3;
    static constexpr int SSA_MINB1 = M::NT <= 4 ? 3 : 2;
    template <int MINB>
    static int ssa_resident_blocks()
    {
        static int blocks = 0;
        if (!blocks) {
            int dev = 0, nsm = 1, per = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_ssa_e1<M, MINB>, SSA_BLOCK, 0);
            blocks = nsm * (per > 0 ? per : 1);
        }
        return blocks;
    }
    template <int MINB>
    static cudaError_t ssa_e1_with(const DevState &s, int day, double tt, double next,
                                   cudaStream_t st)
    {
        const long long need = (long long) blocks_for(s.Ntot, SSA_BLOCK);
        const int resident = ssa_resident_blocks<MINB>();
        const int grid = (int) (need < resident ? need : resident);
        k_ssa_e1<M, MINB><<<grid, SSA_BLOCK, 0, st>>>(s, day, tt, next);
        return cudaGetLastError();
    }
    static cudaError_t quick(const DevState &s, int day, double tt, double next, cudaStream_t st)
    {
        k_quick<M><<<blocks_for(s.Ntot, 256), 256, 0, st>>>(s, day, tt, next);
        return cudaGetLastError();
    }
    static cudaError_t ssa_e1(const DevState &s, int day, double tt, double next, cudaStream_t st)
    {
        return s.ssa_variant == 1 ? ssa_e1_with<SSA_MINB1>(s, day, tt, next, st)
                                  : ssa_e1_with<SSA_MINB0>(s, day, tt, next, st);
    }
    static cudaError_t e2_tail(const DevState &s, const E2Rec *ev, const E2Tail &tail, int day,
                               double tt, cudaStream_t st)
    {
        k_e2_tail<M><<<1, 1024, 0, st>>>(s, ev, tail, day, tt);
        return cudaGetLastError();
    }
    static cudaError_t e2_wave(const DevState &s, const E2Rec *ev, int count, int day, double tt,
                               cudaStream_t st)
    {
        const long long n = (long long) count * s.Nrep;
        if (n == 0)
            return cudaSuccess;
        const int b = (s.wave_block == 128 || s.wave_block == 512) ? s.wave_block : 256;
        k_e2_wave<M><<<blocks_for(n, b), b, 0, st>>>(s, ev, count, day, tt);
        return cudaGetLastError();
    }
    static cudaError_t pts_store(const DevState &s, int day, double tt, int c0, int c1,
                                 const double *v_in, double *v_out, cudaStream_t st)
    {
        k_pts_store<M><<<blocks_for(s.Ntot, 256), 256, 0, st>>>(s, day, tt, c0, c1, v_in, v_out);
        return cudaGetLastError();
    }
    static cudaError_t aem_init(const DevState &s, double tt0, cudaStream_t st)
    {
        k_aem_init<M><<<blocks_for(s.Ntot, 256), 256, 0, st>>>(s, tt0);
        return cudaGetLastError();
    }
    static int aem_resident_blocks()
    {
        static int blocks = 0;
        if (!blocks) {
            int dev = 0, nsm = 1, per = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_aem_day<M>, SSA_BLOCK, 0);
            blocks = nsm * (per > 0 ? per : 1);
        }
        return blocks;
    }
    static cudaError_t aem_day(const DevState &s, int day, double tt, double next, cudaStream_t st)
    {
        const long long need = (long long) blocks_for(s.Ntot, SSA_BLOCK);
        const int grid = (int) (need < aem_resident_blocks() ? need : aem_resident_blocks());
        k_aem_day<M><<<grid, SSA_BLOCK, 0, st>>>(s, day, tt, next);
        return cudaGetLastError();
    }
    static cudaError_t aem_pts(const DevState &s, int day, double tt, int c0, int c1,
                               const double *v_in, double *v_out, cudaStream_t st)
    {
        k_aem_pts<M><<<blocks_for(s.Ntot, 256), 256, 0, st>>>(s, day, tt, c0, c1, v_in, v_out);
        return cudaGetLastError();
    }
    static const Launchers *table()
    {
        static const Launchers t = {M::NC, M::NT, M::ND, M::NGD, M::PTS_LOCAL,
                                    M::RATES_TIME_INVARIANT,
                                    init, horizon, quick, ssa_e1, e2_wave, pts_store,
                                    aem_init, aem_day, aem_pts, e2_tail};
        return &t;
    }
};

}  // namespace siminf

#endif
