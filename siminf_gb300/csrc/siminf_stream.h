/*
 * siminf_stream.h -- the random source of the solver, shared by the CUDA
 * kernels and by host C code.
 *
 * The reference solver draws from one GSL generator per OpenMP thread
 * (src/solvers/SimInf_solver.c:474-477) through three calls:
 * gsl_rng_uniform_pos (src/solvers/SimInf_solver_ssm.c:155,165,
 * src/solvers/SimInf_solver.c:184,298), gsl_ran_binomial
 * (src/solvers/SimInf_solver.c:98,274) and gsl_ran_hypergeometric
 * (src/solvers/SimInf_solver.c:149).  Here every draw comes instead from a
 * counter-based stream keyed by (seed, stream id, draw index), where the
 * stream id is replicate * Nn + node.  A node's draws therefore do not
 * depend on how nodes are split over threads, warps or kernels, which is
 * what lets a GPU run reproduce a CPU run bit for bit.
 *
 *  - Philox4x32-10: J. K. Salmon, M. A. Moraes, R. O. Dror, D. E. Shaw,
 *    "Parallel random numbers: as easy as 1, 2, 3", SC 2011.
 *  - uniform_pos: (2w + 1) * 2^-33 for a 32-bit word w, so 0 < u < 1 with
 *    the 32-bit resolution of a 32-bit Mersenne twister draw.
 *  - si_log: natural logarithm by table reduction (Tang's method: x =
 *    2^e f, f ~ c_j, ln f = -ln r_j + ln(1 + (f r_j - 1))) followed by the
 *    Taylor series of ln(1+z)/z, all in 64/128-bit integer fixed point.
 *    Pure integer arithmetic makes it bit-identical on every CPU and GPU,
 *    and on GB300 integer ALUs are ~40x faster than the FP64 pipe.
 *  - si_hypergeometric: sequential urn draws without replacement (one
 *    word per draw, compared exactly in integers), sampling the smaller of
 *    the draw and its complement.
 *  - si_binomial: sequential-search inversion (L. Devroye, Non-Uniform
 *    Random Variate Generation, 1986, ch. X.4) on chunks of at most 512
 *    trials, summed; Binomial(a + b, p) = Binomial(a, p) + Binomial(b, p).
 *
 * The header compiles as C99 (gcc) and as CUDA C++ (nvcc).  Host code that
 * includes it must be compiled with -ffp-contract=off and device code with
 * -fmad=false so that the few floating-point operations round identically.
 */
#ifndef SIMINF_STREAM_H
#define SIMINF_STREAM_H

#include <stdint.h>
#ifndef __CUDACC__
#  include <string.h>
#endif

#include "siminf_log_table.h"

#ifdef __CUDACC__
#  define SI_HD __host__ __device__ __forceinline__
#else
#  define SI_HD static inline
#endif

/* ---------------------------------------------------------------- */
/* Integer helpers that give the same bits on host and device.       */
/* ---------------------------------------------------------------- */

SI_HD uint64_t si_double_bits(double x)
{
#ifdef __CUDA_ARCH__
    return (uint64_t) __double_as_longlong(x);
#else
    uint64_t b;
    memcpy(&b, &x, sizeof(b));
    return b;
#endif
}

SI_HD double si_bits_double(uint64_t b)
{
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long) b);
#else
    double x;
    memcpy(&x, &b, sizeof(x));
    return x;
#endif
}

SI_HD uint32_t si_umulhi32(uint32_t a, uint32_t b)
{
#ifdef __CUDA_ARCH__
    return __umulhi(a, b);
#else
    return (uint32_t) (((uint64_t) a * b) >> 32);
#endif
}

/* High 64 bits of the unsigned 128-bit product. */
SI_HD uint64_t si_umulhi64(uint64_t a, uint64_t b)
{
#ifdef __CUDA_ARCH__
    return __umul64hi(a, b);
#else
    return (uint64_t) (((unsigned __int128) a * b) >> 64);
#endif
}

/* High 64 bits of the signed 128-bit product (floor of a*b / 2^64). */
SI_HD int64_t si_mulhi64(int64_t a, int64_t b)
{
#ifdef __CUDA_ARCH__
    return (int64_t) __mul64hi((long long) a, (long long) b);
#else
    return (int64_t) (((__int128) a * b) >> 64);
#endif
}

SI_HD int si_clz64(uint64_t x)
{
#ifdef __CUDA_ARCH__
    return __clzll((long long) x);
#else
    return x ? __builtin_clzll(x) : 64;
#endif
}

/* floor(a * b / 2^62) for signed Q62 operands whose product fits. */
SI_HD int64_t si_mul_q62(int64_t a, int64_t b)
{
    const uint64_t hi = (uint64_t) si_mulhi64(a, b);
    const uint64_t lo = (uint64_t) a * (uint64_t) b;
    return (int64_t) ((hi << 2) | (lo >> 62));
}

/* ---------------------------------------------------------------- */
/* Philox4x32-10.                                                    */
/* ---------------------------------------------------------------- */

#define SI_PHILOX_M0 0xD2511F53u
#define SI_PHILOX_M1 0xCD9E8D57u
#define SI_PHILOX_W0 0x9E3779B9u
#define SI_PHILOX_W1 0xBB67AE85u

SI_HD void si_philox4x32_10(uint32_t *c0, uint32_t *c1, uint32_t *c2,
                            uint32_t *c3, uint32_t k0, uint32_t k1)
{
    uint32_t x0 = *c0, x1 = *c1, x2 = *c2, x3 = *c3;
#ifdef __CUDA_ARCH__
#  pragma unroll
#endif
    for (int round = 0; round < 10; round++) {
        const uint32_t hi0 = si_umulhi32(SI_PHILOX_M0, x0);
        const uint32_t lo0 = SI_PHILOX_M0 * x0;
        const uint32_t hi1 = si_umulhi32(SI_PHILOX_M1, x2);
        const uint32_t lo1 = SI_PHILOX_M1 * x2;
        const uint32_t y0 = hi1 ^ x1 ^ k0;
        const uint32_t y2 = hi0 ^ x3 ^ k1;
        x0 = y0;
        x1 = lo1;
        x2 = y2;
        x3 = lo0;
        k0 += SI_PHILOX_W0;
        k1 += SI_PHILOX_W1;
    }
    *c0 = x0;
    *c1 = x1;
    *c2 = x2;
    *c3 = x3;
}

/* ---------------------------------------------------------------- */
/* The per-node stream.                                              */
/* ---------------------------------------------------------------- */

/* Draw i of stream sid under seed is word (i & 3) of
 * Philox4x32-10(counter = {i >> 2 (64 bits), sid (64 bits)},
 *               key = seed (64 bits)).
 *
 * Stream ids: node g = replicate * Nn + node draws from sid g; with common
 * random numbers (mssm_crn) its SSA draws come from sid SI_CRN_SID | g
 * instead, so that they do not shift when its events draw; the
 * all-events method's transition j uses 2^63 | (g * Nt + j) and particle
 * filter interval i resamples from 2^62 + i.  SI_CRN_SID only sets bits
 * of the high word s1. */
#define SI_CRN_SID (3ULL << 61)
#define SI_CRN_S1 ((uint32_t) (SI_CRN_SID >> 32))
typedef struct si_rng {
    uint32_t k0, k1;            /* seed */
    uint32_t s0, s1;            /* stream id */
    uint64_t ctr;               /* index of the next draw */
    uint32_t b0, b1, b2, b3;    /* block (ctr >> 2), valid when have != 0 */
    uint32_t have;
} si_rng;

SI_HD void si_rng_fill(si_rng *r)
{
    const uint64_t blk = r->ctr >> 2;
    uint32_t c0 = (uint32_t) blk, c1 = (uint32_t) (blk >> 32);
    uint32_t c2 = r->s0, c3 = r->s1;
    si_philox4x32_10(&c0, &c1, &c2, &c3, r->k0, r->k1);
    r->b0 = c0;
    r->b1 = c1;
    r->b2 = c2;
    r->b3 = c3;
    r->have = 1;
}

SI_HD void si_rng_init(si_rng *r, uint64_t seed, uint64_t sid, uint64_t ctr)
{
    r->k0 = (uint32_t) seed;
    r->k1 = (uint32_t) (seed >> 32);
    r->s0 = (uint32_t) sid;
    r->s1 = (uint32_t) (sid >> 32);
    r->ctr = ctr;
    r->b0 = r->b1 = r->b2 = r->b3 = 0;
    r->have = 0;
}

/* The next draw, without consuming it. */
SI_HD uint32_t si_peek_u32(si_rng *r)
{
    if (!r->have)
        si_rng_fill(r);
    const uint32_t i = (uint32_t) r->ctr & 3u;
    return (i == 0) ? r->b0 : (i == 1) ? r->b1 : (i == 2) ? r->b2 : r->b3;
}

/* Consume the next draw. */
SI_HD void si_skip(si_rng *r)
{
    r->ctr++;
    if ((r->ctr & 3) == 0)
        r->have = 0;
}

SI_HD uint32_t si_next_u32(si_rng *r)
{
    const uint32_t w = si_peek_u32(r);
    si_skip(r);
    return w;
}

/* Word w -> (2w + 1) * 2^-33, built from integer bits (exact). */
SI_HD double si_u32_to_uniform_pos(uint32_t w)
{
    const uint64_t v = 2 * (uint64_t) w + 1;          /* 1 .. 2^33 - 1 */
    const int p = 63 - si_clz64(v);                    /* 0 .. 32 */
    const uint64_t mant = v << (52 - p);
    const uint64_t expo = (uint64_t) (p - 33 + 1023);
    return si_bits_double((expo << 52) | (mant & 0x000FFFFFFFFFFFFFULL));
}

SI_HD double si_uniform_pos(si_rng *r)
{
    return si_u32_to_uniform_pos(si_next_u32(r));
}

/* ---------------------------------------------------------------- */
/* Natural logarithm in integer fixed point.                         */
/* ---------------------------------------------------------------- */

/* M * 2^-scale for M = (hi, lo) > 0 whose top set bit is bit p, to the
 * nearest double (ties to even); the result must be normal. */
SI_HD double si_u128_to_double_at(uint64_t hi, uint64_t lo, int p, int scale)
{
    uint64_t m;
    int e = p;
    if (p <= 52) {
        m = lo << (52 - p);
    } else {
        const int sh = p - 52;                 /* 1 .. 75 */
        uint64_t rnd, sticky;
        if (sh < 64) {
            m = (lo >> sh) | (hi << (64 - sh));
            rnd = (lo >> (sh - 1)) & 1;
            sticky = (sh > 1) ? (lo & ((1ULL << (sh - 1)) - 1)) : 0;
        } else if (sh == 64) {
            m = hi;
            rnd = lo >> 63;
            sticky = lo & 0x7FFFFFFFFFFFFFFFULL;
        } else {
            m = hi >> (sh - 64);
            rnd = (hi >> (sh - 65)) & 1;
            sticky = (hi & ((1ULL << (sh - 65)) - 1)) | lo;
        }
        m += rnd & ((sticky != 0) | (m & 1));
        if (m >> 53) {
            m >>= 1;
            e++;
        }
    }
    const uint64_t expo = (uint64_t) (e - scale + 1023);
    return si_bits_double((expo << 52) | (m & 0x000FFFFFFFFFFFFFULL));
}

/* |M| * 2^-scale, M = (hi, lo) unsigned 128-bit, to the nearest double
 * (ties to even).  The caller guarantees a result in the normal range. */
SI_HD double si_u128_to_double(uint64_t hi, uint64_t lo, int scale, int negative)
{
    const uint64_t sign = negative ? 0x8000000000000000ULL : 0;
    if (hi == 0 && lo == 0)
        return si_bits_double(sign);
    const int p = hi ? 127 - si_clz64(hi) : 63 - si_clz64(lo);
    uint64_t m;
    int e = p;
    if (p <= 52) {
        m = lo << (52 - p);
    } else {
        const int sh = p - 52;                 /* 1 .. 75 */
        uint64_t rnd, sticky;
        if (sh < 64) {
            m = (lo >> sh) | (sh ? (hi << (64 - sh)) : 0);
            rnd = (lo >> (sh - 1)) & 1;
            sticky = (sh > 1) ? (lo & ((1ULL << (sh - 1)) - 1)) : 0;
        } else if (sh == 64) {
            m = hi;
            rnd = lo >> 63;
            sticky = lo & 0x7FFFFFFFFFFFFFFFULL;
        } else {
            m = hi >> (sh - 64);
            rnd = (hi >> (sh - 65)) & 1;
            sticky = (hi & ((1ULL << (sh - 65)) - 1)) | lo;
        }
        m += rnd & ((sticky != 0) | (m & 1));
        if (m >> 53) {
            m >>= 1;
            e++;
        }
    }
    const uint64_t expo = (uint64_t) (e - scale + 1023);
    return si_bits_double(sign | (expo << 52) | (m & 0x000FFFFFFFFFFFFFULL));
}

/* One copy of the tables for host code and, under nvcc, one in device
 * global memory (both compilation passes must see the declaration). */
static const uint32_t si_log_r_host[128] = SI_LOG_R_INIT;
static const uint64_t si_log_l_host[128] = SI_LOG_L_INIT;
#ifdef __CUDACC__
static __device__ const uint32_t si_log_r_dev[128] = SI_LOG_R_INIT;
static __device__ const uint64_t si_log_l_dev[128] = SI_LOG_L_INIT;
#endif
#ifdef __CUDA_ARCH__
#  define SI_LOG_R(j) si_log_r_dev[j]
#  define SI_LOG_L(j) si_log_l_dev[j]
#else
#  define SI_LOG_R(j) si_log_r_host[j]
#  define SI_LOG_L(j) si_log_l_host[j]
#endif

/* ln(x) for a double x: -inf at 0, NaN below 0 or for NaN, +inf at +inf.
 * Error below one unit in the last place over the positive doubles
 * (checked against a 200-bit reference in the test suite). */
SI_HD double si_log(double x)
{
    const uint64_t bits = si_double_bits(x);
    const uint32_t bexp = (uint32_t) (bits >> 52) & 0x7FFu;
    uint64_t F = bits & 0x000FFFFFFFFFFFFFULL;
    int e;

    if (bits >> 63) {
        if ((bits << 1) == 0)
            return si_bits_double(0xFFF0000000000000ULL);   /* -0 -> -inf */
        return si_bits_double(0x7FF8000000000000ULL);       /* x < 0 -> NaN */
    }
    if (bexp == 0x7FF)
        return x + x;                                        /* inf or NaN */
    if (bexp == 0) {
        if (F == 0)
            return si_bits_double(0xFFF0000000000000ULL);   /* +0 -> -inf */
        const int s = si_clz64(F) - 11;                     /* subnormal */
        F <<= s;
        e = 1 - 1023 - s;
    } else {
        F |= 0x0010000000000000ULL;
        e = (int) bexp - 1023;
    }

    /* f = F / 2^52 in [1, 2); bucket j from the top 7 fraction bits. */
    const int j = (int) ((F >> 45) & 127);
    const uint32_t rd = SI_LOG_R(j);
    const uint64_t R = rd & 0xFFFFu;
    const int K = e + (int) (rd >> 16);
    const uint64_t Lj = SI_LOG_L(j);

    /* z = f R / 2^10 - 1 in Q62, exact. */
    const int64_t Z = (int64_t) (F * R) - (int64_t) 0x4000000000000000LL;

    /* P(z) = ln(1+z)/z = sum (-1)^i z^i / (i+1), Horner in Q62. */
    int64_t P = SI_LOG_C8;
    P = SI_LOG_C7 + si_mul_q62(Z, P);
    P = SI_LOG_C6 + si_mul_q62(Z, P);
    P = SI_LOG_C5 + si_mul_q62(Z, P);
    P = SI_LOG_C4 + si_mul_q62(Z, P);
    P = SI_LOG_C3 + si_mul_q62(Z, P);
    P = SI_LOG_C2 + si_mul_q62(Z, P);
    P = SI_LOG_C1 + si_mul_q62(Z, P);
    P = SI_LOG_C0 + si_mul_q62(Z, P);

    /* W = Z * P, signed 128-bit in Q124 (= ln(1+z)). */
    const uint64_t Whi = (uint64_t) si_mulhi64(Z, P);
    const uint64_t Wlo = (uint64_t) Z * (uint64_t) P;

    if (K == 0 && Lj == 0) {
        /* x in [1 - 2^-8, 1 + 2^-7): ln x = ln(1+z), full relative precision. */
        if ((int64_t) Whi < 0) {
            const uint64_t nlo = ~Wlo + 1;
            const uint64_t nhi = ~Whi + (nlo == 0);
            return si_u128_to_double(nhi, nlo, 124, 1);
        }
        return si_u128_to_double(Whi, Wlo, 124, 0);
    }

    /* T = |K| ln 2 in Q64 (128-bit), then the sign of K. */
    const uint64_t aK = (uint64_t) (K < 0 ? -K : K);
    uint64_t Thi = si_umulhi64(aK, SI_LN2_Q128_HI);
    uint64_t Tlo = aK * SI_LN2_Q128_HI;
    const uint64_t c = si_umulhi64(aK, SI_LN2_Q128_LO);
    Tlo += c;
    Thi += (Tlo < c);
    if (K < 0) {
        Tlo = ~Tlo + 1;
        Thi = ~Thi + (Tlo == 0);
    }
    /* + L_j (Q64, non-negative). */
    Tlo += Lj;
    Thi += (Tlo < Lj);
    /* + ln(1+z): W >> 60 with sign extension. */
    const uint64_t slo = (Wlo >> 60) | (Whi << 4);
    const uint64_t shi = (uint64_t) ((int64_t) Whi >> 60);
    Tlo += slo;
    Thi += shi + (Tlo < slo);

    if ((int64_t) Thi < 0) {
        const uint64_t nlo = ~Tlo + 1;
        const uint64_t nhi = ~Thi + (nlo == 0);
        return si_u128_to_double(nhi, nlo, 64, 1);
    }
    return si_u128_to_double(Thi, Tlo, 64, 0);
}

/* ---------------------------------------------------------------- */
/* -log of a 32-bit uniform, for the SSA's exponential waiting time.  */
/* ---------------------------------------------------------------- */

static const uint32_t si_nl_r1_host[128] = SI_NL_R1_INIT;
static const uint64_t si_nl_l1_host[128] = SI_NL_L1_INIT;
static const uint32_t si_nl_r2_host[256] = SI_NL_R2_INIT;
static const int64_t si_nl_l2_host[256] = SI_NL_L2_INIT;
static const uint64_t si_nl_kln2_host[34][2] = SI_NL_KLN2_INIT;
#ifdef __CUDACC__
static __device__ const uint32_t si_nl_r1_dev[128] = SI_NL_R1_INIT;
static __device__ const uint64_t si_nl_l1_dev[128] = SI_NL_L1_INIT;
static __device__ const uint32_t si_nl_r2_dev[256] = SI_NL_R2_INIT;
static __device__ const int64_t si_nl_l2_dev[256] = SI_NL_L2_INIT;
static __device__ const uint64_t si_nl_kln2_dev[34][2] = SI_NL_KLN2_INIT;
#endif
#ifdef __CUDA_ARCH__
#  define SI_NL(tab) si_nl_##tab##_dev
#else
#  define SI_NL(tab) si_nl_##tab##_host
#endif

SI_HD int si_clz32(uint32_t x)
{
#ifdef __CUDA_ARCH__
    return __clz((int) x);
#else
    return x ? __builtin_clz(x) : 32;
#endif
}

/* 32x32 -> 64-bit product (one wide multiply-add on the GPU). */
SI_HD uint64_t si_mulw(uint32_t a, uint32_t b)
{
    return (uint64_t) a * (uint64_t) b;
}

/* -ln(u) for u = (2w + 1) * 2^-33, the value si_u32_to_uniform_pos(w)
 * gives.  The logarithm of x = 2w + 1 = 2^k m is reduced twice by tables
 * (m r1 r2 = 1 + z, |z| < 2^-14.5, all products exact in 64-bit integers),
 * ln(1 + z) takes four series terms from 32-bit multiplies, and the sum
 * (33 - k) ln 2 - ln(m) is formed in Q64.64 with an absolute error below
 * 2^-61.  That is within one ulp for u <= 1 - 2^-8 (0.97 ulp at worst over
 * all 2^32 words); si_neglog_u32 sends larger u (probability 2^-8) to
 * si_log.  Integer-only: the same bits on every host and device. */
SI_HD double si_neglog_u32_tab(uint32_t w)
{
    const uint64_t x = 2 * (uint64_t) w + 1;
    int k;
    uint64_t M;                                  /* m * 2^32, in [2^32, 2^33) */
    if (x >> 32) {
        k = 32;
        M = x;
    } else {
        const uint32_t xl = (uint32_t) x;
        k = 31 - si_clz32(xl);
        M = (uint64_t) xl << (32 - k);
    }
    const int j1 = (int) ((M >> 25) & 127);
    const uint64_t M1 = M * (uint64_t) SI_NL(r1)[j1];          /* (m r1) * 2^42 */
    const int64_t Z1 = (int64_t) M1 - ((int64_t) 1 << 42);    /* |Z1| < 2^35 */
    const int j2 = (int) (((uint64_t) (Z1 + ((int64_t) 1 << 35)) >> 28) & 255);
    const uint64_t M2 = M1 * (uint64_t) SI_NL(r2)[j2];         /* (m r1 r2) * 2^58 */
    const int64_t Z2 = (int64_t) M2 - ((int64_t) 1 << 58);    /* z * 2^58, |.| < 2^43.5 */

    /* ln(1 + z) * 2^64 = z - z^2/2 + z^3/3 - z^4/4 */
    const uint64_t a = (uint64_t) (Z2 < 0 ? -Z2 : Z2);
    const uint32_t ah = (uint32_t) (a >> 22), al = (uint32_t) (a & 0x3FFFFF);
    /* z^2/2 * 2^64 = a^2 / 2^53, from a = ah 2^22 + al */
    const uint64_t t2 = (si_mulw(ah, ah) >> 9) + (si_mulw(ah, al) >> 30) +
                        (si_mulw(al, al) >> 53);
    const uint32_t b = (uint32_t) (a >> 12);                  /* |z| * 2^46 */
    const uint32_t c = (uint32_t) (si_mulw(b, b) >> 32);      /* z^2 * 2^60 */
    const uint64_t z3 = si_mulw(c, b) >> 42;                  /* |z|^3 * 2^64 */
    const uint64_t t3v = si_umulhi64(z3, 0x5555555555555556ULL);   /* z3 / 3 */
    const uint64_t t4 = (si_mulw(c, c) >> 56) >> 2;           /* z^4 / 4 * 2^64 */
    const int64_t z1t = Z2 * 64;                              /* z * 2^64 */
    const int64_t s3 = Z2 < 0 ? -(int64_t) t3v : (int64_t) t3v;
    const int64_t ln1p = z1t - (int64_t) t2 + s3 - (int64_t) t4;

    /* (33 - k) ln 2 - L1 - L2 - ln(1+z) in Q64.64 */
    uint64_t hi = SI_NL(kln2)[33 - k][0], lo = SI_NL(kln2)[33 - k][1];
    const uint64_t l1 = SI_NL(l1)[j1];
    hi -= (lo < l1);
    lo -= l1;
    const int64_t l2 = SI_NL(l2)[j2] + ln1p;                 /* |.| < 2^58 */
    const uint64_t l2u = (uint64_t) l2;
    const uint64_t l2h = (uint64_t) (l2 >> 63);              /* sign extension */
    hi -= l2h + (lo < l2u);
    lo -= l2u;
    /* to double: the value lies in [2^-8, 23), so its top bit p is at
     * 64 + (0..4) or at 56..63 of lo, and the rounding of
     * si_u128_to_double_at(hi, lo, p, 64) takes the shift sh = p - 52 in
     * 4..16 -- written out here as straight-line code */
    const int p = hi ? 64 + 31 - si_clz32((uint32_t) hi)
                     : 63 - si_clz32((uint32_t) (lo >> 32));
    const int sh = p - 52;
    uint64_t m = (lo >> sh) | (hi << (64 - sh));
    const uint64_t rnd = (lo >> (sh - 1)) & 1;
    const uint64_t sticky = lo & ((1ULL << (sh - 1)) - 1);
    m += rnd & ((sticky != 0) | (m & 1));
    const int ov = (int) (m >> 53);
    m >>= ov;
    const uint64_t expo = (uint64_t) (p + ov - 64 + 1023);
    return si_bits_double((expo << 52) | (m & 0x000FFFFFFFFFFFFFULL));
}

/* si_neglog_u32 for a speculative step: the table value in straight-line
 * code, with *slow set when w is one of the words (probability 2^-8) that
 * si_neglog_u32 hands to si_log instead. */
SI_HD double si_neglog_u32_spec(uint32_t w, int *slow)
{
    const uint64_t x = 2 * (uint64_t) w + 1;
    *slow |= x >= ((uint64_t) 1 << 33) - ((uint64_t) 1 << 25);
    return si_neglog_u32_tab(w);
}

#ifdef __CUDACC__
/* The rare hand-over to si_log, kept out of line on the device: it is
 * taken by 1 word in 256, and inlined it would double the code of the SSA
 * step that every warp keeps in its instruction cache. */
static __device__ __noinline__ double si_neglog_slow(uint32_t w)
{
    return -si_log(si_u32_to_uniform_pos(w));
}
#endif

SI_HD double si_neglog_u32(uint32_t w)
{
    const uint64_t x = 2 * (uint64_t) w + 1;
    if (x >= ((uint64_t) 1 << 33) - ((uint64_t) 1 << 25)) {
#ifdef __CUDA_ARCH__
        return si_neglog_slow(w);
#else
        return -si_log(si_u32_to_uniform_pos(w));
#endif
    }
    return si_neglog_u32_tab(w);
}

/* ---------------------------------------------------------------- */
/* Exact comparisons and conversions on the integer pipes.           */
/* ---------------------------------------------------------------- */

/* Order key of a non-NaN double: keys compare like the doubles, and
 * +0 and -0 share a key. */
SI_HD int64_t si_dkey(uint64_t b)
{
    return (b >> 63) ? -(int64_t) (b & 0x7FFFFFFFFFFFFFFFULL) : (int64_t) b;
}

SI_HD int si_isnan_bits(uint64_t b)
{
    return (b << 1) > 0xFFE0000000000000ULL;
}

/* a > b with IEEE semantics (false when either is NaN). */
SI_HD int si_dgt(double a, double b)
{
    const uint64_t A = si_double_bits(a), B = si_double_bits(b);
    if (si_isnan_bits(A) || si_isnan_bits(B))
        return 0;
    return si_dkey(A) > si_dkey(B);
}

/* a >= b with IEEE semantics (false when either is NaN). */
SI_HD int si_dge(double a, double b)
{
    const uint64_t A = si_double_bits(a), B = si_double_bits(b);
    if (si_isnan_bits(A) || si_isnan_bits(B))
        return 0;
    return si_dkey(A) >= si_dkey(B);
}

/* (double) x for a 32-bit integer, exact, from integer bits. */
SI_HD double si_i2d(int32_t x)
{
    if (x == 0)
        return 0.0;
    const uint64_t sign = x < 0 ? 0x8000000000000000ULL : 0;
    const uint64_t m = x < 0 ? (uint64_t) (0u - (uint32_t) x) : (uint64_t) (uint32_t) x;
    const int p = 63 - si_clz64(m);
    return si_bits_double(sign | ((uint64_t) (p + 1023) << 52) |
                          ((m << (52 - p)) & 0x000FFFFFFFFFFFFFULL));
}

/* (double) x for |x| < 2^53, exact, from integer bits. */
SI_HD double si_l2d(int64_t x)
{
    if (x == 0)
        return 0.0;
    const uint64_t sign = x < 0 ? 0x8000000000000000ULL : 0;
    const uint64_t m = x < 0 ? (uint64_t) 0 - (uint64_t) x : (uint64_t) x;
    const int p = 63 - si_clz64(m);
    return si_bits_double(sign | ((uint64_t) (p + 1023) << 52) |
                          ((m << (52 - p)) & 0x000FFFFFFFFFFFFFULL));
}

/* !isfinite(x) || x < 0.0, the reference's invalid-rate test. */
SI_HD int si_bad_rate(double x)
{
    const uint64_t b = si_double_bits(x);
    return ((b >> 52) & 0x7FF) == 0x7FF || ((b >> 63) && (b << 1) != 0);
}

/* 0 < x < +inf (false for NaN). */
SI_HD int si_finite_pos(double x)
{
    const uint64_t b = si_double_bits(x);
    return !(b >> 63) && b != 0 && ((b >> 52) & 0x7FF) != 0x7FF;
}

/* x == 0.0 (either sign). */
SI_HD int si_is_zero(double x)
{
    return (si_double_bits(x) << 1) == 0;
}

/* ---------------------------------------------------------------- */
/* IEEE-754 binary64 division on the integer pipes.                  */
/* ---------------------------------------------------------------- */

/* Approximate 2^86 / m for m in [2^23, 2^24), good to about 2^-22
 * relative, from the single-precision reciprocal (exact IEEE on the host,
 * the hardware approximation on the GPU; both are within the bound the
 * Newton steps below need). */
SI_HD uint64_t si_recip_seed(uint32_t m24)
{
#ifdef __CUDA_ARCH__
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"((float) m24));
#else
    const float r = 1.0f / (float) m24;
#endif
    /* r = 1.f * 2^(E-127); r * 2^86 as a 64-bit integer (at most 2^63) */
    uint32_t rb;
#ifdef __CUDA_ARCH__
    rb = __float_as_uint(r);
#else
    memcpy(&rb, &r, sizeof(rb));
#endif
    const int E = (int) ((rb >> 23) & 0xFF);
    const uint64_t mant = (uint64_t) ((rb & 0x7FFFFF) | 0x800000);   /* 24 bits */
    const int sh = E - 127 + 86 - 23;                                  /* 39..40 */
    return mant << sh;
}

/* The divisor side of si_div: the divisor's bits, its 53-bit mantissa (0
 * when the divisor is zero, subnormal, infinite or NaN) and y ~ 2^115 / mb
 * in (2^62, 2^63], from the seed in two Newton steps
 * y <- y + y * (2^115 - mb * y) / 2^115.  Newton's iteration for a
 * reciprocal approaches from below and every truncation here rounds down,
 * so y never exceeds 2^115 / mb. */
typedef struct si_recip {
    uint64_t B;
    uint64_t mb;
    uint64_t y;
} si_recip;

SI_HD si_recip si_recip_prep(double b)
{
    si_recip r;
    r.B = si_double_bits(b);
    const int eb = (int) ((r.B >> 52) & 0x7FF);
    /* straight-line: the steps run on any bits, and a divisor without
     * a normal mantissa keeps mb = y = 0 */
    const int normal = (eb != 0) & (eb != 0x7FF);
    const uint64_t mb = (r.B & 0x000FFFFFFFFFFFFFULL) | 0x0010000000000000ULL;
    uint64_t y = si_recip_seed((uint32_t) (mb >> 29));
    for (int it = 0; it < 2; it++) {
        const uint64_t plo = mb * y;
        const uint64_t phi = si_umulhi64(mb, y);           /* mb*y = phi:plo, ~2^115 */
        /* d = 2^115 - mb*y, |d| < 2^95: keep bits 32..95 as a signed value */
        const uint64_t dlo = 0 - plo;
        const uint64_t dhi = ((uint64_t) 1 << 51) - phi - (plo != 0);
        const int64_t d32 = (int64_t) ((dhi << 32) | (dlo >> 32));    /* d / 2^32 */
        /* y * d / 2^115 = (y/2 * d32 / 2^64) / 2^18 */
        const int64_t hi = si_mulhi64((int64_t) (y >> 1), d32);
        y = (uint64_t) ((int64_t) y + (hi >> 18));
    }
    r.mb = normal ? mb : 0;
    r.y = normal ? y : 0;
    return r;
}

/* a / b for the divisor prepared in r (r = si_recip_prep(b)), correctly
 * rounded to nearest even, bit-identical to the IEEE division of any
 * conforming host or device.  Normal operands whose quotient is normal
 * take the integer path: Q = 2 ma y / 2^64 is at most one unit below
 * ma 2^52 / mb (y is a lower bound good to ~2^-60), and the exact
 * remainder fixes it; the fix-ups are selects, so the path is straight
 * code.  Every other case (zero, subnormal, infinite, NaN operands or an
 * overflowing or underflowing quotient) sets *special, and the value
 * returned is then meaningless: si_div_r takes the hardware division for
 * it, a speculative step redoes its work on the exact path. */
SI_HD double si_div_r_spec(double a, const si_recip *r, int *special)
{
    const uint64_t A = si_double_bits(a);
    const int ea = (int) ((A >> 52) & 0x7FF), eb = (int) ((r->B >> 52) & 0x7FF);
    const uint64_t mb = r->mb;
    uint64_t ma = (A & 0x000FFFFFFFFFFFFFULL) | 0x0010000000000000ULL;
    const int lt = ma < mb;                  /* quotient of the mantissas in [1, 2) */
    ma <<= lt;
    const int e = ea - eb - lt;
    *special |= (mb == 0) | (ea == 0) | (ea == 0x7FF) | (e > 1022) | (e < -1022);
    const uint64_t sign = (A ^ r->B) & 0x8000000000000000ULL;
    uint64_t Q = si_umulhi64(ma << 1, r->y);
    int64_t R = (int64_t) ((ma << 52) - Q * mb);
    /* at most one step up is needed; one more each way is kept as margin */
    if (R < 0) {
        Q--;
        R += (int64_t) mb;
    }
    if (R >= (int64_t) mb) {
        Q++;
        R -= (int64_t) mb;
    }
    if (R >= (int64_t) mb) {
        Q++;
        R -= (int64_t) mb;
    }
    /* round to nearest, ties to even */
    const uint64_t twoR = (uint64_t) R << 1;
    Q += (twoR > mb) | ((twoR == mb) & (uint32_t) Q & 1u);
    const int carry = (int) (Q >> 53);
    Q >>= carry;
    const uint64_t expo = (uint64_t) (e + carry + 1023);
    return si_bits_double(sign | (expo << 52) | (Q & 0x000FFFFFFFFFFFFFULL));
}

SI_HD double si_div_r(double a, const si_recip *r, double b)
{
    int special = 0;
    const double q = si_div_r_spec(a, r, &special);
    return special ? a / b : q;
}

SI_HD double si_div(double a, double b)
{
    const si_recip r = si_recip_prep(b);
    return si_div_r(a, &r, b);
}

/* a / b on the integer path alone, *special set where si_div would take
 * the hardware division. */
SI_HD double si_div_spec(double a, double b, int *special)
{
    const si_recip r = si_recip_prep(b);
    return si_div_r_spec(a, &r, special);
}

/* a / b through a one-entry cache of prepared divisors: a rate that
 * divides by a population count which the transitions keep constant
 * prepares it once. */
SI_HD double si_div_cached(double a, double b, si_recip *c)
{
    if (si_double_bits(b) != c->B)
        *c = si_recip_prep(b);
    return si_div_r(a, c, b);
}

#ifdef __cplusplus
/* The divisor cache as a speculative step reads it: the prepared divisor
 * is used as it is, and a division by another divisor, or one that
 * leaves the integer path, sets flag instead of branching (the step is
 * then redone with the si_recip itself). */
struct si_recip_spec {
    const si_recip *c;
    int flag;
};

SI_HD double si_div_cached(double a, double b, si_recip_spec *s)
{
    s->flag |= si_double_bits(b) != s->c->B;
    return si_div_r_spec(a, s->c, &s->flag);
}
#endif

/* An empty cache (no divisor has these bits and a zero mantissa). */
SI_HD si_recip si_recip_none(void)
{
    si_recip r;
    r.B = 0xFFFFFFFFFFFFFFFFULL;
    r.mb = 0;
    r.y = 0;
    return r;
}

/* ---------------------------------------------------------------- */
/* Exponential and log-factorials for the particle filter's weights. */
/* ---------------------------------------------------------------- */

#ifdef __CUDACC__
static __device__ const uint64_t si_exp_inv_fact_dev[14] = SI_EXP_INV_FACT_INIT;
#endif
static const uint64_t si_exp_inv_fact_host[14] = SI_EXP_INV_FACT_INIT;
#ifdef __CUDA_ARCH__
#  define SI_EXP_INV_FACT(j) si_exp_inv_fact_dev[j]
#else
#  define SI_EXP_INV_FACT(j) si_exp_inv_fact_host[j]
#endif

/* exp(x) by Cody-Waite reduction x = k ln2 + r, |r| <= ln(2)/2, with ln 2
 * split into a 32-bit head (k * head exact) and a tail, the Taylor series of
 * exp(r) to degree 13 in Horner form (separate multiply and add), and an
 * exact scaling by 2^k.  Only IEEE add/multiply, so host and device agree
 * bit for bit; about one ulp from the true value. */
SI_HD double si_exp(double x)
{
    const uint64_t xb = si_double_bits(x);
    if (si_isnan_bits(xb))
        return x + x;
    if (x > 709.782712893384)
        return si_bits_double(0x7FF0000000000000ULL);
    if (x < -745.1332191019412)
        return 0.0;
    const double magic = 6755399441055744.0;            /* 2^52 + 2^51 */
    const double kf = (x * si_bits_double(SI_EXP_INV_LN2) + magic) - magic;
    const int k = (int) kf;
    const double r = (x - kf * si_bits_double(SI_EXP_LN2_HI)) - kf * si_bits_double(SI_EXP_LN2_LO);
    double p = si_bits_double(SI_EXP_INV_FACT(13));
    for (int n = 12; n >= 0; n--)
        p = p * r + si_bits_double(SI_EXP_INV_FACT(n));
    /* p * 2^k, in two exact steps when 2^k alone is not a normal double */
    if (k >= -1021 && k <= 1023)
        return p * si_bits_double((uint64_t) (k + 1023) << 52);
    const int k1 = k < 0 ? -1000 : 1000;
    return (p * si_bits_double((uint64_t) (k1 + 1023) << 52)) *
           si_bits_double((uint64_t) (k - k1 + 1023) << 52);
}

/* tab[i] = ln(i!) for i < n, accumulated in order with si_log, the same
 * bits wherever it is computed. */
SI_HD void si_lfact_fill(double *tab, int n)
{
    double acc = 0.0;
    for (int i = 0; i < n; i++) {
        if (i >= 2)
            acc = acc + si_log((double) i);
        tab[i] = acc;
    }
}

/* ---------------------------------------------------------------- */
/* Samplers.                                                         */
/* ---------------------------------------------------------------- */

/* Number of type-1 items in t draws without replacement from an urn with
 * n1 type-1 and n2 type-2 items; 0 <= t <= n1 + n2.  A draw takes a
 * type-1 item iff (2w + 1) * remaining < a * 2^33, i.e. iff
 * uniform_pos < a / remaining, evaluated exactly in 64-bit integers. */
SI_HD int si_hypergeometric(si_rng *r, int n1, int n2, int t)
{
    const int64_t N = (int64_t) n1 + n2;
    int complement = 0;
    if (t <= 0 || n1 <= 0)
        return 0;
    if ((int64_t) t >= N)
        return n1;
    if (2 * (int64_t) t > N) {
        t = (int) (N - t);
        complement = 1;
    }
    uint64_t a = (uint64_t) n1, rem = (uint64_t) N;
    int k = 0;
    for (int i = 0; i < t; i++) {
        if (a == 0)
            break;
        if (a == rem) {
            k += t - i;
            break;
        }
        const uint32_t w = si_next_u32(r);
        if ((2 * (uint64_t) w + 1) * rem < (a << 33)) {
            k++;
            a--;
        }
        rem--;
    }
    return complement ? n1 - k : k;
}

/* Binomial(n, p) by chunked sequential-search inversion.  One draw per
 * chunk of at most 512 trials; none when p <= 0, p >= 1 or n <= 0. */
SI_HD int si_binomial(si_rng *r, double p, int n)
{
    if (n <= 0 || !(p > 0.0))
        return 0;
    if (p >= 1.0)
        return n;
    const int flip = p > 0.5;
    const double q = flip ? 1.0 - p : p;
    const double qc = 1.0 - q;
    const double s = q / qc;
    int total = 0, rem = n;
    while (rem > 0) {
        const int m = rem < 512 ? rem : 512;
        rem -= m;
        /* f0 = qc^m by binary powering. */
        double f = 1.0, b = qc;
        for (int e = m; e; e >>= 1) {
            if (e & 1)
                f = f * b;
            b = b * b;
        }
        double u = si_uniform_pos(r);
        int k = 0;
        while (u > f && k < m) {
            u = u - f;
            k++;
            f = f * ((s * (double) (m - k + 1)) / (double) k);
        }
        total += k;
    }
    return flip ? n - total : total;
}

#endif /* SIMINF_STREAM_H */
