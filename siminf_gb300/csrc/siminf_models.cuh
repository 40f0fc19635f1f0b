/*
 * siminf_models.cuh -- __device__ transition-rate and post-time-step code
 * of the models the library ships.
 *
 * Each model is a struct with compile-time sizes NC (compartments), NT
 * (transitions), ND (continuous state variables), a rate(k, ...) function
 * with the TRFun signature of inst/include/SimInf.h:92-97 plus the
 * transition index k, and pts(...) with the PTSFun signature of
 * inst/include/SimInf.h:100-107.  k is always a compile-time constant at the
 * call sites (unrolled loops), so the switch folds away.
 *
 * The expressions, and their evaluation order, are those of the reference
 * model files (cited per model); the library is compiled with -fmad=false so
 * that no multiply-add is fused and every double rounds as it does in the
 * reference's C.  Three exact substitutions move work off GB300's slow FP64
 * pipe without changing a single bit of any result: int -> double
 * conversions are built from integer bits (si_i2d), a double sum of integer
 * counts that stays below 2^53 is formed as an integer sum and converted once
 * (every partial sum is exact either way), and divisions use si_div, an
 * IEEE round-to-nearest division on the integer pipes.  rate() takes a
 * one-entry cache of the prepared divisor (si_div_cached): a population
 * count, which the transitions keep constant, is prepared once per change.
 * The cache is an si_recip, or in the SSA's speculative step an
 * si_recip_spec, which reads the prepared divisor and flags a stale one
 * instead of preparing it (the step is then redone on the exact path).
 */
#ifndef SIMINF_MODELS_CUH
#define SIMINF_MODELS_CUH

namespace siminf {

/* SIR, src/models/SIR.c:43-87; ldata = (beta, gamma). */
struct ModelSIR {
    static constexpr int NC = 3, NT = 2, ND = 0;
    static constexpr int NGD = 0;  /* gdata entries read */
    static constexpr bool PTS_LOCAL = true;
    static constexpr bool RATES_TIME_INVARIANT = true;  /* rate() ignores t */
    template <class DC>
    __device__ __forceinline__ static double rate(int k, const int *u, const double *v,
                                                  const double *ldata, const double *gdata,
                                                  double t, DC &dc)
    {
        if (k == 0) {
            const double S_n = si_i2d(u[0]);
            const double I_n = si_i2d(u[1]);
            const long long n = (long long) u[0] + u[1] + u[2];     /* S_n + I_n + u[R] */
            /* the population divides every call: its reciprocal is cached */
            const double q = si_div_cached(ldata[0] * S_n * I_n, si_l2d(n > 0 ? n : 1), &dc);
            return n > 0 ? q : 0.0;
        }
        return ldata[1] * si_i2d(u[1]);
    }
    __device__ __forceinline__ static int pts(double *, const int *, const double *,
                                              const double *, const double *, int, double)
    {
        return 0;
    }
};

/* SEIR, src/models/SEIR.c:43-112; ldata = (beta, epsilon, gamma). */
struct ModelSEIR {
    static constexpr int NC = 4, NT = 3, ND = 0;
    static constexpr int NGD = 0;  /* gdata entries read */
    static constexpr bool PTS_LOCAL = true;
    static constexpr bool RATES_TIME_INVARIANT = true;  /* rate() ignores t */
    template <class DC>
    __device__ __forceinline__ static double rate(int k, const int *u, const double *v,
                                                  const double *ldata, const double *gdata,
                                                  double t, DC &dc)
    {
        if (k == 0) {
            const double S_n = si_i2d(u[0]);
            const double I_n = si_i2d(u[2]);
            const long long n = (long long) u[0] + u[1] + u[2] + u[3];  /* S_n + u[E] + I_n + u[R] */
            /* the population divides every call: its reciprocal is cached */
            const double q = si_div_cached(ldata[0] * S_n * I_n, si_l2d(n > 0 ? n : 1), &dc);
            return n > 0 ? q : 0.0;
        }
        if (k == 1)
            return ldata[1] * si_i2d(u[1]);
        return ldata[2] * si_i2d(u[2]);
    }
    __device__ __forceinline__ static int pts(double *, const int *, const double *,
                                              const double *, const double *, int, double)
    {
        return 0;
    }
};

/* SIS, src/models/SIS.c; ldata = (beta, gamma). */
struct ModelSIS {
    static constexpr int NC = 2, NT = 2, ND = 0;
    static constexpr int NGD = 0;  /* gdata entries read */
    static constexpr bool PTS_LOCAL = true;
    static constexpr bool RATES_TIME_INVARIANT = true;  /* rate() ignores t */
    template <class DC>
    __device__ __forceinline__ static double rate(int k, const int *u, const double *v,
                                                  const double *ldata, const double *gdata,
                                                  double t, DC &dc)
    {
        if (k == 0) {
            const double S_n = si_i2d(u[0]);
            const double I_n = si_i2d(u[1]);
            const long long n = (long long) u[0] + u[1];               /* S_n + I_n */
            /* the population divides every call: its reciprocal is cached */
            const double q = si_div_cached(ldata[0] * S_n * I_n, si_l2d(n > 0 ? n : 1), &dc);
            return n > 0 ? q : 0.0;
        }
        return ldata[1] * si_i2d(u[1]);
    }
    __device__ __forceinline__ static int pts(double *, const int *, const double *,
                                              const double *, const double *, int, double)
    {
        return 0;
    }
};

/* src/misc/SimInf_forward_euler_linear_decay.c:57-93 */
__device__ __forceinline__ double forward_euler_linear_decay(
    double phi, int day, int end_t1, int end_t2, int end_t3, int end_t4,
    double b1, double b2, double b3, double b4)
{
    if (day < end_t2) {
        if (day < end_t1) {
            if (end_t1 < end_t4)
                return phi * (1.0 - b1);
            if (day < end_t4) {
                if (end_t4 < end_t3)
                    return phi * (1.0 - b4);
                if (day < end_t3)
                    return phi * (1.0 - b3);
                return phi * (1.0 - b4);
            }
            return phi * (1.0 - b1);
        }
        return phi * (1.0 - b2);
    }
    if (end_t3 < end_t1 || day < end_t3)
        return phi * (1.0 - b3);
    if (end_t4 < end_t1 || day < end_t4)
        return phi * (1.0 - b4);
    return phi * (1.0 - b1);
}

/* SISe, src/models/SISe.c:51-144; ldata = (end_t1..end_t4), gdata = (upsilon,
 * gamma, alpha, beta_t1..beta_t4, epsilon), v = (phi). */
struct ModelSISe {
    static constexpr int NC = 2, NT = 2, ND = 1;
    static constexpr int NGD = 8;  /* gdata entries read */
    static constexpr bool PTS_LOCAL = true;
    static constexpr bool RATES_TIME_INVARIANT = true;  /* rate() ignores t */
    template <class DC>
    __device__ __forceinline__ static double rate(int k, const int *u, const double *v,
                                                  const double *ldata, const double *gdata,
                                                  double t, DC &dc)
    {
        if (k == 0)
            return gdata[0] * v[0] * si_i2d(u[0]);
        return gdata[1] * si_i2d(u[1]);
    }
    __device__ __forceinline__ static int pts(double *v_new, const int *u, const double *v,
                                              const double *ldata, const double *gdata,
                                              int node, double t)
    {
        const int day = (int) t % 365;
        const double I_n = u[1];
        const double n = u[0] + I_n;
        const double phi = v[0];
        v_new[0] = forward_euler_linear_decay(phi, day, (int) ldata[0], (int) ldata[1],
                                              (int) ldata[2], (int) ldata[3], gdata[3],
                                              gdata[4], gdata[5], gdata[6]);
        if (n > 0.0)
            v_new[0] += gdata[2] * I_n / n + gdata[7];
        else
            v_new[0] += gdata[7];
        if (!isfinite(v_new[0]))
            return -7;          /* SIMINF_ERR_V_IS_NOT_FINITE */
        if (v_new[0] < 0.0)
            return -10;         /* SIMINF_ERR_V_IS_NEGATIVE */
        return phi != v_new[0];
    }
};

/* SISe3, src/models/SISe3.c:51-250; u = (S_1, I_1, S_2, I_2, S_3, I_3),
 * v = (phi), ldata = (end_t1..end_t4), gdata = (upsilon_1..3, gamma_1..3,
 * alpha, beta_t1..beta_t4, epsilon); transitions in SISe3_run's order. */
struct ModelSISe3 {
    static constexpr int NC = 6, NT = 6, ND = 1;
    static constexpr int NGD = 12;  /* gdata entries read */
    static constexpr bool PTS_LOCAL = true;
    static constexpr bool RATES_TIME_INVARIANT = true;  /* rate() ignores t */
    template <class DC>
    __device__ __forceinline__ static double rate(int k, const int *u, const double *v,
                                                  const double *ldata, const double *gdata,
                                                  double t, DC &dc)
    {
        switch (k) {
        case 0: return gdata[0] * v[0] * si_i2d(u[0]);
        case 1: return gdata[3] * si_i2d(u[1]);
        case 2: return gdata[1] * v[0] * si_i2d(u[2]);
        case 3: return gdata[4] * si_i2d(u[3]);
        case 4: return gdata[2] * v[0] * si_i2d(u[4]);
        default: return gdata[5] * si_i2d(u[5]);
        }
    }
    __device__ __forceinline__ static int pts(double *v_new, const int *u, const double *v,
                                              const double *ldata, const double *gdata,
                                              int node, double t)
    {
        const int day = (int) t % 365;
        const double I_n = u[1] + u[3] + u[5];
        const double n = I_n + u[0] + u[2] + u[4];
        const double phi = v[0];
        v_new[0] = forward_euler_linear_decay(phi, day, (int) ldata[0], (int) ldata[1],
                                              (int) ldata[2], (int) ldata[3], gdata[7],
                                              gdata[8], gdata[9], gdata[10]);
        if (n > 0.0)
            v_new[0] += gdata[6] * I_n / n + gdata[11];
        else
            v_new[0] += gdata[11];
        if (!isfinite(v_new[0]))
            return -7;
        if (v_new[0] < 0.0)
            return -10;
        return phi != v_new[0];
    }
};

/* The spread of the environmental pressure phi from proximal nodes
 * (src/misc/SimInf_local_spread.c:43-71): neighbors is the node's list of
 * (index, distance) pairs ended by a negative index; phi and u point at
 * the first node of the replicate, so the neighbours' current phi and
 * compartments are read where every node of the replicate keeps them.
 * Each neighbour j that holds individuals adds
 * ((phi_j * N_j - phi_i * N_i) * D) / (N_i * distance), in list order. */
__device__ __forceinline__ double local_spread(const double *neighbors, const double *phi,
                                               const int *u, double N_i, double phi_i,
                                               int Nc, double D)
{
    double ls = 0.0;
    const double phi_i_N_i = phi_i * N_i;
    int j = (int) neighbors[0];
    while (j >= 0) {
        double N_j = 0;
        for (int k = j * Nc; k < (j + 1) * Nc; k++)
            N_j += u[k];
        if (N_j > 0.0)
            ls += ((phi[j] * N_j - phi_i_N_i) * D) / (N_i * neighbors[1]);
        neighbors += 2;
        j = (int) neighbors[0];
    }
    return ls;
}

/* SISe_sp, src/models/SISe_sp.c:40-160: SISe whose post-time-step adds
 * the local spread from the neighbours listed in ldata after end_t1..4.
 * gdata = (upsilon, gamma, alpha, beta_t1..beta_t4, coupling), v = (phi).
 * The post-time-step reads other nodes: u and v are the replicate's
 * arrays at this node (PTS_LOCAL false), as in the reference. */
struct ModelSISe_sp {
    static constexpr int NC = 2, NT = 2, ND = 1;
    static constexpr int NGD = 8;  /* gdata entries read */
    static constexpr bool PTS_LOCAL = false;
    static constexpr bool RATES_TIME_INVARIANT = true;  /* rate() ignores t */
    template <class DC>
    __device__ __forceinline__ static double rate(int k, const int *u, const double *v,
                                                  const double *ldata, const double *gdata,
                                                  double t, DC &dc)
    {
        if (k == 0)
            return gdata[0] * v[0] * si_i2d(u[0]);
        return gdata[1] * si_i2d(u[1]);
    }
    __device__ __forceinline__ static int pts(double *v_new, const int *u, const double *v,
                                              const double *ldata, const double *gdata,
                                              int node, double t)
    {
        const int day = (int) t % 365;
        const double I_i = u[1];
        const double N_i = u[0] + I_i;
        const double phi = v[0];
        v_new[0] = forward_euler_linear_decay(phi, day, (int) ldata[0], (int) ldata[1],
                                              (int) ldata[2], (int) ldata[3], gdata[3],
                                              gdata[4], gdata[5], gdata[6]);
        if (N_i > 0.0)
            v_new[0] += gdata[2] * I_i / N_i +
                        local_spread(ldata + 4, v - node, u - 2 * node, N_i, phi, 2, gdata[7]);
        if (!isfinite(v_new[0]))
            return -7;          /* SIMINF_ERR_V_IS_NOT_FINITE */
        if (v_new[0] < 0.0)
            return -10;         /* SIMINF_ERR_V_IS_NEGATIVE */
        return phi != v_new[0];
    }
};

/* SISe3_sp, src/models/SISe3_sp.c:50-255: SISe3 with the local spread of
 * SISe_sp.  gdata = (upsilon_1..3, gamma_1..3, alpha, beta_t1..beta_t4,
 * coupling), ldata = (end_t1..end_t4, neighbours), v = (phi). */
struct ModelSISe3_sp {
    static constexpr int NC = 6, NT = 6, ND = 1;
    static constexpr int NGD = 12;  /* gdata entries read */
    static constexpr bool PTS_LOCAL = false;
    static constexpr bool RATES_TIME_INVARIANT = true;  /* rate() ignores t */
    template <class DC>
    __device__ __forceinline__ static double rate(int k, const int *u, const double *v,
                                                  const double *ldata, const double *gdata,
                                                  double t, DC &dc)
    {
        return ModelSISe3::rate(k, u, v, ldata, gdata, t, dc);
    }
    __device__ __forceinline__ static int pts(double *v_new, const int *u, const double *v,
                                              const double *ldata, const double *gdata,
                                              int node, double t)
    {
        const int day = (int) t % 365;
        const double I_i = u[1] + u[3] + u[5];
        const double N_i = u[0] + u[2] + u[4] + I_i;
        const double phi = v[0];
        v_new[0] = forward_euler_linear_decay(phi, day, (int) ldata[0], (int) ldata[1],
                                              (int) ldata[2], (int) ldata[3], gdata[7],
                                              gdata[8], gdata[9], gdata[10]);
        if (N_i > 0.0)
            v_new[0] += gdata[6] * I_i / N_i +
                        local_spread(ldata + 4, v - node, u - 6 * node, N_i, phi, 6, gdata[11]);
        if (!isfinite(v_new[0]))
            return -7;
        if (v_new[0] < 0.0)
            return -10;
        return phi != v_new[0];
    }
};

/* mparse SIR (R/C-generator.R:204-247 output for "S -> beta*S*I/N -> I",
 * "I -> gamma*I -> R", N <- S+I+R); gdata = (beta, gamma). */
struct ModelSIRmparse {
    static constexpr int NC = 3, NT = 2, ND = 0;
    static constexpr int NGD = 2;  /* gdata entries read */
    static constexpr bool PTS_LOCAL = true;
    static constexpr bool RATES_TIME_INVARIANT = true;  /* rate() ignores t */
    template <class DC>
    __device__ __forceinline__ static double rate(int k, const int *u, const double *v,
                                                  const double *ldata, const double *gdata,
                                                  double t, DC &dc)
    {
        if (k == 0) {
            const double N = si_i2d(u[0] + u[1] + u[2]);             /* int sum, as in C */
            return si_div_cached(gdata[0] * si_i2d(u[0]) * si_i2d(u[1]), N, &dc);
        }
        return gdata[1] * si_i2d(u[1]);
    }
    __device__ __forceinline__ static int pts(double *, const int *, const double *,
                                              const double *, const double *, int, double)
    {
        return 0;
    }
};

/* mparse SISe for the particle filter: "S -> upsilon*phi*S -> I",
 * "I -> gamma*I -> S", pts_fun phi <- phi*(1-0.03) + 0.05*I/(S+I);
 * gdata = (upsilon, gamma), v = (phi). */
struct ModelSISePF {
    static constexpr int NC = 2, NT = 2, ND = 1;
    static constexpr int NGD = 2;  /* gdata entries read */
    static constexpr bool PTS_LOCAL = true;
    static constexpr bool RATES_TIME_INVARIANT = true;  /* rate() ignores t */
    template <class DC>
    __device__ __forceinline__ static double rate(int k, const int *u, const double *v,
                                                  const double *ldata, const double *gdata,
                                                  double t, DC &dc)
    {
        if (k == 0)
            return gdata[0] * v[0] * si_i2d(u[0]);
        return gdata[1] * si_i2d(u[1]);
    }
    __device__ __forceinline__ static int pts(double *v_new, const int *u, const double *v,
                                              const double *ldata, const double *gdata,
                                              int node, double t)
    {
        const double S_n = u[0];
        const double I_n = u[1];
        const double n = S_n + I_n;
        v_new[0] = v[0] * (1.0 - 0.03);
        if (n > 0.0)
            v_new[0] += 0.05 * I_n / n;
        return v[0] != v_new[0];
    }
};

}  // namespace siminf

#endif
