/*
 * siminf_kernels.cu -- the lookup of the models the library ships
 * (siminf_models.cuh; their kernels are instantiated in siminf_models_a.cu,
 * _b.cu and _c.cu), and the particle filter's kernels, which do not depend
 * on the model.
 */
#include "siminf_kernels.cuh"

namespace siminf {

/* ------------------------------------------------------------------ */
/* Particle filter (R/pfilter.R:417-452, src/misc/SimInf_particle_filter.c: */
/* 33-67): log-weights, normalisation, ESS, systematic resampling and   */
/* the ancestors' state copy.  Sums run in particle or node order on one */
/* thread so that every bit matches the CPU restatement.                */
/* ------------------------------------------------------------------ */
#define PF_LOG_FLOOR (-690.0)

__device__ __forceinline__ double pf_logdens(const double *lfact, int tablen, int k, int n,
                                             double logp, double logq)
{
    if (k < 0 || n < 0 || k > n || n >= tablen)
        return PF_LOG_FLOOR;
    return (((lfact[n] - lfact[k]) - lfact[n - k]) + (double) k * logp) +
           (double) (n - k) * logq;
}

__global__ void k_pf_weights(const int *U, int tlen, int Nn, int Nc, int Np, const int *obs_row,
                             int obs_c, const double *lfact, int tablen, double logp, double logq,
                             double *w, const int *interval)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= Np)
        return;
    if (interval)
        obs_row += (size_t) *interval * Nn;     /* obs_row is the first interval's row */
    const int *last = U + ((size_t) p * tlen + tlen - 1) * (size_t) Nn * Nc;
    double acc = 0.0;
    for (int node = 0; node < Nn; node++)
        acc = acc + pf_logdens(lfact, tablen, obs_row[node], last[(size_t) node * Nc + obs_c],
                               logp, logq);
    w[p] = acc;
}

/* One block: max (exact in any order), exp in parallel, then the serial
 * sums, log-likelihood, ESS and resampling on thread 0. */
__global__ void k_pf_finalize(double *w, int Np, double log_np, double *loglik, double *ess,
                              int i, uint64_t seed, uint64_t sid, int *anc, int *anc_out,
                              int *interval, const uint64_t *seed_dev)
{
    if (seed_dev)
        seed = *seed_dev;               /* graph replay: the pass's seed */
    if (interval) {
        /* graph replay: the interval, its resampling stream and its row of
         * ancestors come from the device counter, which moves on at the end */
        i = *interval;
        sid += (uint64_t) i;
        if (anc_out)
            anc_out += (size_t) i * Np;
    }
    __shared__ double red[1024];
    __shared__ double s_sum;
    double m = -INFINITY;
    for (int p = threadIdx.x; p < Np; p += blockDim.x)
        m = fmax(m, w[p]);
    red[threadIdx.x] = m;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o)
            red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + o]);
        __syncthreads();
    }
    const double max_w = red[0];
    for (int p = threadIdx.x; p < Np; p += blockDim.x)
        w[p] = si_exp(w[p] - max_w);
    __syncthreads();
    if (threadIdx.x == 0) {
        double sum = 0.0;
        for (int p = 0; p < Np; p++)
            sum = sum + w[p];
        *loglik = ((*loglik + max_w) + si_log(sum)) - log_np;
        s_sum = sum;
    }
    __syncthreads();
    for (int p = threadIdx.x; p < Np; p += blockDim.x)
        w[p] = w[p] / s_sum;
    __syncthreads();
    if (threadIdx.x == 0) {
        double sq = 0.0;
        for (int p = 0; p < Np; p++)
            sq = sq + w[p] * w[p];
        ess[i] = 1.0 / sq;
        /* systematic resampling */
        double cumsum_w = 0;
        for (int p = 0; p < Np; p++)
            cumsum_w += w[p];
        si_rng r;
        si_rng_init(&r, seed, sid, 0);
        const double du = cumsum_w / (double) Np;
        double u = du * si_uniform_pos(&r);
        cumsum_w = w[0];
        for (int p = 0, j = 0; p < Np; p++) {
            while (u > cumsum_w && j < Np - 1)
                cumsum_w += w[++j];
            anc[p] = j;
            if (anc_out)
                anc_out[p] = j + 1;
            u += du;
        }
        if (interval)
            *interval = i + 1;
    }
}

__global__ void k_pf_gather(const int *U, const double *V, int tlen, long long nu, long long nv,
                            const int *anc, int Np, int *u0, double *v0)
{
    const long long idx = blockIdx.x * (long long) blockDim.x + threadIdx.x;
    if (idx < (long long) Np * nu) {
        const int p = (int) (idx / nu);
        const long long r = idx - (long long) p * nu;
        u0[idx] = U[((size_t) anc[p] * tlen + tlen - 1) * nu + r];
    }
    if (V && idx < (long long) Np * nv) {
        const int p = (int) (idx / nv);
        const long long r = idx - (long long) p * nv;
        v0[idx] = V[((size_t) anc[p] * tlen + tlen - 1) * nv + r];
    }
}

cudaError_t pf_weights(const int *U, int tlen, int Nn, int Nc, int Np, const int *obs_row,
                       int obs_c, const double *lfact, int tablen, double logp, double logq,
                       double *w, cudaStream_t st, const int *interval)
{
    k_pf_weights<<<(Np + 127) / 128, 128, 0, st>>>(U, tlen, Nn, Nc, Np, obs_row, obs_c, lfact,
                                                   tablen, logp, logq, w, interval);
    return cudaGetLastError();
}

cudaError_t pf_finalize(double *w, int Np, double log_np, double *loglik, double *ess, int i,
                        uint64_t seed, uint64_t sid, int *anc, int *anc_out, cudaStream_t st,
                        int *interval, const uint64_t *seed_dev)
{
    k_pf_finalize<<<1, 1024, 0, st>>>(w, Np, log_np, loglik, ess, i, seed, sid, anc, anc_out,
                                      interval, seed_dev);
    return cudaGetLastError();
}

cudaError_t pf_gather(const int *U, const double *V, int tlen, long long nu, long long nv,
                      const int *anc, int Np, int *u0, double *v0, cudaStream_t st)
{
    const long long n = (long long) Np * (nu > nv ? nu : nv);
    k_pf_gather<<<(unsigned) ((n + 255) / 256), 256, 0, st>>>(U, V, tlen, nu, nv, anc, Np, u0, v0);
    return cudaGetLastError();
}

/* The shipped models' launcher tables, instantiated in three translation
 * units (siminf_models_a.cu, _b.cu, _c.cu) that compile in parallel. */
const Launchers *launchers_shipped_a(const char *name);
const Launchers *launchers_shipped_b(const char *name);
const Launchers *launchers_shipped_c(const char *name);

const Launchers *launchers_for(const char *name)
{
    const Launchers *t = launchers_shipped_a(name);
    if (!t)
        t = launchers_shipped_b(name);
    return t ? t : launchers_shipped_c(name);
}

}  // namespace siminf
