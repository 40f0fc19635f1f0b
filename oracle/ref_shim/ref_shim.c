/*
 * ref_shim.c -- the R and GSL symbols the reference solver sources need,
 * for building them unmodified into oracle/_ref (oracle test
 * infrastructure; never part of the product).
 *
 * Generators: gsl_rng_alloc is called once for the master generator
 * (src/solvers/SimInf_solver_ssm.c:391, src/solvers/SimInf_solver_mssm.c:
 * 420) and then once per solver thread (src/solvers/SimInf_solver.c:474).
 * Thread i's generator serves nodes [Ni, Ni + Nn_i) with local node
 * indices (Ni = i * (Nn / Nthread), src/solvers/SimInf_solver.c:1096) or,
 * for replicated models run with Nthread == Nrep, replicate i.  Its offset
 * turns the local `node` at a draw site into the global stream id
 * replicate * Nn + node, so draws match siminf_stream.h's keying.
 *
 * Independent mode (shim_set_independent(1)), for the distribution tests
 * against the reference: every generator is instead a 32-bit Mersenne
 * twister (M. Matsumoto and T. Nishimura, ACM TOMACS 8(1), 1998: the
 * published MT19937 recurrence, tempering and initialisation), the master
 * seeded with the run's seed and each thread's generator from the master,
 * as the reference seeds its GSL generators (src/solvers/SimInf_solver.c:
 * 474-477); uniforms are word / 2^32 with zero rejected, and the samplers
 * draw from a stream keyed by two of the thread's words.
 */
#include <stdarg.h>
#include <stdint.h>
#include <stdlib.h>
#include <stdio.h>
#ifdef _OPENMP
#  include <omp.h>
#endif
#include "R.h"
#include "gsl/gsl_rng.h"
#include "gsl/gsl_randist.h"
#include "../../siminf_gb300/csrc/siminf_stream.h"

enum { MT_N = 624, MT_M = 397 };

struct gsl_rng {
    long offset;
    int crn;                /* one of mssm_crn's per-(replicate, node) generators */
    uint32_t mt[MT_N];
    int mti;
};

static void mt_seed(gsl_rng *r, uint32_t s)
{
    r->mt[0] = s;
    for (int i = 1; i < MT_N; i++)
        r->mt[i] = 1812433253u * (r->mt[i - 1] ^ (r->mt[i - 1] >> 30)) + (uint32_t) i;
    r->mti = MT_N;
}

static uint32_t mt_next(gsl_rng *r)
{
    static const uint32_t mag01[2] = {0x0u, 0x9908b0dfu};
    uint32_t y;
    if (r->mti >= MT_N) {
        int kk;
        for (kk = 0; kk < MT_N - MT_M; kk++) {
            y = (r->mt[kk] & 0x80000000u) | (r->mt[kk + 1] & 0x7fffffffu);
            r->mt[kk] = r->mt[kk + MT_M] ^ (y >> 1) ^ mag01[y & 1u];
        }
        for (; kk < MT_N - 1; kk++) {
            y = (r->mt[kk] & 0x80000000u) | (r->mt[kk + 1] & 0x7fffffffu);
            r->mt[kk] = r->mt[kk + (MT_M - MT_N)] ^ (y >> 1) ^ mag01[y & 1u];
        }
        y = (r->mt[MT_N - 1] & 0x80000000u) | (r->mt[0] & 0x7fffffffu);
        r->mt[MT_N - 1] = r->mt[MT_M - 1] ^ (y >> 1) ^ mag01[y & 1u];
        r->mti = 0;
    }
    y = r->mt[r->mti++];
    y ^= (y >> 11);
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= (y >> 18);
    return y;
}

static int g_independent;

void shim_set_independent(int on)
{
    g_independent = on;
}

static const gsl_rng_type type_mt = {"mt19937"};
static const gsl_rng_type type_taus = {"taus2"};
const gsl_rng_type *gsl_rng_mt19937 = &type_mt;
const gsl_rng_type *gsl_rng_taus2 = &type_taus;

static struct {
    uint64_t seed;
    int Nn, Nthread, Nrep, threads, verbose;
    int allocs;
    si_rng *streams;
    si_rng *crn_streams;    /* replicated models: the SSA streams of mssm_crn */
} g;

int shim_configure(uint64_t seed, int Nn, int Nthread, int Nrep, int threads)
{
    const long n = (long) Nn * (Nrep > 0 ? Nrep : 1);
    g.seed = seed;
    g.Nn = Nn;
    g.Nthread = Nthread;
    g.Nrep = Nrep;
    g.threads = threads > 0 ? threads : 1;
    g.allocs = 0;
    g.verbose = getenv("SIMINF_REF_VERBOSE") != NULL;
    free(g.streams);
    g.streams = malloc((size_t) (n > 0 ? n : 1) * sizeof(si_rng));
    if (!g.streams)
        return -1;
    for (long i = 0; i < n; i++)
        si_rng_init(&g.streams[i], seed, (uint64_t) i, 0);
    free(g.crn_streams);
    g.crn_streams = NULL;
    if (Nrep > 1) {
        g.crn_streams = malloc((size_t) n * sizeof(si_rng));
        if (!g.crn_streams)
            return -1;
        for (long i = 0; i < n; i++)
            si_rng_init(&g.crn_streams[i], seed, SI_CRN_SID | (uint64_t) i, 0);
    }
    return 0;
}

void shim_release(void)
{
    free(g.streams);
    g.streams = NULL;
    free(g.crn_streams);
    g.crn_streams = NULL;
}

gsl_rng *gsl_rng_alloc(const gsl_rng_type *T)
{
    (void) T;
    gsl_rng *r = malloc(sizeof(*r));
    if (!r)
        return NULL;
    const int k = g.allocs++;
    mt_seed(r, (uint32_t) (g.seed ^ (g.seed >> 32)) + (uint32_t) k);
    r->crn = 0;
    if (k == 0) {
        r->offset = -1;                        /* master: never draws */
    } else if (k - 1 >= g.Nthread) {
        /* mssm_crn allocates one generator per (replicate, node) after the
         * threads' event generators (src/solvers/SimInf_solver_mssm_crn.c:
         * 459-473), replicate by replicate, node by node: the j-th is
         * stream j = replicate * Nn + node */
        r->crn = 1;
        r->offset = k - 1 - g.Nthread;
    } else {
        const long i = k - 1;
        r->offset = (g.Nrep > 1) ? i * g.Nn : i * (g.Nn / g.Nthread);
    }
    return r;
}

void gsl_rng_free(gsl_rng *r) { free(r); }
void gsl_rng_set(const gsl_rng *r, unsigned long int s)
{
    if (g_independent)
        mt_seed((gsl_rng *) r, (uint32_t) s);
}
unsigned long int gsl_rng_max(const gsl_rng *r) { (void) r; return 0xFFFFFFFFUL; }
unsigned long int gsl_rng_uniform_int(const gsl_rng *r, unsigned long int n)
{
    if (!g_independent || n == 0)
        return 0;
    return (unsigned long int) mt_next((gsl_rng *) r) % n;
}

static si_rng *stream(const gsl_rng *r, long node)
{
    if (r->crn)
        return &g.crn_streams[r->offset];      /* its own stream, whatever `node` says */
    return &g.streams[r->offset + node];
}

/* Independent mode: a stream keyed by two of the generator's words. */
static si_rng independent_stream(const gsl_rng *r)
{
    si_rng s;
    const uint64_t k = ((uint64_t) mt_next((gsl_rng *) r) << 32) | mt_next((gsl_rng *) r);
    si_rng_init(&s, k, 0x5EEDull, 0);
    return s;
}

double shim_uniform_pos(const gsl_rng *r, long node)
{
    if (g_independent) {
        uint32_t w;
        do
            w = mt_next((gsl_rng *) r);
        while (w == 0);
        return (double) w / 4294967296.0;
    }
    return si_uniform_pos(stream(r, node));
}

unsigned int shim_binomial(const gsl_rng *r, double p, unsigned int n, long node)
{
    if (g_independent) {
        si_rng s = independent_stream(r);
        return (unsigned int) si_binomial(&s, p, (int) n);
    }
    return (unsigned int) si_binomial(stream(r, node), p, (int) n);
}

unsigned int shim_hypergeometric(const gsl_rng *r, unsigned int n1, unsigned int n2,
                                 unsigned int t, long node)
{
    if (g_independent) {
        si_rng s = independent_stream(r);
        return (unsigned int) si_hypergeometric(&s, (int) n1, (int) n2, (int) t);
    }
    return (unsigned int) si_hypergeometric(stream(r, node), (int) n1, (int) n2, (int) t);
}

int SimInf_num_threads(void) { return g.threads; }

void REprintf(const char *fmt, ...)
{
    if (!g.verbose)
        return;
    va_list ap;
    va_start(ap, fmt);
    vfprintf(stderr, fmt, ap);
    va_end(ap);
}

void Rprintf(const char *fmt, ...)
{
    if (!g.verbose)
        return;
    va_list ap;
    va_start(ap, fmt);
    vfprintf(stderr, fmt, ap);
    va_end(ap);
}

void R_FlushConsole(void) {}
