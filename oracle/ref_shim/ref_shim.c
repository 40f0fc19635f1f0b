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

struct gsl_rng {
    long offset;
};

static const gsl_rng_type type_mt = {"mt19937"};
static const gsl_rng_type type_taus = {"taus2"};
const gsl_rng_type *gsl_rng_mt19937 = &type_mt;
const gsl_rng_type *gsl_rng_taus2 = &type_taus;

static struct {
    uint64_t seed;
    int Nn, Nthread, Nrep, threads, verbose;
    int allocs;
    si_rng *streams;
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
    return 0;
}

void shim_release(void)
{
    free(g.streams);
    g.streams = NULL;
}

gsl_rng *gsl_rng_alloc(const gsl_rng_type *T)
{
    (void) T;
    gsl_rng *r = malloc(sizeof(*r));
    if (!r)
        return NULL;
    const int k = g.allocs++;
    if (k == 0) {
        r->offset = -1;                        /* master: never draws */
    } else {
        const long i = k - 1;
        r->offset = (g.Nrep > 1) ? i * g.Nn : i * (g.Nn / g.Nthread);
    }
    return r;
}

void gsl_rng_free(gsl_rng *r) { free(r); }
void gsl_rng_set(const gsl_rng *r, unsigned long int s) { (void) r; (void) s; }
unsigned long int gsl_rng_max(const gsl_rng *r) { (void) r; return 0xFFFFFFFFUL; }
unsigned long int gsl_rng_uniform_int(const gsl_rng *r, unsigned long int n)
{
    (void) r; (void) n;
    return 0;
}

static si_rng *stream(const gsl_rng *r, long node)
{
    return &g.streams[r->offset + node];
}

double shim_uniform_pos(const gsl_rng *r, long node)
{
    return si_uniform_pos(stream(r, node));
}

unsigned int shim_binomial(const gsl_rng *r, double p, unsigned int n, long node)
{
    return (unsigned int) si_binomial(stream(r, node), p, (int) n);
}

unsigned int shim_hypergeometric(const gsl_rng *r, unsigned int n1, unsigned int n2,
                                 unsigned int t, long node)
{
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
