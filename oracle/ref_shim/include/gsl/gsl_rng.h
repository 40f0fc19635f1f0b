/* Stub of gsl/gsl_rng.h (oracle test infrastructure).
 *
 * Every draw the reference solver makes is routed to the per-node
 * Philox4x32-10 stream of siminf_stream.h.  The stream is chosen from the
 * generator's thread offset plus the variable `node`, which is in scope at
 * every draw site of the solver sources (src/solvers/SimInf_solver_ssm.c:
 * 155,165, src/solvers/SimInf_solver_mssm.c:172,183,
 * src/solvers/SimInf_solver.c:98,149,184,274,298). */
#ifndef SHIM_GSL_RNG_H
#define SHIM_GSL_RNG_H
typedef struct gsl_rng_type { const char *name; } gsl_rng_type;
typedef struct gsl_rng gsl_rng;
extern const gsl_rng_type *gsl_rng_mt19937;
extern const gsl_rng_type *gsl_rng_taus2;
gsl_rng *gsl_rng_alloc(const gsl_rng_type *T);
void gsl_rng_free(gsl_rng *r);
void gsl_rng_set(const gsl_rng *r, unsigned long int s);
unsigned long int gsl_rng_max(const gsl_rng *r);
unsigned long int gsl_rng_uniform_int(const gsl_rng *r, unsigned long int n);
double shim_uniform_pos(const gsl_rng *r, long node);
#define gsl_rng_uniform_pos(r) shim_uniform_pos((r), (long) (node))
#endif
