/*
 * ref_solver_aem.c -- the reference's aem solver
 * (src/solvers/SimInf_solver_aem.c), compiled unmodified by including it
 * (oracle test infrastructure).  Its calcTimes draws with no `node` in
 * scope, and the stub's draw macro names one: this file-scope `node` is the
 * one it finds.  The aem solver is only run with independent generators
 * (shim_set_independent(1)), which ignore the node.
 */
static const long node = 0;
#include "solvers/SimInf_solver_aem.c"
