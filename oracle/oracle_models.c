/*
 * oracle_models.c -- host model code for the oracle (test infrastructure).
 *
 * Rate and post-time-step functions follow the reference model files
 * expression for expression:
 *   SIR   src/models/SIR.c:43-87     (ldata: beta, gamma)
 *   SEIR  src/models/SEIR.c:43-112   (ldata: beta, epsilon, gamma)
 *   SIS   src/models/SIS.c           (ldata: beta, gamma)
 *   SISe3 src/models/SISe3.c:51-250 (N shift matrix, block-diagonal G)
 *   SISe  src/models/SISe.c:51-144   (ldata: end_t1..end_t4; gdata: upsilon,
 *         gamma, alpha, beta_t1..beta_t4, epsilon) with
 *         src/misc/SimInf_forward_euler_linear_decay.c:57-93
 * and two mparse models, written as R/C-generator.R:204-297 would emit them:
 *   SIR_mparse  "S -> beta*S*I/N -> I", "I -> gamma*I -> R", N <- S+I+R
 *   SISe_pf     "S -> upsilon*phi*S -> I", "I -> gamma*I -> S" with
 *               pts_fun phi <- phi*(1-0.03) + 0.05*I/(S+I)
 */
#include <math.h>
#include <string.h>
#include "oracle_models.h"

#define UNUSED(x) ((void) (x))

/* SIR, src/models/SIR.c */
static double sir_s_to_i(const int *u, const double *v, const double *ldata,
                         const double *gdata, double t)
{
    UNUSED(v); UNUSED(gdata); UNUSED(t);
    const double S_n = u[0];
    const double I_n = u[1];
    const double n = S_n + I_n + u[2];
    if (n > 0.0)
        return (ldata[0] * S_n * I_n) / n;
    return 0.0;
}

static double sir_i_to_r(const int *u, const double *v, const double *ldata,
                         const double *gdata, double t)
{
    UNUSED(v); UNUSED(gdata); UNUSED(t);
    return ldata[1] * u[1];
}

static int pts_none(double *v_new, const int *u, const double *v,
                    const double *ldata, const double *gdata, int node,
                    double t)
{
    UNUSED(v_new); UNUSED(u); UNUSED(v); UNUSED(ldata); UNUSED(gdata);
    UNUSED(node); UNUSED(t);
    return 0;
}

/* SEIR, src/models/SEIR.c */
static double seir_s_to_e(const int *u, const double *v, const double *ldata,
                          const double *gdata, double t)
{
    UNUSED(v); UNUSED(gdata); UNUSED(t);
    const double S_n = u[0];
    const double I_n = u[2];
    const double n = S_n + u[1] + I_n + u[3];
    if (n > 0.0)
        return ldata[0] * S_n * I_n / n;
    return 0.0;
}

static double seir_e_to_i(const int *u, const double *v, const double *ldata,
                          const double *gdata, double t)
{
    UNUSED(v); UNUSED(gdata); UNUSED(t);
    return ldata[1] * u[1];
}

static double seir_i_to_r(const int *u, const double *v, const double *ldata,
                          const double *gdata, double t)
{
    UNUSED(v); UNUSED(gdata); UNUSED(t);
    return ldata[2] * u[2];
}

/* SIS, src/models/SIS.c */
static double sis_s_to_i(const int *u, const double *v, const double *ldata,
                         const double *gdata, double t)
{
    UNUSED(v); UNUSED(gdata); UNUSED(t);
    const double S_n = u[0];
    const double I_n = u[1];
    const double n = S_n + I_n;
    if (n > 0.0)
        return (ldata[0] * S_n * I_n) / n;
    return 0.0;
}

static double sis_i_to_s(const int *u, const double *v, const double *ldata,
                         const double *gdata, double t)
{
    UNUSED(v); UNUSED(gdata); UNUSED(t);
    return ldata[1] * u[1];
}

/* SISe, src/models/SISe.c */
static double sise_s_to_i(const int *u, const double *v, const double *ldata,
                          const double *gdata, double t)
{
    UNUSED(ldata); UNUSED(t);
    return gdata[0] * v[0] * u[0];
}

static double sise_i_to_s(const int *u, const double *v, const double *ldata,
                          const double *gdata, double t)
{
    UNUSED(v); UNUSED(ldata); UNUSED(t);
    return gdata[1] * u[1];
}

/* src/misc/SimInf_forward_euler_linear_decay.c:57-93 */
static double decay(double phi, int day, int end_t1, int end_t2, int end_t3,
                    int end_t4, double b1, double b2, double b3, double b4)
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

static int sise_pts(double *v_new, const int *u, const double *v,
                    const double *ldata, const double *gdata, int node,
                    double t)
{
    UNUSED(node);
    const int day = (int) t % 365;
    const double I_n = u[1];
    const double n = u[0] + I_n;
    const double phi = v[0];
    v_new[0] = decay(phi, day, (int) ldata[0], (int) ldata[1], (int) ldata[2],
                     (int) ldata[3], gdata[3], gdata[4], gdata[5], gdata[6]);
    if (n > 0.0)
        v_new[0] += gdata[2] * I_n / n + gdata[7];
    else
        v_new[0] += gdata[7];
    if (!isfinite(v_new[0]))
        return -7;              /* SIMINF_ERR_V_IS_NOT_FINITE */
    if (v_new[0] < 0.0)
        return -10;             /* SIMINF_ERR_V_IS_NEGATIVE */
    return phi != v_new[0];
}

/* SISe3, src/models/SISe3.c; u = (S_1, I_1, S_2, I_2, S_3, I_3), v = (phi),
 * ldata = (end_t1..end_t4), gdata = (upsilon_1..3, gamma_1..3, alpha,
 * beta_t1..beta_t4, epsilon); transition order of SISe3_run. */
static double sise3_s1(const int *u, const double *v, const double *ldata,
                       const double *gdata, double t)
{
    UNUSED(ldata); UNUSED(t);
    return gdata[0] * v[0] * u[0];
}

static double sise3_i1(const int *u, const double *v, const double *ldata,
                       const double *gdata, double t)
{
    UNUSED(v); UNUSED(ldata); UNUSED(t);
    return gdata[3] * u[1];
}

static double sise3_s2(const int *u, const double *v, const double *ldata,
                       const double *gdata, double t)
{
    UNUSED(ldata); UNUSED(t);
    return gdata[1] * v[0] * u[2];
}

static double sise3_i2(const int *u, const double *v, const double *ldata,
                       const double *gdata, double t)
{
    UNUSED(v); UNUSED(ldata); UNUSED(t);
    return gdata[4] * u[3];
}

static double sise3_s3(const int *u, const double *v, const double *ldata,
                       const double *gdata, double t)
{
    UNUSED(ldata); UNUSED(t);
    return gdata[2] * v[0] * u[4];
}

static double sise3_i3(const int *u, const double *v, const double *ldata,
                       const double *gdata, double t)
{
    UNUSED(v); UNUSED(ldata); UNUSED(t);
    return gdata[5] * u[5];
}

static int sise3_pts(double *v_new, const int *u, const double *v,
                     const double *ldata, const double *gdata, int node, double t)
{
    UNUSED(node);
    const int day = (int) t % 365;
    const double I_n = u[1] + u[3] + u[5];
    const double n = I_n + u[0] + u[2] + u[4];
    const double phi = v[0];
    v_new[0] = decay(phi, day, (int) ldata[0], (int) ldata[1], (int) ldata[2],
                     (int) ldata[3], gdata[7], gdata[8], gdata[9], gdata[10]);
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

/* mparse SIR: N <- S+I+R; beta = gdata[0], gamma = gdata[1]. */
static double mp_sir_1(const int *u, const double *v, const double *ldata,
                       const double *gdata, double t)
{
    UNUSED(v); UNUSED(ldata); UNUSED(t);
    const double N = u[0] + u[1] + u[2];
    return gdata[0] * u[0] * u[1] / N;
}

static double mp_sir_2(const int *u, const double *v, const double *ldata,
                       const double *gdata, double t)
{
    UNUSED(v); UNUSED(ldata); UNUSED(t);
    return gdata[1] * u[1];
}

/* mparse SISe for the particle filter: upsilon = gdata[0], gamma = gdata[1],
 * phi = v[0]. */
static double pf_s_to_i(const int *u, const double *v, const double *ldata,
                        const double *gdata, double t)
{
    UNUSED(ldata); UNUSED(t);
    return gdata[0] * v[0] * u[0];
}

static double pf_i_to_s(const int *u, const double *v, const double *ldata,
                        const double *gdata, double t)
{
    UNUSED(v); UNUSED(ldata); UNUSED(t);
    return gdata[1] * u[1];
}

static int pf_pts(double *v_new, const int *u, const double *v,
                  const double *ldata, const double *gdata, int node, double t)
{
    UNUSED(ldata); UNUSED(gdata); UNUSED(node); UNUSED(t);
    const double S_n = u[0];
    const double I_n = u[1];
    const double n = S_n + I_n;
    v_new[0] = v[0] * (1.0 - 0.03);
    if (n > 0.0)
        v_new[0] += 0.05 * I_n / n;
    return v[0] != v_new[0];
}

/* src/misc/SimInf_local_spread.c:43-71: neighbours' contribution to phi
 * of node i; neighbors is (index, distance) pairs ended by index -1, phi
 * and u point at the first node. */
static double local_spread(const double *neighbors, const double *phi, const int *u,
                           double N_i, double phi_i, int Nc, double D)
{
    double ls = 0.0;
    const double phi_i_N_i = phi_i * N_i;
    for (int j = (int) neighbors[0]; j >= 0; j = (int) neighbors[0]) {
        double N_j = 0;
        for (int k = j * Nc; k < (j + 1) * Nc; k++)
            N_j += u[k];
        if (N_j > 0.0)
            ls += ((phi[j] * N_j - phi_i_N_i) * D) / (N_i * neighbors[1]);
        neighbors += 2;
    }
    return ls;
}

/* SISe_sp, src/models/SISe_sp.c:108-160: the SISe rates; the post time
 * step adds the local spread from the neighbours after end_t1..end_t4 in
 * ldata; gdata = (upsilon, gamma, alpha, beta_t1..beta_t4, coupling).  It
 * reads other nodes through offsets from its own node's u and v. */
static int sise_sp_pts(double *v_new, const int *u, const double *v,
                       const double *ldata, const double *gdata, int node, double t)
{
    const int day = (int) t % 365;
    const double I_i = u[1];
    const double N_i = u[0] + I_i;
    const double phi = v[0];
    v_new[0] = decay(phi, day, (int) ldata[0], (int) ldata[1], (int) ldata[2],
                     (int) ldata[3], gdata[3], gdata[4], gdata[5], gdata[6]);
    if (N_i > 0.0)
        v_new[0] += gdata[2] * I_i / N_i +
                    local_spread(&ldata[4], &v[-node], &u[-2 * node], N_i, phi, 2, gdata[7]);
    if (!isfinite(v_new[0]))
        return -7;
    if (v_new[0] < 0.0)
        return -10;
    return phi != v_new[0];
}

/* SISe3_sp, src/models/SISe3_sp.c:207-255: the SISe3 rates with the local
 * spread; gdata = (upsilon_1..3, gamma_1..3, alpha, beta_t1..4, coupling). */
static int sise3_sp_pts(double *v_new, const int *u, const double *v,
                        const double *ldata, const double *gdata, int node, double t)
{
    const int day = (int) t % 365;
    const double I_i = u[1] + u[3] + u[5];
    const double N_i = u[0] + u[2] + u[4] + I_i;
    const double phi = v[0];
    v_new[0] = decay(phi, day, (int) ldata[0], (int) ldata[1], (int) ldata[2],
                     (int) ldata[3], gdata[7], gdata[8], gdata[9], gdata[10]);
    if (N_i > 0.0)
        v_new[0] += gdata[6] * I_i / N_i +
                    local_spread(&ldata[4], &v[-node], &u[-6 * node], N_i, phi, 6, gdata[11]);
    if (!isfinite(v_new[0]))
        return -7;
    if (v_new[0] < 0.0)
        return -10;
    return phi != v_new[0];
}

static const oracle_model models[] = {
    {"SIR", 3, 2, 0, {sir_s_to_i, sir_i_to_r}, pts_none},
    {"SEIR", 4, 3, 0, {seir_s_to_e, seir_e_to_i, seir_i_to_r}, pts_none},
    {"SIS", 2, 2, 0, {sis_s_to_i, sis_i_to_s}, pts_none},
    {"SISe", 2, 2, 1, {sise_s_to_i, sise_i_to_s}, sise_pts},
    {"SISe3", 6, 6, 1, {sise3_s1, sise3_i1, sise3_s2, sise3_i2, sise3_s3, sise3_i3}, sise3_pts},
    {"SIR_mparse", 3, 2, 0, {mp_sir_1, mp_sir_2}, pts_none},
    {"SISe_pf", 2, 2, 1, {pf_s_to_i, pf_i_to_s}, pf_pts},
    {"SISe_sp", 2, 2, 1, {sise_s_to_i, sise_i_to_s}, sise_sp_pts},
    {"SISe3_sp", 6, 6, 1, {sise3_s1, sise3_i1, sise3_s2, sise3_i2, sise3_s3, sise3_i3},
     sise3_sp_pts},
};

/* Models registered at run time: host builds of generated model code,
 * whose rate and post-time-step functions the test suite hands over. */
enum { MAX_REGISTERED = 64 };
static oracle_model registered[MAX_REGISTERED];
static char registered_names[MAX_REGISTERED][64];
static int n_registered;

int oracle_register_model(const char *name, int Nc, int Nt, int Nd, const oracle_trfun *tr,
                          oracle_ptsfun pts)
{
    if (Nt < 1 || Nt > 32 || strlen(name) >= 64)
        return -1;
    int k = 0;
    while (k < n_registered && strcmp(registered_names[k], name) != 0)
        k++;
    if (k == n_registered) {
        if (n_registered == MAX_REGISTERED)
            return -1;
        n_registered++;
    }
    strcpy(registered_names[k], name);
    oracle_model *m = &registered[k];
    m->name = registered_names[k];
    m->Nc = Nc;
    m->Nt = Nt;
    m->Nd = Nd;
    for (int j = 0; j < 32; j++)
        m->tr[j] = j < Nt ? tr[j] : NULL;
    m->pts = pts;
    return 0;
}

const oracle_model *oracle_model_lookup(const char *name)
{
    for (size_t i = 0; i < sizeof(models) / sizeof(models[0]); i++)
        if (strcmp(models[i].name, name) == 0)
            return &models[i];
    for (int k = 0; k < n_registered; k++)
        if (strcmp(registered_names[k], name) == 0)
            return &registered[k];
    return NULL;
}
