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

static const oracle_model models[] = {
    {"SIR", 3, 2, 0, {sir_s_to_i, sir_i_to_r}, pts_none},
    {"SEIR", 4, 3, 0, {seir_s_to_e, seir_e_to_i, seir_i_to_r}, pts_none},
    {"SIS", 2, 2, 0, {sis_s_to_i, sis_i_to_s}, pts_none},
    {"SISe", 2, 2, 1, {sise_s_to_i, sise_i_to_s}, sise_pts},
    {"SISe3", 6, 6, 1, {sise3_s1, sise3_i1, sise3_s2, sise3_i2, sise3_s3, sise3_i3}, sise3_pts},
    {"SIR_mparse", 3, 2, 0, {mp_sir_1, mp_sir_2}, pts_none},
    {"SISe_pf", 2, 2, 1, {pf_s_to_i, pf_i_to_s}, pf_pts},
};

const oracle_model *oracle_model_lookup(const char *name)
{
    for (size_t i = 0; i < sizeof(models) / sizeof(models[0]); i++)
        if (strcmp(models[i].name, name) == 0)
            return &models[i];
    return NULL;
}
