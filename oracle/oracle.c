/*
 * oracle.c -- CPU restatement of the cuda_mcmc MCMC-RE hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: it is loaded by the
 * tests, by __graft_entry__.smoke() and by bench.py's cpu_baseline /
 * --impl reference legs, and never by the cuda_mcmc_gb300 product path.
 *
 * What it restates (paths are relative to the MITHaystack/cuda_mcmc tree):
 *   - the Sgr A* crescent + Gaussian visibility models in FP64:
 *       sgra_model9   examples/sgra_model_fit/model.cuh:322-462
 *                     (same maths as xringaus, src/obsdatafit.py:1476-1608)
 *       sgra_model13  examples/sgra_model_fit/model.cuh:120-315
 *                     (the GPU variant, i.e. WITHOUT the d1*V inner-ring
 *                     shift that xringaus2 has at obsdatafit.py:1690-1691)
 *     and the model() dispatcher with its two passes and closure phases,
 *     examples/sgra_model_fit/model.cuh:9-115;
 *   - the other plugin models: Rosenbrock (examples/search_Rosenbrock/
 *     model.cuh:40-41, generalised to N dimensions), the two-equation
 *     system (examples/solvsys/model.cuh:51-54) and the n-equation
 *     nonlinear system r_k = sum_j A_kj sin x_j + B_kj x_j^2 - b_k;
 *   - one chi^2 term, src/gpu_mcmc.cu:299-323;
 *   - the sweep: init_pcur :245-267, gen_proposal :361-411,
 *     spmp_mcmc :426-474, adjust_steps :480-526, replica_exchange
 *     :533-626, driven in the order of run_mcmc :682-763.
 *
 * A second arithmetic (or_problem.arith = OR_ARITH_F32, Sgr A* sgra_model9
 * only) evaluates the model and the chi^2 sum in float32 as the reference's
 * kernels do: float model values from float Bessel functions (j0f, j1f,
 * jnf), float closure wrap and terms (gpu_mcmc.cu:305-323) and the serial
 * float sum of a chi2m row (spmp_mcmc, :447-448).  The CPU baseline of the
 * benchmark times the sweep in that arithmetic.
 *
 * Random numbers are INJECTED: every replica ist = ibeta*nseq + iseq owns a
 * stream of uniforms in (0,1] and a stream of standard normals, consumed in
 * exactly the order in which the reference's kernels call curand_uniform()
 * and curand_normal() on rndst[ist].  Model values and chi^2 are computed in
 * double precision; parameters stay float32 as in the reference, and the
 * proposal step p + pstp*N(0,1) and the prior draw pmin + (pmax-pmin)*u are
 * single fused multiply-adds (fmaf), which is what nvcc emits for the
 * reference's float expressions.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define OR_PI 3.14159265358979323846

enum { OR_MODEL_SGRA = 1, OR_MODEL_ROSEN = 2, OR_MODEL_SOLVSYS = 3,
       OR_MODEL_NLSYS = 4 };

enum { OR_OK = 0, OR_ERR_ARG = 1, OR_ERR_STREAM = 2 };

/* ------------------------------------------------------------------------ */
/* Sgr A* visibility models (FP64).                                          */
/* ------------------------------------------------------------------------ */

/* sgra_model9, examples/sgra_model_fit/model.cuh:322-462 (xringaus). */
void or_sgra_model9(double ul, double vl, const double *prm,
                    double *vamp, double *vpha)
{
    const double pi = OR_PI, pi4 = 4.0 * OR_PI;
    double Zsp = prm[0], Rex = prm[1], rq = prm[2], ecc = prm[3];
    double fade = prm[4], gax = prm[5], aq = prm[6], gq = prm[7];
    double th = prm[8];
    double Rin, d, gsy, gsx, gcoef, h, h0, U, V, rho;
    double ree, ime, rei = 0.0, imi = 0.0, Fr_re, Fr_im, Vre, Vim;

    Rex = (pi / 180.0) * (Rex / 3600.0) * 1e3;   /* uas -> nrad */
    Rin = rq * Rex;
    d = ecc * (Rex - Rin);
    gsy = gax * Rex;
    gsx = aq * gsy;
    gcoef = 2.0 * pow(pi / (2.0 * sqrt(2.0 * log(2.0))), 2);
    h = (2.0 / pi) / ((Rex * Rex - Rin * Rin * (1.0 + d / Rex)) * fade
                      + (Rex * Rex - Rin * Rin * (1.0 - d / Rex)));
    h0 = fade * h;

    U = ul * cos(th) + vl * sin(th);
    V = -ul * sin(th) + vl * cos(th);
    rho = sqrt(U * U + V * V);

    if (rho > 1e-7) {
        double arg = 2.0 * pi * rho, aRex = arg * Rex;
        ree = 0.5 * (h + h0) * Rex * j1(aRex) / rho;
        ime = (h - h0) / pi4 * (pi * Rex * (j0(aRex) - jn(2, aRex)) / (rho * rho)
                                - j1(aRex) / (rho * rho * rho)) * U;
        if (Rin != 0.0) {
            double aRin = arg * Rin;
            rei = 0.5 * (h + h0 - d * (h - h0) / Rex) * Rin * j1(aRin) / rho;
            imi = (h - h0) / pi4 * rq * (pi * Rin * (j0(aRin) - jn(2, aRin))
                                         / (rho * rho)
                                         - j1(aRin) / (rho * rho * rho)) * U;
        }
    } else {                                      /* rho -> 0 limits */
        ree = 0.5 * (h + h0) * pi * Rex * Rex;
        ime = -0.25 * pi * pi * (h - h0) * Rex * Rex * Rex * U;
        if (Rin != 0.0) {
            rei = 0.5 * (h + h0 - d * (h - h0) / Rex) * pi * Rin * Rin;
            imi = -0.25 * pi * pi * (h - h0) * (pow(Rin, 4) / Rex) * U;
        }
    }
    if (Rin != 0.0) {
        double dre = cos(2.0 * pi * d * U), dim = sin(2.0 * pi * d * U);
        double fin_re = rei * dre - imi * dim, fin_im = rei * dim + imi * dre;
        Fr_re = ree - fin_re;
        Fr_im = ime - fin_im;
    } else {
        Fr_re = ree;
        Fr_im = ime;
    }
    if (gax == 0.0 || aq == 0.0 || gq == 0.0) {
        Vre = Zsp * Fr_re;
        Vim = Zsp * Fr_im;
    } else {
        double gshift = Rin - d;
        double Gamp = exp(-gcoef * (pow(U * gsx, 2) + pow(V * gsy, 2)));
        double Gph = -2.0 * pi * gshift * U;
        double Fg_re = Gamp * cos(Gph), Fg_im = Gamp * sin(Gph);
        Vre = Zsp * ((1.0 - gq) * Fr_re + gq * Fg_re);
        Vim = Zsp * ((1.0 - gq) * Fr_im + gq * Fg_im);
    }
    *vamp = sqrt(Vre * Vre + Vim * Vim);
    *vpha = atan2(Vim, Vre);
}

/* sgra_model13, examples/sgra_model_fit/model.cuh:120-315. */
void or_sgra_model13(double ul, double vl, const double *prm,
                     double *vamp, double *vpha)
{
    const double pi = OR_PI, pi4 = 4.0 * OR_PI;
    double Zsp = prm[0], Rex = prm[1], rq = prm[2], ecc = prm[3];
    double fade = prm[4], gr = prm[5], gax = prm[6], aq = prm[7];
    double gq = prm[8], alpha = prm[9], beta = prm[10], eta = prm[11];
    double th = prm[12];
    double Rin, D, d, h, h0, U, V, rho, ree, ime, rei = 0.0, imi = 0.0;
    double Fr_re, Fr_im, Fg_re = 0.0, Fg_im = 0.0, Vre, Vim;

    Rex = (pi / 180.0) * (Rex / 3600.0) * 1e3;
    Rin = rq * Rex;
    if (gax != 0.0 && aq != 0.0 && gq != 0.0) {
        double gsy = gax * Rex, gsx = aq * gsy;
        double Ub = ul * cos(beta) + vl * sin(beta);
        double Vb = -ul * sin(beta) + vl * cos(beta);
        double gshift = gr * Rex * (cos(alpha) * ul + sin(alpha) * vl);
        double fwhm2std = 2.0 * pow(pi / (2.0 * sqrt(2.0 * log(2.0))), 2);
        double Gamp = exp(-fwhm2std * (pow(Ub * gsx, 2) + pow(Vb * gsy, 2)));
        double Gph = -2.0 * pi * gshift;
        Fg_re = Gamp * cos(Gph);
        Fg_im = Gamp * sin(Gph);
    }
    if (gq == 1.0) {                              /* Gaussian only */
        Vre = Zsp * Fg_re;
        Vim = Zsp * Fg_im;
        *vamp = sqrt(Vre * Vre + Vim * Vim);
        *vpha = atan2(Vim, Vre);
        return;
    }
    D = ecc * (Rex - Rin);
    d = D * cos(eta - th);
    h = (2.0 / pi) / ((Rex * Rex - Rin * Rin * (1.0 + d / Rex)) * fade
                      + (Rex * Rex - Rin * Rin * (1.0 - d / Rex)));
    h0 = fade * h;
    U = ul * cos(th) + vl * sin(th);
    V = -ul * sin(th) + vl * cos(th);
    rho = sqrt(U * U + V * V);
    if (rho > 1e-7) {
        double arg = 2.0 * pi * rho, aRex = arg * Rex;
        ree = 0.5 * (h + h0) * Rex * j1(aRex) / rho;
        ime = (h - h0) / pi4 * (pi * Rex * (j0(aRex) - jn(2, aRex)) / (rho * rho)
                                - j1(aRex) / (rho * rho * rho)) * U;
        if (Rin != 0.0) {
            double aRin = arg * Rin;
            rei = 0.5 * (h + h0 - d * (h - h0) / Rex) * Rin * j1(aRin) / rho;
            imi = (h - h0) / pi4 * rq * (pi * Rin * (j0(aRin) - jn(2, aRin))
                                         / (rho * rho)
                                         - j1(aRin) / (rho * rho * rho)) * U;
        }
    } else {
        ree = 0.5 * (h + h0) * pi * Rex * Rex;
        ime = -0.25 * pi * pi * (h - h0) * Rex * Rex * Rex * U;
        if (Rin != 0.0) {
            rei = 0.5 * (h + h0 - d * (h - h0) / Rex) * pi * Rin * Rin;
            imi = -0.25 * pi * pi * (h - h0) * (pow(Rin, 4) / Rex) * U;
        }
    }
    if (Rin != 0.0) {
        double dre = cos(2.0 * pi * d * U), dim = sin(2.0 * pi * d * U);
        double fin_re = rei * dre - imi * dim, fin_im = rei * dim + imi * dre;
        Fr_re = ree - fin_re;
        Fr_im = ime - fin_im;
    } else {
        Fr_re = ree;
        Fr_im = ime;
    }
    if (gax == 0.0 || aq == 0.0 || gq == 0.0) {
        Vre = Zsp * Fr_re;
        Vim = Zsp * Fr_im;
    } else {
        Vre = Zsp * ((1.0 - gq) * Fr_re + gq * Fg_re);
        Vim = Zsp * ((1.0 - gq) * Fr_im + gq * Fg_im);
    }
    *vamp = sqrt(Vre * Vre + Vim * Vim);
    *vpha = atan2(Vim, Vre);
}

/* Batch helper for fixtures: one parameter vector, n uv points. */
int or_sgra_vis(int imodel, const double *prm, int n, const double *u,
                const double *v, double *amp, double *pha)
{
    int i;
    if (imodel != 1 && imodel != 2) return OR_ERR_ARG;
    for (i = 0; i < n; i++) {
        if (imodel == 1) or_sgra_model9(u[i], v[i], prm, &amp[i], &pha[i]);
        else or_sgra_model13(u[i], v[i], prm, &amp[i], &pha[i]);
    }
    return OR_OK;
}

/* sgra_model9 in float32 arithmetic (the reference's kernels compute in
 * float, examples/sgra_model_fit/model.cuh:322-462): the same maths as
 * or_sgra_model9 with float operations and float Bessel functions. */
void or_sgra_model9_f(float ul, float vl, const float *prm, float *vamp, float *vpha)
{
    const float pi = (float)OR_PI, pi4 = 4.0f * (float)OR_PI;
    float Zsp = prm[0], Rex = prm[1], rq = prm[2], ecc = prm[3];
    float fade = prm[4], gax = prm[5], aq = prm[6], gq = prm[7], th = prm[8];
    float Rin, d, gsy, gsx, gcoef, h, h0, U, V, rho, cth, sth;
    float ree, ime, rei = 0.0f, imi = 0.0f, Fr_re, Fr_im, Vre, Vim;

    Rex = (pi / 180.0f) * (Rex / 3600.0f) * 1e3f;
    Rin = rq * Rex;
    d = ecc * (Rex - Rin);
    gsy = gax * Rex;
    gsx = aq * gsy;
    gcoef = 2.0f * powf(pi / (2.0f * sqrtf(2.0f * logf(2.0f))), 2.0f);
    h = (2.0f / pi) / ((Rex * Rex - Rin * Rin * (1.0f + d / Rex)) * fade
                       + (Rex * Rex - Rin * Rin * (1.0f - d / Rex)));
    h0 = fade * h;
    cth = cosf(th);
    sth = sinf(th);
    U = ul * cth + vl * sth;
    V = -ul * sth + vl * cth;
    rho = sqrtf(U * U + V * V);
    if (rho > 1e-7f) {
        float arg = 2.0f * pi * rho, aRex = arg * Rex, r2 = rho * rho, r3 = r2 * rho;
        float b1 = j1f(aRex);
        ree = 0.5f * (h + h0) * Rex * b1 / rho;
        ime = (h - h0) / pi4 * (pi * Rex * (j0f(aRex) - jnf(2, aRex)) / r2 - b1 / r3) * U;
        if (Rin != 0.0f) {
            float aRin = arg * Rin, c1 = j1f(aRin);
            rei = 0.5f * (h + h0 - d * (h - h0) / Rex) * Rin * c1 / rho;
            imi = (h - h0) / pi4 * rq * (pi * Rin * (j0f(aRin) - jnf(2, aRin)) / r2 - c1 / r3) * U;
        }
    } else {
        ree = 0.5f * (h + h0) * pi * Rex * Rex;
        ime = -0.25f * pi * pi * (h - h0) * Rex * Rex * Rex * U;
        if (Rin != 0.0f) {
            rei = 0.5f * (h + h0 - d * (h - h0) / Rex) * pi * Rin * Rin;
            imi = -0.25f * pi * pi * (h - h0) * (Rin * Rin * Rin * Rin / Rex) * U;
        }
    }
    if (Rin != 0.0f) {
        float dre = cosf(2.0f * pi * d * U), dim = sinf(2.0f * pi * d * U);
        Fr_re = ree - (rei * dre - imi * dim);
        Fr_im = ime - (rei * dim + imi * dre);
    } else {
        Fr_re = ree;
        Fr_im = ime;
    }
    if (gax == 0.0f || aq == 0.0f || gq == 0.0f) {
        Vre = Zsp * Fr_re;
        Vim = Zsp * Fr_im;
    } else {
        float gshift = Rin - d, ug = U * gsx, vg = V * gsy;
        float Gamp = expf(-gcoef * (ug * ug + vg * vg));
        float Gph = -2.0f * pi * gshift * U;
        Vre = Zsp * ((1.0f - gq) * Fr_re + gq * Gamp * cosf(Gph));
        Vim = Zsp * ((1.0f - gq) * Fr_im + gq * Gamp * sinf(Gph));
    }
    *vamp = sqrtf(Vre * Vre + Vim * Vim);
    *vpha = atan2f(Vim, Vre);
}

/* ------------------------------------------------------------------------ */
/* Problem description and one replica's model row.                          */
/* ------------------------------------------------------------------------ */

typedef struct {
    int model;                 /* OR_MODEL_* */
    int imodel;                /* passed through to the model (sgra: 1 or 2) */
    int ncoor, ndat, nicoor, nidat, nptot, npass;
    const float *coor, *dat, *std2r;
    const int *icoor, *idat;
    int arith;                 /* OR_ARITH_F64 (checker) or OR_ARITH_F32 */
} or_problem;

enum { OR_ARITH_F64 = 0, OR_ARITH_F32 = 1 };

static double wrap_angle(double x) { return atan2(sin(x), cos(x)); }

/*
 * Evaluate one replica's model over all data, the way calc_chi2_terms
 * (src/gpu_mcmc.cu:273-325) drives model() pass by pass.
 *   p      : nptot float parameters
 *   datm   : ndat model values (out); entries with no term keep their value
 *   phase  : nvis model phases for sgra (out, may be NULL otherwise)
 *   iret   : ndat return codes of the pass that produced the term (out)
 * Returns OR_OK or OR_ERR_ARG (unknown sgra imodel).
 */
static int model_row_d(const or_problem *pb, const double *prm, double *datm,
                       double *phase, int *iret, int pass_mask)
{
    int id, j, k, n = pb->nptot;
    for (id = 0; id < pb->ndat; id++) iret[id] = 0;

    switch (pb->model) {
    case OR_MODEL_SGRA: {
        int nvis = pb->idat[0], cpext = pb->idat[2];
        if (pb->imodel != 1 && pb->imodel != 2) return OR_ERR_ARG;
        if (pass_mask & 1) {                      /* pass 0: amp + phase */
            for (id = 0; id < nvis && id < pb->ndat; id++) {
                double a, ph;
                double ul = pb->coor[2 * id], vl = pb->coor[2 * id + 1];
                if (pb->imodel == 1) or_sgra_model9(ul, vl, prm, &a, &ph);
                else or_sgra_model13(ul, vl, prm, &a, &ph);
                datm[id] = a;
                phase[id] = ph;
                iret[id] = 1;
            }
        }
        if (pass_mask & 2) {                      /* pass 1: closures */
            for (id = nvis; id < pb->ndat; id++) {
                double cph;
                if (cpext == 0) {
                    int c = 3 * (id - nvis);
                    cph = phase[pb->icoor[c]] + phase[pb->icoor[c + 1]]
                        - phase[pb->icoor[c + 2]];
                } else {
                    int c = 4 * (id - nvis) + 2 * nvis;
                    double u1 = pb->coor[c], v1 = pb->coor[c + 1];
                    double u2 = pb->coor[c + 2], v2 = pb->coor[c + 3];
                    double u3 = -(u1 + u2), v3 = -(v1 + v2), a, p1, p2, p3;
                    if (pb->imodel == 1) {
                        or_sgra_model9(u1, v1, prm, &a, &p1);
                        or_sgra_model9(u2, v2, prm, &a, &p2);
                        or_sgra_model9(u3, v3, prm, &a, &p3);
                    } else {
                        or_sgra_model13(u1, v1, prm, &a, &p1);
                        or_sgra_model13(u2, v2, prm, &a, &p2);
                        or_sgra_model13(u3, v3, prm, &a, &p3);
                    }
                    cph = p1 + p2 - p3;
                }
                datm[id] = wrap_angle(cph);
                iret[id] = 2;
            }
        }
        return OR_OK;
    }
    case OR_MODEL_ROSEN: {                        /* datum 0 only */
        if ((pass_mask & 1) && pb->ndat > 0) {
            double f = 0.0;
            for (j = 0; j + 1 < n; j++) {
                double a = prm[j + 1] - prm[j] * prm[j], b = 1.0 - prm[j];
                f += 100.0 * a * a + b * b;
            }
            datm[0] = f;
            for (id = 0; id < pb->ndat; id++) iret[id] = 1;
        }
        return OR_OK;
    }
    case OR_MODEL_SOLVSYS: {
        if (pass_mask & 1) {
            for (id = 0; id < pb->ndat; id++) {
                if (id == 0)
                    datm[id] = pow(prm[0], pb->coor[0]) + pow(prm[1], pb->coor[1]);
                else
                    datm[id] = -(double)pb->coor[2] * prm[0] + prm[1];
                iret[id] = 1;
            }
        }
        return OR_OK;
    }
    case OR_MODEL_NLSYS: {
        if (pass_mask & 1) {
            const float *A = pb->coor, *B = pb->coor + (size_t)pb->ndat * n;
            for (k = 0; k < pb->ndat; k++) {
                double s = 0.0;
                for (j = 0; j < n; j++)
                    s += A[k * n + j] * sin(prm[j]) + B[k * n + j] * prm[j] * prm[j];
                datm[k] = s;
                iret[k] = 1;
            }
        }
        return OR_OK;
    }
    default:
        return OR_ERR_ARG;
    }
}

/* model_row_d at the float parameters the reference's kernels receive. */
static int model_row(const or_problem *pb, const float *p, double *datm,
                     double *phase, int *iret, int pass_mask)
{
    int j;
    double prm[16] = {0};
    for (j = 0; j < pb->nptot && j < 16; j++) prm[j] = (double)p[j];
    return model_row_d(pb, prm, datm, phase, iret, pass_mask);
}

static int pass_mask_for(const or_problem *pb)
{
    return pb->npass >= 2 ? 3 : 1;
}

/* chi^2 terms of one row: src/gpu_mcmc.cu:305-323. */
static double chi2_row(const or_problem *pb, const double *datm,
                       const int *iret, double *chi2m_row)
{
    int id;
    double s = 0.0;
    for (id = 0; id < pb->ndat; id++) {
        if (iret[id] != 0) {
            double dif = (double)pb->dat[id] - datm[id];
            if (iret[id] == 2) dif = wrap_angle(dif);
            chi2m_row[id] = dif * dif * (double)pb->std2r[id];
        }
        s += chi2m_row[id];
    }
    return s;
}

/*
 * calc_modchi2 semantics (src/mcmcjob.cu:227-254 + gpu_mcmc.cu:769-783):
 * model values, chi^2 terms and per-replica chi^2 for nrep parameter sets.
 *   pcur  [nrep][nptot]
 *   datm  [nrep][ndat]  model values; phase [nrep][nvis] (sgra, or NULL)
 *   chi2m [nrep][ndat]  (in/out: entries without a term keep their value)
 *   chi2c [nrep]
 */
int or_calc_modchi2(const or_problem *pb, int nrep, const float *pcur,
                    const int *flag, double *datm, double *phase,
                    double *chi2m, double *chi2c)
{
    int r, rc, nvis = (pb->model == OR_MODEL_SGRA) ? pb->idat[0] : 0;
    int *iret = (int *)malloc(sizeof(int) * (pb->ndat > 0 ? pb->ndat : 1));
    double dummy_phase[1];
    if (!iret) return OR_ERR_ARG;
    for (r = 0; r < nrep; r++) {
        if (flag && flag[r] == 0) continue;
        rc = model_row(pb, pcur + (size_t)r * pb->nptot, datm + (size_t)r * pb->ndat,
                       phase ? phase + (size_t)r * nvis : dummy_phase, iret,
                       pass_mask_for(pb));
        if (rc) { free(iret); return rc; }
        chi2c[r] = chi2_row(pb, datm + (size_t)r * pb->ndat, iret,
                            chi2m + (size_t)r * pb->ndat);
    }
    free(iret);
    return OR_OK;
}

/* calc_model semantics (gpu_mcmc.cu:633-658): pass 0 only, no chi^2. */
int or_calc_model(const or_problem *pb, int nrep, const float *pcur,
                  double *datm, double *phase)
{
    int r, rc, nvis = (pb->model == OR_MODEL_SGRA) ? pb->idat[0] : 0;
    int *iret = (int *)malloc(sizeof(int) * (pb->ndat > 0 ? pb->ndat : 1));
    double dummy_phase[1];
    if (!iret) return OR_ERR_ARG;
    for (r = 0; r < nrep; r++) {
        rc = model_row(pb, pcur + (size_t)r * pb->nptot, datm + (size_t)r * pb->ndat,
                       phase ? phase + (size_t)r * nvis : dummy_phase, iret, 1);
        if (rc) { free(iret); return rc; }
    }
    free(iret);
    return OR_OK;
}

/*
 * chi^2 at FP64 parameters p[nrep][nptot] (no rounding of p to float): the
 * function whose central differences check the gradient.  Same terms as
 * or_calc_modchi2 (src/gpu_mcmc.cu:305-323).
 */
int or_chi2_d(const or_problem *pb, int nrep, const double *p, double *chi2c)
{
    int r, rc, nvis = (pb->model == OR_MODEL_SGRA) ? pb->idat[0] : 0;
    size_t nd = (size_t)(pb->ndat > 0 ? pb->ndat : 1);
    int *iret = (int *)malloc(sizeof(int) * nd);
    double *datm = (double *)malloc(sizeof(double) * nd);
    double *row = (double *)malloc(sizeof(double) * nd);
    double *phase = (double *)malloc(sizeof(double) * (size_t)(nvis > 0 ? nvis : 1));
    double prm[16];
    rc = OR_OK;
    if (!iret || !datm || !row || !phase || pb->nptot > 16) rc = OR_ERR_ARG;
    for (r = 0; r < nrep && rc == OR_OK; r++) {
        int j;
        for (j = 0; j < pb->nptot; j++) prm[j] = p[(size_t)r * pb->nptot + j];
        for (j = 0; j < pb->ndat; j++) row[j] = 0.0;
        rc = model_row_d(pb, prm, datm, phase, iret, pass_mask_for(pb));
        if (rc == OR_OK) chi2c[r] = chi2_row(pb, datm, iret, row);
    }
    free(iret); free(datm); free(row); free(phase);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* Injected random streams.                                                  */
/* ------------------------------------------------------------------------ */

typedef struct {
    const float *u;   /* [nrep][lu] uniforms in (0,1] */
    const float *n;   /* [nrep][ln] standard normals   */
    int lu, ln;
    int *cu, *cn;     /* [nrep] cursors (in/out)      */
    int overflow;
} or_streams;

static float draw_u(or_streams *s, int ist)
{
    int c = s->cu[ist];
    if (c >= s->lu) { s->overflow = 1; return 1.0f; }
    s->cu[ist] = c + 1;
    return s->u[(size_t)ist * s->lu + c];
}

static float draw_n(or_streams *s, int ist)
{
    int c = s->cn[ist];
    if (c >= s->ln) { s->overflow = 1; return 0.0f; }
    s->cn[ist] = c + 1;
    return s->n[(size_t)ist * s->ln + c];
}

static float wrap_angle_f(float p) { return (float)atan2(sin((double)p), cos((double)p)); }

/* ------------------------------------------------------------------------ */
/* The sweep.                                                                */
/* ------------------------------------------------------------------------ */

typedef struct {
    /* sizes */
    int nprm, nadj, nbeta, nseq, niter_total;
    /* parameter description, [nptot] / [nprm] / [nbeta] */
    const int *pdescr, *ivar, *invar;
    const float *pmint, *pmaxt, *beta;
    /* state, reference layouts (in/out) */
    float *pcur;      /* [nbeta][nseq][nptot] */
    double *chi2c;    /* [nbeta][nseq] */
    int *flag;        /* [nbeta][nseq] */
    float *ptent;     /* [nbeta][nseq] */
    int *ptentn;      /* [nbeta][nseq] */
    float *pstp;      /* [nprm][nbeta][nseq] */
    int *n_acpt;      /* [nprm][nbeta][nseq] */
    int *n_exch;      /* [nbeta][nseq] */
    int *n_cnt;       /* [nprm][nbeta][nseq] */
    int *n_hist;      /* [nadj][nprm][nbeta][nseq] */
    int *tcur;        /* [nbeta][nseq] */
    /* outputs */
    float *pout;      /* [nprm][nbeta][nseq][niter_total] */
    int *tout;        /* [nbeta][nseq][niter_total] */
    float *chi2;      /* [nseq][niter_total] */
    /* last evaluated model rows (datm/chi2m semantics of the reference) */
    double *datm;     /* [nbeta][nseq][ndat] or NULL */
    double *chi2m;    /* [nbeta][nseq][ndat] or NULL */
    /* optional decision traces */
    signed char *tr_dec;   /* [nstep][nprm][nrep]: -1 prior, 0 reject, 1 accept */
    double *tr_margin;     /* [nstep][nprm][nrep]: u - alpha */
    signed char *tr_xk;    /* [nstep][nseq][nbeta]: pair index k */
    signed char *tr_xdec;  /* [nstep][nseq][nbeta]: swapped? */
    double *tr_xmargin;    /* [nstep][nseq][nbeta]: u - alpha */
    /* proposal kind: 0 = the reference's one-parameter proposals; 1 = block
       proposals p_ivar[i] += pstp[0] * (L z)_i, L = prop_chol[iseq] (lower,
       row-major [nprm][nprm]), z ~ N(0, I) drawn z_0..z_{nprm-1}, (L z)_i
       accumulated over j = 0..i with fmaf; bookkeeping on slot k = 0.  This
       mode is the library's extension, restated here as its checker. */
    int prop_mode;
    const float *prop_chol;  /* [nseq][nprm][nprm] */
} or_sweep_state;

/* One replica's chi^2 in float32, as calc_chi2_terms (src/gpu_mcmc.cu:273-325)
 * over examples/sgra_model_fit/model.cuh and the serial float sum of
 * spmp_mcmc (:447-448): sgra_model9 only.  The buffers hold the float values
 * widened to double. */
static int chi2_of_f32(const or_problem *pb, const float *p, double *datm_row,
                       double *phase, int *iret, double *chi2m_row, double *out)
{
    const int nvis = pb->idat[0], cpext = pb->nidat > 2 ? pb->idat[2] : 0;
    int id;
    float sum = 0.0f;
    for (id = 0; id < pb->ndat; id++) iret[id] = 0;
    for (id = 0; id < nvis && id < pb->ndat; id++) {
        float a, ph;
        or_sgra_model9_f(pb->coor[2 * id], pb->coor[2 * id + 1], p, &a, &ph);
        datm_row[id] = a;
        phase[id] = ph;
        iret[id] = 1;
    }
    if (pass_mask_for(pb) & 2) {
        for (id = nvis; id < pb->ndat; id++) {
            float cph;
            if (cpext == 0) {
                int c = 3 * (id - nvis);
                cph = (float)phase[pb->icoor[c]] + (float)phase[pb->icoor[c + 1]]
                    - (float)phase[pb->icoor[c + 2]];
            } else {
                int c = 4 * (id - nvis) + 2 * nvis;
                float u1 = pb->coor[c], v1 = pb->coor[c + 1];
                float u2 = pb->coor[c + 2], v2 = pb->coor[c + 3], a, p1, p2, p3;
                or_sgra_model9_f(u1, v1, p, &a, &p1);
                or_sgra_model9_f(u2, v2, p, &a, &p2);
                or_sgra_model9_f(-(u1 + u2), -(v1 + v2), p, &a, &p3);
                cph = p1 + p2 - p3;
            }
            datm_row[id] = atan2f(sinf(cph), cosf(cph));
            iret[id] = 2;
        }
    }
    for (id = 0; id < pb->ndat; id++) {
        if (iret[id] != 0) {
            float dif = pb->dat[id] - (float)datm_row[id];
            if (iret[id] == 2) dif = atan2f(sinf(dif), cosf(dif));
            chi2m_row[id] = (dif * dif) * pb->std2r[id];
        }
        sum += (float)chi2m_row[id];
    }
    *out = sum;
    return OR_OK;
}

static int chi2_of(const or_problem *pb, const float *p, double *datm_row,
                   double *phase, int *iret, double *chi2m_row, double *out)
{
    if (pb->arith == OR_ARITH_F32 && pb->model == OR_MODEL_SGRA && pb->imodel == 1)
        return chi2_of_f32(pb, p, datm_row, phase, iret, chi2m_row, out);
    int rc = model_row(pb, p, datm_row, phase, iret, pass_mask_for(pb));
    if (rc) return rc;
    *out = chi2_row(pb, datm_row, iret, chi2m_row);
    return OR_OK;
}

/*
 * Run do_init (init_pcur + initial chi^2), then nburn burn-in iterations and
 * niter main iterations; main iteration t writes pout/tout/chi2 at index
 * itr0 + t.  Returns OR_OK, OR_ERR_ARG or OR_ERR_STREAM (stream exhausted).
 */
int or_sweep(const or_problem *pb, or_sweep_state *st, or_streams *rs,
             int do_init, int nburn, int niter, int itr0)
{
    const int nbeta = st->nbeta, nseq = st->nseq, nprm = st->nprm;
    const int nptot = pb->nptot, ndat = pb->ndat, nrep = nbeta * nseq;
    const int nvis = (pb->model == OR_MODEL_SGRA) ? pb->idat[0] : 0;
    int ist, i, k, t, step, itr, ipm, rc = OR_OK;
    double *datm_tmp, *chi2m_tmp, *phase_tmp;
    int *iret;
    float bk[64];   /* block mode: the pre-proposal parameters */

    if (nbeta < 2 || nseq < 1 || nprm < 1 || nptot < nprm || st->nadj < 1)
        return OR_ERR_ARG;
    if (st->prop_mode == 1 && (!st->prop_chol || nptot > 64)) return OR_ERR_ARG;
    datm_tmp = (double *)calloc((size_t)nrep * (ndat > 0 ? ndat : 1), sizeof(double));
    chi2m_tmp = (double *)calloc((size_t)nrep * (ndat > 0 ? ndat : 1), sizeof(double));
    phase_tmp = (double *)calloc((size_t)(nvis > 0 ? nvis : 1), sizeof(double));
    iret = (int *)calloc((size_t)(ndat > 0 ? ndat : 1), sizeof(int));
    if (!datm_tmp || !chi2m_tmp || !phase_tmp || !iret) { rc = OR_ERR_ARG; goto done; }
    if (st->datm) memcpy(datm_tmp, st->datm, sizeof(double) * (size_t)nrep * ndat);
    if (st->chi2m) memcpy(chi2m_tmp, st->chi2m, sizeof(double) * (size_t)nrep * ndat);

    if (do_init) {
        /* init_pcur, gpu_mcmc.cu:245-267 */
        for (ist = 0; ist < nrep; ist++) {
            st->flag[ist] = 1;
            for (i = 0; i < nprm; i++) {
                float u, p;
                k = st->ivar[i];
                u = draw_u(rs, ist);
                p = fmaf(st->pmaxt[k] - st->pmint[k], u, st->pmint[k]);
                if (st->pdescr[k] == 2) p = wrap_angle_f(p);
                st->pcur[(size_t)ist * nptot + k] = p;
            }
        }
        /* initial calc_chi2_terms x npass + calc_chi2, gpu_mcmc.cu:716-719 */
        for (ist = 0; ist < nrep; ist++) {
            rc = chi2_of(pb, st->pcur + (size_t)ist * nptot, datm_tmp + (size_t)ist * ndat,
                         phase_tmp, iret, chi2m_tmp + (size_t)ist * ndat, &st->chi2c[ist]);
            if (rc) goto done;
        }
    }

    for (step = 0; step < nburn + niter; step++) {
        int burn = step < nburn;
        itr = burn ? step : step - nburn;
        for (ipm = 0; ipm < nprm; ipm++) {
            for (ist = 0; ist < nrep; ist++) {
                int ibeta = ist / nseq, iseq = ist % nseq, kk, pt, ip;
                float r, p, sd, rn;
                size_t tix = ((size_t)step * nprm + ipm) * nrep + ist;
                if (st->prop_mode == 1) {
                    const float *L = st->prop_chol + (size_t)iseq * nprm * nprm;
                    float acc[64], zj, sdb;
                    int out = 0, j2;
                    if (nprm > 64) { rc = OR_ERR_ARG; goto done; }
                    for (i = 0; i < nprm; i++) acc[i] = 0.0f;
                    for (j2 = 0; j2 < nprm; j2++) {
                        zj = draw_n(rs, ist);
                        for (i = j2; i < nprm; i++) acc[i] = fmaf(L[i * nprm + j2], zj, acc[i]);
                    }
                    if (rs->overflow) { rc = OR_ERR_STREAM; goto done; }
                    for (i = 0; i < nptot; i++) bk[i] = st->pcur[(size_t)ist * nptot + i];
                    sdb = st->pstp[(size_t)ibeta * nseq + iseq];     /* slot k = 0 */
                    for (i = 0; i < nprm; i++) {
                        int tt = st->ivar[i];
                        float pp = fmaf(sdb, acc[i], bk[tt]);
                        if (st->pdescr[tt] == 2) pp = wrap_angle_f(pp);
                        if (pp < st->pmint[tt] || pp > st->pmaxt[tt]) out = 1;
                        st->pcur[(size_t)ist * nptot + tt] = pp;
                    }
                    t = st->ivar[0];
                    st->ptentn[ist] = t;
                    st->ptent[ist] = bk[t];
                    if (out) {
                        for (i = 0; i < nptot; i++) st->pcur[(size_t)ist * nptot + i] = bk[i];
                        st->flag[ist] = 0;
                    } else {
                        st->flag[ist] = 1;
                    }
                    pt = ist * nptot + t;
                    goto evaluate;
                }
                /* gen_proposal, gpu_mcmc.cu:361-411 */
                do {
                    r = draw_u(rs, ist);
                    kk = (int)((float)nprm * r);
                } while (kk >= nprm && !rs->overflow);
                if (rs->overflow) { rc = OR_ERR_STREAM; goto done; }
                t = st->ivar[kk];
                st->ptentn[ist] = t;
                pt = ist * nptot + t;
                p = st->pcur[pt];
                st->ptent[ist] = p;
                sd = st->pstp[(nbeta * kk + ibeta) * nseq + iseq];
                rn = draw_n(rs, ist);
                p = fmaf(sd, rn, p);
                if (st->pdescr[t] == 2) p = wrap_angle_f(p);
                if (p < st->pmint[t] || p > st->pmaxt[t]) {
                    st->flag[ist] = 0;
                } else {
                    st->flag[ist] = 1;
                    st->pcur[pt] = p;
                }
            evaluate:
                /* calc_chi2_terms + spmp_mcmc, gpu_mcmc.cu:273-325, 426-474 */
                if (st->flag[ist] != 0) {
                    double c2, a, alpha;
                    float u;
                    rc = chi2_of(pb, st->pcur + (size_t)ist * nptot,
                                 datm_tmp + (size_t)ist * ndat, phase_tmp, iret,
                                 chi2m_tmp + (size_t)ist * ndat, &c2);
                    if (rc) goto done;
                    a = exp(-0.5 * (double)st->beta[ibeta] * (c2 - st->chi2c[ist]));
                    alpha = a < 1.0 ? a : 1.0;
                    u = draw_u(rs, ist);
                    if (st->tr_margin) st->tr_margin[tix] = (double)u - alpha;
                    if ((double)u <= alpha) {
                        st->chi2c[ist] = c2;
                        st->n_acpt[(nbeta * st->invar[t] + ibeta) * nseq + iseq]++;
                        if (st->tr_dec) st->tr_dec[tix] = 1;
                    } else {
                        if (st->prop_mode == 1)
                            for (i = 0; i < nptot; i++) st->pcur[(size_t)ist * nptot + i] = bk[i];
                        else
                            st->pcur[pt] = st->ptent[ist];
                        st->flag[ist] = 0;
                        if (st->tr_dec) st->tr_dec[tix] = 0;
                    }
                } else {
                    if (st->tr_dec) st->tr_dec[tix] = -1;
                    if (st->tr_margin) st->tr_margin[tix] = 0.0;
                }
                /* adjust_steps (burn-in only), gpu_mcmc.cu:480-526 */
                if (burn) {
                    int kp = st->invar[st->ptentn[ist]], modn, sumh = 0, iadj, den;
                    float rate;
                    ip = (nbeta * kp + ibeta) * nseq + iseq;
                    modn = st->n_cnt[ip] % st->nadj;
                    st->n_hist[((nprm * modn + kp) * nbeta + ibeta) * nseq + iseq] =
                        st->flag[ist] != 0 ? 1 : 0;
                    for (iadj = 0; iadj < st->nadj; iadj++)
                        sumh += st->n_hist[((nprm * iadj + kp) * nbeta + ibeta) * nseq + iseq];
                    den = st->nadj < st->n_cnt[ip] ? st->nadj : st->n_cnt[ip];
                    rate = (float)sumh / (float)den;
                    if (rate < 0.30f) st->pstp[ip] = (float)((double)st->pstp[ip] / 1.01);
                    else st->pstp[ip] = (float)((double)st->pstp[ip] * 1.01);
                    st->n_cnt[ip] += 1;
                }
            }
        }
        /* replica_exchange, gpu_mcmc.cu:533-626 (the ibeta = 0 stream) */
        for (i = 0; i < nseq; i++) {
            int ib, nb1 = nbeta - 1;
            for (ib = 0; ib < nbeta; ib++) {
                float r, u;
                int k0, k1, j;
                double a, alpha;
                size_t xix = ((size_t)step * nseq + i) * nbeta + ib;
                do {
                    r = draw_u(rs, i);
                    k = (int)((float)nb1 * r);
                } while (k >= nb1 && !rs->overflow);
                if (rs->overflow) { rc = OR_ERR_STREAM; goto done; }
                k0 = k * nseq + i;
                k1 = (k + 1) * nseq + i;
                a = exp(-0.5 * ((double)st->beta[k + 1] - (double)st->beta[k])
                        * (st->chi2c[k0] - st->chi2c[k1]));
                alpha = a < 1.0 ? a : 1.0;
                u = draw_u(rs, i);
                if (st->tr_xk) st->tr_xk[xix] = (signed char)k;
                if (st->tr_xmargin) st->tr_xmargin[xix] = (double)u - alpha;
                if ((double)u <= alpha) {
                    int idum = st->tcur[k0];
                    double dc;
                    st->tcur[k0] = st->tcur[k1];
                    st->tcur[k1] = idum;
                    for (j = 0; j < nptot; j++) {
                        float dum = st->pcur[(size_t)k0 * nptot + j];
                        st->pcur[(size_t)k0 * nptot + j] = st->pcur[(size_t)k1 * nptot + j];
                        st->pcur[(size_t)k1 * nptot + j] = dum;
                    }
                    dc = st->chi2c[k0];
                    st->chi2c[k0] = st->chi2c[k1];
                    st->chi2c[k1] = dc;
                    if (!burn) st->n_exch[k * nseq + i]++;
                    if (st->tr_xdec) st->tr_xdec[xix] = 1;
                } else if (st->tr_xdec) {
                    st->tr_xdec[xix] = 0;
                }
            }
            if (!burn) {
                int ib2, j;
                size_t it = (size_t)(itr0 + itr);
                for (ib2 = 0; ib2 < nbeta; ib2++) {
                    for (j = 0; j < nptot; j++) {
                        if (st->invar[j] != -1) {
                            size_t ipo = (((size_t)nbeta * st->invar[j] + ib2) * nseq + i)
                                         * st->niter_total + it;
                            st->pout[ipo] = st->pcur[((size_t)nseq * ib2 + i) * nptot + j];
                        }
                    }
                    st->tout[((size_t)nseq * ib2 + i) * st->niter_total + it] =
                        st->tcur[nseq * ib2 + i];
                }
                st->chi2[(size_t)st->niter_total * i + it] = (float)st->chi2c[i];
            }
        }
    }
done:
    if (rc == OR_OK && st->datm) memcpy(st->datm, datm_tmp, sizeof(double) * (size_t)nrep * ndat);
    if (rc == OR_OK && st->chi2m) memcpy(st->chi2m, chi2m_tmp, sizeof(double) * (size_t)nrep * ndat);
    free(datm_tmp);
    free(chi2m_tmp);
    free(phase_tmp);
    free(iret);
    return rc;
}

/* Size of the structs, so the ctypes mirror can check its layout. */
/* chi^2 of nrep float parameter sets in the float32 arithmetic of
 * chi2_of_f32 (sgra_model9 only); chi2c [nrep]. */
int or_chi2_f32(const or_problem *pb, int nrep, const float *pcur, double *chi2c)
{
    int r, rc = OR_OK;
    double *datm, *phase, *chi2m;
    int *iret;
    if (pb->model != OR_MODEL_SGRA || pb->imodel != 1) return OR_ERR_ARG;
    datm = (double *)calloc((size_t)pb->ndat, sizeof(double));
    phase = (double *)calloc((size_t)pb->ndat + 1, sizeof(double));
    chi2m = (double *)calloc((size_t)pb->ndat, sizeof(double));
    iret = (int *)calloc((size_t)pb->ndat, sizeof(int));
    if (!datm || !phase || !chi2m || !iret) rc = OR_ERR_ARG;
    for (r = 0; rc == OR_OK && r < nrep; r++)
        rc = chi2_of_f32(pb, pcur + (size_t)r * pb->nptot, datm, phase, iret, chi2m, &chi2c[r]);
    free(datm);
    free(phase);
    free(chi2m);
    free(iret);
    return rc;
}

int or_sizeof_problem(void) { return (int)sizeof(or_problem); }
int or_sizeof_sweep_state(void) { return (int)sizeof(or_sweep_state); }
int or_sizeof_streams(void) { return (int)sizeof(or_streams); }
