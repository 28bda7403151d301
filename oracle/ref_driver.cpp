/*
 * ref_driver.cpp -- CPU emulation driver for the reference's own kernels.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/ref_build.py compiles the kernels of the
 * reference's src/gpu_mcmc.cu (lines up to run_mcmc, read in place and fed to
 * g++ on stdin, together with one of the reference's examples/<m>/model.cuh)
 * as plain C++, and links them with this file into oracle/_ref/libref_<m>.so.
 * This driver plays the role of run_mcmc (src/gpu_mcmc.cu:682-763),
 * run_calcmodchi2 (:769-783) and run_calcmodel (:790-802): it launches each
 * kernel by looping over its blocks and threads, one thread at a time, in
 * the same kernel order.  Random draws come from injected streams
 * (oracle/ref_shim/curand_kernel.h).  The job object is the reference's
 * CMcmcFit class from src/mcmcjob.cuh with host arrays in place of device
 * arrays.
 */
#include <cstdlib>
#include <cstring>
#include <cuda.h>
#include <curand_kernel.h>
#include "mcmcjob.cuh"

/* Kernels compiled from the reference's gpu_mcmc.cu (other translation unit). */
void init_rng(CMcmcFit *mc);
void init_pcur(CMcmcFit *mc);
void calc_chi2_terms(CCalcModel *mc, int ipass);
void calc_chi2(CCalcModel *mc);
void gen_proposal(CMcmcFit *mc);
void spmp_mcmc(CMcmcFit *mc);
void adjust_steps(CMcmcFit *mc);
void replica_exchange(CMcmcFit *mc, int burn, int itr);
void calc_model(CCalcModel *mc);

ref_dim3 blockIdx, threadIdx, blockDim, gridDim;
curandState *g_ref_rndst_base;
const float *g_ref_u, *g_ref_n;
int g_ref_lu, g_ref_ln, g_ref_overflow;

template <class F>
static void launch(unsigned nb, unsigned nt, F f)
{
    gridDim = {nb, 1, 1};
    blockDim = {nt, 1, 1};
    for (unsigned b = 0; b < nb; b++)
        for (unsigned t = 0; t < nt; t++) {
            blockIdx = {b, 0, 0};
            threadIdx = {t, 0, 0};
            f();
        }
}

extern "C" int ref_mcmc(
    float *coor, float *dat, float *std2r, int *icoor, int *idat, float *datm,
    float *chi2m, int *pdescr, int *ivar, int *invar, float *ptotal, float *pmint,
    float *pmaxt, float *pout, int *tout, float *chi2, float *chi2c, int *tcur,
    int *flag, int *n_acpt, int *n_exch, int *n_cnt, int *n_hist, float *beta,
    float *pstp, float *ptent, int *ptentn, float *pcur,
    int *cursors, const float *su, const float *sn, int lu, int ln,
    int imodel, int ncoor, int ndat, int nicoor, int nidat, int ndatm, int nptot,
    int nprm, int nadj, int npass, int nbeta, int nseq, int nburn, int niter,
    int do_init, int itr0, int niter_total)
{
    int nrep = nbeta * nseq;
    if (nbeta < 2 || nseq < 1 || nprm < 1) return 1;
    CMcmcFit *mc = static_cast<CMcmcFit *>(std::calloc(1, sizeof(CMcmcFit)));
    curandState *rs = static_cast<curandState *>(std::calloc(nrep, sizeof(curandState)));
    if (!mc || !rs) { std::free(mc); std::free(rs); return 1; }
    for (int i = 0; i < nrep; i++) { rs[i].cu = cursors[2 * i]; rs[i].cn = cursors[2 * i + 1]; }

    mc->imodel = imodel; mc->ncoor = ncoor; mc->ndat = ndat; mc->nicoor = nicoor;
    mc->nidat = nidat; mc->ndatm = ndatm; mc->nptot = nptot; mc->nbeta = nbeta;
    mc->nseq = nseq; mc->nchi2m = nbeta * nseq * ndat;
    mc->coor = coor; mc->dat = dat; mc->std2r = std2r; mc->icoor = icoor;
    mc->idat = idat; mc->datm = datm; mc->chi2m = chi2m; mc->pcur = pcur;
    mc->flag = flag; mc->chi2c = chi2c;
    mc->nprm = nprm; mc->nadj = nadj; mc->npass = npass; mc->nburn = nburn;
    mc->niter = niter_total; mc->nrndst = nrep; mc->ipm = 0; mc->itr = 0;
    mc->seed = 0; mc->rndst = rs;
    mc->pdescr = pdescr; mc->ivar = ivar; mc->invar = invar; mc->ptotal = ptotal;
    mc->pmint = pmint; mc->pmaxt = pmaxt; mc->pout = pout; mc->tout = tout;
    mc->chi2 = chi2; mc->tcur = tcur; mc->n_acpt = n_acpt; mc->n_exch = n_exch;
    mc->n_cnt = n_cnt; mc->n_hist = n_hist; mc->pstp = pstp; mc->beta = beta;
    mc->ptent = ptent; mc->ptentn = ptentn;

    g_ref_rndst_base = rs; g_ref_u = su; g_ref_n = sn; g_ref_lu = lu; g_ref_ln = ln;
    g_ref_overflow = 0;

    unsigned nblocks = mc->nchi2m / 128 + 1;
    if (do_init) {
        launch(nseq, nbeta, [&] { init_rng(mc); });
        for (int i = 0; i < nrep; i++) { rs[i].cu = cursors[2 * i]; rs[i].cn = cursors[2 * i + 1]; }
        launch(nseq, nbeta, [&] { init_pcur(mc); });
        for (int ip = 0; ip < npass; ip++) launch(nblocks, 128, [&] { calc_chi2_terms(mc, ip); });
        launch(nseq, nbeta, [&] { calc_chi2(mc); });
    }
    for (int step = 0; step < nburn + niter && !g_ref_overflow; step++) {
        int burn = step < nburn;
        int itr = burn ? step : itr0 + step - nburn;
        for (int ipm = 0; ipm < nprm; ipm++) {
            launch(nseq, nbeta, [&] { gen_proposal(mc); });
            for (int ip = 0; ip < npass; ip++) launch(nblocks, 128, [&] { calc_chi2_terms(mc, ip); });
            launch(nseq, nbeta, [&] { spmp_mcmc(mc); });
            if (burn) launch(nseq, nbeta, [&] { adjust_steps(mc); });
        }
        launch(nseq, 1, [&] { replica_exchange(mc, burn, itr); });
    }
    for (int i = 0; i < nrep; i++) { cursors[2 * i] = rs[i].cu; cursors[2 * i + 1] = rs[i].cn; }
    int rc = g_ref_overflow ? 2 : 0;
    std::free(rs);
    std::free(mc);
    return rc;
}

static CCalcModel *new_calc(float *coor, float *dat, float *std2r, int *icoor,
                            int *idat, float *datm, float *chi2m, float *pcur,
                            float *chi2c, int *flag, int imodel, int ncoor,
                            int ndat, int nicoor, int nidat, int ndatm,
                            int nptot, int nbeta, int nseq)
{
    CCalcModel *mc = static_cast<CCalcModel *>(std::calloc(1, sizeof(CCalcModel)));
    if (!mc) return nullptr;
    mc->imodel = imodel; mc->ncoor = ncoor; mc->ndat = ndat; mc->nicoor = nicoor;
    mc->nidat = nidat; mc->ndatm = ndatm; mc->nptot = nptot; mc->nbeta = nbeta;
    mc->nseq = nseq; mc->nchi2m = nbeta * nseq * ndat;
    mc->coor = coor; mc->dat = dat; mc->std2r = std2r; mc->icoor = icoor;
    mc->idat = idat; mc->datm = datm; mc->chi2m = chi2m; mc->pcur = pcur;
    mc->flag = flag; mc->chi2c = chi2c;
    return mc;
}

/* calc_modchi2 (src/mcmcjob.cu:227-254) as run by run_calcmodchi2. */
extern "C" int ref_calc_modchi2(
    float *coor, float *dat, float *std2r, int *icoor, int *idat, float *datm,
    float *chi2m, float *pcur, float *chi2c, int *flag, int imodel, int ncoor,
    int ndat, int nicoor, int nidat, int ndatm, int nptot, int nbeta, int nseq)
{
    CCalcModel *mc = new_calc(coor, dat, std2r, icoor, idat, datm, chi2m, pcur,
                              chi2c, flag, imodel, ncoor, ndat, nicoor, nidat,
                              ndatm, nptot, nbeta, nseq);
    if (!mc) return 1;
    unsigned nblocks = mc->nchi2m / 128 + 1;
    launch(nblocks, 128, [&] { calc_chi2_terms(mc, 0); });
    launch(nblocks, 128, [&] { calc_chi2_terms(mc, 1); });
    launch(nseq, nbeta, [&] { calc_chi2(mc); });
    std::free(mc);
    return 0;
}

/* calc_model (src/mcmcjob.cu:257-298) as run by run_calcmodel; every
 * replica's flag is set to 1 here (the reference leaves it uninitialised). */
extern "C" int ref_calc_model(
    float *coor, int *idat, float *datm, float *pcur, int imodel, int ncoor,
    int ndat, int nidat, int ndatm, int nptot, int nbeta, int nseq)
{
    int nrep = nbeta * nseq;
    int *flag = static_cast<int *>(std::malloc(sizeof(int) * nrep));
    if (!flag) return 1;
    for (int i = 0; i < nrep; i++) flag[i] = 1;
    CCalcModel *mc = new_calc(coor, nullptr, nullptr, nullptr, idat, datm, nullptr,
                              pcur, nullptr, flag, imodel, ncoor, ndat, 1, nidat,
                              ndatm, nptot, nbeta, nseq);
    if (!mc) { std::free(flag); return 1; }
    unsigned nblocks = mc->nchi2m / 128 + 1;
    launch(nblocks, 128, [&] { calc_model(mc); });
    std::free(mc);
    std::free(flag);
    return 0;
}
