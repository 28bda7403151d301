// cmc_job.h -- the plain-C description of one MCMC-RE job on the device.
//
// Shared by the CUDA kernels, the C-ABI host layer and (through ctypes) the
// Python device API.  Every array is a DEVICE pointer in the reference's
// layout (src/gpu_mcmc.cu:100-188); ist = ibeta*nseq + iseq indexes replicas.
#pragma once
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum cmc_status {
  CMC_OK = 0,
  CMC_ERR_ARG = 1,        /* invalid sizes / pointers                         */
  CMC_ERR_CUDA = 2,       /* a CUDA runtime call failed                       */
  CMC_ERR_STREAM = 3,     /* an injected random stream ran out                */
  CMC_ERR_MODEL = 4,      /* the model reported an error (e.g. bad imodel)    */
  CMC_ERR_NOMEM = 5,      /* device allocation failed                         */
  CMC_ERR_UNSUPPORTED = 6, /* no kernel configuration fits these sizes        */
  CMC_ERR_TIMEOUT = 7,    /* a wait between the CTAs of a spread-layout sweep
                             ran out (cmc_set_layout)                         */
  CMC_ERR_CANCELLED = 8   /* the batch was cancelled (cmc_batch_cancel)      */
};

enum cmc_prop_mode {
  CMC_PROP_SINGLE = 0,    /* the reference's proposals: one parameter k drawn
                             per proposal, p_k += pstp[k] * N(0,1)
                             (src/gpu_mcmc.cu:361-411)                        */
  CMC_PROP_BLOCK = 1      /* no counterpart in the reference: all nprm
                             parameters at once, p += pstp[0] * L z with
                             z ~ N(0, I) and L = prop_chol[iseq]; acceptance
                             bookkeeping and step adaptation on slot k = 0    */
};

enum cmc_rng_mode {
  CMC_RNG_CURAND = 0,     /* cuRAND XORWOW, curand_init(seed, ist, 0): the
                             reference's generator (src/gpu_mcmc.cu:228-239)  */
  CMC_RNG_INJECTED = 1    /* uniforms / normals read from caller streams      */
};

typedef struct cmc_job {
  /* sizes, reference meaning (src/mcmc.h:7-20) */
  int ncoor, ndat, nicoor, nidat, ndatm;
  int nptot, nprm, nadj, npass, nbeta, nseq;
  int imodel;
  /* this launch: do_init (init_rng + init_pcur + first chi^2), then nburn
     burn-in and niter main iterations; main iteration m is recorded at
     pout/tout/chi2 index itr0 + m of an array with niter_total columns */
  int do_init, nburn, niter, itr0, niter_total;
  int rng_mode;
  unsigned long long seed;

  /* data */
  const float *coor, *dat, *std2r;
  const int *icoor, *idat;
  /* parameter description */
  const int *pdescr, *ivar, *invar;
  const float *pmint, *pmaxt, *beta;
  /* host copy of idat[0..3] (the built-in Sgr A* path sizes its buffers
     from nvis = idat[0] and cpExt = idat[2] before launching) */
  int hidat[4];

  /* sampler state (in/out) */
  float *pcur;          /* [nbeta][nseq][nptot] */
  float *chi2c;         /* [nbeta][nseq]        */
  int *flag;            /* [nbeta][nseq]        */
  float *ptent;         /* [nbeta][nseq]        */
  int *ptentn;          /* [nbeta][nseq]        */
  float *pstp;          /* [nprm][nbeta][nseq]  */
  int *n_acpt;          /* [nprm][nbeta][nseq]  */
  int *n_exch;          /* [nbeta][nseq]        */
  int *n_cnt;           /* [nprm][nbeta][nseq]  */
  int *n_hist;          /* [nadj][nprm][nbeta][nseq] */
  int *tcur;            /* [nbeta][nseq]        */
  unsigned char *rndst; /* [nbeta][nseq][48]: curandStateXORWOW */

  /* outputs */
  float *pout;          /* [nprm][nbeta][nseq][niter_total] */
  int *tout;            /* [nbeta][nseq][niter_total]       */
  float *chi2;          /* [nseq][niter_total]              */
  float *datm;          /* [ndatm]: model rows of the last evaluation (may be NULL) */
  float *chi2m;         /* [nbeta][nseq][ndat]                  (may be NULL) */

  /* injected random streams (rng_mode == CMC_RNG_INJECTED) */
  const float *inj_u;   /* [nbeta*nseq][inj_lu] uniforms in (0,1] */
  const float *inj_n;   /* [nbeta*nseq][inj_ln] standard normals  */
  int inj_lu, inj_ln;
  int *inj_cur;         /* [nbeta*nseq][2] cursors (in/out)        */

  /* library-owned scratch: packed data for the built-in fast models */
  void *work;
  size_t work_bytes;

  /* device status word (CMC_* code), written by the kernels */
  int *status;

  /* proposal kind (enum cmc_prop_mode) and, for CMC_PROP_BLOCK, the lower
     Cholesky factors of the proposal covariance of each sequence in ivar
     order: prop_chol[(iseq*nprm + i)*nprm + j], j <= i (the upper triangle is
     not read).  Typically (2.38^2/nprm) F^-1 for the Fisher information F of
     the beta = 1 target; replica ibeta scales it by pstp[0][ibeta][iseq]. */
  int prop_mode;
  int prop_reserved;
  const float *prop_chol;

  /* sequence sharding (no counterpart in the reference): when nseq_total > 0
     this job holds sequences [seq_offset, seq_offset + nseq) of a run with
     nseq_total sequences, and replica (ibeta, iseq) seeds its generator with
     curand_init(seed, ibeta*nseq_total + seq_offset + iseq, 0), the
     subsequence it has in the unsharded run, so that the shards of a run
     together walk exactly the unsharded run's chains.  0: unsharded. */
  int seq_offset;
  int nseq_total;
} cmc_job;

#ifdef __cplusplus
}
#endif
