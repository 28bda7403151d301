// mcmcjob.cuh -- what a user model.cuh plugin sees.
//
// A plugin is a file defining
//     __device__ int model(CCalcModel *mc, int id, int ipt, int imd, int ipass);
// exactly as for the reference (template/model.cuh:21, src/gpu_mcmc.cu:202-221):
//   id    index into mc->dat (one datum),
//   ipt   offset of this replica's parameters: mc->pcur[ipt .. ipt+nptot-1],
//   imd   "through index" ist*ndat + id into mc->datm, where the model stores
//         its value before returning,
//   ipass pass number 0 .. npass-1,
// returning 0 (no term in this pass), 1 (plain term) or 2 (phase term whose
// residual is wrapped to [-pi, pi]).
//
// CCalcModel here carries the reference's member names and meanings
// (src/mcmcjob.cuh:30-72) so that existing model.cuh files compile unchanged;
// the layout is this library's own.  The device pointers refer to the running
// job's arrays: coor, dat, std2r, icoor, idat (read-only data), datm and
// chi2m (model rows, [nbeta][nseq][ndat] plus any tail a model uses, e.g. the
// Sgr A* phase tail at datm + nchi2m), and pcur (parameters of the replicas
// being evaluated).  flag and chi2c point at the job's state arrays, which
// are brought up to date at the end of each launch, not during it.
#pragma once

#ifdef __cplusplus
class CCalcModel {
 public:
  int imodel;
  int ncoor;
  int ndat;
  int nicoor;
  int nidat;
  int ndatm;
  int nptot;
  int nbeta;
  int nseq;
  int nchi2m;   /* nbeta*nseq*ndat */

  /* array sizes in bytes */
  int s_coor, s_dat, s_icoor, s_idat, s_datm, s_chi2m, s_pcur, s_bsint, s_bsflt;

  /* device arrays of the running job */
  float *coor;    /* [ncoor]  */
  float *dat;     /* [ndat]   */
  float *std2r;   /* [ndat]   */
  int *icoor;     /* [nicoor] */
  int *idat;      /* [nidat]  */
  float *datm;    /* [ndatm]  */
  float *chi2m;   /* [nbeta][nseq][ndat] */
  float *pcur;    /* [nbeta][nseq][nptot] */
  int *flag;      /* [nbeta][nseq] */
  float *chi2c;   /* [nbeta][nseq] */

  /* host-side pointers of the reference's class; unused on the device */
  float *coor_h, *dat_h, *std2r_h;
  int *icoor_h, *idat_h;
  float *datm_h, *chi2m_h, *pcur_h;
  int *flag_h;
  float *chi2c_h;
};
#endif

