// model_plugin.cuh -- the fused sweep driven by a user model.cuh plugin.
//
// The translation unit that includes this header must first include the
// plugin (see lib_plugin.cu), which defines
//     __device__ int model(CCalcModel *mc, int id, int ipt, int imd, int ipass);
// The sweep then calls model() once per (replica, datum, pass) exactly as the
// reference's calc_chi2_terms does (src/gpu_mcmc.cu:273-325): the model
// writes datm[imd], the kernel forms the term (dat - datm)^2 * std2r (the
// residual wrapped to [-pi, pi] when model() returns 2) into chi2m[imd], and
// a replica's chi^2 is the sum of its chi2m row (:331-350, :447-448), so a
// datum that gets no term in any pass keeps contributing its old chi2m value
// as in the reference.  datm / chi2m / pcur live in global memory because
// the plugin addresses them by the global indices imd and ipt.
#pragma once
#include <cuda_runtime.h>

#include "cmc_job.h"
#include "mcmcjob.cuh"

namespace cmc {

struct PluginModel {
  struct Consts { int unused; };
  struct Packed { int ndat, npass, phasor; };

  static constexpr bool kRowsInEval = true;
  static constexpr int kMaxR = 32;  // instantiated replicas-per-CTA counts: 1 .. 32
  static constexpr bool kSpread = false;   // cluster layout only

  // data points one replica's evaluation runs over
  __host__ __device__ static int points(const Packed &pk) { return pk.ndat * pk.npass; }

  __host__ __device__ static unsigned scratch_bytes(const Packed &, int)
  {
    return (unsigned)sizeof(CCalcModel);
  }

  // ---- host side ----------------------------------------------------------
  static int host_dims(const cmc_job &j, int mode, Packed &pk, const char **err)
  {
    pk.ndat = j.ndat;
    pk.npass = (mode == 0) ? j.npass : 2;
    const long long nchi2m = (long long)j.nbeta * j.nseq * j.ndat;
    if (j.datm == nullptr || j.ndatm < nchi2m) {
      *err = "plugin model: datm must hold at least nbeta*nseq*ndat values";
      return CMC_ERR_ARG;
    }
    if (mode != 2 && j.chi2m == nullptr) {
      *err = "plugin model: chi2m is required";
      return CMC_ERR_ARG;
    }
    return CMC_OK;
  }

  static size_t host_work_bytes(const Packed &) { return 0; }
  static size_t host_work_bytes_min(const Packed &) { return 0; }
  static constexpr bool kGlobalPhases = false;

  static int host_pack(const cmc_job &, Packed &, void *, cudaStream_t) { return CMC_OK; }

  template <class Cta>
  __device__ static void setup(Cta &cta, int tid, int)
  {
    if (tid != 0) return;
    const cmc_job &j = *cta.job;
    CCalcModel *mc = reinterpret_cast<CCalcModel *>(cta.scratch);
    mc->imodel = j.imodel;
    mc->ncoor = j.ncoor;
    mc->ndat = j.ndat;
    mc->nicoor = j.nicoor;
    mc->nidat = j.nidat;
    mc->ndatm = j.ndatm;
    mc->nptot = j.nptot;
    mc->nbeta = j.nbeta;
    mc->nseq = j.nseq;
    mc->nchi2m = j.nbeta * j.nseq * j.ndat;
    mc->s_coor = 4 * j.ncoor;
    mc->s_dat = 4 * j.ndat;
    mc->s_icoor = 4 * j.nicoor;
    mc->s_idat = 4 * j.nidat;
    mc->s_datm = 4 * j.ndatm;
    mc->s_chi2m = 4 * mc->nchi2m;
    mc->s_pcur = 4 * j.nbeta * j.nseq * j.nptot;
    mc->s_bsint = 4 * j.nbeta * j.nseq;
    mc->s_bsflt = 4 * j.nbeta * j.nseq;
    mc->coor = const_cast<float *>(j.coor);
    mc->dat = const_cast<float *>(j.dat);
    mc->std2r = const_cast<float *>(j.std2r);
    mc->icoor = const_cast<int *>(j.icoor);
    mc->idat = const_cast<int *>(j.idat);
    mc->datm = j.datm;
    mc->chi2m = j.chi2m;
    mc->pcur = j.pcur;
    mc->flag = j.flag;
    mc->chi2c = j.chi2c;
    mc->coor_h = mc->dat_h = mc->std2r_h = nullptr;
    mc->icoor_h = mc->idat_h = nullptr;
    mc->datm_h = mc->chi2m_h = mc->pcur_h = nullptr;
    mc->flag_h = nullptr;
    mc->chi2c_h = nullptr;
  }

  template <class Cta>
  __device__ static void after_exchange(Cta &) {}

  // Publish the replica's parameter row where the plugin reads it (pcur[ipt]).
  template <class Cta>
  __device__ static void prepare(Cta &cta, int r, const float *p)
  {
    const int nptot = cta.job->nptot;
    float *dst = cta.job->pcur + (size_t)cta.ist[r] * nptot;
    for (int j = 0; j < nptot; ++j) dst[j] = p[j];
  }

  template <int R, class Cta>
  __device__ static void eval(Cta &cta, float (&acc)[R])
  {
    const cmc_job &job = *cta.job;
    CCalcModel *mc = reinterpret_cast<CCalcModel *>(cta.scratch);
    const int tid = cta.tid, T = cta.nthreads, ndat = job.ndat, nptot = job.nptot;
    bool act[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      acc[r] = 0.0f;
      act[r] = cta.flag[r] != 0;
    }
    __threadfence_block();
    for (int ipass = 0; ipass < cta.pk->npass; ++ipass) {
      for (int i = tid; i < ndat; i += T) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
          if (!act[r]) continue;
          const int ist = cta.ist[r];
          const int imd = ist * ndat + i;
          const int iret = model(mc, i, ist * nptot, imd, ipass);
          if (iret == 0) continue;
          float dif = job.dat[i] - job.datm[imd];
          if (iret == 2) dif = atan2f(sinf(dif), cosf(dif));
          job.chi2m[imd] = (dif * dif) * job.std2r[i];
        }
      }
      __syncthreads();
    }
    for (int i = tid; i < ndat; i += T) {
#pragma unroll
      for (int r = 0; r < R; ++r)
        if (act[r]) acc[r] += job.chi2m[(size_t)cta.ist[r] * ndat + i];
    }
  }

  // calc_model: model() with ipass = 0 for every datum (gpu_mcmc.cu:633-658).
  template <int R, class Cta>
  __device__ static void model_rows(Cta &cta, const int *flags)
  {
    const cmc_job &job = *cta.job;
    CCalcModel *mc = reinterpret_cast<CCalcModel *>(cta.scratch);
    const int tid = cta.tid, T = cta.nthreads, ndat = job.ndat, nptot = job.nptot;
    for (int i = tid; i < ndat; i += T) {
#pragma unroll
      for (int r = 0; r < R; ++r) {
        if (!flags[r]) continue;
        const int ist = cta.ist[r];
        model(mc, i, ist * nptot, ist * ndat + i, 0);
      }
    }
  }

  template <int R, class Cta>
  __device__ static void final_rows(Cta &, const float *, const int *) {}
};

}  // namespace cmc
