// cmc_eval.cuh -- batch model evaluation kernels behind calc_modchi2 and
// calc_model (src/mcmcjob.cu:227-298, src/gpu_mcmc.cu:769-802).
//
// One CTA evaluates R parameter sets (replicas ist = blockIdx.x*R + r) over
// all data with the same model code as the sweep:
//   mode 0 (calc_modchi2): model values, chi^2 terms and chi2c = sum of the
//          chi2m row, both passes (run_calcmodchi2 runs passes 0 and 1);
//   mode 1 (calc_model):   pass 0 only, model values (and, for Sgr A*, the
//          phase tail) without chi^2.
// Replicas with flag == 0 are skipped, as calc_chi2_terms does.
#pragma once
#include "cmc_sweep.cuh"

namespace cmc {

template <class Model, int R>
__device__ __forceinline__ void eval_body(const cmc_job &job, const typename Model::Packed &pk,
                                          int mode)
{
  extern __shared__ __align__(16) unsigned char smem[];
  const int tid = threadIdx.x, T = blockDim.x, NW = T >> 5;
  const int nptot = job.nptot, nrep = job.nbeta * job.nseq;
  const SmemPlan P = make_plan(R, T, nptot, 1, 1, 1, sizeof(typename Model::Consts),
                               Model::scratch_bytes(pk, R));
  float *params = (float *)(smem + P.params);
  int *ri = (int *)(smem + P.ri);
  int *s_flag = ri + R;
  float *s_red = (float *)(smem + P.red);

  Cta<Model, R> cta;
  cta.job = &job;
  cta.pk = &pk;
  cta.consts = (typename Model::Consts *)(smem + P.consts);
  cta.flag = s_flag;
  cta.scratch = (float *)(smem + P.scratch);
  cta.tid = tid;
  cta.nthreads = T;
#pragma unroll
  for (int r = 0; r < R; ++r) cta.ist[r] = blockIdx.x * R + r;
  cta.ph_region = blockIdx.x * R;

  for (int i = tid; i < R * nptot; i += T) {
    int r = i / nptot, j = i - r * nptot;
    int ist = blockIdx.x * R + r;
    params[i] = (ist < nrep) ? job.pcur[(size_t)ist * nptot + j] : 0.0f;
  }
  Model::setup(cta, tid, T);
  if (tid < R) {
    int ist = blockIdx.x * R + tid;
    s_flag[tid] = (ist < nrep && (job.flag == nullptr || job.flag[ist] != 0)) ? 1 : 0;
  }
  __syncthreads();
  if (tid < R && s_flag[tid]) Model::prepare(cta, tid, &params[tid * nptot]);
  __syncthreads();
  if (mode == 1) {
    Model::template model_rows<R>(cta, s_flag);
    return;
  }
  float acc[R];
  if (Model::kRowsInEval) {
    Model::template eval<R>(cta, acc);
  } else {
    // Rows first, then chi2c as the sum of each chi2m row (calc_chi2, :331-350).
    Model::template final_rows<R>(cta, params, s_flag);
    __syncthreads();
#pragma unroll
    for (int r = 0; r < R; ++r) acc[r] = 0.0f;
    for (int i = tid; i < job.ndat; i += T) {
#pragma unroll
      for (int r = 0; r < R; ++r)
        if (s_flag[r]) acc[r] += job.chi2m[(size_t)cta.ist[r] * job.ndat + i];
    }
  }
  block_reduce<Model, R>(acc, s_red, tid, NW);
  __syncthreads();
  if (tid < R && s_flag[tid]) {
    float s = 0.f;
    for (int w = 0; w < NW; ++w) s += s_red[tid * NW + w];
    job.chi2c[blockIdx.x * R + tid] = s;
  }
}

template <class Model, int R>
__global__ void __launch_bounds__(kMaxThreads)
eval_kernel(const cmc_job job, const typename Model::Packed pk, int mode)
{
  eval_body<Model, R>(job, pk, mode);
}

}  // namespace cmc
