// cmc_launch_impl.cuh -- definitions behind cmc_launch.cuh.  Included by the
// instance translation units only (inst_sgra.cu, inst_plugin.cu), each of
// which instantiates one value of R for its model.
#pragma once
#include <cstdlib>
#include <string>

#include "cmc_eval.cuh"
#include "cmc_launch.cuh"
#include "cmc_sweep.cuh"

namespace cmc {

int fail(int code, const std::string &msg);   // cmc_host.cuh (library TU)

template <class Model, int R>
int sweep_capacity(int G, int T, size_t smem, int nseq)
{
  auto kern = sweep_kernel<Model, R>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  if (G > 8 &&
      cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = G;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3(G * nseq);
  cfg.blockDim = dim3(T);
  cfg.dynamicSmemBytes = smem;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, (void *)kern, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

template <class Model, int R>
int launch_sweep(const cmc_job &j, const typename Model::Packed &pk, const LaunchCfg &c,
                 cudaStream_t s)
{
  auto kern = sweep_kernel<Model, R>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)c.smem);
  if (e == cudaSuccess && c.G > 8)
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  if (e != cudaSuccess)
    return fail(CMC_ERR_CUDA, std::string("sweep kernel attributes: ") + cudaGetErrorString(e));
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = c.G;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3(c.G * j.nseq);
  cfg.blockDim = dim3(c.T);
  cfg.dynamicSmemBytes = c.smem;
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  e = cudaLaunchKernelEx(&cfg, kern, j, pk);
  if (e != cudaSuccess)
    return fail(CMC_ERR_CUDA, std::string("sweep kernel launch: ") + cudaGetErrorString(e));
  return CMC_OK;
}

template <class Model, int R>
int batch_capacity(int G, int T, size_t smem)
{
  auto kern = batch_kernel<Model, R>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  if (G > 8 &&
      cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = G;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3(G);
  cfg.blockDim = dim3(T);
  cfg.dynamicSmemBytes = smem;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, (void *)kern, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

template <class Model, int R>
int launch_batch(const cmc_job *jobs, const typename Model::Packed *pks, const int2 *items,
                 int nitems, int *counter, int G, int T, size_t smem, int nclusters, int do_init,
                 int nburn, int niter, int itr0, cudaStream_t s)
{
  auto kern = batch_kernel<Model, R>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess && G > 8)
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  if (e != cudaSuccess)
    return fail(CMC_ERR_CUDA, std::string("batch kernel attributes: ") + cudaGetErrorString(e));
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = G;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3(G * nclusters);
  cfg.blockDim = dim3(T);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  e = cudaLaunchKernelEx(&cfg, kern, jobs, pks, items, nitems, counter, do_init, nburn, niter,
                         itr0);
  if (e != cudaSuccess)
    return fail(CMC_ERR_CUDA, std::string("batch kernel launch: ") + cudaGetErrorString(e));
  return CMC_OK;
}

template <class Model, int R>
int spread_capacity(int T, size_t smem)
{
  auto kern = spread_kernel<Model, R>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  int dev = 0, coop = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, T, smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return coop ? per_sm * sms : 0;
}

template <class Model, int R>
int launch_spread(const cmc_job &j, const typename Model::Packed &pk, const LaunchCfg &c,
                  void *ctl, cudaStream_t s)
{
  auto kern = spread_kernel<Model, R>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)c.smem);
  if (e != cudaSuccess)
    return fail(CMC_ERR_CUDA, std::string("spread kernel attributes: ") + cudaGetErrorString(e));
  e = cudaMemsetAsync(ctl, 0, spread_ctl_counter_bytes(j.nseq), s);
  if (e != cudaSuccess)
    return fail(CMC_ERR_CUDA, std::string("spread counters: ") + cudaGetErrorString(e));
  SpreadCtl x = spread_ctl_at(static_cast<unsigned char *>(ctl), j.nseq, j.nbeta, j.nptot);
  if (const char *h = std::getenv("CMC_SPREAD_HOLD_SEQ")) x.hold = std::atoi(h);   // test hook
  x.ngroups = c.groups;
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.gridDim = dim3(c.nblocks);
  cfg.blockDim = dim3(c.T);
  cfg.dynamicSmemBytes = c.smem;
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  e = cudaLaunchKernelEx(&cfg, kern, j, pk, x);
  if (e != cudaSuccess)
    return fail(CMC_ERR_CUDA, std::string("spread kernel launch: ") + cudaGetErrorString(e));
  return CMC_OK;
}

template <class Model, int R>
int launch_eval(const cmc_job &j, const typename Model::Packed &pk, int model_only, int T,
                size_t smem, cudaStream_t s)
{
  auto kern = eval_kernel<Model, R>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess)
    return fail(CMC_ERR_CUDA, std::string("eval kernel attributes: ") + cudaGetErrorString(e));
  const int nrep = j.nbeta * j.nseq;
  kern<<<(nrep + R - 1) / R, T, smem, s>>>(j, pk, model_only);
  e = cudaGetLastError();
  if (e != cudaSuccess)
    return fail(CMC_ERR_CUDA, std::string("eval kernel launch: ") + cudaGetErrorString(e));
  return CMC_OK;
}

#define CMC_INSTANTIATE(MODEL, RV)                                                        \
  template int sweep_capacity<MODEL, RV>(int, int, size_t, int);                          \
  template int launch_sweep<MODEL, RV>(const cmc_job &, const MODEL::Packed &,           \
                                       const LaunchCfg &, cudaStream_t);                  \
  template int launch_eval<MODEL, RV>(const cmc_job &, const MODEL::Packed &, int, int,  \
                                      size_t, cudaStream_t);                              \
  template int batch_capacity<MODEL, RV>(int, int, size_t);                               \
  template int launch_batch<MODEL, RV>(const cmc_job *, const MODEL::Packed *, const int2 *, \
                                       int, int *, int, int, size_t, int, int, int, int, int, \
                                       cudaStream_t);

// The spread-layout sweep for one R (every R of 1..Model::kMaxR of a model
// with Model::kSpread).
#define CMC_INSTANTIATE_SPREAD(MODEL, RV)                                                  \
  template int spread_capacity<MODEL, RV>(int, size_t);                                    \
  template int launch_spread<MODEL, RV>(const cmc_job &, const MODEL::Packed &,           \
                                        const LaunchCfg &, void *, cudaStream_t);

}  // namespace cmc
