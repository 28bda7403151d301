// module_plugin.cu -- a model.cuh plugin's kernels as a loadable CUDA module.
//
// Compiled with -DCMC_PLUGIN_FILE='"path/model.cuh"' to a cubin (or PTX):
//     nvcc -cubin -arch=sm_103a -DCMC_PLUGIN_FILE=... module_plugin.cu
// it holds the sweep, batch and evaluation kernels of the replicas-per-CTA
// counts 1 .. CMC_MODULE_MAX_R under plain C names
// (cmc_mod_{sweep,batch,eval}_r<R>).  The module library libcmc_module.so
// (lib_plugin.cu + inst_module.cu) loads such a file at run time and launches
// these kernels through the CUDA driver API, so a model can be compiled where
// its source is and run wherever the module file is copied, with the same
// C-ABI as a library that has the model compiled in.
#include "plugin_prelude.cuh"
#include "cmc_eval.cuh"

#define CMC_MODULE_KERNELS(RV)                                                                  \
  extern "C" __global__ void __launch_bounds__(cmc::kMaxThreads, CMC_MIN_BLOCKS)               \
      cmc_mod_sweep_r##RV(const cmc_job job, const cmc::PluginModel::Packed pk)                \
  {                                                                                             \
    cmc::sweep_body<cmc::PluginModel, RV>(job, pk);                                             \
  }                                                                                             \
  extern "C" __global__ void __launch_bounds__(cmc::kMaxThreads, CMC_MIN_BLOCKS)               \
      cmc_mod_batch_r##RV(const cmc_job *jobs, const cmc::PluginModel::Packed *pks,            \
                          const int2 *items, int nitems, int *counter, int do_init, int nburn, \
                          int niter, int itr0)                                                  \
  {                                                                                             \
    cmc::batch_body<cmc::PluginModel, RV>(jobs, pks, items, nitems, counter, do_init, nburn,   \
                                          niter, itr0);                                         \
  }                                                                                             \
  extern "C" __global__ void __launch_bounds__(cmc::kMaxThreads)                               \
      cmc_mod_eval_r##RV(const cmc_job job, const cmc::PluginModel::Packed pk, int mode)       \
  {                                                                                             \
    cmc::eval_body<cmc::PluginModel, RV>(job, pk, mode);                                        \
  }

// A heavy model (the reference's Sgr A* file: Bessel functions in every
// model call, one call per replica unrolled) compiles much faster with fewer
// counts; the library skips the counts a module lacks when it picks a shape.
#ifndef CMC_MODULE_MAX_R
#define CMC_MODULE_MAX_R 32
#endif
CMC_MODULE_KERNELS(1)
#if CMC_MODULE_MAX_R >= 2
CMC_MODULE_KERNELS(2)
#endif
#if CMC_MODULE_MAX_R >= 4
CMC_MODULE_KERNELS(4)
#endif
#if CMC_MODULE_MAX_R >= 8
CMC_MODULE_KERNELS(8)
#endif
#if CMC_MODULE_MAX_R >= 16
CMC_MODULE_KERNELS(16)
#endif
#if CMC_MODULE_MAX_R >= 32
CMC_MODULE_KERNELS(32)
#endif
