// cmc_launch.cuh -- launch entry points of the kernel instances.
//
// Each (model, R) kernel instance is compiled in its own translation unit
// (inst_*.cu with -DCMC_R=R, see cmc_launch_impl.cuh) so that a library builds
// in parallel; the host layer only sees these declarations.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>

#include "cmc_job.h"

namespace cmc {

struct LaunchCfg {
  int R = 0, G = 0, T = 0, phasor = 1, clusters_per_wave = 0;
  size_t smem = 0;
  int spread = 0;    // 1: spread layout (cooperative launch of nblocks CTAs, G = 0)
  int nblocks = 0;
  int groups = 1;    // spread layout: sequence groups run one after the other
};

// Clusters of G CTAs (T threads, smem bytes) that can be resident at once;
// 0 when the configuration does not fit.
template <class Model, int R>
int sweep_capacity(int G, int T, size_t smem, int nseq);

template <class Model, int R>
int launch_sweep(const cmc_job &j, const typename Model::Packed &pk, const LaunchCfg &c,
                 cudaStream_t s);

// Resident clusters of the batch kernel at this shape (0: does not fit).
template <class Model, int R>
int batch_capacity(int G, int T, size_t smem);

template <class Model, int R>
int launch_batch(const cmc_job *jobs, const typename Model::Packed *pks, const int2 *items,
                 int nitems, int *counter, int G, int T, size_t smem, int nclusters, int do_init,
                 int nburn, int niter, int itr0, cudaStream_t s);

// Spread layout (cmc_sweep.cuh): CTAs of T threads and smem bytes resident
// at once on the device (0: does not fit), and the cooperative launch of
// c.nblocks CTAs over the job's SpreadCtl area `ctl` (whose counters the
// launch zeroes first, on the same stream).
template <class Model, int R>
int spread_capacity(int T, size_t smem);

template <class Model, int R>
int launch_spread(const cmc_job &j, const typename Model::Packed &pk, const LaunchCfg &c,
                  void *ctl, cudaStream_t s);

template <class Model, int R>
int launch_eval(const cmc_job &j, const typename Model::Packed &pk, int model_only, int T,
                size_t smem, cudaStream_t s);

}  // namespace cmc
