// lib_sgra.cu -- libcmc_sgra.so: the C-ABI with the built-in Sgr A* crescent
// + Gaussian model (the reference's examples/sgra_model_fit/model.cuh).
#include "cmc_host.cuh"
#include "model_sgra.cuh"

#define CMC_MODEL cmc::SgraModel
#define CMC_MODEL_NAME "sgra"
#include "cmc_abi.inc"

// ---- allocation-free entry point --------------------------------------------
//
// cmc_run takes every device array from its caller except one: job->work, the
// scratch that holds the packed Sgr A* data.  Some callers cannot hand out new
// device memory at run time -- for example a process whose device memory is
// reserved up front by another framework's caching allocator (a fresh
// cudaMalloc there fails or fragments that pool), or a latency-critical
// pipeline that cannot let cudaMalloc / cudaFree synchronise the device between
// its stages.  cmc_run_noalloc is cmc_run with that scratch taken from a fixed
// array compiled into this library (kStaticWorkBytes = 4 MiB, enough for about
// 80,000 visibility + triangle points with their closures).  It calls no
// cudaMalloc, cudaFree or other allocating routine.
//
// The array's device address is looked up once per device, by the first call
// made with that device current (so that first call should come before any
// stream capture).  Every GPU that loads this library keeps the 4 MiB until
// the process exits.  All calls share the one array and it keeps the last
// call's contents; nothing in it needs to start at zero (each call rewrites
// every element it reads).  Calls that overlap on the GPU race on it: issue
// them on one stream, or otherwise order them.
#include <mutex>

namespace {
constexpr size_t kStaticWorkBytes = size_t(4) << 20;
__device__ __align__(256) unsigned char g_static_work[kStaticWorkBytes];
constexpr int kMaxDevices = 64;
std::mutex g_static_work_mu;
void *g_static_work_ptr[kMaxDevices] = {};
}  // namespace

extern "C" int cmc_run_noalloc(const cmc_job *job, void *stream)
{
  cmc::last_error().clear();
  if (!job) return cmc::fail(CMC_ERR_ARG, "cmc_run_noalloc: job is NULL");
  const size_t need = cmc::work_bytes<cmc::SgraModel>(*job, 0);
  if (need > kStaticWorkBytes)
    return cmc::fail(CMC_ERR_ARG,
                     "cmc_run_noalloc: the packed data needs " + std::to_string(need) +
                         " bytes of scratch, more than its fixed 4 MiB array (about 80,000 "
                         "points); use cmc_run with a caller-provided job->work");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cmc::cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices)
    return cmc::fail(CMC_ERR_ARG, "cmc_run_noalloc: device ordinal out of range");
  void *p = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_static_work_mu);
    if (g_static_work_ptr[dev] == nullptr) {
      e = cudaGetSymbolAddress(&g_static_work_ptr[dev], g_static_work);
      if (e != cudaSuccess) {
        g_static_work_ptr[dev] = nullptr;
        return cmc::cuda_fail(e, "cudaGetSymbolAddress(static scratch)");
      }
    }
    p = g_static_work_ptr[dev];
  }
  cmc_job j = *job;
  j.work = p;
  j.work_bytes = kStaticWorkBytes;
  return cmc::run_sweep<cmc::SgraModel>(j, (cudaStream_t)stream);
}
