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
// array compiled into this library (kStaticWorkBytes = 4 MiB).  The packed
// data takes 52 bytes per point and 32 per closure, so at most about 80,000
// points; the closure phases of all replicas then need the rest of the array
// ((nbeta*nseq + 8)*points*4 bytes, used from 2048 points on) or, failing that,
// shared memory (R*points*4 bytes per CTA, R >= nbeta/16: up to about 27,000
// points at 32 temperatures).  Where cmc_run with a full job->work would keep
// the phases in global memory and they do not fit in the array, this call
// keeps them in shared memory, so its launch shape and speed can differ from
// cmc_run's.  It calls no cudaMalloc, cudaFree or other allocating routine.
//
// The array's device address is looked up once per device, by the first call
// made with that device current (so that first call should come before any
// stream capture), and cached for the life of the process: after a
// cudaDeviceReset the cached address is stale.  Every GPU that loads this
// library keeps the 4 MiB until the process exits.  All calls share the one array and it keeps the last
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
  const size_t need = cmc::work_bytes_min<cmc::SgraModel>(*job, 0);
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
  // The closure phases of every replica must fit too: beside the packed data
  // in the array (from 2048 points on, when (nbeta*nseq + 8)*points floats fit
  // there) or else in shared memory, where each CTA keeps the phases of its
  // R >= nbeta/16 replicas.  A job that fits neither is refused here with a
  // message that names the array.
  {
    int rc = cmc::validate_common(j, 0);
    if (rc) return rc;
    cmc::SgraModel::Packed pk;
    const char *err = nullptr;
    rc = cmc::SgraModel::host_dims(j, 0, pk, &err);
    if (rc) return cmc::fail(rc, err);
    cmc::LaunchCfg c;
    if (cmc::pick_sweep_config<cmc::SgraModel>(j, pk, c) != CMC_OK)
      return cmc::fail(CMC_ERR_UNSUPPORTED,
                       "cmc_run_noalloc: the closure phases of this job fit neither beside "
                       "the packed data in the fixed 4 MiB array ((nbeta*nseq + 8)*points*4 bytes) "
                       "nor in shared memory (R*points*4 bytes per CTA with R >= nbeta/16 "
                       "replicas); use cmc_run with job->work of cmc_work_bytes() bytes");
  }
  return cmc::run_sweep<cmc::SgraModel>(j, (cudaStream_t)stream);
}

// ---- chi^2 gradient (no counterpart in the reference) -----------------------
//
// cmc_grad: chi2c[ist] and dchi2/dp into grad[ist*nptot + k] at pcur for every
// replica ist < nbeta*nseq (flag[ist] == 0 with flag non-NULL: zeros), with the
// job's npass (npass < 2: amplitude terms only).  job->work holds the packed
// data followed by the per-point phases and adjoints of every replica:
// cmc_grad_work_bytes(job) bytes.
#include "model_sgra_grad.cuh"

namespace {
size_t grad_extra_offset(const cmc::SgraModel::Packed &pk)
{
  return cmc::SgraModel::host_work_bytes_min(pk);
}

int grad_dims(const cmc_job &j, cmc::SgraModel::Packed &pk)
{
  int rc = cmc::validate_common(j, 1);
  if (rc) return rc;
  const char *err = nullptr;
  cmc_job k = j;
  k.datm = nullptr;   // the gradient writes no model rows
  rc = cmc::SgraModel::host_dims(k, 0, pk, &err);
  if (rc) return cmc::fail(rc, err);
  if (j.nptot > cmc::kMaxGradParams)
    return cmc::fail(CMC_ERR_ARG, "cmc_grad: nptot must be <= 16");
  return CMC_OK;
}
}  // namespace

extern "C" size_t cmc_grad_work_bytes(const cmc_job *job)
{
  if (!job) return 0;
  cmc::SgraModel::Packed pk;
  const char *err = nullptr;
  cmc_job k = *job;
  k.datm = nullptr;
  if (cmc::SgraModel::host_dims(k, 0, pk, &err)) return 0;
  const size_t nrep = (size_t)job->nbeta * job->nseq;
  return grad_extra_offset(pk) + nrep * 3 * (size_t)pk.npts * sizeof(float);
}

extern "C" int cmc_grad(const cmc_job *job, float *grad, void *stream)
{
  cmc::last_error().clear();
  if (!job) return cmc::fail(CMC_ERR_ARG, "cmc_grad: job is NULL");
  if (!grad) return cmc::fail(CMC_ERR_ARG, "cmc_grad: grad must be a device pointer");
  const cmc_job &j = *job;
  cmc::SgraModel::Packed pk;
  int rc = grad_dims(j, pk);
  if (rc) return rc;
  const size_t need = cmc_grad_work_bytes(job);
  if (j.work == nullptr || j.work_bytes < need)
    return cmc::fail(CMC_ERR_ARG, "cmc_grad: job.work is smaller than cmc_grad_work_bytes()");
  cudaStream_t s = (cudaStream_t)stream;
  rc = cmc::SgraModel::host_pack(j, pk, j.work, s);
  if (rc) return cmc::fail(rc, "packing the model data failed");
  float *gwork = (float *)((unsigned char *)j.work + grad_extra_offset(pk));
  const int T = 256;
  const size_t smem = cmc::sgra_grad_smem(j.nptot, T);
  const unsigned nrep = (unsigned)(j.nbeta * j.nseq);
  cmc::sgra_grad_kernel<<<nrep, T, smem, s>>>(j, pk, grad, gwork);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? CMC_OK : cmc::cuda_fail(e, "sgra_grad_kernel launch");
}

// cmc_fisher: Gauss-Newton Fisher information of chi^2/2 at pcur for every
// replica into fisher[ist][nptot][nptot] (zeros for flag[ist] == 0 with flag
// non-NULL).  job->work: the packed data followed by per-point derivative rows
// of every replica, cmc_fisher_work_bytes(job) bytes.
extern "C" size_t cmc_fisher_work_bytes(const cmc_job *job)
{
  if (!job) return 0;
  cmc::SgraModel::Packed pk;
  const char *err = nullptr;
  cmc_job k = *job;
  k.datm = nullptr;
  if (cmc::SgraModel::host_dims(k, 0, pk, &err)) return 0;
  const size_t nrep = (size_t)job->nbeta * job->nseq;
  return grad_extra_offset(pk) + nrep * cmc::sgra_fisher_gwork_floats(pk) * sizeof(float);
}

extern "C" int cmc_fisher(const cmc_job *job, float *fisher, void *stream)
{
  cmc::last_error().clear();
  if (!job) return cmc::fail(CMC_ERR_ARG, "cmc_fisher: job is NULL");
  if (!fisher) return cmc::fail(CMC_ERR_ARG, "cmc_fisher: fisher must be a device pointer");
  const cmc_job &j = *job;
  cmc::SgraModel::Packed pk;
  int rc = grad_dims(j, pk);
  if (rc) return rc;
  const size_t need = cmc_fisher_work_bytes(job);
  if (j.work == nullptr || j.work_bytes < need)
    return cmc::fail(CMC_ERR_ARG, "cmc_fisher: job.work is smaller than cmc_fisher_work_bytes()");
  cudaStream_t s = (cudaStream_t)stream;
  rc = cmc::SgraModel::host_pack(j, pk, j.work, s);
  if (rc) return cmc::fail(rc, "packing the model data failed");
  float *gwork = (float *)((unsigned char *)j.work + grad_extra_offset(pk));
  const unsigned nrep = (unsigned)(j.nbeta * j.nseq);
  cmc::sgra_fisher_kernel<<<nrep, 256, cmc::sgra_fisher_smem(j.nptot), s>>>(j, pk, fisher, gwork);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? CMC_OK : cmc::cuda_fail(e, "sgra_fisher_kernel launch");
}
