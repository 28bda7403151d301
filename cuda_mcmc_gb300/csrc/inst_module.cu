// inst_module.cu -- kernel launches of the module library libcmc_module.so.
//
// Where a plugin library has its model compiled in (inst_plugin.cu), the
// module library takes the kernels from a CUDA module built from
// module_plugin.cu with the model (a cubin or PTX file), loaded at the first
// launch from the path given to cmc_module_set() or, failing that, in the
// environment variable CMC_PLUGIN_MODULE.  The launches are the same as the
// compiled-in ones -- clusters of G CTAs, T threads, the dynamic shared memory
// of the plan -- issued with the CUDA driver API (cuLaunchKernelEx) in the
// runtime's current context on the caller's stream.  The driver functions are
// looked up through the runtime (cudaGetDriverEntryPointByVersion) at the
// first launch, so the library loads on a machine without a GPU driver.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <cstdlib>
#include <mutex>
#include <string>

#define CMC_PLUGIN_DECLARE_ONLY 1
#include "plugin_prelude.cuh"
#include "cmc_launch.cuh"

namespace cmc {

int fail(int code, const std::string &msg);   // cmc_host.cuh (library TU)

namespace {
std::mutex g_mu;
std::string g_path;
CUmodule g_mod = nullptr;
CUfunction g_fn[3][6] = {};   // [sweep, batch, eval][R index]

// the CUDA driver functions this library calls
struct Driver {
  PFN_cuModuleLoad_v2000 moduleLoad = nullptr;
  PFN_cuModuleGetFunction_v2000 moduleGetFunction = nullptr;
  PFN_cuFuncSetAttribute_v9000 funcSetAttribute = nullptr;
  PFN_cuOccupancyMaxActiveClusters_v11070 occupancyMaxActiveClusters = nullptr;
  PFN_cuLaunchKernelEx_v11060 launchKernelEx = nullptr;
  PFN_cuGetErrorString_v6000 getErrorString = nullptr;
  bool ok = false;
};
Driver g_drv;

template <class F>
bool entry(const char *name, F &f)
{
  void *p = nullptr;
  cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
  if (cudaGetDriverEntryPointByVersion(name, &p, 12080, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || p == nullptr) {
    cudaGetLastError();
    return false;
  }
  f = reinterpret_cast<F>(p);
  return true;
}

// Resolves the driver functions once (called with g_mu held).
bool driver()
{
  if (g_drv.ok) return true;
  g_drv.ok = entry("cuModuleLoad", g_drv.moduleLoad) &&
             entry("cuModuleGetFunction", g_drv.moduleGetFunction) &&
             entry("cuFuncSetAttribute", g_drv.funcSetAttribute) &&
             entry("cuOccupancyMaxActiveClusters", g_drv.occupancyMaxActiveClusters) &&
             entry("cuLaunchKernelEx", g_drv.launchKernelEx) &&
             entry("cuGetErrorString", g_drv.getErrorString);
  return g_drv.ok;
}

int r_index(int R)
{
  switch (R) {
    case 1: return 0;
    case 2: return 1;
    case 4: return 2;
    case 8: return 3;
    case 16: return 4;
    case 32: return 5;
    default: return -1;
  }
}

const char *cu_err(CUresult r)
{
  const char *s = nullptr;
  if (g_drv.getErrorString) g_drv.getErrorString(r, &s);
  return s ? s : "unknown CUDA driver error";
}

// The function `kind` (0 sweep, 1 batch, 2 eval) at R, loading the module on
// first use; nullptr (with the library's last error set) when the module is
// missing or lacks that count.
CUfunction function(int kind, int R)
{
  static const char *names[3] = {"cmc_mod_sweep_r", "cmc_mod_batch_r", "cmc_mod_eval_r"};
  const int ri = r_index(R);
  if (ri < 0) {
    fail(CMC_ERR_UNSUPPORTED, "module library: no kernel for this replicas-per-CTA count");
    return nullptr;
  }
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_mod) {
    std::string path = g_path;
    if (path.empty()) {
      const char *e = std::getenv("CMC_PLUGIN_MODULE");
      if (e) path = e;
    }
    if (path.empty()) {
      fail(CMC_ERR_ARG, "module library: no module file (cmc_module_set or CMC_PLUGIN_MODULE)");
      return nullptr;
    }
    cudaFree(nullptr);   // the runtime's primary context is current from here on
    if (!driver()) {
      fail(CMC_ERR_CUDA, "module library: the CUDA driver functions are not available");
      return nullptr;
    }
    CUresult r = g_drv.moduleLoad(&g_mod, path.c_str());
    if (r != CUDA_SUCCESS) {
      g_mod = nullptr;
      fail(CMC_ERR_CUDA, "module library: loading " + path + ": " + cu_err(r));
      return nullptr;
    }
  }
  if (!g_fn[kind][ri]) {
    const std::string name = names[kind] + std::to_string(R);
    CUresult r = g_drv.moduleGetFunction(&g_fn[kind][ri], g_mod, name.c_str());
    if (r != CUDA_SUCCESS) {
      g_fn[kind][ri] = nullptr;
      fail(CMC_ERR_UNSUPPORTED, "module library: " + name + ": " + cu_err(r));
      return nullptr;
    }
  }
  return g_fn[kind][ri];
}

int set_attrs(CUfunction f, size_t smem, int G)
{
  CUresult r = g_drv.funcSetAttribute(f, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)smem);
  if (r == CUDA_SUCCESS && G > 8)
    r = g_drv.funcSetAttribute(f, CU_FUNC_ATTRIBUTE_NON_PORTABLE_CLUSTER_SIZE_ALLOWED, 1);
  return r == CUDA_SUCCESS ? CMC_OK
                           : fail(CMC_ERR_CUDA, std::string("kernel attributes: ") + cu_err(r));
}

CUlaunchConfig config(int G, int grid, int T, size_t smem, cudaStream_t s, CUlaunchAttribute *attr)
{
  CUlaunchConfig cfg = {};
  attr[0].id = CU_LAUNCH_ATTRIBUTE_CLUSTER_DIMENSION;
  attr[0].value.clusterDim.x = G > 0 ? G : 1;
  attr[0].value.clusterDim.y = 1;
  attr[0].value.clusterDim.z = 1;
  cfg.gridDimX = grid;
  cfg.gridDimY = cfg.gridDimZ = 1;
  cfg.blockDimX = T;
  cfg.blockDimY = cfg.blockDimZ = 1;
  cfg.sharedMemBytes = (unsigned)smem;
  cfg.hStream = (CUstream)s;
  cfg.attrs = attr;
  cfg.numAttrs = G > 0 ? 1 : 0;
  return cfg;
}

int capacity(int kind, int R, int G, int T, size_t smem, int grid)
{
  CUfunction f = function(kind, R);
  if (!f || set_attrs(f, smem, G) != CMC_OK) return 0;
  CUlaunchAttribute attr[1];
  CUlaunchConfig cfg = config(G, grid, T, smem, nullptr, attr);
  int n = 0;
  return g_drv.occupancyMaxActiveClusters(&n, f, &cfg) == CUDA_SUCCESS ? n : 0;
}

int launch(int kind, int R, int G, int grid, int T, size_t smem, cudaStream_t s, void **args)
{
  CUfunction f = function(kind, R);
  if (!f) return g_mod ? CMC_ERR_UNSUPPORTED : CMC_ERR_CUDA;   // no such count / no module
  int rc = set_attrs(f, smem, G);
  if (rc) return rc;
  CUlaunchAttribute attr[1];
  CUlaunchConfig cfg = config(G, grid, T, smem, s, attr);
  CUresult r = g_drv.launchKernelEx(&cfg, f, args, nullptr);
  return r == CUDA_SUCCESS ? CMC_OK
                           : fail(CMC_ERR_CUDA, std::string("kernel launch: ") + cu_err(r));
}
}  // namespace

#define CMC_MODULE_LAUNCHERS(RV)                                                                 \
  template <>                                                                                    \
  int sweep_capacity<PluginModel, RV>(int G, int T, size_t smem, int nseq)                       \
  {                                                                                              \
    return capacity(0, RV, G, T, smem, G * nseq);                                                \
  }                                                                                              \
  template <>                                                                                    \
  int launch_sweep<PluginModel, RV>(const cmc_job &j, const PluginModel::Packed &pk,             \
                                    const LaunchCfg &c, cudaStream_t s)                          \
  {                                                                                              \
    cmc_job jj = j;                                                                              \
    PluginModel::Packed pp = pk;                                                                 \
    void *args[] = {&jj, &pp};                                                                   \
    return launch(0, RV, c.G, c.G * j.nseq, c.T, c.smem, s, args);                               \
  }                                                                                              \
  template <>                                                                                    \
  int batch_capacity<PluginModel, RV>(int G, int T, size_t smem)                                 \
  {                                                                                              \
    return capacity(1, RV, G, T, smem, G);                                                       \
  }                                                                                              \
  template <>                                                                                    \
  int launch_batch<PluginModel, RV>(const cmc_job *jobs, const PluginModel::Packed *pks,         \
                                    const int2 *items, int nitems, int *counter, int G, int T,   \
                                    size_t smem, int nclusters, int do_init, int nburn,          \
                                    int niter, int itr0, cudaStream_t s)                         \
  {                                                                                              \
    void *args[] = {&jobs, &pks, &items, &nitems, &counter, &do_init, &nburn, &niter, &itr0};   \
    return launch(1, RV, G, G * nclusters, T, smem, s, args);                                    \
  }                                                                                              \
  template <>                                                                                    \
  int launch_eval<PluginModel, RV>(const cmc_job &j, const PluginModel::Packed &pk,              \
                                   int model_only, int T, size_t smem, cudaStream_t s)           \
  {                                                                                              \
    cmc_job jj = j;                                                                              \
    PluginModel::Packed pp = pk;                                                                 \
    void *args[] = {&jj, &pp, &model_only};                                                      \
    const int nrep = j.nbeta * j.nseq;                                                           \
    return launch(2, RV, 0, (nrep + RV - 1) / RV, T, smem, s, args);                             \
  }

CMC_MODULE_LAUNCHERS(1)
CMC_MODULE_LAUNCHERS(2)
CMC_MODULE_LAUNCHERS(4)
CMC_MODULE_LAUNCHERS(8)
CMC_MODULE_LAUNCHERS(16)
CMC_MODULE_LAUNCHERS(32)

}  // namespace cmc

// See include/cuda_mcmc.h.
extern "C" int cmc_module_set(const char *path)
{
  std::lock_guard<std::mutex> lock(cmc::g_mu);
  const std::string p = path ? path : "";
  if (cmc::g_mod && p != cmc::g_path)
    return cmc::fail(CMC_ERR_ARG, "cmc_module_set: another module is already loaded");
  cmc::g_path = p;
  return CMC_OK;
}
