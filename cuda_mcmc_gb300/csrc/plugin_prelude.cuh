// plugin_prelude.cuh -- compiles a model.cuh plugin (CMC_PLUGIN_FILE) unchanged,
// with the helpers the reference's mcmcjob.cuh gives plugins (pi, pi4, min,
// max; src/mcmcjob.cuh:9-21) defined only while it is being read, then the
// plugin model policy.
#pragma once
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <curand_kernel.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "mcmcjob.cuh"

// The plugin is read inside an unnamed namespace: every kernel-instance object
// of a library holds its own internal copy of model(), so the objects link
// together.  Headers a plugin might include are included above first.
#ifdef CMC_PLUGIN_DECLARE_ONLY
namespace {
__device__ int model(CCalcModel *mc, int id, int ipt, int imd, int ipass);
}
#else
namespace {
#define pi (3.1415926535897931f)
#define pi4 (12.566370614359172f)
#define min(a, b) ((a) < (b) ? (a) : (b))
#define max(a, b) ((a) > (b) ? (a) : (b))
#include CMC_PLUGIN_FILE
#undef pi
#undef pi4
#undef min
#undef max
}  // namespace
#endif

#include "model_plugin.cuh"
