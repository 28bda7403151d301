/* Force-included before the reference's kernels when oracle/ref_build.py
 * compiles them as plain C++ for the CPU (test infrastructure).  Kernel
 * qualifiers vanish and the launch coordinates become globals that the
 * emulation driver (oracle/ref_driver.cpp) sets before each "thread". */
#pragma once
#include <cmath>
/* the C++ <math.h> also brings the float overloads (expf for exp(float)...)
 * into the global namespace, as CUDA's device math headers do */
#include <math.h>
#include <cstdio>
#include <cstdlib>
#define __global__
#define __device__
#define __host__
struct ref_dim3 { unsigned x, y, z; };
extern ref_dim3 blockIdx, threadIdx, blockDim, gridDim;
