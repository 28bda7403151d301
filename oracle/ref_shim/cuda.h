/* Host stand-in for <cuda.h>, used only when oracle/ref_build.py compiles the
 * reference's kernels as plain C++ on the CPU (test infrastructure). */
#pragma once
typedef enum cudaError { cudaSuccess = 0 } cudaError;
typedef cudaError cudaError_t;
