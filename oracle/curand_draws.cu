/*
 * curand_draws.cu -- the uniforms that cuRAND XORWOW states give next.
 *
 * TEST INFRASTRUCTURE ONLY.  The lock-step test against the reference's own
 * CUDA build (tests/test_gpu_ref_cuda.py) snapshots the reference's
 * generator states (curandState, src/gpu_mcmc.cu:228-239) just before its
 * spmp_mcmc and replica_exchange kernels; these are then read here, through
 * cuRAND's own curand_uniform() on a copy of each state, to learn the uniform
 * u each Metropolis or exchange decision compares with its acceptance
 * probability (src/gpu_mcmc.cu:451, :563).  A decision whose u lies within a
 * relative 1e-3 of its probability is a near tie, which float32 rounding of
 * chi^2 may legitimately flip.
 */
#include <cuda_runtime.h>
#include <curand_kernel.h>

__global__ void next_uniforms_kernel(const curandStateXORWOW *st, int n, int per, float *out)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  curandStateXORWOW s = st[i];
  for (int j = 0; j < per; ++j) out[(size_t)i * per + j] = curand_uniform(&s);
}

/* out[i*per + j] = the j-th uniform state i gives (states and out are device
 * pointers; the states are not modified).  Returns a cudaError_t. */
extern "C" int cd_next_uniforms(const void *states, int n, int per, float *out, void *stream)
{
  if (n <= 0 || per <= 0) return 0;
  next_uniforms_kernel<<<(n + 127) / 128, 128, 0, (cudaStream_t)stream>>>(
      (const curandStateXORWOW *)states, n, per, out);
  return (int)cudaGetLastError();
}
