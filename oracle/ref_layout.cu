/*
 * ref_layout.cu -- prints the byte layout of the reference's job object.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/ref_build.py compiles this file against
 * the reference's src/mcmcjob.cuh (read in place through -I) and runs it once
 * in the build container; the JSON it prints (oracle/_ref/ref_gpu_layout.json)
 * lets oracle/ref_gpu.py build a CMcmcFit object (src/mcmcjob.cuh:121-279,
 * derived from CCalcModel :30-118) in device memory for the reference's own
 * kernels, which take a CMcmcFit* / CCalcModel* (src/gpu_mcmc.cu:228-626).
 * Both machines are LP64, so the layout is the same on the x86 build host and
 * the Arm GPU host.
 */
#include <cstddef>
#include <cstdio>

#include <cuda_runtime.h>
#include <curand_kernel.h>

#include "mcmcjob.cuh"

static int first = 1;
#define FIELD(m)                                                                      \
  do {                                                                                \
    std::printf("%s\n    \"%s\": %zu", first ? "" : ",", #m, offsetof(CMcmcFit, m)); \
    first = 0;                                                                        \
  } while (0)

int main()
{
  std::printf("{\n  \"sizeof_CMcmcFit\": %zu,\n  \"sizeof_curandState\": %zu,\n"
              "  \"sizeof_pointer\": %zu,\n  \"offsets\": {",
              sizeof(CMcmcFit), sizeof(curandState), sizeof(void *));
  /* CCalcModel */
  FIELD(imodel); FIELD(ncoor); FIELD(ndat); FIELD(nicoor); FIELD(nidat); FIELD(ndatm);
  FIELD(nptot); FIELD(nbeta); FIELD(nseq); FIELD(nchi2m);
  FIELD(coor); FIELD(dat); FIELD(std2r); FIELD(icoor); FIELD(idat); FIELD(datm);
  FIELD(chi2m); FIELD(pcur); FIELD(flag); FIELD(chi2c);
  /* CMcmcFit */
  FIELD(nprm); FIELD(nadj); FIELD(npass); FIELD(nburn); FIELD(niter); FIELD(nrndst);
  FIELD(ipm); FIELD(itr); FIELD(seed); FIELD(ntitr);
  FIELD(rndst); FIELD(pdescr); FIELD(ivar); FIELD(invar); FIELD(ptotal); FIELD(pmint);
  FIELD(pmaxt); FIELD(pout); FIELD(tout); FIELD(chi2); FIELD(tcur); FIELD(n_acpt);
  FIELD(n_exch); FIELD(n_cnt); FIELD(n_hist); FIELD(pstp); FIELD(beta); FIELD(ptent);
  FIELD(ptentn);
  std::printf("\n  }\n}\n");
  return 0;
}
