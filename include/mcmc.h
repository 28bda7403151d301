/*
 * mcmc.h -- the reference's header name for its three entry points.
 *
 * Code written against the reference (MITHaystack/cuda_mcmc) includes
 * "mcmc.h" (src/mcmc.h:1-39), e.g. its Cython bridge src/mcmc_interf.pyx
 * (`cdef extern from "mcmc.h"`, :213, :285, :318).  With this directory on
 * the include path, that code compiles unchanged against this library's
 * declarations (identical signatures) and links against libcmc_<model>.so.
 */
#ifndef CMC_REFERENCE_MCMC_H
#define CMC_REFERENCE_MCMC_H
#include "cuda_mcmc.h"
#endif
