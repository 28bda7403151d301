// lib_sgra.cu -- libcmc_sgra.so: the C-ABI with the built-in Sgr A* crescent
// + Gaussian model (the reference's examples/sgra_model_fit/model.cuh).
#include "cmc_host.cuh"
#include "model_sgra.cuh"

#define CMC_MODEL cmc::SgraModel
#define CMC_MODEL_NAME "sgra"
#include "cmc_abi.inc"
