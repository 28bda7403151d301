// inst_sgra.cu -- kernel instances of the built-in Sgr A* model for one
// replicas-per-CTA count R (compiled once per R with -DCMC_R=R): the cluster
// layout's sweep, batch and evaluation kernels for R = 1, 2, 4, 8 and the
// spread layout's sweep for every R of 1..8.
#define CMC_INSTANCE_TU 1
#include "model_sgra.cuh"
#include "cmc_launch_impl.cuh"

namespace cmc {
#if (CMC_R & (CMC_R - 1)) == 0
CMC_INSTANTIATE(SgraModel, CMC_R)
#endif
CMC_INSTANTIATE_SPREAD(SgraModel, CMC_R)
}
