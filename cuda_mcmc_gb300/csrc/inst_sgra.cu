// inst_sgra.cu -- kernel instances of the built-in Sgr A* model for one
// replicas-per-CTA count R (compiled once per R with -DCMC_R=R).
#define CMC_INSTANCE_TU 1
#include "model_sgra.cuh"
#include "cmc_launch_impl.cuh"

namespace cmc {
CMC_INSTANTIATE(SgraModel, CMC_R)
}
