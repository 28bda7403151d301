// inst_plugin.cu -- kernel instances of a model.cuh plugin for one
// replicas-per-CTA count R (compiled once per R with -DCMC_R=R and the same
// -DCMC_PLUGIN_FILE as lib_plugin.cu).
#define CMC_INSTANCE_TU 1
#include "plugin_prelude.cuh"
#include "cmc_launch_impl.cuh"

namespace cmc {
CMC_INSTANTIATE(PluginModel, CMC_R)
}
