// lib_plugin.cu -- libcmc_<name>.so: the C-ABI with a model.cuh plugin compiled
// in.  Build with -DCMC_PLUGIN_FILE='"path/to/model.cuh"' and
// -DCMC_PLUGIN_NAME='"name"', linked with the inst_plugin.cu objects.
#define CMC_PLUGIN_DECLARE_ONLY 1
#include "plugin_prelude.cuh"
#include "cmc_host.cuh"

#define CMC_MODEL cmc::PluginModel
#define CMC_MODEL_NAME CMC_PLUGIN_NAME
#include "cmc_abi.inc"
