// CUDACONV::RunConfig -- the reference's runtime configuration
// (src/GpuConvolver/cuda/cudaConv2.h:13-26), layout-compatible with
// pisco_run_config of the C ABI.
#ifndef PISCO_CUDACONV2_H
#define PISCO_CUDACONV2_H

#include <stddef.h>

#include "../../../pisco_gb300.h"

namespace CUDACONV {
struct CUDACONVConf_t {
    int nStreams;
    size_t maxMemUsage;
    int deviceId;
    int gridSizeX;
    int gridSizeY;
    int blockSizeX;
    int blockSizeY;
    int ptgPerConv;
    int pixelsPerDisc;
};
typedef struct CUDACONVConf_t RunConfig;
static_assert(sizeof(RunConfig) == sizeof(pisco_run_config), "RunConfig layout");
}  // namespace CUDACONV

#endif
