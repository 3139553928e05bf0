// Kernel launches with programmatic stream serialization (programmatic
// dependent launch): the kernel may be scheduled while the previous kernel in
// the stream finishes, and waits in JC_PDL_ENTRY (common.cuh) before touching
// shared data. In a captured graph the dependency becomes a programmatic
// edge. JC_PDL=0 in the environment launches without the attribute.
#pragma once

#include <cuda_runtime.h>

#include <cstdlib>
#include <cstring>
#include <utility>

namespace jc {

inline bool pdl_enabled() {
    static const bool on = [] {
        const char* e = std::getenv("JC_PDL");
        return !(e && std::strcmp(e, "0") == 0);
    }();
    return on;
}

// Launches kernel<<<grid, block, smem, s>>>(args...) with the attribute and,
// when cluster > 1, a 1-D cluster of that many CTAs.
template <class... KArgs, class... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, unsigned cluster,
                       Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[2];
    unsigned n = 0;
    if (pdl_enabled()) {
        at[n].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[n].val.programmaticStreamSerializationAllowed = 1;
        n++;
    }
    if (cluster > 1) {
        at[n].id = cudaLaunchAttributeClusterDimension;
        at[n].val.clusterDim.x = cluster;
        at[n].val.clusterDim.y = 1;
        at[n].val.clusterDim.z = 1;
        n++;
    }
    cfg.attrs = at;
    cfg.numAttrs = n;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

}  // namespace jc
