// Kernel launches with explicit launch attributes.  The priority travels as a
// per-launch attribute so that CUDA-graph capture keeps it in the kernel node
// (a stream's own priority is a property of the stream, not of the captured
// work); cluster kernels add their cluster shape the same way.
#pragma once
#include <utility>
#include <cuda_runtime.h>

namespace hdb {

template <typename... KArgs, typename... Args>
cudaError_t launch_ex(void (*kernel)(KArgs...), unsigned grid, unsigned block, size_t smem, cudaStream_t stream,
                      int priority, unsigned cluster, Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[2];
    unsigned count = 0;
    attr[count].id = cudaLaunchAttributePriority;
    attr[count].val.priority = priority;
    ++count;
    if (cluster > 1) {
        attr[count].id = cudaLaunchAttributeClusterDimension;
        attr[count].val.clusterDim.x = cluster;
        attr[count].val.clusterDim.y = 1;
        attr[count].val.clusterDim.z = 1;
        ++count;
    }
    cfg.attrs = attr;
    cfg.numAttrs = count;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

}  // namespace hdb
