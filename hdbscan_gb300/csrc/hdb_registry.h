// Host-side registry of the compiled kernel variants (one table per precision).
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>
#include <cuda_runtime.h>

#include "hdb_args.h"

namespace hdb {

struct ForwardVariant {
    int threads;
    int v;        // vertices per thread
    int dp;       // padded register dimensions; 0 = matrix variant
    const void* func;
    void (*launch)(const ForwardArgs&, int grid, size_t smem, cudaStream_t);
};

struct CoreVariant {
    int k;        // list length (max ms)
    int dp;       // padded register dimensions; 0 = matrix variant
    const void* func;
    void (*launch)(const CoreArgs&, int grid, cudaStream_t);
};

struct PrecisionKernels {
    int real_bytes;
    const ForwardVariant* forward;
    int n_forward;
    const CoreVariant* core;
    int n_core;
    void (*launch_distance)(const DistanceArgs&, int grid, cudaStream_t);
    void (*launch_select)(const CoreArgs&, int grid, size_t smem, cudaStream_t);
    const void* select_func;
    void (*launch_backward)(const BackwardArgs&, int grid, cudaStream_t);
    size_t (*forward_smem)(int n, int dp, bool x_in_smem, bool unit_core);
};

const PrecisionKernels& kernels_f32();
const PrecisionKernels& kernels_f64();

// Raise (never lower) a kernel's dynamic shared-memory limit; thread-safe.
cudaError_t raise_dynamic_smem(const void* func, size_t bytes);

// Message returned by hdb_last_error() on the calling thread.
void set_last_error(const char* message);
inline void set_last_error(const std::string& message) { set_last_error(message.c_str()); }

}  // namespace hdb
