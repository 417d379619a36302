// Host-side registry of the compiled kernel variants (one table per precision).
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>
#include <cuda_runtime.h>

#include "hdb_args.h"

namespace hdb {

// Dynamic shared-memory layout of one forward launch.
struct ForwardLayout {
    int n_arenas;
    int x_in_smem;
    size_t arena_stride;
    size_t x_off;
    size_t core_off;
    size_t bytes;
};

struct ForwardVariant {
    int threads;  // Prim threads; the CTA has threads + 32 (one tree warp)
    int v;        // vertices (slots) per Prim thread
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
    // Best layout for windows of up to n points within `budget` bytes; false if none fits.
    bool (*forward_layout)(int n, int dp, bool unit_core, size_t budget, ForwardLayout* out);
};

const PrecisionKernels& kernels_f32();
const PrecisionKernels& kernels_f64();

// Raise (never lower) a kernel's dynamic shared-memory limit; thread-safe.
cudaError_t raise_dynamic_smem(const void* func, size_t bytes);

// Message returned by hdb_last_error() on the calling thread.
void set_last_error(const char* message);
inline void set_last_error(const std::string& message) { set_last_error(message.c_str()); }

}  // namespace hdb
