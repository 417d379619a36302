// Host-side registry of the compiled kernel variants (one table per precision).
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>
#include <cuda_runtime.h>

#include "hdb_args.h"

namespace hdb {

// Every launcher takes the launch priority (numerically as stream priorities).
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
    int cluster;  // CTAs per window (1 = hdb_forward_kernel, else a cluster of hdb_cluster_forward_kernel)
    int per_sm;   // CTAs per SM the variant is built for (launch bounds, shared-memory budget)
    const void* func;
    cudaError_t (*launch)(const ForwardArgs&, int grid, size_t smem, cudaStream_t, int priority);
    // Shared-memory layout for windows of up to n points within `budget` bytes; false if none fits.
    bool (*layout)(int n, bool unit_core, size_t budget, ForwardLayout* out);
};

struct CoreVariant {
    int k;        // list length (max ms)
    int dp;       // padded register dimensions; 0 = matrix variant
    int rows;     // rows per CTA (work items start every `rows` rows)
    const void* func;
    cudaError_t (*launch)(const CoreArgs&, int grid, cudaStream_t, int priority);
};

struct PrecisionKernels {
    int real_bytes;
    const ForwardVariant* forward;   // single-CTA variants
    int n_forward;
    const ForwardVariant* cluster;   // cluster variants (windows above 1024 points)
    int n_cluster;
    const CoreVariant* core;
    int n_core;
    cudaError_t (*launch_distance)(const DistanceArgs&, int grid, cudaStream_t, int priority);
    cudaError_t (*launch_select)(const CoreArgs&, int grid, size_t smem, cudaStream_t, int priority);
    const void* select_func;
    cudaError_t (*launch_backward)(const BackwardArgs&, int grid, cudaStream_t, int priority);
    // Producer stage: input (compute type / bfloat16 / float16) -> compute type, optionally L2-normalised.
    cudaError_t (*launch_prepare)(const void* X, int input_type, void* out, int64_t points, int D, int normalize,
                                  cudaStream_t, int priority);
    // Best single-CTA layout (at most max_arenas arenas) for windows of up to n
    // points within `budget` bytes; false if none fits.
    bool (*forward_layout)(int n, int dp, bool unit_core, size_t budget, int max_arenas, ForwardLayout* out);
};

const PrecisionKernels& kernels_f32();
const PrecisionKernels& kernels_f64();
// Cluster variants, compiled in their own translation units.
const ForwardVariant* cluster_variants_f32(int* count);
const ForwardVariant* cluster_variants_f64(int* count);

// Raise (never lower) a kernel's dynamic shared-memory limit; thread-safe.
cudaError_t raise_dynamic_smem(const void* func, size_t bytes);

// Message returned by hdb_last_error() on the calling thread.
void set_last_error(const char* message);
inline void set_last_error(const std::string& message) { set_last_error(message.c_str()); }

}  // namespace hdb
