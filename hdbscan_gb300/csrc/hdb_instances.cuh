// Explicit kernel variants and their host launchers, one table per precision
// (instantiated by hdb_kernels_f32.cu / hdb_kernels_f64.cu).
#pragma once
#include "hdb_backward.cuh"
#include "hdb_distance.cuh"
#include "hdb_forward.cuh"
#include "hdb_registry.h"

namespace hdb {

template <typename Real, int THREADS, int V, int DP>
void launch_forward(const ForwardArgs& a, int grid, size_t smem, cudaStream_t s) {
    hdb_forward_kernel<Real, THREADS, V, DP><<<grid, THREADS, smem, s>>>(a);
}

template <typename Real, int THREADS, int V, int DP>
constexpr ForwardVariant forward_variant() {
    return ForwardVariant{THREADS, V, DP, (const void*)hdb_forward_kernel<Real, THREADS, V, DP>,
                          launch_forward<Real, THREADS, V, DP>};
}

template <typename Real, int K, int DP>
void launch_core_points(const CoreArgs& a, int grid, cudaStream_t s) {
    hdb_core_points_kernel<Real, K, DP><<<grid, kCoreRows, 0, s>>>(a);
}

template <typename Real, int K>
void launch_core_matrix(const CoreArgs& a, int grid, cudaStream_t s) {
    hdb_core_matrix_kernel<Real, K><<<grid, kCoreRows, 0, s>>>(a);
}

template <typename Real, int K, int DP>
constexpr CoreVariant core_points_variant() {
    return CoreVariant{K, DP, (const void*)hdb_core_points_kernel<Real, K, DP>, launch_core_points<Real, K, DP>};
}

template <typename Real, int K>
constexpr CoreVariant core_matrix_variant() {
    return CoreVariant{K, 0, (const void*)hdb_core_matrix_kernel<Real, K>, launch_core_matrix<Real, K>};
}

template <typename Real>
void launch_distance(const DistanceArgs& a, int grid, cudaStream_t s) {
    hdb_distance_kernel<Real><<<grid, 256, 0, s>>>(a);
}

template <typename Real>
void launch_select(const CoreArgs& a, int grid, size_t smem, cudaStream_t s) {
    hdb_core_select_kernel<Real><<<grid, 256, smem, s>>>(a);
}

template <typename Real>
void launch_backward(const BackwardArgs& a, int grid, cudaStream_t s) {
    hdb_backward_kernel<Real><<<grid, 256, 0, s>>>(a);
}

template <typename Real>
size_t forward_smem_dispatch(int n, int dp, bool x_in_smem, bool unit_core) {
    size_t bytes = Arena<Real>::bytes(n);
    bytes = (bytes + 15) & ~size_t(15);
    if (x_in_smem && dp > 0) bytes += (size_t)n * dp * sizeof(Real);
    if (!unit_core) bytes += (size_t)Arena<Real>::round_cap(n) * sizeof(Real);
    return bytes;
}

}  // namespace hdb
