// Explicit kernel variants and their host launchers, one table per precision
// (instantiated by hdb_kernels_f32.cu / hdb_kernels_f64.cu).
#pragma once
#include "hdb_backward.cuh"
#include "hdb_distance.cuh"
#include "hdb_forward.cuh"
#include "hdb_launch.h"
#include "hdb_prepare.cuh"
#include "hdb_registry.h"

namespace hdb {

template <typename Real>
bool forward_layout(int n, int dp, bool unit_core, size_t budget, int max_arenas, ForwardLayout* out);

template <typename Real, int THREADS, int V, int DP, int MINB>
cudaError_t launch_forward(const ForwardArgs& a, int grid, size_t smem, cudaStream_t s, int priority) {
    return launch_ex(hdb_forward_kernel<Real, THREADS, V, DP, MINB>, grid, THREADS + 32, smem, s, priority, 1, a);
}

// Several CTAs per SM keep one arena each: the other CTAs provide the overlap.
template <typename Real, int DP, int MINB>
bool single_layout(int n, bool unit_core, size_t budget, ForwardLayout* out) {
    return forward_layout<Real>(n, DP, unit_core, budget, MINB > 1 ? 1 : 2, out);
}

template <typename Real, int THREADS, int V, int DP, int MINB = 1>
constexpr ForwardVariant forward_variant() {
    return ForwardVariant{THREADS, V, DP, 1, MINB, (const void*)hdb_forward_kernel<Real, THREADS, V, DP, MINB>,
                          launch_forward<Real, THREADS, V, DP, MINB>, single_layout<Real, DP, MINB>};
}

template <typename Real, int K, int DP>
cudaError_t launch_core_points(const CoreArgs& a, int grid, cudaStream_t s, int priority) {
    return launch_ex(hdb_core_points_kernel<Real, K, DP>, grid, kCoreRows, 0, s, priority, 1, a);
}

template <typename Real, int K>
cudaError_t launch_core_matrix(const CoreArgs& a, int grid, cudaStream_t s, int priority) {
    return launch_ex(hdb_core_rows_kernel<Real, K>, grid, 32 * kCoreRowsWarps, 0, s, priority, 1, a);
}

template <typename Real, int K, int DP>
constexpr CoreVariant core_points_variant() {
    return CoreVariant{K, DP, kCoreRows, (const void*)hdb_core_points_kernel<Real, K, DP>, launch_core_points<Real, K, DP>};
}

template <typename Real, int K>
constexpr CoreVariant core_matrix_variant() {
    return CoreVariant{K, 0, kCoreMatrixRows, (const void*)hdb_core_rows_kernel<Real, K>, launch_core_matrix<Real, K>};
}

template <typename Real>
cudaError_t launch_distance(const DistanceArgs& a, int grid, cudaStream_t s, int priority) {
    if constexpr (sizeof(Real) == 4) {
        if (a.tile == kDistTile128) return launch_ex(hdb_distance128_kernel<float>, grid, 256, 0, s, priority, 1, a);
    }
    return launch_ex(hdb_distance_kernel<Real>, grid, 256, 0, s, priority, 1, a);
}

template <typename Real>
cudaError_t launch_select(const CoreArgs& a, int grid, size_t smem, cudaStream_t s, int priority) {
    return launch_ex(hdb_core_select_kernel<Real>, grid, 256, smem, s, priority, 1, a);
}

template <typename Real>
cudaError_t launch_prepare(const void* X, int input_type, void* out, int64_t points, int D, int normalize,
                           cudaStream_t s, int priority) {
    const unsigned grid = (unsigned)((points + 255) / 256);
    Real* y = static_cast<Real*>(out);
    if (input_type == kInputBF16)
        return launch_ex(hdb_prepare_kernel<Real, __nv_bfloat16>, grid, 256, 0, s, priority, 1,
                         static_cast<const __nv_bfloat16*>(X), y, points, D, normalize);
    if (input_type == kInputF16)
        return launch_ex(hdb_prepare_kernel<Real, __half>, grid, 256, 0, s, priority, 1, static_cast<const __half*>(X), y,
                         points, D, normalize);
    return launch_ex(hdb_prepare_kernel<Real, Real>, grid, 256, 0, s, priority, 1, static_cast<const Real*>(X), y,
                     points, D, normalize);
}

template <typename Real>
cudaError_t launch_backward(const BackwardArgs& a, int grid, cudaStream_t s, int priority) {
    return launch_ex(hdb_backward_kernel<Real>, grid, 32 * kBackwardWarps, 0, s, priority, 1, a);
}

// Two arenas (Prim/tree overlap) when they fit next to the staged window,
// else one arena with the staged window, else one arena alone.
template <typename Real>
bool forward_layout(int n, int dp, bool unit_core, size_t budget, int max_arenas, ForwardLayout* out) {
    const size_t arena = (Arena<Real>::bytes(n) + 127) & ~size_t(127);
    const size_t x = dp > 0 ? (((size_t)n * dp * sizeof(Real) + 127) & ~size_t(127)) : 0;
    const size_t core = unit_core ? 0 : (((size_t)Arena<Real>::round_cap(n) * sizeof(Real) + 127) & ~size_t(127));
    const int nbs[3] = {2, 1, 1};
    const int xss[3] = {1, 1, 0};
    for (int c = 0; c < 3; ++c) {
        if (nbs[c] > max_arenas) continue;
        const int xs = dp > 0 ? xss[c] : 0;
        const size_t bytes = nbs[c] * arena + (xs ? x : 0) + core;
        if (bytes <= budget) {
            out->n_arenas = nbs[c];
            out->x_in_smem = xs;
            out->arena_stride = arena;
            out->x_off = nbs[c] * arena;
            out->core_off = out->x_off + (xs ? x : 0);
            out->bytes = bytes;
            return true;
        }
    }
    return false;
}

}  // namespace hdb
