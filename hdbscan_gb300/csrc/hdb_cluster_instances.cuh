// Cluster forward variants and their host launchers (instantiated by
// hdb_cluster_f32.cu / hdb_cluster_f64.cu).
#pragma once
#include "hdb_cluster.cuh"
#include "hdb_launch.h"
#include "hdb_registry.h"

namespace hdb {

template <typename Real, int PT, int SV, int DP, int CS>
cudaError_t launch_cluster_forward(const ForwardArgs& a, int grid, size_t smem, cudaStream_t s, int priority) {
    return launch_ex(hdb_cluster_forward_kernel<Real, PT, SV, DP, CS>, grid, PT + 32, smem, s, priority, CS, a);
}

// One arena, the record buffers ([2][CS] plus the vertex-0 record) and the
// compaction staging of PT*SV slots.
template <typename Real, int PT, int SV, int DP, int CS>
bool cluster_layout(int n, bool /*unit_core*/, size_t budget, ForwardLayout* out) {
    if (n > CS * PT * SV) return false;
    const size_t arena = (Arena<Real>::bytes(n) + 127) & ~size_t(127);
    constexpr size_t rec = (size_t)Record<Real, DP>::kBytes;
    const size_t recs = 2 * CS * rec + ((rec + 15) & ~size_t(15));
    const size_t stage = (size_t)PT * SV * (sizeof(Real) + 2 * sizeof(int16_t));
    const size_t bytes = arena + recs + stage;
    if (bytes > budget) return false;
    out->n_arenas = 1;
    out->x_in_smem = 0;
    out->arena_stride = arena;
    out->x_off = arena;
    out->core_off = arena;
    out->bytes = bytes;
    return true;
}

template <typename Real, int PT, int SV, int DP, int CS>
constexpr ForwardVariant cluster_variant() {
    return ForwardVariant{PT, SV, DP, CS, 1, (const void*)hdb_cluster_forward_kernel<Real, PT, SV, DP, CS>,
                          launch_cluster_forward<Real, PT, SV, DP, CS>, cluster_layout<Real, PT, SV, DP, CS>};
}

}  // namespace hdb
