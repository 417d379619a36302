// float32 kernel variants.  Register budget: SV*DP floats of coordinates per
// Prim thread stay <= 64.
#include "hdb_instances.cuh"

namespace hdb {
namespace {
const ForwardVariant kForward[] = {
    forward_variant<float, 32, 2, 8>(),
    forward_variant<float, 32, 2, 16>(),
    forward_variant<float, 32, 2, 32>(),
    forward_variant<float, 32, 2, 0>(),
    forward_variant<float, 64, 2, 8>(),
    forward_variant<float, 64, 2, 16>(),
    forward_variant<float, 64, 2, 32>(),
    forward_variant<float, 64, 2, 0>(),
    forward_variant<float, 128, 2, 8>(),
    forward_variant<float, 128, 2, 16>(),
    forward_variant<float, 128, 2, 32>(),
    forward_variant<float, 128, 2, 0>(),
    forward_variant<float, 256, 2, 8>(),
    forward_variant<float, 256, 2, 16>(),
    forward_variant<float, 256, 2, 32>(),
    forward_variant<float, 256, 2, 0>(),
    forward_variant<float, 512, 2, 8>(),
    forward_variant<float, 512, 2, 16>(),
    forward_variant<float, 512, 2, 32>(),
    forward_variant<float, 512, 2, 0>(),
    forward_variant<float, 512, 4, 8>(),
    forward_variant<float, 512, 4, 16>(),
    forward_variant<float, 512, 4, 0>(),
    forward_variant<float, 512, 8, 8>(),
    forward_variant<float, 512, 8, 0>(),
    // Two CTAs per SM.
    forward_variant<float, 256, 4, 8, 2>(),
    forward_variant<float, 256, 4, 16, 2>(),
    forward_variant<float, 128, 4, 8, 2>(),
    forward_variant<float, 128, 4, 16, 2>(),
    forward_variant<float, 128, 4, 32, 2>(),
};
const CoreVariant kCore[] = {
    core_points_variant<float, 8, 8>(),   core_points_variant<float, 8, 16>(),
    core_points_variant<float, 8, 32>(),  core_points_variant<float, 8, 64>(),
    core_points_variant<float, 16, 8>(),  core_points_variant<float, 16, 16>(),
    core_points_variant<float, 16, 32>(), core_points_variant<float, 16, 64>(),
    core_points_variant<float, 32, 8>(),  core_points_variant<float, 32, 16>(),
    core_points_variant<float, 32, 32>(), core_points_variant<float, 32, 64>(),
    core_points_variant<float, 64, 8>(),  core_points_variant<float, 64, 16>(),
    core_points_variant<float, 64, 32>(), core_points_variant<float, 64, 64>(),
    core_matrix_variant<float, 8>(),      core_matrix_variant<float, 16>(),
    core_matrix_variant<float, 32>(),     core_matrix_variant<float, 64>(),
};
}  // namespace
const PrecisionKernels& kernels_f32() {
    static const PrecisionKernels table = [] {
        PrecisionKernels t = {
            4, kForward, (int)(sizeof(kForward) / sizeof(kForward[0])), nullptr, 0, kCore,
            (int)(sizeof(kCore) / sizeof(kCore[0])), launch_distance<float>, launch_select<float>,
            (const void*)hdb_core_select_kernel<float>, launch_backward<float>, launch_prepare<float>,
            forward_layout<float>,
        };
        t.cluster = cluster_variants_f32(&t.n_cluster);
        return t;
    }();
    return table;
}
}  // namespace hdb
