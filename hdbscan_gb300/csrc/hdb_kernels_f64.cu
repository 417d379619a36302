// float64 kernel variants.  Register budget: SV*DP doubles of coordinates per
// Prim thread stay <= 32 (64 registers).
#include "hdb_instances.cuh"

namespace hdb {
namespace {
const ForwardVariant kForward[] = {
    forward_variant<double, 32, 2, 8>(),
    forward_variant<double, 32, 2, 16>(),
    forward_variant<double, 32, 2, 0>(),
    forward_variant<double, 64, 2, 8>(),
    forward_variant<double, 64, 2, 16>(),
    forward_variant<double, 64, 2, 0>(),
    forward_variant<double, 128, 2, 8>(),
    forward_variant<double, 128, 2, 16>(),
    forward_variant<double, 128, 2, 0>(),
    forward_variant<double, 256, 2, 8>(),
    forward_variant<double, 256, 2, 16>(),
    forward_variant<double, 256, 2, 0>(),
    forward_variant<double, 512, 2, 8>(),
    forward_variant<double, 512, 2, 16>(),
    forward_variant<double, 512, 2, 0>(),
    forward_variant<double, 512, 4, 8>(),
    forward_variant<double, 512, 4, 0>(),
    forward_variant<double, 512, 8, 0>(),
};
const CoreVariant kCore[] = {
    core_points_variant<double, 8, 8>(),   core_points_variant<double, 8, 16>(),
    core_points_variant<double, 8, 32>(),
    core_points_variant<double, 16, 8>(),  core_points_variant<double, 16, 16>(),
    core_points_variant<double, 16, 32>(),
    core_points_variant<double, 32, 8>(),  core_points_variant<double, 32, 16>(),
    core_points_variant<double, 32, 32>(),
    core_points_variant<double, 64, 8>(),  core_points_variant<double, 64, 16>(),
    core_points_variant<double, 64, 32>(),
    core_matrix_variant<double, 8>(),      core_matrix_variant<double, 16>(),
    core_matrix_variant<double, 32>(),     core_matrix_variant<double, 64>(),
};
}  // namespace
const PrecisionKernels& kernels_f64() {
    static const PrecisionKernels table = [] {
        PrecisionKernels t = {
            8, kForward, (int)(sizeof(kForward) / sizeof(kForward[0])), nullptr, 0, kCore,
            (int)(sizeof(kCore) / sizeof(kCore[0])), launch_distance<double>, launch_select<double>,
            (const void*)hdb_core_select_kernel<double>, launch_backward<double>, launch_prepare<double>,
            forward_layout<double>,
        };
        t.cluster = cluster_variants_f64(&t.n_cluster);
        return t;
    }();
    return table;
}
}  // namespace hdb
