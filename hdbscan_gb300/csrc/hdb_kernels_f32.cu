// float32 kernel variants.  Register budget: V*DP floats of coordinates per
// thread stay <= 32 at 1024 threads and <= 64 below.
#include "hdb_instances.cuh"

namespace hdb {
namespace {
const ForwardVariant kForward[] = {
    forward_variant<float, 128, 1, 8>(),  forward_variant<float, 128, 1, 16>(),
    forward_variant<float, 128, 1, 32>(), forward_variant<float, 128, 1, 0>(),
    forward_variant<float, 256, 1, 8>(),  forward_variant<float, 256, 1, 16>(),
    forward_variant<float, 256, 1, 32>(), forward_variant<float, 256, 1, 0>(),
    forward_variant<float, 512, 1, 8>(),  forward_variant<float, 512, 1, 16>(),
    forward_variant<float, 512, 1, 32>(), forward_variant<float, 512, 1, 0>(),
    forward_variant<float, 512, 2, 8>(),  forward_variant<float, 512, 2, 16>(),
    forward_variant<float, 512, 2, 32>(), forward_variant<float, 512, 2, 0>(),
    forward_variant<float, 1024, 2, 8>(), forward_variant<float, 1024, 2, 16>(),
    forward_variant<float, 1024, 2, 0>(),
    forward_variant<float, 1024, 4, 8>(), forward_variant<float, 1024, 4, 0>(),
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
const PrecisionKernels kTable = {
    4, kForward, (int)(sizeof(kForward) / sizeof(kForward[0])), kCore, (int)(sizeof(kCore) / sizeof(kCore[0])),
    launch_distance<float>, launch_select<float>, (const void*)hdb_core_select_kernel<float>,
    launch_backward<float>, forward_smem_dispatch<float>,
};
}  // namespace
const PrecisionKernels& kernels_f32() { return kTable; }
}  // namespace hdb
