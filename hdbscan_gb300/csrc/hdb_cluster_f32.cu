// float32 cluster forward variants: 512 Prim threads x 2 slots per CTA,
// 2 or 4 CTAs per window (up to 2048 / 4096 points), register dimensions
// 8/16/32 or the matrix variant.
#include "hdb_cluster_instances.cuh"

namespace hdb {
namespace {
const ForwardVariant kCluster[] = {
    cluster_variant<float, 512, 2, 8, 2>(),  cluster_variant<float, 512, 2, 16, 2>(),
    cluster_variant<float, 512, 2, 32, 2>(), cluster_variant<float, 512, 2, 0, 2>(),
    cluster_variant<float, 512, 2, 8, 4>(),  cluster_variant<float, 512, 2, 16, 4>(),
    cluster_variant<float, 512, 2, 32, 4>(), cluster_variant<float, 512, 2, 0, 4>(),
};
}  // namespace
const ForwardVariant* cluster_variants_f32(int* count) {
    *count = (int)(sizeof(kCluster) / sizeof(kCluster[0]));
    return kCluster;
}
}  // namespace hdb
