// float64 cluster forward variants: 512 Prim threads x 2 slots per CTA,
// 2 or 4 CTAs per window, register dimensions 8/16 or the matrix variant.
#include "hdb_cluster_instances.cuh"

namespace hdb {
namespace {
const ForwardVariant kCluster[] = {
    cluster_variant<double, 512, 2, 8, 2>(), cluster_variant<double, 512, 2, 16, 2>(),
    cluster_variant<double, 512, 2, 0, 2>(), cluster_variant<double, 512, 2, 8, 4>(),
    cluster_variant<double, 512, 2, 16, 4>(), cluster_variant<double, 512, 2, 0, 4>(),
};
}  // namespace
const ForwardVariant* cluster_variants_f64(int* count) {
    *count = (int)(sizeof(kCluster) / sizeof(kCluster[0]));
    return kCluster;
}
}  // namespace hdb
