// Backward of the linkage merge weights with respect to the input points.
//
// The reference has no gradients (hdbscan_gpu README: "no gradients"); this
// kernel has no reference counterpart.  The discrete structure (MST edges,
// sort order, core neighbours) is held fixed.  Merge weight i of a window is
// w = max(core_u, core_v, d_uv) for the i-th sorted MST edge (u, v).  The
// gradient follows the term that attains the maximum, distance first:
//   d_uv == w              -> pair (u, v)
//   else core_u == w       -> pair (u, nbr_u)   (nbr = ms-th nearest neighbour)
//   else core_v == w       -> pair (v, nbr_v)
// and for the chosen pair (a, b) with d_ab > 0:
//   dX[a] += g (x_a - x_b) / d_ab,  dX[b] -= g (x_a - x_b) / d_ab.
// d_uv is recomputed with the forward's exact arithmetic (k-order sum, no FMA,
// correctly rounded sqrt) so the equality tests see the forward's bits; the
// dense distance buffer is never kept.
#pragma once
#include "hdb_common.cuh"

namespace hdb {


template <typename Real>
__device__ __forceinline__ Real exact_distance(const Real* xa, const Real* xb, int D) {
    using T = RealTraits<Real>;
    Real acc = Real(0);
    for (int k = 0; k < D; ++k) {
        const Real delta = T::sub(xa[k], xb[k]);
        acc = T::add(acc, T::mul(delta, delta));
    }
    return T::sqrt_rn(acc);
}

// Each warp takes 32 consecutive linkage rows.  First every lane decides the
// pair of its own row: the chosen pair's distance is the merge weight itself
// (the distance term, or the core distance, which is the distance to the core
// neighbour computed with the same arithmetic), so the exact distance d_uv is
// recomputed only when a core distance ties the weight and the
// distance-first rule needs to know whether d_uv ties it too.  Then the warp
// scatters the rows one after another with the lanes over the coordinates:
// the terms g (x_a - x_b) / w are independent per coordinate, so the loads of
// x_a and x_b and the atomics on dX are coalesced.
template <typename Real>
__global__ void __launch_bounds__(32 * kBackwardWarps) hdb_backward_kernel(const BackwardArgs args) {
    const int lane = threadIdx.x & 31;
    const int first = (blockIdx.x * kBackwardWarps + (threadIdx.x >> 5)) * 32;
    if (first >= args.n_edges) return;  // warp-uniform
    const int r = first + lane;
    const int D = args.D;
    const Real* X = static_cast<const Real*>(args.X);
    int64_t row_a = -1, row_b = -1;  // global point rows of the pair, -1 = no gradient
    Real scale = Real(0);
    if (r < args.n_edges) {
        const Real g = static_cast<const Real*>(args.grad)[r];
        const Real wgt = static_cast<const Real*>(args.link_w)[r];
        if (g != Real(0) && wgt > Real(0)) {
            const int w = args.edge_window[r];
            const int64_t base = args.offsets[w];
            const int64_t ebase = base - w;
            const int e = args.order[r];
            const int u = args.edges_uv[2 * (ebase + e)], v = args.edges_uv[2 * (ebase + e) + 1];
            int a = u, b = v;
            if (!args.unit_core) {
                const Real* core = static_cast<const Real*>(args.core);
                const Real cu = core[base + u], cv = core[base + v];
                if ((cu == wgt || cv == wgt) &&
                    !(exact_distance<Real>(X + (base + u) * D, X + (base + v) * D, D) == wgt)) {
                    if (cu == wgt) { a = u; b = args.core_nbr[base + u]; }
                    else { a = v; b = args.core_nbr[base + v]; }
                }
            }
            if (b >= 0 && a != b) {
                row_a = base + a;
                row_b = base + b;
                scale = g / wgt;
            }
        }
    }
    Real* dX = static_cast<Real*>(args.dX);
    for (int t = 0; t < 32; ++t) {
        const int64_t ra = __shfl_sync(0xffffffffu, row_a, t);
        if (ra < 0) continue;  // warp-uniform
        const int64_t rb = __shfl_sync(0xffffffffu, row_b, t);
        const Real sc = __shfl_sync(0xffffffffu, scale, t);
        const Real* xa = X + ra * D;
        const Real* xb = X + rb * D;
        for (int k = lane; k < D; k += 32) {
            const Real c = sc * (xa[k] - xb[k]);
            atomicAdd(dX + ra * D + k, c);
            atomicAdd(dX + rb * D + k, -c);
        }
    }
}

}  // namespace hdb
