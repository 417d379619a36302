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

// One thread per linkage row.
template <typename Real>
__global__ void __launch_bounds__(256) hdb_backward_kernel(const BackwardArgs args) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= args.n_edges) return;
    const int w = args.edge_window[r];
    const int64_t base = args.offsets[w];
    const int64_t ebase = base - w;
    const int D = args.D;
    const Real* X = static_cast<const Real*>(args.X);
    const Real g = static_cast<const Real*>(args.grad)[r];
    if (g == Real(0)) return;
    const Real wgt = static_cast<const Real*>(args.link_w)[r];
    const int e = args.order[r];
    const int u = args.edges_uv[2 * (ebase + e)], v = args.edges_uv[2 * (ebase + e) + 1];
    int a = u, b = v;
    const Real duv = exact_distance<Real>(X + (base + u) * D, X + (base + v) * D, D);
    if (!args.unit_core && !(duv == wgt)) {
        const Real* core = static_cast<const Real*>(args.core);
        if (core[base + u] == wgt) { a = u; b = args.core_nbr[base + u]; }
        else if (core[base + v] == wgt) { a = v; b = args.core_nbr[base + v]; }
    }
    if (b < 0 || a == b) return;
    const Real* xa = X + (base + a) * D;
    const Real* xb = X + (base + b) * D;
    const Real d = (a == u && b == v) ? duv : exact_distance<Real>(xa, xb, D);
    if (!(d > Real(0))) return;
    const Real scale = g / d;
    Real* dX = static_cast<Real*>(args.dX);
    for (int k = 0; k < D; ++k) {
        const Real c = scale * (xa[k] - xb[k]);
        atomicAdd(dX + (base + a) * D + k, c);
        atomicAdd(dX + (base + b) * D + k, -c);
    }
}

}  // namespace hdb
