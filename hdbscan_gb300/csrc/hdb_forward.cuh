// Fused per-window forward kernel: Prim MST over the mutual-reachability
// graph (distances recomputed on chip, never written to HBM) followed by the
// hierarchy stages of hdb_tree.cuh, persistent over a size-sorted work queue.
//
// Reference path replaced: hdbscan_gpu/_cuda.py:110-127 (dense distance
// buffer + cluster kernel) and hdbscan_gpu/_kernels.py:164-760.
//
// Prim (reference _kernels.py:164-320, register variant :194-209):
//  * each thread owns V vertices j = tid + v*THREADS with their coordinates
//    (padded to DP, zero padding is exact) in registers, best weight, source
//    and an in-tree bit;
//  * per iteration the current vertex's coordinates come from the window
//    staged in shared memory (or from global memory for large windows);
//  * DP == 0 selects the matrix variant instead: weights come from row
//    `current` of a materialized distance matrix (hdb_distance.cuh), read
//    coalesced, exactly as the reference reads distances[current*n + j];
//  * strict '<' update keeps the older source on equal weights;
//  * argmin by (weight, vertex index) with redux.sync in every warp, warp
//    winners double-buffered in shared memory, ONE __syncthreads per
//    iteration, and every warp re-reduces the warp winners so the next
//    vertex is known without a second barrier;
//  * the owner of the winning vertex writes the edge (source, vertex, weight).
#pragma once
#include "hdb_common.cuh"
#include "hdb_tree.cuh"

namespace hdb {


template <typename Real, int DP>
__host__ __device__ constexpr int stage_stride() { return DP > 0 ? DP : 1; }

// Bytes of dynamic shared memory for a window of n points.
template <typename Real, int DP>
__host__ __device__ inline size_t forward_smem_bytes(int n, bool x_in_smem, bool unit_core) {
    size_t bytes = Arena<Real>::bytes(n);
    bytes = (bytes + 15) & ~size_t(15);
    if (x_in_smem && DP > 0) bytes += (size_t)n * DP * sizeof(Real);
    if (!unit_core) bytes += (size_t)Arena<Real>::round_cap(n) * sizeof(Real);
    return bytes;
}

template <typename Real, int THREADS, int V, int DP>
__global__ void __launch_bounds__(THREADS) hdb_forward_kernel(const ForwardArgs args) {
    using T = RealTraits<Real>;
    using Key = typename T::Bits;
    constexpr int NW = THREADS / 32;
    constexpr int VEC = 16 / (int)sizeof(Real);
    static_assert(DP % VEC == 0, "DP must be a multiple of one 16-byte vector");
    constexpr Key SENTINEL = (Key)~(Key)0;
    constexpr int DPS = DP > 0 ? DP : 1;  // stride of the staged window

    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ Key s_key[2][NW];
    __shared__ uint32_t s_idx[2][NW];
    __shared__ int s_item;
    __shared__ int s_counter;
    __shared__ int s_next_label;

    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int warp = tid >> 5;
    const Real* __restrict__ X = static_cast<const Real*>(args.X);
    const Real* __restrict__ core_g = static_cast<const Real*>(args.core);
    const int D = args.D;
    const Real epsilon = (Real)args.eps;  // the reference casts options to Real (_cuda.py:105)

    for (int guard = 0; guard < (1 << 30); ++guard) {
        if (tid == 0) s_item = atomicAdd(args.ticket, 1);
        __syncthreads();
        const int item = s_item;
        if (item >= args.queue_len) return;
        const int w = args.queue[item];
        const int64_t base = args.offsets[w];
        const int n = (int)(args.offsets[w + 1] - base);
        const Real* __restrict__ Xw = X + base * D;
        const Real* __restrict__ Dw = DP > 0 ? nullptr : static_cast<const Real*>(args.dist) + args.dist_offsets[w];

        // ---- shared-memory carve-up ------------------------------------
        Arena<Real> arena = Arena<Real>::carve(smem, n);
        size_t off = (Arena<Real>::bytes(n) + 15) & ~size_t(15);
        Real* s_x = nullptr;
        const bool xs = DP > 0 && args.x_in_smem;
        if (xs) { s_x = reinterpret_cast<Real*>(smem + off); off += (size_t)n * DP * sizeof(Real); }
        Real* s_core = nullptr;
        if (!args.unit_core) s_core = reinterpret_cast<Real*>(smem + off);

        // ---- stage coordinates / cores, validate input ------------------
        int bad = 0;
        if (xs) {
            for (int t = tid; t < n * DPS; t += THREADS) {
                const int j = t / DPS, k = t - j * DPS;
                Real v = Real(0);
                if (k < D) { v = Xw[(int64_t)j * D + k]; bad |= !isfinite(v); }
                s_x[t] = v;
            }
        } else {
            for (int t = tid; t < n * D; t += THREADS) bad |= !isfinite(Xw[t]);
        }
        if (!args.unit_core)
            for (int j = tid; j < n; j += THREADS) s_core[j] = core_g[base + j];
        if (__syncthreads_or(bad)) {
            if (tid == 0) atomic_status(args.status, kNonFinite);
            for (int j = tid; j < n; j += THREADS) args.labels[base + j] = -1;
            continue;
        }

        Real xr[V][DP > 0 ? DP : 1];
        Real best[V];
        Real core_r[V];
        int src[V];
        uint32_t in_tree = 0;
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const int j = tid + v * THREADS;
            best[v] = T::inf();
            src[v] = 1;  // reference initial source (_kernels.py:167)
            core_r[v] = Real(0);
            if (DP > 0) {
#pragma unroll
                for (int k = 0; k < (DP > 0 ? DP : 1); ++k) {
                    Real value = Real(0);
                    if (j < n) value = xs ? s_x[j * DPS + k] : (k < D ? Xw[(int64_t)j * D + k] : Real(0));
                    xr[v][k] = value;
                }
            }
            if (!args.unit_core && j < n) core_r[v] = s_core[j];
        }
        if (tid == 0) in_tree = 1u;  // vertex 0 starts the tree (_kernels.py:210-213)

        // ---- Prim -------------------------------------------------------
        int cur = 0;
        int overflow = 0;
        for (int it = 0; it < n - 1; ++it) {
            const Real core_cur = args.unit_core ? Real(0) : s_core[cur];
            Real acc[V];
#pragma unroll
            for (int v = 0; v < V; ++v) acc[v] = Real(0);
            if (DP > 0) {
#pragma unroll
                for (int k0 = 0; k0 < (DP > 0 ? DP : VEC); k0 += VEC) {
                    Real c[VEC];
                    if (xs) {
                        if constexpr (sizeof(Real) == 4) {
                            const float4 q = *reinterpret_cast<const float4*>(s_x + cur * DPS + k0);
                            c[0] = q.x; c[1] = q.y; c[2 % VEC] = q.z; c[3 % VEC] = q.w;
                        } else {
                            const double2 q = *reinterpret_cast<const double2*>(s_x + cur * DPS + k0);
                            c[0] = q.x; c[1 % VEC] = q.y;
                        }
                    } else {
#pragma unroll
                        for (int kk = 0; kk < VEC; ++kk)
                            c[kk] = (k0 + kk < D) ? Xw[(int64_t)cur * D + k0 + kk] : Real(0);
                    }
#pragma unroll
                    for (int v = 0; v < V; ++v) {
#pragma unroll
                        for (int kk = 0; kk < VEC; ++kk) {
                            const Real delta = T::sub(c[kk], xr[v][(k0 + kk) % (DP > 0 ? DP : 1)]);
                            acc[v] = T::add(acc[v], T::mul(delta, delta));
                        }
                    }
                }
            } else {
                // Matrix variant: row `cur` of the window's distance block.
                const Real* __restrict__ row = Dw + (int64_t)cur * (int64_t)((n + 3) & ~3);  // padded stride
#pragma unroll
                for (int v = 0; v < V; ++v) {
                    const int j = tid + v * THREADS;
                    if (j < n && !((in_tree >> v) & 1u)) acc[v] = __ldcg(row + j);
                }
            }
            Key lkey = SENTINEL;
            uint32_t lidx = 0xffffffffu;
#pragma unroll
            for (int v = 0; v < V; ++v) {
                const int j = tid + v * THREADS;
                if (j < n && !((in_tree >> v) & 1u)) {
                    const Real d = DP > 0 ? T::sqrt_rn(acc[v]) : acc[v];
                    overflow |= !(d <= T::kMax);
                    const Real wgt = args.unit_core ? d : T::maxr(T::maxr(core_cur, core_r[v]), d);
                    if (wgt < best[v]) { best[v] = wgt; src[v] = cur; }
                    const Key k = T::key(best[v]);
                    if (k < lkey) { lkey = k; lidx = (uint32_t)j; }
                }
            }
            warp_argmin(lkey, lidx);
            const int buf = it & 1;
            if (lane == 0) { s_key[buf][warp] = lkey; s_idx[buf][warp] = lidx; }
            __syncthreads();
            Key gk = lane < NW ? s_key[buf][lane] : SENTINEL;
            uint32_t gi = lane < NW ? s_idx[buf][lane] : 0xffffffffu;
            warp_argmin(gk, gi);
            const int next = (int)gi;
            // Owner of the winner records the edge and joins the tree.
            if ((next % THREADS) == tid) {
                const int v = next / THREADS;
#pragma unroll
                for (int vv = 0; vv < V; ++vv) {
                    if (vv == v) {
                        arena.s0[it] = (int16_t)src[vv];
                        arena.s1[it] = (int16_t)next;
                        arena.r0[it] = best[vv];
                        in_tree |= 1u << vv;
                    }
                }
            }
            if (next < 0 || next >= n) {  // unreachable: one non-tree vertex always remains
                overflow |= 2;
                break;
            }
            cur = next;
        }
        if (__syncthreads_or(overflow)) {
            if (tid == 0) atomic_status(args.status, (overflow & 2) ? kInternal : kOverflow);
            for (int j = tid; j < n; j += THREADS) args.labels[base + j] = -1;
            continue;
        }

        const int m = n - 1;
        const int64_t ebase = base - w;
        if (args.edges_uv) {
            for (int i = tid; i < m; i += THREADS) {
                args.edges_uv[2 * (ebase + i)] = arena.s0[i];
                args.edges_uv[2 * (ebase + i) + 1] = arena.s1[i];
                static_cast<Real*>(args.edge_w)[ebase + i] = arena.r0[i];
            }
        }

        // ---- hierarchy ---------------------------------------------------
        sort_edges<Real>(arena, m, &s_counter);
        if (args.order)
            for (int i = tid; i < m; i += THREADS) args.order[ebase + i] = arena.s2[i];
        for (int i = tid; i < m; i += THREADS) {
            const int e = arena.s2[i];
            const int16_t u = arena.s0[e], v = arena.s1[e];
            arena.s2[i] = u;
            arena.s8[i] = v;
        }
        for (int i = tid; i < n; i += THREADS) { arena.s6[i] = (int16_t)i; arena.s7[i] = (int16_t)i; }
        __syncthreads();
        if (tid == 0) linkage_serial<Real>(arena, n);
        __syncthreads();
        if (args.link_lr) {
            for (int i = tid; i < m; i += THREADS) {
                args.link_lr[2 * (ebase + i)] = arena.s3[i];
                args.link_lr[2 * (ebase + i) + 1] = arena.s4[i];
                args.link_size[ebase + i] = arena.s5[i];
                static_cast<Real*>(args.link_w)[ebase + i] = arena.r0[i];
            }
        }
        __syncthreads();
        if (tid == 0) s_next_label = condense_serial<Real>(arena, n, args.mcs);
        __syncthreads();
        const int next_label = s_next_label;
        if (args.cl_parent) {
            // Condensed state before selection overwrites the arrays it shares.
            for (int c = tid; c < next_label - n; c += THREADS) {
                args.cl_parent[base + c] = c == 0 ? -1 : arena.s8[c];
                static_cast<Real*>(args.cl_birth)[base + c] = arena.r1[c];
            }
        }
        __syncthreads();
        if (tid == 0) select_and_label<Real>(arena, n, next_label, epsilon, nullptr);
        __syncthreads();
        for (int i = tid; i < n; i += THREADS) args.labels[base + i] = arena.s6[arena.s9[i] - n];
        if (args.cl_parent) {
            for (int c = tid; c < next_label - n; c += THREADS) {
                static_cast<Real*>(args.cl_stability)[base + c] = arena.r2[c];
                args.cl_selected[base + c] = arena.sel[c];
            }
            for (int i = tid; i < n; i += THREADS) args.point_parent[base + i] = arena.s9[i];
            if (tid == 0) args.n_clusters[w] = next_label - n;
        }
        __syncthreads();
    }
}

}  // namespace hdb
