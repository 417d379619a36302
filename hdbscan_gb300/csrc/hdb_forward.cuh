// Fused per-window forward kernel, warp-specialized and persistent.
//
// Reference path replaced: hdbscan_gpu/_cuda.py:110-127 (dense distance
// buffer + cluster kernel) and hdbscan_gpu/_kernels.py:164-760.
//
// One CTA = PT "Prim" threads + one "tree" warp, looping over a size-sorted
// window queue (atomic ticket, bounded by the queue length):
//  * the Prim warps build window k's minimum spanning tree of the
//    mutual-reachability graph (reference _kernels.py:164-320) into arena k%2;
//  * the tree warp turns window k-1's edges into labels (hdb_tree.cuh) in the
//    other arena at the same time.
// Hand-off uses named barriers only (bar.arrive / bar.sync with fixed thread
// counts): FULL[b] (Prim arrives, tree waits) and EMPTY[b] (tree arrives, Prim
// waits before reusing arena b).  With one arena (large windows) the two
// roles simply alternate.  In matrix variants of at most 4 slots per thread
// the next ticket is taken before each hand-off; when the CTA has no window
// left, the Prim warps join the tree warp for that last window's sort (HELP,
// the whole CTA) and exit, and the tree warp finishes the window alone.
//
// Prim details:
//  * slot s lives in thread s / SV (vertex id vid; the matrix variant lays
//    slots out lane-major so that row reads coalesce); the thread keeps the
//    vertex's coordinates (zero-padded to DP, exact) in registers, its best
//    weight, source and an in-tree bit;
//  * the current vertex's coordinates come from the window staged in shared
//    memory (or from global memory for large windows); DP == 0 selects the
//    matrix variant, which reads row `current` of a materialized distance
//    block instead (hdb_distance.cuh);
//  * strict '<' update keeps the older source on equal weights; argmin by
//    (weight, vertex id) with redux.sync, one barrier per iteration, every
//    active warp re-reduces the warp winners so the next vertex is known
//    without a second barrier;
//  * a candidate skips the correctly rounded sqrt when acc >= RU(best^2):
//    then sqrt_rn(acc) >= best (sqrt_rn is monotone, best representable), so
//    no strict improvement is possible;
//  * whenever one warp's worth of slots (matrix variant) or two (register
//    variants) has joined the tree, the vertices still outside are re-packed
//    into the lowest slots and the warps left without slots stop taking part
//    in the iteration barrier.
#pragma once
#include "hdb_common.cuh"
#include "hdb_tree.cuh"

namespace hdb {

constexpr int kBarStart = 1;  // Prim threads: window start / staging / post-Prim
constexpr int kBarIter = 2;   // active Prim warps: per-iteration barrier
constexpr int kBarFull = 3;   // 3, 4: Prim -> tree hand-off of arena 0 / 1
constexpr int kBarEmpty = 5;  // 5, 6: tree -> Prim release of arena 0 / 1
constexpr int kBarHelp = 7;   // whole CTA: the last window's sort with the Prim warps helping
// A CTA's last window sorts with every warp when it has at least this many
// edges, in matrix variants of at most 4 slots per thread: with 8 slots the
// float32 matrix Prim measured 3.4x slower per iteration in a build with this
// path, and the register variants keep their Prim code as measured.
constexpr int kHelpMinEdges = 256;
constexpr int kHelpMaxSlots = 4;

__device__ __forceinline__ void bar_sync(int id, int count) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}
__device__ __forceinline__ void bar_arrive(int id, int count) {
    asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(count) : "memory");
}

__device__ __forceinline__ int64_t global_ns() {
    int64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Exclusive scan of one int per thread over the first `warps` warps (all of
// them must call); `total` receives the sum.  Uses barrier kBarIter.
__device__ __forceinline__ int active_exclusive_scan(int value, int warps, int* s_scan, int& total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = value;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_scan[warp] = x;
    bar_sync(kBarIter, warps * 32);
    int t = lane < warps ? s_scan[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, t, o);
        if (lane >= o) t += y;
    }
    total = __shfl_sync(0xffffffffu, t, 31);
    const int before = __shfl_sync(0xffffffffu, t, warp > 0 ? warp - 1 : 0);
    return (warp > 0 ? before : 0) + x - value;
}

// Coordinates of vertex j (padded to DPS with zeros) into registers.
template <typename Real, int DP, int DPS, int VEC>
__device__ __forceinline__ void load_coords(Real (&xr)[DPS], int j, bool xs, const Real* s_x, const Real* Xw, int D) {
    if (DP == 0) return;
    if (j < 0) {
#pragma unroll
        for (int k = 0; k < DPS; ++k) xr[k] = Real(0);
        return;
    }
    if (xs) {
#pragma unroll
        for (int k0 = 0; k0 < DPS; k0 += VEC) {
            if constexpr (sizeof(Real) == 4) {
                const float4 q = *reinterpret_cast<const float4*>(s_x + j * DPS + k0);
                xr[k0] = q.x; xr[(k0 + 1) % DPS] = q.y; xr[(k0 + 2) % DPS] = q.z; xr[(k0 + 3) % DPS] = q.w;
            } else {
                const double2 q = *reinterpret_cast<const double2*>(s_x + j * DPS + k0);
                xr[k0] = q.x; xr[(k0 + 1) % DPS] = q.y;
            }
        }
    } else {
#pragma unroll
        for (int k = 0; k < DPS; ++k) xr[k] = k < D ? Xw[(int64_t)j * D + k] : Real(0);
    }
}

// Coordinates of the current vertex, 16 bytes at a time.
template <typename Real, int VEC>
__device__ __forceinline__ void load_vec(Real (&c)[VEC], const Real* s_x, const Real* Xw, int cur, int k0, int DPS,
                                         bool xs, int D) {
    if (xs) {
        if constexpr (sizeof(Real) == 4) {
            const float4 q = *reinterpret_cast<const float4*>(s_x + cur * DPS + k0);
            c[0] = q.x; c[1 % VEC] = q.y; c[2 % VEC] = q.z; c[3 % VEC] = q.w;
        } else {
            const double2 q = *reinterpret_cast<const double2*>(s_x + cur * DPS + k0);
            c[0] = q.x; c[1 % VEC] = q.y;
        }
    } else {
#pragma unroll
        for (int kk = 0; kk < VEC; ++kk) c[kk] = (k0 + kk < D) ? Xw[(int64_t)cur * D + k0 + kk] : Real(0);
    }
}

// Prim over one window by the active Prim warps (reference _kernels.py:164-320).
// Writes edge `it` = (source, vertex, weight) into arena s0/s1/r0.  Returns
// overflow flags (1 = a distance overflowed, 2 = internal inconsistency).
template <typename Real, int PT, int SV, int DP, bool UNIT, typename Key>
__device__ __forceinline__ int prim_window(const ForwardArgs& args, const Arena<Real>& arena, const Real* s_x,
                                           const Real* s_core, const Real* Xw, const Real* Dw, int n, bool xs,
                                           Key (*s_key)[PT / 32], uint32_t (*s_idx)[PT / 32], int* s_scan) {
    using T = RealTraits<Real>;
    constexpr int PW = PT / 32;
    constexpr int VEC = 16 / (int)sizeof(Real);
    constexpr int DPS = DP > 0 ? DP : VEC;
    constexpr Key SENTINEL = (Key)~(Key)0;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int D = args.D;

    // Per-slot state.  Register variants: slot s = tid*SV + v.  Matrix variant:
    // slot s = warp*32*SV + v*32 + lane (lane-major), so that for each v the
    // warp's 32 row reads fall on consecutive slots, whose vertex ids increase
    // (one 128-byte line before any vertex left the tree) instead of one float
    // per 32-byte sector SV times over.  Either way warp w owns slots
    // [w*32*SV, (w+1)*32*SV).  xr holds the coordinates, act marks slots
    // holding a vertex outside the tree.  Float distances use packed
    // f32x2 instructions for the differences and squares only; the sum stays a
    // chain of scalar round-to-nearest adds in k order (a packed multiply
    // feeding a packed add may be contracted into a packed FMA, which would
    // change the rounding).
    constexpr bool kLaneMajor = DP == 0;
    auto slot_of = [&](int v) { return kLaneMajor ? warp * 32 * SV + v * 32 + lane : tid * SV + v; };
    Real xr[SV][DPS];
    Real best[SV], thr[SV], core_r[SV];
    int src[SV], vid[SV];
    bool act[SV];
    auto load_slot = [&](int v, int j) {
        load_coords<Real, DP, DPS, VEC>(xr[v], j, xs, s_x, Xw, D);
        if (!UNIT) core_r[v] = j >= 0 ? s_core[j] : Real(0);
    };
#pragma unroll
    for (int v = 0; v < SV; ++v) {
        const int j = slot_of(v);
        vid[v] = j < n ? j : -1;
        act[v] = j < n && j != 0;  // vertex 0 starts the tree (_kernels.py:210-213)
        best[v] = T::inf();
        thr[v] = T::inf();
        src[v] = 1;  // reference initial source (_kernels.py:167)
        core_r[v] = Real(0);
        load_slot(v, vid[v]);
    }

    int cur = 0;
    int overflow = 0;
    Real acc_max = Real(0);
    int live = n;
    int aw = (n + 32 * SV - 1) / (32 * SV);
    if (aw > PW) aw = PW;
    if (warp >= aw) return 0;
    // Re-pack after one warp's worth of slots left the tree (matrix variant), or
    // two (register variants: their re-pack reloads coordinates, c2 +1.3%).
    constexpr int kCompactAfter = (DP > 0 ? 64 : 32) * SV;
    for (int it = 0; it < n - 1; ++it) {
        const int remaining = n - 1 - it;  // vertices still outside the tree
        if (live - remaining >= kCompactAfter) {
            // ---- compaction over the active warps ----------------------------
            // Live vertices are staged in slot order (so slots keep increasing
            // vertex ids) and re-packed into slots [0, live).
            int16_t* stage_j = arena.s2;
            int16_t* stage_src = arena.s3;
            Real* stage_best = arena.r1;
            int total = 0;
            if constexpr (kLaneMajor) {
                unsigned bal[SV];
                int wcount = 0;
#pragma unroll
                for (int v = 0; v < SV; ++v) { bal[v] = __ballot_sync(0xffffffffu, act[v]); wcount += __popc(bal[v]); }
                int pos = active_exclusive_scan(lane == 0 ? wcount : 0, aw, s_scan, total);
                pos = __shfl_sync(0xffffffffu, pos, 0);  // slots of the warps before this one
                const unsigned below = lanemask_lt();
#pragma unroll
                for (int v = 0; v < SV; ++v) {
                    if (act[v]) {
                        const int at = pos + __popc(bal[v] & below);
                        stage_j[at] = (int16_t)vid[v];
                        stage_src[at] = (int16_t)src[v];
                        stage_best[at] = best[v];
                    }
                    pos += __popc(bal[v]);
                }
            } else {
                int count = 0;
#pragma unroll
                for (int v = 0; v < SV; ++v) count += act[v] ? 1 : 0;
                int pos = active_exclusive_scan(count, aw, s_scan, total);
#pragma unroll
                for (int v = 0; v < SV; ++v) {
                    if (act[v]) {
                        stage_j[pos] = (int16_t)vid[v];
                        stage_src[pos] = (int16_t)src[v];
                        stage_best[pos] = best[v];
                        ++pos;
                    }
                }
            }
            bar_sync(kBarIter, aw * 32);
            live = total;
#pragma unroll
            for (int v = 0; v < SV; ++v) {
                const int slot = slot_of(v);
                if (slot < live) {
                    vid[v] = stage_j[slot];
                    src[v] = stage_src[slot];
                    best[v] = stage_best[slot];
                    thr[v] = T::mul_ru(best[v], best[v]);
                    act[v] = true;
                } else {
                    vid[v] = -1;
                    act[v] = false;
                }
                load_slot(v, vid[v]);
            }
            bar_sync(kBarIter, aw * 32);  // staging slots may be rewritten afterwards
            const int naw = (live + 32 * SV - 1) / (32 * SV);
            aw = naw < 1 ? 1 : naw;
            if (warp >= aw) break;  // this warp has no slots left (warp-uniform)
        }
        const Real core_cur = UNIT ? Real(0) : s_core[cur];
        Real acc[SV];
        if constexpr (DP > 0) {
#pragma unroll
            for (int v = 0; v < SV; ++v) acc[v] = Real(0);
#pragma unroll
            for (int k0 = 0; k0 < DPS; k0 += VEC) {
                Real c[VEC];
                load_vec<Real, VEC>(c, s_x, Xw, cur, k0, DPS, xs, D);
#pragma unroll
                for (int v = 0; v < SV; ++v) {
                    if constexpr (sizeof(Real) == 4) {
                        // Two coordinates per packed instruction: x - c as
                        // fma(c, -1, x) (exact product, one rounding: RN(x - c)
                        // = -RN(c - x), same square), the squares as one packed
                        // multiply, then the k-ordered scalar sum.
#pragma unroll
                        for (int kk = 0; kk < VEC; kk += 2) {
                            const float2 delta = __ffma2_rn(make_float2(c[kk], c[kk + 1]), make_float2(-1.0f, -1.0f),
                                                            make_float2(xr[v][k0 + kk], xr[v][k0 + kk + 1]));
                            const float2 sq = __fmul2_rn(delta, delta);
                            acc[v] = T::add(acc[v], sq.x);
                            acc[v] = T::add(acc[v], sq.y);
                        }
                    } else {
#pragma unroll
                        for (int kk = 0; kk < VEC; ++kk) {
                            const Real delta = T::sub(c[kk], xr[v][k0 + kk]);
                            acc[v] = T::add(acc[v], T::mul(delta, delta));
                        }
                    }
                }
            }
        } else {
            // Matrix variant: row `cur` of the window's distance block (slots
            // outside the tree set read entry 0 and ignore it).
            const Real* __restrict__ row = Dw + (int64_t)cur * (int64_t)((n + 3) & ~3);
#pragma unroll
            for (int v = 0; v < SV; ++v) acc[v] = __ldcg(row + (act[v] ? vid[v] : 0));
        }
        Key lkey = SENTINEL;
        uint32_t lidx = 0xffffffffu;
#pragma unroll
        for (int v = 0; v < SV; ++v) {
            if constexpr (DP > 0) {
                // sqrt_rn is monotone and best representable: acc >= RU(best^2)
                // gives sqrt_rn(acc) >= best, so no strict improvement.
                acc_max = T::sel(act[v], T::vmax(acc_max, acc[v]), acc_max);
                const Real cm = UNIT ? Real(0) : T::vmax(core_cur, core_r[v]);
                if (act[v] && T::lt(acc[v], thr[v]) && (UNIT || T::lt(cm, best[v]))) {
                    const Real d = T::sqrt_rn(acc[v]);
                    const Real wgt = UNIT ? d : T::vmax(cm, d);
                    if (T::lt(wgt, best[v])) {  // strict: equal weights keep the older source
                        best[v] = wgt;
                        src[v] = cur;
                        thr[v] = T::mul_ru(wgt, wgt);
                    }
                }
            } else {
                if (act[v]) {
                    const Real d = acc[v];
                    overflow |= !T::finite_nn(d);
                    const Real wgt = UNIT ? d : T::vmax(T::vmax(core_cur, core_r[v]), d);
                    if (T::lt(wgt, best[v])) { best[v] = wgt; src[v] = cur; }
                }
            }
            const Key key = act[v] ? T::key(best[v]) : SENTINEL;
            const uint32_t j = (uint32_t)vid[v];
            if (key_idx_lt(key, j, lkey, lidx)) { lkey = key; lidx = j; }
        }
        warp_argmin(lkey, lidx);
        const int buf = it & 1;
        if (lane == 0) { s_key[buf][warp] = lkey; s_idx[buf][warp] = lidx; }
        bar_sync(kBarIter, aw * 32);
        Key gk = lane < aw ? s_key[buf][lane] : SENTINEL;
        uint32_t gi = lane < aw ? s_idx[buf][lane] : 0xffffffffu;
        warp_argmin(gk, gi);
        const int next = (int)gi;
        // The owner of the winner records the edge; its slot leaves the tree set.
#pragma unroll
        for (int v = 0; v < SV; ++v) {
            if (vid[v] == next && act[v]) {
                arena.s0[it] = (int16_t)src[v];
                arena.s1[it] = (int16_t)next;
                arena.r0[it] = best[v];
                act[v] = false;
            }
        }
        if (next < 0 || next >= n) {  // unreachable: a non-tree vertex always remains
            overflow |= 2;
            break;
        }
        cur = next;
    }
    if (DP > 0) overflow |= !(acc_max <= T::kMax);
    return overflow;
}

// The hierarchy of one window by the tree warp: exports of the Prim edges,
// NumPy-order sort, linkage, condensation, selection and labels
// (reference _kernels.py:358-760), on the arena at `base`.
template <typename Real>
__device__ __noinline__ void tree_window(const ForwardArgs& args, unsigned char* base_ptr, int w, int n,
                                         int* help_ctr = nullptr) {
    const int lane = threadIdx.x & 31;
    const Real epsilon = (Real)args.eps;  // the reference casts options to Real (_cuda.py:105)
    const int m = n - 1;
    if (args.stage_ns && lane == 0) args.stage_ns[8 * w + 3] = global_ns();
    const int64_t base = args.offsets[w];
    const int64_t ebase = base - w;
    Arena<Real> a = Arena<Real>::carve(base_ptr, n);
    if (args.edges_uv) {
        for (int i = lane; i < m; i += 32) {
            args.edges_uv[2 * (ebase + i)] = a.s0[i];
            args.edges_uv[2 * (ebase + i) + 1] = a.s1[i];
            static_cast<Real*>(args.edge_w)[ebase + i] = a.r0[i];
        }
    }
    if (help_ctr)  // the Prim warps have no window left and join the sort (whole CTA)
        sort_edges_cta<Real>(a, m, (int)blockDim.x, kBarHelp, help_ctr);
    else
        sort_edges_warp<Real>(a, m, args.unit_core != 0);
    if (args.stage_ns && lane == 0) args.stage_ns[8 * w + 4] = global_ns();
    if (args.order)
        for (int i = lane; i < m; i += 32) args.order[ebase + i] = a.s2[i];
    __syncwarp();
    for (int i = lane; i < m; i += 32) {
        const int e = a.s2[i];
        const int16_t u = a.s0[e], v = a.s1[e];
        a.s2[i] = u;
        a.s3[i] = v;
    }
    __syncwarp();
    linkage_warp<Real>(a, n);
    if (args.stage_ns && lane == 0) args.stage_ns[8 * w + 5] = global_ns();
    if (args.link_lr) {
        for (int i = lane; i < m; i += 32) {
            args.link_lr[2 * (ebase + i)] = a.s4[i];
            args.link_lr[2 * (ebase + i) + 1] = a.s5[i];
            args.link_size[ebase + i] = a.s6[i];
            static_cast<Real*>(args.link_w)[ebase + i] = a.r0[i];
        }
    }
    __syncwarp();
    const int next_label = condense_warp<Real>(a, n, args.mcs, args.cl_size ? args.cl_size + base : nullptr);
    if (args.stage_ns && lane == 0) args.stage_ns[8 * w + 6] = global_ns();
    if (args.point_lambda) {  // s8: the linkage node each point was pruned at; r0: lambda per node
        Real* out = static_cast<Real*>(args.point_lambda) + base;
        for (int i = lane; i < n; i += 32) out[i] = a.r0[a.s8[i] - n];
    }
    if (args.cl_parent) {
        for (int c = lane; c < next_label - n; c += 32) {
            args.cl_parent[base + c] = a.s2[c];
            static_cast<Real*>(args.cl_birth)[base + c] = a.r1[c];
        }
    }
    __syncwarp();
    select_and_label_warp<Real>(a, n, next_label, epsilon, args.method, args.allow_single != 0, args.labels + base,
                                args.probabilities ? static_cast<Real*>(args.probabilities) + base : nullptr);
    if (args.cl_parent) {
        for (int c = lane; c < next_label - n; c += 32) {
            static_cast<Real*>(args.cl_stability)[base + c] = a.r2[c];
            args.cl_selected[base + c] = a.sel[c];
        }
        for (int i = lane; i < n; i += 32) args.point_parent[base + i] = a.s9[i];
        if (lane == 0) args.n_clusters[w] = next_label - n;
    }
    if (args.stage_ns && lane == 0) args.stage_ns[8 * w + 7] = global_ns();
}

struct WindowMeta {
    int w;      // window index, -1 = queue exhausted
    int n;
    int skip;   // labels already written (invalid input / overflow)
    int help;   // the CTA's last window: the Prim warps join its sort, then both sides exit
};

// Dynamic shared memory: n_arenas arenas of arena_stride bytes, then the
// staged window (x_off) and its core distances (core_off); see the plan layer.
// MINB CTAs share an SM (register budget from the launch bounds): with two,
// one window's barrier and reduction latency hides behind another's distance
// arithmetic.
template <typename Real, int PT, int SV, int DP, int MINB>
__global__ void __launch_bounds__(PT + 32, MINB) hdb_forward_kernel(const __grid_constant__ ForwardArgs args) {
    using T = RealTraits<Real>;
    using Key = typename T::Bits;
    constexpr int PW = PT / 32;
    constexpr int VEC = 16 / (int)sizeof(Real);
    constexpr int DPS = DP > 0 ? DP : VEC;
    static_assert(DPS % VEC == 0, "DP must be a multiple of one 16-byte vector");
    static_assert(PT % 32 == 0 && PT + 32 <= 1024, "Prim threads plus the tree warp must fit one CTA");
    static_assert(SV <= 16, "in-tree bits are kept in one 16-bit mask");
    constexpr Key SENTINEL = (Key)~(Key)0;
    constexpr bool kJoinSort = DP == 0 && SV <= kHelpMaxSlots;

    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ Key s_key[2][PW];
    __shared__ uint32_t s_idx[2][PW];
    __shared__ int s_scan[32];
    __shared__ int s_item;
    __shared__ int s_flags[2];  // by window parity: a reset never races a late read
    __shared__ WindowMeta s_meta[2];

    const int tid = threadIdx.x;
    const int warp = tid >> 5;
    const Real* __restrict__ X = static_cast<const Real*>(args.X);
    const int D = args.D;
    const int nb = args.n_arenas;

    if (warp == PW) {
        // =================== tree warp (consumer) ============================
        for (int k = 0; k < (1 << 30); ++k) {
            const int b = nb == 2 ? (k & 1) : 0;
            bar_sync(kBarFull + b, PT + 32);
            const WindowMeta meta = s_meta[b];
            if (meta.w < 0) return;
            if constexpr (kJoinSort) {
                if (meta.help) {  // no release: the Prim warps consumed every earlier one and exit too
                    tree_window<Real>(args, smem + (size_t)b * args.arena_stride, meta.w, meta.n, s_scan);
                    return;
                }
            }
            if (!meta.skip) tree_window<Real>(args, smem + (size_t)b * args.arena_stride, meta.w, meta.n);
            __syncwarp();
            __threadfence_block();
            bar_arrive(kBarEmpty + b, PT + 32);
        }
        return;
    }

    // ====================== Prim warps (producer) ============================
    const Real* __restrict__ core_g = static_cast<const Real*>(args.core);
    const bool xs = DP > 0 && args.x_in_smem;
    Real* s_x = reinterpret_cast<Real*>(smem + args.x_off);
    Real* s_core = reinterpret_cast<Real*>(smem + args.core_off);

    if constexpr (kJoinSort) {
        if (tid == 0) s_item = atomicAdd(args.ticket, 1);
    }
    for (int k = 0; k < (1 << 30); ++k) {
        const int b = nb == 2 ? (k & 1) : 0;
        const int par = k & 1;
        if constexpr (kJoinSort) {
            if (tid == 0) s_flags[par] = 0;  // the ticket was taken before the last hand-off
        } else {
            if (tid == 0) { s_item = atomicAdd(args.ticket, 1); s_flags[par] = 0; }
        }
        bar_sync(kBarStart, PT);
        const int item = s_item;
        if (item >= args.queue_len) {
            if (k >= nb) bar_sync(kBarEmpty + b, PT + 32);
            if (tid == 0) s_meta[b].w = -1;
            __threadfence_block();
            bar_arrive(kBarFull + b, PT + 32);
            // Take the tree warp's release of the previous window so no
            // arrival is left pending when the CTA exits.
            if (nb == 2 && k >= 1) bar_sync(kBarEmpty + (b ^ 1), PT + 32);
            return;
        }
        const int w = args.queue[item];
        const int64_t base = args.offsets[w];
        const int n = (int)(args.offsets[w + 1] - base);
        const Real* __restrict__ Xw = X + base * D;
        const Real* __restrict__ Dw = DP > 0 ? nullptr : static_cast<const Real*>(args.dist) + args.dist_offsets[w];
        if (args.stage_ns && tid == 0) args.stage_ns[8 * w + 0] = global_ns();

        // ---- stage coordinates / cores, validate input -----------------------
        int bad = 0;
        if (xs) {
            // Eight independent loads in flight per thread before the stores.
            constexpr int U = 8;
            const int total = n * DPS;
            int t = tid;
            for (; t + (U - 1) * PT < total; t += U * PT) {
                Real v[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const int tt = t + u * PT, j = tt / DPS, kk = tt - j * DPS;
                    v[u] = kk < D ? Xw[(int64_t)j * D + kk] : Real(0);
                }
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    bad |= !isfinite(v[u]);
                    s_x[t + u * PT] = v[u];
                }
            }
            for (; t < total; t += PT) {
                const int j = t / DPS, kk = t - j * DPS;
                Real v = Real(0);
                if (kk < D) { v = Xw[(int64_t)j * D + kk]; bad |= !isfinite(v); }
                s_x[t] = v;
            }
        } else {
            for (int t = tid; t < n * D; t += PT) bad |= !isfinite(Xw[t]);
        }
        if (!args.unit_core)
            for (int j = tid; j < n; j += PT) s_core[j] = core_g[base + j];
        if (bad) atomicOr(&s_flags[par], 1);
        bar_sync(kBarStart, PT);
        const bool invalid = s_flags[par] & 1;

        if (k >= nb) bar_sync(kBarEmpty + b, PT + 32);  // arena b released by the tree warp
        Arena<Real> arena = Arena<Real>::carve(smem + (size_t)b * args.arena_stride, n);

        int overflow = 0;
        if (!invalid) {
            if (args.stage_ns && tid == 0) args.stage_ns[8 * w + 1] = global_ns();
            if (args.unit_core)
                overflow = prim_window<Real, PT, SV, DP, true>(args, arena, s_x, s_core, Xw, Dw, n, xs, s_key, s_idx, s_scan);
            else
                overflow = prim_window<Real, PT, SV, DP, false>(args, arena, s_x, s_core, Xw, Dw, n, xs, s_key, s_idx, s_scan);
        }
        if (overflow) atomicOr(&s_flags[par], overflow << 1);
        if constexpr (kJoinSort) {
            // The next window's ticket, taken before the hand-off so that the
            // CTA's last window is known as such.
            if (tid == 0) s_item = atomicAdd(args.ticket, 1);
        }
        bar_sync(kBarStart, PT);
        const int flags = s_flags[par];
        if (args.stage_ns && tid == 0) args.stage_ns[8 * w + 2] = global_ns();
        int skip = 0;
        if (flags) {
            const int code = (flags & 1) ? kNonFinite : ((flags & 4) ? kInternal : kOverflow);
            if (tid == 0) atomic_status(args.status, code);
            for (int j = tid; j < n; j += PT) args.labels[base + j] = -1;
            skip = 1;
        }
        int help = 0;
        if constexpr (kJoinSort)
            help = s_item >= args.queue_len && !skip && !args.unit_core && n - 1 >= kHelpMinEdges;
        if (tid == 0) { s_meta[b].w = w; s_meta[b].n = n; s_meta[b].skip = skip; s_meta[b].help = help; }
        __threadfence_block();
        bar_arrive(kBarFull + b, PT + 32);
        if constexpr (kJoinSort) {
            if (help) {
                // Take the tree warp's release of the previous window (nothing
                // may stay pending at exit), then sort this one with it.
                if (nb == 2 && k >= 1) bar_sync(kBarEmpty + (b ^ 1), PT + 32);
                sort_edges_cta<Real>(arena, n - 1, PT + 32, kBarHelp, s_scan);
                return;
            }
        }
    }
}

}  // namespace hdb
