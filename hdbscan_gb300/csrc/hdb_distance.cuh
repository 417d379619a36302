// Pairwise distances and self-inclusive core distances.
//
// * hdb_distance_kernel: materializes each window's distance block with a
//   64x64 register-blocked tile per CTA over the upper triangle (tile i <= j)
//   and writes every off-diagonal tile twice (direct and mirrored), both with
//   16-byte coalesced stores.  Replaces the one-thread-per-element
//   DISTANCE_SOURCE (hdbscan_gpu/_kernels.py:45-88) with bit-identical values:
//   per pair the coordinates are accumulated in k order with
//   total = total + delta*delta and no FMA, then a correctly rounded sqrt.
//   Block row stride ld = round_up(n, 4) keeps every row 16-byte aligned.
// * hdb_distance128_kernel: the same blocks for float32 windows of 384 points
//   and more, 128x128 tiles with 8x8 pairs per thread (same arithmetic).
// * hdb_core_points_kernel / hdb_core_rows_kernel: core_i = the (ms-1)-th
//   smallest distance of row i, self (0) included (reference:
//   hdbscan_gpu/_cuda.py:114-118, cp.partition), from a list of the K
//   smallest (value, index) pairs; the value at position ms-1 is the order
//   statistic, the index is the ms-th nearest neighbour in (distance, index)
//   order (used by the backward pass).  The points kernel recomputes the
//   distances (one thread per row, a sorted register list); the rows kernel
//   reads the materialized block (one warp per row, the list across lanes).
// * hdb_core_select_kernel: any ms, one CTA per row, radix select on the
//   order-preserving bit pattern of the non-negative distances.
#pragma once
#include "hdb_common.cuh"

namespace hdb {

__host__ __device__ inline int64_t dist_ld(int n) { return (int64_t)((n + 3) & ~3); }


constexpr int kDistTile = 64;

template <typename Real>
struct DistVec;
template <> struct DistVec<float> {
    static constexpr int KC = 32;
    __device__ static void load4(const float* p, float* out) {
        const float4 q = *reinterpret_cast<const float4*>(p);
        out[0] = q.x; out[1] = q.y; out[2] = q.z; out[3] = q.w;
    }
    __device__ static void store4(float* p, float a, float b, float c, float d) {
        *reinterpret_cast<float4*>(p) = make_float4(a, b, c, d);
    }
};
template <> struct DistVec<double> {
    static constexpr int KC = 16;
    __device__ static void load4(const double* p, double* out) {
        const double2 q0 = *reinterpret_cast<const double2*>(p);
        const double2 q1 = *reinterpret_cast<const double2*>(p + 2);
        out[0] = q0.x; out[1] = q0.y; out[2] = q1.x; out[3] = q1.y;
    }
    __device__ static void store4(double* p, double a, double b, double c, double d) {
        *reinterpret_cast<double2*>(p) = make_double2(a, b);
        *reinterpret_cast<double2*>(p + 2) = make_double2(c, d);
    }
};

// 256 threads = 16x16; thread (ty, tx) owns rows ty*4..+3 and cols tx*4..+3.
// float64: 64 registers, 4 CTAs per SM (the integer-pipe arithmetic is
// latency-bound at 3 CTAs; 5 would spill).
template <typename Real>
__global__ void __launch_bounds__(256, sizeof(Real) == 8 ? 4 : 1) hdb_distance_kernel(const DistanceArgs args) {
    using T = RealTraits<Real>;
    constexpr int KC = DistVec<Real>::KC;
    __shared__ __align__(16) Real s_i[KC][kDistTile];
    __shared__ __align__(16) Real s_j[KC][kDistTile];
    const int tile = blockIdx.x;
    if (tile >= args.n_tiles) return;
    const int w = args.tiles[3 * tile], ti = args.tiles[3 * tile + 1], tj = args.tiles[3 * tile + 2];
    const int64_t base = args.offsets[w];
    const int n = (int)(args.offsets[w + 1] - base);
    const int D = args.D;
    const Real* __restrict__ Xw = static_cast<const Real*>(args.X) + base * D;
    Real* __restrict__ Dw = static_cast<Real*>(args.dist) + args.dist_offsets[w];
    const int64_t ld = dist_ld(n);
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int i0 = ti * kDistTile, j0 = tj * kDistTile;

    Real acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = Real(0);

    for (int k0 = 0; k0 < D; k0 += KC) {
        // Stage [64 rows x KC coords] of each block, transposed to [KC][64]:
        // lanes walk the row index, so each shared store instruction writes
        // consecutive words (no bank conflicts); every thread covers KC/4
        // coordinates of one row (row reads hit L1/L2: the window is reused
        // by every tile of its block row).
        bool safe = true;
        {
            constexpr int KQ = KC / 4;
            const int r = tid & (kDistTile - 1), kq = tid >> 6;
            const int gi = i0 + r, gj = j0 + r;
#pragma unroll
            for (int kk = 0; kk < KQ; ++kk) {
                const int k = kq * KQ + kk, gk = k0 + k;
                const Real vi = (gi < n && gk < D) ? Xw[(int64_t)gi * D + gk] : Real(0);
                const Real vj = (gj < n && gk < D) ? Xw[(int64_t)gj * D + gk] : Real(0);
                safe = safe && T::operand_safe(vi) && T::operand_safe(vj);
                s_i[k][r] = vi;
                s_j[k][r] = vj;
            }
        }
        // Chunk-uniform choice of the square: the integer-pipe one when every
        // staged coordinate keeps all squares normal and every float64
        // accumulator is in the fused square-and-add's domain (hdb_exact.h),
        // else the hardware multiply.
        if constexpr (sizeof(Real) == 8) {
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) safe = safe && sqr_add_acc_safe(acc[a][b]);
        }
        const bool int_square = __syncthreads_and(safe);
        const int kend = min(KC, D - k0);
        if constexpr (sizeof(Real) == 4) {
            // Packed differences and squares (x_i - x_j = fma(x_j, -1, x_i),
            // exact product and one rounding), scalar k-ordered sums.  Full
            // chunks run unrolled so the shared loads of later k issue early.
            auto step = [&](int k) {
                float xi[4], xj[4];
                DistVec<float>::load4(&s_i[k][ty * 4], xi);
                DistVec<float>::load4(&s_j[k][tx * 4], xj);
#pragma unroll
                for (int a = 0; a < 4; ++a) {
                    const float2 xa = make_float2(xi[a], xi[a]);
#pragma unroll
                    for (int b = 0; b < 4; b += 2) {
                        const float2 d = __ffma2_rn(make_float2(xj[b], xj[b + 1]), make_float2(-1.0f, -1.0f), xa);
                        const float2 q = __fmul2_rn(d, d);
                        acc[a][b] = T::add(acc[a][b], q.x);
                        acc[a][b + 1] = T::add(acc[a][b + 1], q.y);
                    }
                }
            };
            if (kend == KC) {
#pragma unroll 8
                for (int k = 0; k < KC; ++k) step(k);
            } else {
                for (int k = 0; k < kend; ++k) step(k);
            }
        } else {
            auto accumulate = [&](auto square) {
                for (int k = 0; k < kend; ++k) {
                    Real xi[4], xj[4];
                    DistVec<Real>::load4(&s_i[k][ty * 4], xi);
                    DistVec<Real>::load4(&s_j[k][tx * 4], xj);
#pragma unroll
                    for (int a = 0; a < 4; ++a)
#pragma unroll
                        for (int b = 0; b < 4; ++b) {
                            const Real delta = T::sub(xi[a], xj[b]);
                            acc[a][b] = T::add(acc[a][b], square(delta));
                        }
                }
            };
            if (int_square) {
                // Squares on the integer pipes (hdb_exact.h); 12 of the 16
                // running sums add on the integer pipes too, fused with their
                // square (sqr_add_rn: the square is never packed), the other
                // 4 on the FP64 pipe, which balances the two pipes (10, 13,
                // 14 or 16 of 16 is slower).
                for (int k = 0; k < kend; ++k) {
                    Real xi[4], xj[4];
                    DistVec<Real>::load4(&s_i[k][ty * 4], xi);
                    DistVec<Real>::load4(&s_j[k][tx * 4], xj);
#pragma unroll
                    for (int a = 0; a < 4; ++a)
#pragma unroll
                        for (int b = 0; b < 4; ++b) {
                            const Real delta = T::sub(xi[a], xj[b]);
                            acc[a][b] = (((a * 4 + b) & 3) != 0) ? sqr_add_rn(acc[a][b], delta)
                                                                 : T::add(acc[a][b], T::sqr(delta));
                        }
                }
            } else {
                accumulate([](Real d) { return T::mul(d, d); });
            }
        }
        __syncthreads();
    }
    int overflow = 0;
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            acc[a][b] = T::sqrt_rn(acc[a][b]);
            const int gi = i0 + ty * 4 + a, gj = j0 + tx * 4 + b;
            if (gi < n && gj < n) overflow |= !(acc[a][b] <= T::kMax);
        }
    const int cj = j0 + tx * 4;
    if (cj < ld) {
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const int gi = i0 + ty * 4 + a;
            if (gi < n) DistVec<Real>::store4(Dw + gi * ld + cj, acc[a][0], acc[a][1], acc[a][2], acc[a][3]);
        }
    }
    if (ti != tj) {
        const int ci = i0 + ty * 4;
        if (ci < ld) {
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const int gj = j0 + tx * 4 + b;
                if (gj < n) DistVec<Real>::store4(Dw + gj * ld + ci, acc[0][b], acc[1][b], acc[2][b], acc[3][b]);
            }
        }
    }
    if (__syncthreads_or(overflow) && tid == 0) atomic_status(args.status, kOverflow);
}

// Float32 blocks of larger windows: 128x128 tiles, 256 threads, 8x8 pairs per
// thread (rows ty*4..+3 and 64+ty*4..+3, columns likewise from tx), so every
// shared load feeds 16 pair updates and the accumulators give 64-way
// independence.  Per pair the arithmetic is that of hdb_distance_kernel: the
// difference x_i - x_j as fma(x_j, -1, x_i) (exact product, one rounding) and
// its square in packed f32x2 instructions, the k-ordered sum in scalar
// round-to-nearest adds, a correctly rounded sqrt.
constexpr int kDistTile128 = 128;

template <typename Real>
__global__ void __launch_bounds__(256, 2) hdb_distance128_kernel(const DistanceArgs args) {
    static_assert(sizeof(Real) == 4, "the 128x128 tile kernel is float32 only");
    using T = RealTraits<float>;
    constexpr int KC = 32;
    constexpr int TS = kDistTile128;
    __shared__ __align__(16) float s_i[KC][TS];
    __shared__ __align__(16) float s_j[KC][TS];
    const int tile = blockIdx.x;
    if (tile >= args.n_tiles) return;
    const int w = args.tiles[3 * tile], ti = args.tiles[3 * tile + 1], tj = args.tiles[3 * tile + 2];
    const int64_t base = args.offsets[w];
    const int n = (int)(args.offsets[w + 1] - base);
    const int D = args.D;
    const float* __restrict__ Xw = static_cast<const float*>(args.X) + base * D;
    float* __restrict__ Dw = static_cast<float*>(args.dist) + args.dist_offsets[w];
    const int64_t ld = dist_ld(n);
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int i0 = ti * TS, j0 = tj * TS;

    float acc[8][8];
#pragma unroll
    for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int b = 0; b < 8; ++b) acc[a][b] = 0.0f;

    for (int k0 = 0; k0 < D; k0 += KC) {
        // Stage [128 rows x KC coords] of each block transposed to [KC][128]:
        // lanes walk the row index (conflict-free stores); each thread covers
        // KC/2 coordinates of one row.
        {
            const int r = tid & (TS - 1), kq = tid >> 7;
            const int gi = i0 + r, gj = j0 + r;
#pragma unroll
            for (int kk = 0; kk < KC / 2; ++kk) {
                const int k = kq * (KC / 2) + kk, gk = k0 + k;
                s_i[k][r] = (gi < n && gk < D) ? Xw[(int64_t)gi * D + gk] : 0.0f;
                s_j[k][r] = (gj < n && gk < D) ? Xw[(int64_t)gj * D + gk] : 0.0f;
            }
        }
        __syncthreads();
        const int kend = min(KC, D - k0);
        auto step = [&](int k) {
            float xi[8], xj[8];
            DistVec<float>::load4(&s_i[k][ty * 4], xi);
            DistVec<float>::load4(&s_i[k][64 + ty * 4], xi + 4);
            DistVec<float>::load4(&s_j[k][tx * 4], xj);
            DistVec<float>::load4(&s_j[k][64 + tx * 4], xj + 4);
#pragma unroll
            for (int a = 0; a < 8; ++a) {
                const float2 xa = make_float2(xi[a], xi[a]);
#pragma unroll
                for (int b = 0; b < 8; b += 2) {
                    const float2 d = __ffma2_rn(make_float2(xj[b], xj[b + 1]), make_float2(-1.0f, -1.0f), xa);
                    const float2 q = __fmul2_rn(d, d);
                    acc[a][b] = T::add(acc[a][b], q.x);
                    acc[a][b + 1] = T::add(acc[a][b + 1], q.y);
                }
            }
        };
        if (kend == KC) {
#pragma unroll 4
            for (int k = 0; k < KC; ++k) step(k);
        } else {
            for (int k = 0; k < kend; ++k) step(k);
        }
        __syncthreads();
    }
    int overflow = 0;
#pragma unroll
    for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int b = 0; b < 8; ++b) {
            acc[a][b] = T::sqrt_rn(acc[a][b]);
            const int gi = i0 + (a < 4 ? ty * 4 + a : 64 + ty * 4 + a - 4);
            const int gj = j0 + (b < 4 ? tx * 4 + b : 64 + tx * 4 + b - 4);
            if (gi < n && gj < n) overflow |= !(acc[a][b] <= T::kMax);
        }
    // Direct block: row gi, columns cj..cj+3 (ld is a multiple of 4, so a
    // column group that starts below ld ends below it).
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int cj = j0 + h * 64 + tx * 4;
        if (cj < ld) {
#pragma unroll
            for (int a = 0; a < 8; ++a) {
                const int gi = i0 + (a < 4 ? ty * 4 + a : 64 + ty * 4 + a - 4);
                if (gi < n)
                    DistVec<float>::store4(Dw + gi * ld + cj, acc[a][4 * h], acc[a][4 * h + 1], acc[a][4 * h + 2],
                                           acc[a][4 * h + 3]);
            }
        }
    }
    if (ti != tj) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int ci = i0 + h * 64 + ty * 4;
            if (ci < ld) {
#pragma unroll
                for (int b = 0; b < 8; ++b) {
                    const int gj = j0 + (b < 4 ? tx * 4 + b : 64 + tx * 4 + b - 4);
                    if (gj < n)
                        DistVec<float>::store4(Dw + gj * ld + ci, acc[4 * h][b], acc[4 * h + 1][b], acc[4 * h + 2][b],
                                               acc[4 * h + 3][b]);
                }
            }
        }
    }
    if (__syncthreads_or(overflow) && tid == 0) atomic_status(args.status, kOverflow);
}

// ---------------------------------------------------------------------------
// Core distances.
// ---------------------------------------------------------------------------

constexpr int kCoreRows = 128;        // rows per CTA of the points kernel
constexpr int kCoreMatrixRows = 32;   // rows per work item of the matrix (rows) kernel

template <typename Real, int K>
__device__ __forceinline__ void topk_insert(Real (&L)[K], int (&LI)[K], Real d, int j) {
    using T = RealTraits<Real>;
    if (!T::lt(d, L[K - 1])) return;
#pragma unroll
    for (int t = K - 1; t > 0; --t) {
        const bool shift = T::lt(d, L[t - 1]);
        const bool place = !shift && T::lt(d, L[t]);
        L[t] = T::sel(shift, L[t - 1], T::sel(place, d, L[t]));
        LI[t] = shift ? LI[t - 1] : (place ? j : LI[t]);
    }
    const bool first = T::lt(d, L[0]);
    L[0] = T::sel(first, d, L[0]);
    LI[0] = first ? j : LI[0];
}

template <typename Real, int K>
__device__ __forceinline__ void topk_pick(const Real (&L)[K], const int (&LI)[K], int k, Real& value, int& index) {
#pragma unroll
    for (int t = 0; t < K; ++t)
        if (t == k) { value = L[t]; index = LI[t]; }
}

// Rows from points: 128 rows per CTA, j tiles staged in shared memory.
template <typename Real, int K, int DP>
__global__ void __launch_bounds__(kCoreRows) hdb_core_points_kernel(const CoreArgs args) {
    using T = RealTraits<Real>;
    constexpr int TJ = 64;
    constexpr int VEC = 16 / (int)sizeof(Real);
    static_assert(DP % VEC == 0, "DP must be a multiple of one 16-byte vector");
    __shared__ __align__(16) Real s_x[TJ * DP];
    const int item = blockIdx.x;
    if (item >= args.n_items) return;
    const int w = args.items[2 * item], r0 = args.items[2 * item + 1];
    const int64_t base = args.offsets[w];
    const int n = (int)(args.offsets[w + 1] - base);
    const int D = args.D;
    const Real* __restrict__ Xw = static_cast<const Real*>(args.X) + base * D;
    const int i = r0 + threadIdx.x;
    Real xi[DP];
#pragma unroll
    for (int k = 0; k < DP; ++k) xi[k] = (i < n && k < D) ? Xw[(int64_t)i * D + k] : Real(0);
    Real L[K];
    int LI[K];
#pragma unroll
    for (int t = 0; t < K; ++t) { L[t] = T::inf(); LI[t] = -1; }
    int overflow = 0;
    for (int j0 = 0; j0 < n; j0 += TJ) {
        const int cnt = min(TJ, n - j0);
        for (int t = threadIdx.x; t < TJ * DP; t += kCoreRows) {
            const int r = t / DP, k = t - r * DP;
            s_x[t] = (r < cnt && k < D) ? Xw[(int64_t)(j0 + r) * D + k] : Real(0);
        }
        __syncthreads();
        if (i < n) {
            for (int jj = 0; jj < cnt; ++jj) {
                Real acc = Real(0);
#pragma unroll
                for (int k0 = 0; k0 < DP; k0 += VEC) {
                    Real c[VEC];
                    if constexpr (sizeof(Real) == 4) {
                        const float4 q = *reinterpret_cast<const float4*>(&s_x[jj * DP + k0]);
                        c[0] = q.x; c[1 % VEC] = q.y; c[2 % VEC] = q.z; c[3 % VEC] = q.w;
                    } else {
                        const double2 q = *reinterpret_cast<const double2*>(&s_x[jj * DP + k0]);
                        c[0] = q.x; c[1 % VEC] = q.y;
                    }
#pragma unroll
                    for (int kk = 0; kk < VEC; ++kk) {
                        const Real delta = T::sub(xi[k0 + kk], c[kk]);
                        acc = T::add(acc, T::mul(delta, delta));
                    }
                }
                const Real d = T::sqrt_rn(acc);
                overflow |= !(d <= T::kMax);
                topk_insert<Real, K>(L, LI, d, j0 + jj);
            }
        }
        __syncthreads();
    }
    if (i < n) {
        Real value = Real(0);
        int index = -1;
        topk_pick<Real, K>(L, LI, args.ms - 1, value, index);
        static_cast<Real*>(args.core)[base + i] = value;
        if (args.core_nbr) args.core_nbr[base + i] = index;
    }
    if (__syncthreads_or(overflow) && threadIdx.x == 0) atomic_status(args.status, kOverflow);
}

// 64-bit key select on 32-bit words (a 64-bit select is an FP64-pipe instruction on GB300).
__device__ __forceinline__ unsigned long long core_key_sel(bool c, unsigned long long a, unsigned long long b) {
    const uint32_t hi = c ? (uint32_t)(a >> 32) : (uint32_t)(b >> 32);
    const uint32_t lo = c ? (uint32_t)a : (uint32_t)b;
    return ((unsigned long long)hi << 32) | lo;
}

// Rows of the materialized matrix, one warp per row, for lists of K <= 64
// (both precisions).  The warp reads 32 consecutive entries of its row per
// load (coalesced, eight loads in flight per lane), keeps the K smallest (key, index) pairs across the lanes
// (position p = lane + 32*h, ascending), and filters every entry with one
// integer compare against the current K-th key; entries below it are
// inserted one at a time in index order by the whole warp (each position
// takes its predecessor by a shuffle), so the list is exactly the one the
// serial strict-'<' scan in index order builds: the K smallest in
// (value, index) order.  The first 32 entries are placed by a warp bitonic
// sort on (key, index).  Keys are the order-preserving bit patterns of the
// non-negative distances (integer compares only; float64 keys compare as
// 32-bit word pairs).
constexpr int kCoreRowsWarps = 8;  // warps per CTA; an item's 32 rows are shared among them

template <typename Key>
__device__ __forceinline__ Key shfl_key(Key k, int src) {
    if constexpr (sizeof(Key) == 4) {
        return __shfl_sync(0xffffffffu, k, src);
    } else {
        const uint32_t hi = __shfl_sync(0xffffffffu, (uint32_t)(k >> 32), src);
        const uint32_t lo = __shfl_sync(0xffffffffu, (uint32_t)k, src);
        return ((Key)hi << 32) | lo;
    }
}
template <typename Key>
__device__ __forceinline__ Key shfl_key_up(Key k) {
    if constexpr (sizeof(Key) == 4) {
        return __shfl_up_sync(0xffffffffu, k, 1);
    } else {
        const uint32_t hi = __shfl_up_sync(0xffffffffu, (uint32_t)(k >> 32), 1);
        const uint32_t lo = __shfl_up_sync(0xffffffffu, (uint32_t)k, 1);
        return ((Key)hi << 32) | lo;
    }
}
template <typename Key>
__device__ __forceinline__ Key shfl_key_xor(Key k, int mask) {
    if constexpr (sizeof(Key) == 4) {
        return __shfl_xor_sync(0xffffffffu, k, mask);
    } else {
        const uint32_t hi = __shfl_xor_sync(0xffffffffu, (uint32_t)(k >> 32), mask);
        const uint32_t lo = __shfl_xor_sync(0xffffffffu, (uint32_t)k, mask);
        return ((Key)hi << 32) | lo;
    }
}
template <typename Key>
__device__ __forceinline__ Key key_select(bool c, Key a, Key b) {
    if constexpr (sizeof(Key) == 4) {
        return c ? a : b;
    } else {
        return core_key_sel(c, a, b);
    }
}

template <typename Real, int K>
__global__ void __launch_bounds__(32 * kCoreRowsWarps) hdb_core_rows_kernel(const CoreArgs args) {
    static_assert(K <= 64, "at most two list entries per lane");
    using T = RealTraits<Real>;
    using Key = typename T::Bits;
    constexpr int E = (K + 31) / 32;     // list entries per lane
    constexpr Key kNone = (Key)~(Key)0;  // above every distance key (and +inf's)
    constexpr int U = 8;                 // row chunks per group of loads
    const int item = blockIdx.x;
    if (item >= args.n_items) return;
    const int w = args.items[2 * item], r0 = args.items[2 * item + 1];
    const int64_t base = args.offsets[w];
    const int n = (int)(args.offsets[w + 1] - base);
    const Real* __restrict__ Dw = static_cast<const Real*>(args.dist) + args.dist_offsets[w];
    const int64_t ld = dist_ld(n);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int r = warp; r < kCoreMatrixRows; r += kCoreRowsWarps) {
        const int i = r0 + r;
        if (i >= n) break;  // warp-uniform
        const Real* __restrict__ row = Dw + (int64_t)i * ld;
        // First 32 entries: bitonic sort on (key, index), ascending.
        Key lk[E];
        int li[E];
        lk[0] = lane < n ? T::key(__ldcs(row + lane)) : kNone;
        li[0] = lane;
        if constexpr (E > 1) { lk[1] = kNone; li[1] = 32 + lane; }
#pragma unroll
        for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
            for (int j = k >> 1; j > 0; j >>= 1) {
                const Key pk = shfl_key_xor(lk[0], j);
                const int pi = __shfl_xor_sync(0xffffffffu, li[0], j);
                const bool partner_less = key_lt(pk, lk[0]) || (key_eq(pk, lk[0]) && pi < li[0]);
                const bool keep_min = ((lane & k) == 0) == ((lane & j) == 0);
                const bool take = keep_min ? partner_less : !partner_less;
                lk[0] = key_select(take, pk, lk[0]);
                li[0] = take ? pi : li[0];
            }
        }
        Key tau = shfl_key(lk[(K - 1) / 32], (K - 1) % 32);
        for (int j0 = 32; j0 < n; j0 += 32 * U) {
            Key v[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int j = j0 + 32 * u + lane;
                v[u] = j < n ? T::key(__ldcs(row + j)) : kNone;
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                unsigned bal = __ballot_sync(0xffffffffu, key_lt(v[u], tau));
                while (bal) {
                    const int src = __ffs(bal) - 1;
                    bal &= bal - 1;
                    const Key ck = shfl_key(v[u], src);
                    if (key_lt(ck, tau)) {  // warp-uniform; tau only decreases
                        const int cj = j0 + 32 * u + src;
                        // Predecessor of position lane + 32h: lane - 1 of the same h,
                        // or lane 31 of h - 1 for lane 0.
                        Key pk[E];
                        int pi[E];
                        pk[0] = shfl_key_up(lk[0]);
                        pi[0] = __shfl_up_sync(0xffffffffu, li[0], 1);
                        if constexpr (E > 1) {
                            const Key up = shfl_key_up(lk[1]);
                            const int upi = __shfl_up_sync(0xffffffffu, li[1], 1);
                            const Key last = shfl_key(lk[0], 31);
                            const int lasti = __shfl_sync(0xffffffffu, li[0], 31);
                            pk[1] = lane == 0 ? last : up;
                            pi[1] = lane == 0 ? lasti : upi;
                        }
#pragma unroll
                        for (int h = 0; h < E; ++h) {
                            const bool shift = (h > 0 || lane > 0) && key_lt(ck, pk[h]);
                            const bool place = !shift && key_lt(ck, lk[h]);
                            lk[h] = key_select(shift, pk[h], key_select(place, ck, lk[h]));
                            li[h] = shift ? pi[h] : (place ? cj : li[h]);
                        }
                        tau = shfl_key(lk[(K - 1) / 32], (K - 1) % 32);
                    }
                }
            }
        }
        const int pos = args.ms - 1;
#pragma unroll
        for (int h = 0; h < E; ++h) {
            if (pos == lane + 32 * h) {
                static_cast<Real*>(args.core)[base + i] = T::from_key(lk[h]);
                if (args.core_nbr) args.core_nbr[base + i] = li[h];
            }
        }
    }
}

// Any ms: one CTA (256 threads) per row; the row is computed (or read) into
// shared memory, then a most-significant-digit radix select over 8-bit digits
// of the order-preserving key finds the (ms-1)-th value; the neighbour index
// is the position's element in (value, index) order.
template <typename Real>
__global__ void __launch_bounds__(256) hdb_core_select_kernel(const CoreArgs args) {
    using T = RealTraits<Real>;
    using Key = typename T::Bits;
    constexpr int kBits = 8 * (int)sizeof(Key);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Key* s_key = reinterpret_cast<Key*>(smem_raw);
    __shared__ int s_hist[256];
    __shared__ int s_pick[2];
    __shared__ int s_overflow;
    const int row = blockIdx.x;
    // items here are (window, row) pairs, one per CTA.
    if (row >= args.n_items) return;
    const int w = args.items[2 * row], i = args.items[2 * row + 1];
    const int64_t base = args.offsets[w];
    const int n = (int)(args.offsets[w + 1] - base);
    const int D = args.D;
    if (threadIdx.x == 0) s_overflow = 0;
    __syncthreads();
    int overflow = 0;
    if (args.dist) {
        const Real* Dw = static_cast<const Real*>(args.dist) + args.dist_offsets[w] + i * dist_ld(n);
        for (int j = threadIdx.x; j < n; j += 256) s_key[j] = T::key(Dw[j]);
    } else {
        const Real* Xw = static_cast<const Real*>(args.X) + base * D;
        for (int j = threadIdx.x; j < n; j += 256) {
            Real acc = Real(0);
            for (int k = 0; k < D; ++k) {
                const Real delta = T::sub(Xw[(int64_t)i * D + k], Xw[(int64_t)j * D + k]);
                acc = T::add(acc, T::mul(delta, delta));
            }
            const Real d = T::sqrt_rn(acc);
            overflow |= !(d <= T::kMax);
            s_key[j] = T::key(d);
        }
    }
    if (overflow) atomicOr(&s_overflow, 1);
    __syncthreads();
    int k = args.ms - 1;          // rank still to skip inside the current prefix
    Key prefix = 0, mask = 0;
    for (int shift = kBits - 8; shift >= 0; shift -= 8) {
        for (int b = threadIdx.x; b < 256; b += 256) s_hist[b] = 0;
        __syncthreads();
        for (int j = threadIdx.x; j < n; j += 256)
            if ((s_key[j] & mask) == prefix) atomicAdd(&s_hist[(s_key[j] >> shift) & 0xff], 1);
        __syncthreads();
        if (threadIdx.x == 0) {
            int acc = 0, b = 0;
            for (; b < 256; ++b) {
                if (acc + s_hist[b] > k) break;
                acc += s_hist[b];
            }
            s_pick[0] = b;
            s_pick[1] = acc;
        }
        __syncthreads();
        prefix |= (Key)s_pick[0] << shift;
        mask |= (Key)0xff << shift;
        k -= s_pick[1];
        __syncthreads();
    }
    // prefix is the value; k elements equal to it come before the chosen one.
    if (threadIdx.x == 0) {
        int seen = 0, index = -1;
        for (int j = 0; j < n; ++j)
            if (s_key[j] == prefix) {
                if (seen == k) { index = j; break; }
                ++seen;
            }
        static_cast<Real*>(args.core)[base + i] = T::from_key(prefix);
        if (args.core_nbr) args.core_nbr[base + i] = index;
        if (s_overflow) atomic_status(args.status, kOverflow);
    }
}

}  // namespace hdb
