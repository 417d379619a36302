// Thread-block-cluster forward kernel for windows above 1024 points.
//
// Reference path replaced: the same as hdb_forward_kernel
// (hdbscan_gpu/_kernels.py:164-760); the reference runs one block per window
// (hdbscan_gpu/_cuda.py:82-88, 122-127), this kernel spreads the Prim loop of
// one window over the CS CTAs of a cluster.
//
// CTA c of a cluster owns the contiguous vertex range [c*chunk, min(n,
// (c+1)*chunk)), chunk = ceil(n / CS).  Its PT Prim threads keep those
// vertices' coordinates in registers (or, in the matrix variant, read their
// part of row `current` of the distance block), exactly as the single-CTA
// kernel does.  Each Prim iteration ends with one cluster-wide exchange:
//  * the CTA winner (weight key, vertex) comes from the warp argmin and one
//    CTA barrier;
//  * its owner thread sends a record {key, vertex, source, core distance,
//    coordinates} into slot `rank` of every other CTA's record buffer with
//    st.async, whose mbarrier::complete_tx delivers data and signal together
//    (no fence, no round trip), then writes its own copy locally and arrives
//    on its own mbarrier with expect_tx of the CS-1 remote records (one
//    arrival per phase, release at CTA scope);
//  * each Prim thread waits on its local mbarrier (acquire, cluster scope),
//    takes the lexicographic minimum of the CS records and reads the next
//    vertex's coordinates from the local copy of its record, so the next
//    iteration starts without a second round trip.
// Record buffers and mbarriers are double-buffered by exchange parity.  A CTA
// can only send exchange x+2 after it received every CTA's record of x+1, and
// each CTA sends x+1 only after it finished reading the buffers of x, so no
// buffer is overwritten while it is read.
//
// Windows come from the size-sorted queue: CTA rank 0 takes a ticket and
// broadcasts it (DSMEM store + remote mbarrier arrive).  The k-th window of a
// cluster has its home in CTA k % CS: that CTA records the MST edges in its
// arena and its tree warp runs the hierarchy (tree_window) while the cluster
// moves on to windows homed elsewhere, so with one arena per CTA the
// hierarchy of a window overlaps the Prim loops of the next CS-1 windows.
// Two more exchanges per window (before and after Prim) agree on the input
// validation and overflow flags, so every CTA takes the same path.
//
// Every mbarrier wait is bounded (kWaitLimitNs of %globaltimer).  A timeout
// sets the internal-error status and a sticky per-CTA abort flag that makes
// later waits fail at once; control flow (barrier participation, loop trip
// counts, compaction points) never depends on exchanged data, and indices
// read from records are clamped, so an aborted kernel still ends and stays in
// bounds.  All threads of the cluster meet at a hardware cluster barrier
// before exit, so no CTA leaves while another may address its shared memory.
#pragma once
#include "hdb_forward.cuh"

namespace hdb {

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint32_t cluster_ctarank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

// Address of the same shared-memory object in CTA `rank` of the cluster.
__device__ __forceinline__ uint32_t map_rank(uint32_t addr, uint32_t rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
    return r;
}

__device__ __forceinline__ void st_cluster_v4(uint32_t addr, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
    asm volatile("st.shared::cluster.v4.u32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(a), "r"(b), "r"(c), "r"(d)
                 : "memory");
}

// Asynchronous 16-byte store into another CTA's shared memory; its completion
// is a complete_tx of 16 bytes on `bar` (an mbarrier in the same CTA as addr).
__device__ __forceinline__ void st_async_v4(uint32_t addr, uint32_t bar, uint32_t a, uint32_t b, uint32_t c,
                                            uint32_t d) {
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v4.b32 [%0], {%1, %2, %3, %4}, [%5];" ::"r"(addr),
                 "r"(a), "r"(b), "r"(c), "r"(d), "r"(bar)
                 : "memory");
}

// This CTA's one arrival of a phase, announcing `bytes` of remote st.async
// data; orders this thread's earlier shared-memory stores before it.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
    uint64_t state;
    asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 %0, [%1], %2;"
                 : "=l"(state)
                 : "r"(bar), "r"(bytes)
                 : "memory");
    (void)state;
}

__device__ __forceinline__ void st_shared_v4(uint32_t addr, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
    asm volatile("st.shared.v4.u32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(a), "r"(b), "r"(c), "r"(d) : "memory");
}

__device__ __forceinline__ void st_cluster_u32(uint32_t addr, uint32_t v) {
    asm volatile("st.shared::cluster.u32 [%0], %1;" ::"r"(addr), "r"(v) : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Arrive on an mbarrier of any CTA of the cluster; orders this thread's
// earlier stores before the arrival (release, cluster scope).
__device__ __forceinline__ void mbar_arrive_cluster(uint32_t bar) {
    asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ bool mbar_test(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ void cluster_barrier() {
    asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
}

constexpr int64_t kWaitLimitNs = 2000000000ll;  // 2 s: far above any legitimate wait

// Bounded wait for the completion of phase `parity` of a local mbarrier, for
// at most `limit_ns` of %globaltimer (and 2^30 polls).  Returns false when
// this wait or an earlier one of the CTA gave up.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int* abort_flag,
                                          int64_t limit_ns) {
    if (mbar_test(bar, parity)) return true;
    if (*abort_flag) return false;
    const int64_t t0 = global_ns();
    for (int spin = 0; spin < (1 << 30); ++spin) {
        if (mbar_test(bar, parity)) return true;
        if ((spin & 31) == 31) {
            if (*abort_flag) return false;
            if (global_ns() - t0 > limit_ns) break;
        }
    }
    *abort_flag = 1;
    return false;
}

// Exchange record: a header, then DP coordinates (none in the matrix variant).
//   float32 header (16 B): key u32 | vertex u16, source u16 | core f32 | flags u32
//   float64 header (32 B): key u64 | vertex u16, source u16 | flags u32 | core f64 | pad
template <typename Real, int DP>
struct Record {
    static constexpr int kHeader = sizeof(Real) == 4 ? 16 : 32;
    static constexpr int kBytes = kHeader + DP * (int)sizeof(Real);
    static constexpr int kCoreOff = sizeof(Real) == 4 ? 8 : 16;
};

// Sends one record (header, then NC coordinates; NC = 0 for header-only
// records, whose coordinate bytes are then zero) to slot `slot` (a shared
// address valid in every CTA) of every CTA of the cluster: st.async to the
// others, plain stores locally, then this CTA's arrival on full[p].
template <typename Real, int DP, int CS, int NC>
__device__ __forceinline__ void send_record(uint32_t slot, uint32_t bar, uint32_t rank,
                                            typename RealTraits<Real>::Bits key, uint32_t vs, uint32_t flags,
                                            Real core, const Real* x) {
    constexpr int kWords = Record<Real, DP>::kBytes / 16;
    constexpr int kHeaderWords = Record<Real, DP>::kHeader / 16;
    auto word = [&](int i, uint32_t (&q)[4]) {
        if (i < kHeaderWords) {
            if constexpr (sizeof(Real) == 4) {
                q[0] = key; q[1] = vs; q[2] = __float_as_uint(core); q[3] = flags;
            } else {
                const unsigned long long c = (unsigned long long)__double_as_longlong(core);
                if (i == 0) { q[0] = (uint32_t)key; q[1] = (uint32_t)(key >> 32); q[2] = vs; q[3] = flags; }
                else { q[0] = (uint32_t)c; q[1] = (uint32_t)(c >> 32); q[2] = 0u; q[3] = 0u; }
            }
        } else {
            const int k = (i - kHeaderWords) * (16 / (int)sizeof(Real));
            if constexpr (sizeof(Real) == 4) {
                q[0] = NC ? __float_as_uint(x[k]) : 0u; q[1] = NC ? __float_as_uint(x[k + 1]) : 0u;
                q[2] = NC ? __float_as_uint(x[k + 2]) : 0u; q[3] = NC ? __float_as_uint(x[k + 3]) : 0u;
            } else {
                const unsigned long long a = NC ? (unsigned long long)__double_as_longlong(x[k]) : 0ull;
                const unsigned long long b = NC ? (unsigned long long)__double_as_longlong(x[k + 1]) : 0ull;
                q[0] = (uint32_t)a; q[1] = (uint32_t)(a >> 32); q[2] = (uint32_t)b; q[3] = (uint32_t)(b >> 32);
            }
        }
    };
#pragma unroll
    for (uint32_t d = 1; d < (uint32_t)CS; ++d) {
        const uint32_t r = (rank + d) % (uint32_t)CS;
        const uint32_t dst = map_rank(slot, r), rbar = map_rank(bar, r);
#pragma unroll
        for (int i = 0; i < kWords; ++i) {
            uint32_t q[4];
            word(i, q);
            st_async_v4(dst + 16 * i, rbar, q[0], q[1], q[2], q[3]);
        }
    }
#pragma unroll
    for (int i = 0; i < kWords; ++i) {
        uint32_t q[4];
        word(i, q);
        st_shared_v4(slot + 16 * i, q[0], q[1], q[2], q[3]);
    }
    mbar_arrive_expect_tx(bar, (uint32_t)((CS - 1) * Record<Real, DP>::kBytes));
}

// Shared state of one cluster CTA.  The two flag words of a window (input
// validation, then overflow) are separate and double-buffered by window
// parity: thread 0 resets the pair of window k while a slow thread may still
// read the result of window k-1, and a late read of the validation result can
// never see overflow bits of the same window.
struct ClusterShared {
    uint32_t recs;       // shared address of the record buffers [2][CS]
    uint32_t full0;      // shared address of mbarrier full[0] (full[1] = +8)
    unsigned char* recs_ptr;
    unsigned char* rec0;  // local record of vertex 0 (first current vertex)
    volatile int* abort_flag;
    int64_t wait_limit;   // ns, every mbarrier wait
    int* vflags;          // this window's validation flags
    int* oflags;          // this window's overflow flags
    int* xc_out;
};

// One exchange of a header-only record carrying `flags` (thread 0 only);
// returns the OR of all CTAs' flags.  Bit 4 (internal) is added on timeout.
template <typename Real, int DP, int CS>
__device__ __forceinline__ int exchange_flags(const ClusterShared& cs, uint32_t rank, uint32_t xc, int flags) {
    using Rec = Record<Real, DP>;
    const uint32_t p = xc & 1, ph = (xc >> 1) & 1;
    const uint32_t slot = cs.recs + (p * CS + rank) * Rec::kBytes;
    send_record<Real, DP, CS, 0>(slot, cs.full0 + 8 * p, rank, (typename RealTraits<Real>::Bits)0, 0u,
                                 (uint32_t)flags, Real(0), nullptr);
    int all = 0;
    if (!mbar_wait(cs.full0 + 8 * p, ph, cs.abort_flag, cs.wait_limit)) all |= 4;
#pragma unroll
    for (int r = 0; r < CS; ++r) {
        const unsigned char* rp = cs.recs_ptr + (p * CS + r) * Rec::kBytes;
        all |= (int)*reinterpret_cast<const volatile uint32_t*>(rp + (sizeof(Real) == 4 ? 12 : 12));
    }
    return all;
}

// Prim over one window by one CTA of the cluster (reference
// _kernels.py:164-320), sandwiched between the validation and overflow
// exchanges.  Returns the cluster-wide flags (1 non-finite input, 2 overflow,
// 4 internal); the home CTA has written edge `it` into `arena` for every
// iteration when the result is 0.
template <typename Real, int PT, int SV, int DP, int CS, bool UNIT, typename Key>
__device__ __forceinline__ int cluster_window(const ForwardArgs& args, const ClusterShared& cs, uint32_t rank,
                                              uint32_t& xc, int w, int n, bool home, bool wait_empty,
                                              const Arena<Real>& arena, Real* stage_best, int16_t* stage_j,
                                              int16_t* stage_src, Key (*s_key)[PT / 32], uint32_t (*s_idx)[PT / 32],
                                              int* s_scan) {
    using T = RealTraits<Real>;
    using Rec = Record<Real, DP>;
    constexpr int PW = PT / 32;
    constexpr int VEC = 16 / (int)sizeof(Real);
    constexpr int DPS = DP > 0 ? DP : VEC;
    constexpr int L = PT * SV;
    constexpr Key SENTINEL = (Key)~(Key)0;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int D = args.D;
    const int64_t base = args.offsets[w];
    const Real* __restrict__ Xw = static_cast<const Real*>(args.X) + base * D;
    const Real* __restrict__ core_w = UNIT ? nullptr : static_cast<const Real*>(args.core) + base;
    const Real* __restrict__ Dw = DP > 0 ? nullptr : static_cast<const Real*>(args.dist) + args.dist_offsets[w];
    const int64_t ld = (n + 3) & ~3;

    const int chunk = (n + CS - 1) / CS;
    const int lo = min(n, (int)rank * chunk);
    const int hi = min(n, lo + chunk);

    // ---- slots and validation ------------------------------------------------
    // Slot layout as in hdb_forward.cuh: lane-major for the matrix variant
    // (coalesced row reads), thread-major for the register variants.
    constexpr bool kLaneMajor = DP == 0;
    auto slot_of = [&](int v) { return kLaneMajor ? warp * 32 * SV + v * 32 + lane : tid * SV + v; };
    Real xr[SV][DPS];
    Real best[SV], thr[SV], core_r[SV];
    int src[SV], vid[SV];
    bool act[SV];
    int bad = (chunk > L || (DP > 0 && D > DP)) ? 4 : 0;  // the plan never sends such a window here
    auto load_slot = [&](int v, int j) {
        if constexpr (DP > 0) {
#pragma unroll
            for (int k = 0; k < DPS; ++k) xr[v][k] = (j >= 0 && k < D) ? Xw[(int64_t)j * D + k] : Real(0);
        }
        if (!UNIT) core_r[v] = j >= 0 ? core_w[j] : Real(0);
    };
#pragma unroll
    for (int v = 0; v < SV; ++v) {
        const int j = lo + slot_of(v);
        const bool valid = slot_of(v) < L && j < hi;
        vid[v] = valid ? j : -1;
        act[v] = valid && j != 0;  // vertex 0 starts the tree (_kernels.py:210-213)
        best[v] = T::inf();
        thr[v] = T::inf();
        src[v] = 1;  // reference initial source (_kernels.py:167)
        core_r[v] = Real(0);
        load_slot(v, vid[v]);
        if constexpr (DP > 0) {
#pragma unroll
            for (int k = 0; k < DPS; ++k) bad |= !isfinite(xr[v][k]);
        }
    }
    if constexpr (DP == 0) {
        for (int64_t t = (int64_t)lo * D + tid; t < (int64_t)hi * D; t += PT) bad |= !isfinite(Xw[t]);
    }
    // Record of vertex 0, the first current vertex, in every CTA.
    Real* r0x = reinterpret_cast<Real*>(cs.rec0 + Rec::kHeader);
    if (DP > 0 && tid < DP) r0x[tid] = tid < D ? Xw[tid] : Real(0);
    if (tid == 0) *reinterpret_cast<Real*>(cs.rec0 + Rec::kCoreOff) = UNIT ? Real(0) : core_w[0];
    if (bad) atomicOr(cs.vflags, bad);
    bar_sync(kBarStart, PT);
    if (tid == 0) *cs.vflags = exchange_flags<Real, DP, CS>(cs, rank, xc, *cs.vflags);
    ++xc;
    if (home && wait_empty) bar_sync(kBarEmpty, PT + 32);  // arena released by the tree warp
    bar_sync(kBarStart, PT);
    const int vflags = *cs.vflags;  // final for this window: every thread reads the same value
    if (vflags) return vflags;      // every CTA saw the same records
    if (home && args.stage_ns && tid == 0) args.stage_ns[8 * w + 1] = global_ns();

    // ---- Prim ------------------------------------------------------------------
    int overflow = 0;  // 2 = a distance overflowed, 4 = internal inconsistency
    Real acc_max = Real(0);
    int live = hi - lo;
    int aw = (live + 32 * SV - 1) / (32 * SV);
    aw = aw < 1 ? 1 : (aw > PW ? PW : aw);
    const unsigned char* cur_rec = cs.rec0;
    int cur = 0;
    if (warp < aw) {
        for (int it = 0; it < n - 1; ++it) {
            if (it > 0 && (it & 31) == 0) {
                // ---- compaction checkpoint (CTA-uniform decision) -------------
                // Live vertices are staged in slot order and re-packed into
                // slots [0, live).
                unsigned bal[SV];
                int count = 0;
#pragma unroll
                for (int v = 0; v < SV; ++v) {
                    bal[v] = __ballot_sync(0xffffffffu, act[v]);
                    count += kLaneMajor ? __popc(bal[v]) : (act[v] ? 1 : 0);
                }
                int total = 0;
                int pos = active_exclusive_scan(kLaneMajor ? (lane == 0 ? count : 0) : count, aw, s_scan, total);
                if (live - total >= 32 * SV) {
                    if constexpr (kLaneMajor) {
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
                    bar_sync(kBarIter, aw * 32);  // staging may be rewritten afterwards
                    const int naw = (live + 32 * SV - 1) / (32 * SV);
                    aw = naw < 1 ? 1 : naw;
                    if (warp >= aw) break;  // warp-uniform
                }
            }
            const Real core_cur = UNIT ? Real(0) : *reinterpret_cast<const Real*>(cur_rec + Rec::kCoreOff);
            Real acc[SV];
            if constexpr (DP > 0) {
                const Real* cx = reinterpret_cast<const Real*>(cur_rec + Rec::kHeader);
#pragma unroll
                for (int v = 0; v < SV; ++v) acc[v] = Real(0);
#pragma unroll
                for (int k0 = 0; k0 < DPS; k0 += VEC) {
                    Real c[VEC];
                    if constexpr (sizeof(Real) == 4) {
                        const float4 q = *reinterpret_cast<const float4*>(cx + k0);
                        c[0] = q.x; c[1 % VEC] = q.y; c[2 % VEC] = q.z; c[3 % VEC] = q.w;
                    } else {
                        const double2 q = *reinterpret_cast<const double2*>(cx + k0);
                        c[0] = q.x; c[1 % VEC] = q.y;
                    }
#pragma unroll
                    for (int v = 0; v < SV; ++v) {
                        if constexpr (sizeof(Real) == 4) {
                            // Packed differences (fma(c, -1, x) = RN(x - c)) and
                            // squares; scalar k-ordered sum, as in hdb_forward.cuh.
#pragma unroll
                            for (int kk = 0; kk < VEC; kk += 2) {
                                const float2 delta =
                                    __ffma2_rn(make_float2(c[kk], c[kk + 1]), make_float2(-1.0f, -1.0f),
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
                const Real* __restrict__ row = Dw + (int64_t)cur * ld;
#pragma unroll
                for (int v = 0; v < SV; ++v) acc[v] = __ldcg(row + (act[v] ? vid[v] : 0));
            }
            Key lkey = SENTINEL;
            uint32_t lidx = 0xffffffffu;
#pragma unroll
            for (int v = 0; v < SV; ++v) {
                if constexpr (DP > 0) {
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
                        overflow |= T::finite_nn(d) ? 0 : 2;
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

            // ---- cluster exchange ---------------------------------------------
            const uint32_t p = xc & 1, ph = (xc >> 1) & 1;
            ++xc;
            const uint32_t slot = cs.recs + (p * CS + rank) * Rec::kBytes;
            if (!key_eq(gk, SENTINEL)) {
#pragma unroll
                for (int v = 0; v < SV; ++v) {
                    if (act[v] && vid[v] == (int)gi) {
                        const uint32_t vs = (gi & 0xffffu) | ((uint32_t)src[v] << 16);
                        send_record<Real, DP, CS, DP>(slot, cs.full0 + 8 * p, rank, gk, vs, 0u, core_r[v], xr[v]);
                    }
                }
            } else if (tid == 0) {
                send_record<Real, DP, CS, 0>(slot, cs.full0 + 8 * p, rank, SENTINEL, 0xffffffffu, 0u, Real(0),
                                             nullptr);
            }
            if (!mbar_wait(cs.full0 + 8 * p, ph, cs.abort_flag, cs.wait_limit)) overflow |= 4;
            Key wk = SENTINEL;
            uint32_t wv = 0xffffffffu;
            int wr = 0;
#pragma unroll
            for (int r = 0; r < CS; ++r) {
                const unsigned char* rp = cs.recs_ptr + (p * CS + r) * Rec::kBytes;
                const Key k = *reinterpret_cast<const Key*>(rp);
                const uint32_t vs = *reinterpret_cast<const uint32_t*>(rp + sizeof(Key));
                if (key_idx_lt(k, vs & 0xffffu, wk, wv & 0xffffu)) { wk = k; wv = vs; wr = r; }
            }
            int next = (int)(wv & 0xffffu);
            if (key_eq(wk, SENTINEL) || next >= n) {  // unreachable: a non-tree vertex always remains
                overflow |= 4;
                next = 0;
            }
#pragma unroll
            for (int v = 0; v < SV; ++v)
                if (act[v] && vid[v] == next) act[v] = false;
            if (home && tid == 0) {
                int s = (int)(wv >> 16);
                arena.s0[it] = (int16_t)(s < n ? s : 0);
                arena.s1[it] = (int16_t)next;
                arena.r0[it] = T::from_key(wk);
            }
            cur_rec = cs.recs_ptr + (p * CS + wr) * Rec::kBytes;
            cur = next;
        }
    }
    if (DP > 0) overflow |= (acc_max <= T::kMax) ? 0 : 2;
    if (tid == 0) *cs.xc_out = (int)xc;  // warp 0 always runs every iteration
    if (overflow) atomicOr(cs.oflags, overflow);
    bar_sync(kBarStart, PT);
    xc = (uint32_t)*cs.xc_out;
    if (tid == 0) *cs.oflags = exchange_flags<Real, DP, CS>(cs, rank, xc, *cs.oflags);
    ++xc;
    bar_sync(kBarStart, PT);
    return *cs.oflags;
}

// Dynamic shared memory: one arena (arena_stride bytes), the record buffers
// [2][CS] plus the vertex-0 record, then the compaction staging of PT*SV slots.
template <typename Real, int PT, int SV, int DP, int CS>
__global__ void __launch_bounds__(PT + 32, 1) hdb_cluster_forward_kernel(const __grid_constant__ ForwardArgs args) {
    using T = RealTraits<Real>;
    using Key = typename T::Bits;
    using Rec = Record<Real, DP>;
    constexpr int PW = PT / 32;
    constexpr int L = PT * SV;
    static_assert(CS >= 2 && CS <= 8, "portable cluster sizes");
    static_assert(PT % 32 == 0 && PT + 32 <= 1024, "Prim threads plus the tree warp must fit one CTA");
    static_assert(DP == 0 || DP % (16 / (int)sizeof(Real)) == 0, "DP must be a multiple of one 16-byte vector");
    static_assert(DP <= PT, "vertex-0 record is loaded one coordinate per thread");

    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ Key s_key[2][PW];
    __shared__ uint32_t s_idx[2][PW];
    __shared__ int s_scan[32];
    __shared__ __align__(8) uint64_t s_full[2];
    __shared__ __align__(8) uint64_t s_item_bar;
    __shared__ int s_item[2];
    __shared__ int s_vflags[2];
    __shared__ int s_oflags[2];
    __shared__ int s_xc;
    __shared__ int s_abort;
    __shared__ WindowMeta s_meta;

    const int tid = threadIdx.x;
    const int warp = tid >> 5;
    const uint32_t rank = cluster_ctarank();

    ClusterShared cs;
    cs.recs_ptr = smem + args.arena_stride;
    cs.recs = smem_u32(cs.recs_ptr);
    cs.rec0 = cs.recs_ptr + 2 * CS * Rec::kBytes;
    cs.full0 = smem_u32(&s_full[0]);
    cs.abort_flag = &s_abort;
    cs.wait_limit = args.wait_limit_ns > 0 ? args.wait_limit_ns : kWaitLimitNs;
    cs.vflags = &s_vflags[0];
    cs.oflags = &s_oflags[0];
    cs.xc_out = &s_xc;
    Real* stage_best = reinterpret_cast<Real*>(cs.rec0 + ((Rec::kBytes + 15) & ~15));
    int16_t* stage_j = reinterpret_cast<int16_t*>(stage_best + L);
    int16_t* stage_src = stage_j + L;

    if (tid == 0) {
        mbar_init(&s_full[0], 1);  // one local arrival (with expect_tx) per phase
        mbar_init(&s_full[1], 1);
        mbar_init(&s_item_bar, 1);
        s_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    cluster_barrier();  // every CTA's mbarriers exist before the first remote arrive

    if (warp == PW) {
        // ======== tree warp: the hierarchy of the windows homed here ==========
        for (int k = 0; k < (1 << 30); ++k) {
            bar_sync(kBarFull, PT + 32);
            const WindowMeta meta = s_meta;
            if (meta.w < 0) break;
            if (!meta.skip) tree_window<Real>(args, smem, meta.w, meta.n);
            __syncwarp();
            __threadfence_block();
            bar_arrive(kBarEmpty, PT + 32);
        }
        cluster_barrier();
        return;
    }

    // ============================ Prim threads =================================
    uint32_t xc = 0;  // exchange counter, identical in every CTA of the cluster
    int homes = 0;
    for (int k = 0; k < (1 << 30); ++k) {
        if (rank == 0 && tid == 0 && !(args.stall_first_ticket && k == 0)) {
            const int item = s_abort ? args.queue_len : atomicAdd(args.ticket, 1);
#pragma unroll
            for (uint32_t r = 0; r < (uint32_t)CS; ++r) {
                st_cluster_u32(map_rank(smem_u32(&s_item[k & 1]), r), (uint32_t)item);
                mbar_arrive_cluster(map_rank(smem_u32(&s_item_bar), r));
            }
        }
        if (tid == 0) {
            if (!mbar_wait(smem_u32(&s_item_bar), k & 1, &s_abort, cs.wait_limit)) {
                atomic_status(args.status, kInternal);
                s_item[k & 1] = args.queue_len;
            }
            s_vflags[k & 1] = 0;
            s_oflags[k & 1] = 0;
        }
        cs.vflags = &s_vflags[k & 1];
        cs.oflags = &s_oflags[k & 1];
        bar_sync(kBarStart, PT);
        const int item = s_item[k & 1];
        const bool home = (k % CS) == (int)rank;
        if (item < 0 || item >= args.queue_len) {
            if (homes > 0) bar_sync(kBarEmpty, PT + 32);
            if (tid == 0) s_meta.w = -1;
            __threadfence_block();
            bar_arrive(kBarFull, PT + 32);
            break;
        }
        const int w = args.queue[item];
        const int64_t base = args.offsets[w];
        const int n = (int)(args.offsets[w + 1] - base);
        if (home && args.stage_ns && tid == 0) args.stage_ns[8 * w + 0] = global_ns();
        Arena<Real> arena = Arena<Real>::carve(smem, n);
        const bool wait_empty = home && homes > 0;
        int flags;
        if (args.unit_core)
            flags = cluster_window<Real, PT, SV, DP, CS, true>(args, cs, rank, xc, w, n, home, wait_empty, arena,
                                                               stage_best, stage_j, stage_src, s_key, s_idx, s_scan);
        else
            flags = cluster_window<Real, PT, SV, DP, CS, false>(args, cs, rank, xc, w, n, home, wait_empty, arena,
                                                                stage_best, stage_j, stage_src, s_key, s_idx, s_scan);
        if (!home) continue;
        ++homes;
        if (args.stage_ns && tid == 0) args.stage_ns[8 * w + 2] = global_ns();
        int skip = 0;
        if (flags) {
            const int code = (flags & 1) ? kNonFinite : ((flags & 4) ? kInternal : kOverflow);
            if (tid == 0) atomic_status(args.status, code);
            for (int j = tid; j < n; j += PT) args.labels[base + j] = -1;
            skip = 1;
        }
        if (tid == 0) { s_meta.w = w; s_meta.n = n; s_meta.skip = skip; }
        __threadfence_block();
        bar_arrive(kBarFull, PT + 32);
    }
    cluster_barrier();
}

}  // namespace hdb
