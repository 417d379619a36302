// Hierarchy stages of one window, run by ONE warp (the tree warp of the
// forward kernel) on a shared-memory arena: exact NumPy-order introsort ->
// union-find single linkage -> breadth-first condensation -> excess of mass
// -> epsilon merge -> labels.
//
// Semantics follow the reference kernels (hdbscan_gpu/_kernels.py) stage by
// stage; each function cites the lines it reproduces.  The parallel
// decompositions are this project's own:
//  * the introsort runs every Hoare partition warp-parallel.  For a segment
//    whose pivot sits at hi-1, let A be the ascending positions in
//    [lo+1, hi-1] holding w >= pivot (where the i scan stops) and B the
//    descending positions in [lo, hi-2] holding w <= pivot (where the j scan
//    stops).  The serial loop swaps A[k] with B[k] exactly while A[k] < B[k],
//    i.e. an A-stopper of rank k swaps iff more than k B-stoppers lie to its
//    right (and symmetrically for B), and stops at i = min(A[K], B[K-1]) for
//    K swaps.  Ranks come from ballots, so each partition is two passes over
//    the segment plus K/32 swap rounds, with NumPy's exact swap sequence.
//    Segments shorter than a threshold (m/16 clamped to [32, 128]) and
//    depth-exhausted heapsort segments are finished one per lane by the
//    serial algorithm itself (partitions, stack, insertion sort, heapsort);
//    segments are disjoint, so the order in which they finish is irrelevant;
//  * windows whose edge weights are all distinct are sorted by a stable warp
//    LSD radix sort instead (the argsort of distinct keys is unique, so it
//    equals NumPy's); a window with any tied weight falls back to the exact
//    introsort above;
//  * linkage uses union by size over packed 32-bit word pairs
//    {parent | component node << 16, size} without path compression;
//    the roots, hence the tree, are those of the reference's union-find.
//    Batches of 32 edges find their roots in parallel, then one lane
//    commits the unions in order (fixing up roots merged within the batch).
//  * condensation runs the reference's breadth-first queue one level at a
//    time across the warp: every cluster is a path of the dendrogram (it only
//    branches where it ends in a split), so the nodes of one level belong to
//    distinct clusters and each lane's stability sum keeps the reference's
//    addition order; split children take consecutive ids by a ballot prefix
//    over the level, i.e. in queue order.  Pruned points find their cluster
//    afterwards from their lowest large ancestor.
//  * selection uses the binary shape of the condensed tree (every split
//    creates exactly two consecutive ids), as the reference's
//    COOPERATIVE_BINARY_EOM variant does (_kernels.py:648-669), and runs its
//    serial passes in chunks of 32 cluster ids, one lane per cluster, each
//    lane waiting (by ballot) only for its parent or children.
#pragma once
#include "hdb_common.cuh"

namespace hdb {

template <typename Real> struct SortPair;
template <> struct __align__(8) SortPair<float> { float w; int32_t idx; };
template <> struct __align__(16) SortPair<double> { double w; int64_t idx; };

// Shared-memory arena for one window of capacity `cap` points (cap >= n).
//  r0  Real[cap]  Prim edge weights -> weights in sorted order (merge weights)
//  r1  Real[cap]  \  SortPair[cap] during the sort -> union-find words during
//  r2  Real[cap]  /  linkage -> cluster birth (r1) and stability (r2)
//  s0  i16[cap]   Prim edge source  -> prune queue [0, cap)
//  s1  i16[cap]   Prim edge target  -> prune queue [cap, 2cap)
//  s2  i16[cap]   sorted order -> sorted sources -> cluster parent
//  s3  i16[cap]   sort swap list A -> sorted targets -> first child
//  s4  i16[cap]   sort swap list B -> linkage left -> EOM blocked
//  s5  i16[cap]   task lo -> linkage right -> epsilon stop
//  s6  i16[cap]   task hi -> linkage size -> label map
//  s7  i16[cap]   task depth -> relabel -> resolved label
//  s8  i16[cap]   leaf lo -> BFS queue
//  s9  i16[cap]   leaf hi -> point parent
//  sel u8[cap]    cluster selected flag
template <typename Real> struct Arena {
    Real *r0, *r1, *r2;
    int16_t *s0, *s1, *s2, *s3, *s4, *s5, *s6, *s7, *s8, *s9;
    uint8_t* sel;

    __host__ __device__ static int round_cap(int n) { return (n + 7) & ~7; }
    __host__ __device__ static size_t bytes(int n) {
        const size_t cap = (size_t)round_cap(n);
        return (3 * cap * sizeof(Real) + 10 * cap * sizeof(int16_t) + cap + 15) & ~size_t(15);
    }
    __device__ static Arena carve(void* base, int n) {
        Arena a;
        const int cap = round_cap(n);
        Real* r = reinterpret_cast<Real*>(base);
        a.r0 = r;
        a.r1 = r + cap;
        a.r2 = r + 2 * cap;
        int16_t* s = reinterpret_cast<int16_t*>(r + 3 * cap);
        a.s0 = s; a.s1 = s + cap; a.s2 = s + 2 * cap; a.s3 = s + 3 * cap; a.s4 = s + 4 * cap;
        a.s5 = s + 5 * cap; a.s6 = s + 6 * cap; a.s7 = s + 7 * cap; a.s8 = s + 8 * cap; a.s9 = s + 9 * cap;
        a.sel = reinterpret_cast<uint8_t*>(s + 10 * cap);
        return a;
    }
};

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// ---------------------------------------------------------------------------
// Introsort (reference: _kernels.py:358-516; NumPy 2.3.5 aquicksort).
// ---------------------------------------------------------------------------
template <typename Real>
__device__ void heap_sort_pairs(SortPair<Real>* p, int lo, int hi) {
    const int count = hi - lo + 1;
    SortPair<Real>* a = p + lo - 1;  // 1-based
    for (int root = count / 2; root >= 1; --root) {
        SortPair<Real> value = a[root];
        int pos = root, child = 2 * root;
        while (child <= count) {
            if (child < count && RealTraits<Real>::lt(a[child].w, a[child + 1].w)) ++child;
            if (RealTraits<Real>::lt(value.w, a[child].w)) { a[pos] = a[child]; pos = child; child *= 2; } else break;
        }
        a[pos] = value;
    }
    for (int end = count; end > 1;) {
        SortPair<Real> value = a[end];
        a[end] = a[1];
        --end;
        int pos = 1, child = 2;
        while (child <= end) {
            if (child < end && RealTraits<Real>::lt(a[child].w, a[child + 1].w)) ++child;
            if (RealTraits<Real>::lt(value.w, a[child].w)) { a[pos] = a[child]; pos = child; child *= 2; } else break;
        }
        a[pos] = value;
    }
}

template <typename Real>
__device__ void insertion_sort_pairs(SortPair<Real>* p, int lo, int hi) {
    for (int i = lo + 1; i <= hi; ++i) {
        SortPair<Real> value = p[i];
        int j = i;
        while (j > lo && RealTraits<Real>::lt(value.w, p[j - 1].w)) { p[j] = p[j - 1]; --j; }
        p[j] = value;
    }
}

template <typename Real>
__device__ __forceinline__ void swap_pairs(SortPair<Real>* p, int i, int j) {
    SortPair<Real> t = p[i]; p[i] = p[j]; p[j] = t;
}

// One Hoare partition of p[lo..hi] (hi - lo > 15) by one lane: NumPy's
// median-of-three, pivot parked at hi-1, unguarded i/j scans (p[hi-1] and
// p[lo] are the sentinels) and the final swap (_kernels.py:444-462).
template <typename Real>
__device__ int partition_serial(SortPair<Real>* p, int lo, int hi) {
    const int mid = lo + ((hi - lo) >> 1);
    if (RealTraits<Real>::lt(p[mid].w, p[lo].w)) swap_pairs(p, mid, lo);
    if (RealTraits<Real>::lt(p[hi].w, p[mid].w)) swap_pairs(p, hi, mid);
    if (RealTraits<Real>::lt(p[mid].w, p[lo].w)) swap_pairs(p, mid, lo);
    swap_pairs(p, mid, hi - 1);
    const Real pivot = p[hi - 1].w;
    int i = lo, j = hi - 1;
    for (;;) {
        do ++i; while (RealTraits<Real>::lt(p[i].w, pivot));
        do --j; while (RealTraits<Real>::lt(pivot, p[j].w));
        if (i >= j) break;
        swap_pairs(p, i, j);
    }
    swap_pairs(p, i, hi - 1);
    return i;
}

// Segments shorter than this many elements (or depth-exhausted) are sorted by
// one lane.  The lane's stack holds the larger sides while the loop continues
// on the smaller one, so a segment of s elements never stacks more than
// log2(s/16) + 1 entries.
constexpr int kLaneSortMax = 128;
constexpr int kLaneStack = 8;
static_assert((kLaneSortMax >> (kLaneStack - 1)) <= 16, "lane introsort stack too small");

// NumPy's aquicksort loop on one segment by one lane.  code = depth*2 +
// checked: a checked segment with negative depth is heapsorted (the check a
// popped segment gets); an unchecked one (the smaller side that the loop
// continues on) is partitioned first (_kernels.py:433-470).
template <typename Real>
__device__ void introsort_lane(SortPair<Real>* p, int lo, int hi, int code) {
    int depth = code >> 1;  // arithmetic shift keeps negative depths
    bool checked = code & 1;
    int st_lo[kLaneStack], st_hi[kLaneStack], st_depth[kLaneStack];
    int top = 0;
    for (;;) {
        if (checked && depth < 0) {
            heap_sort_pairs(p, lo, hi);
        } else {
            while (hi - lo > 15) {
                const int i = partition_serial(p, lo, hi);
                --depth;
                if (i - lo < hi - i) { st_lo[top] = i + 1; st_hi[top] = hi; hi = i - 1; }
                else { st_lo[top] = lo; st_hi[top] = i - 1; lo = i + 1; }
                st_depth[top++] = depth;
            }
            insertion_sort_pairs(p, lo, hi);
        }
        if (top == 0) return;
        --top;
        lo = st_lo[top]; hi = st_hi[top]; depth = st_depth[top]; checked = true;
    }
}

// One Hoare partition of p[lo..hi] (hi - lo > 15) by the whole warp.
// Returns the pivot's final position (warp-uniform).
template <typename Real>
__device__ int partition_warp(SortPair<Real>* p, int lo, int hi, int16_t* list_a, int16_t* list_b) {
    const int lane = threadIdx.x & 31;
    if (lane == 0) {
        const int mid = lo + ((hi - lo) >> 1);
        if (RealTraits<Real>::lt(p[mid].w, p[lo].w)) swap_pairs(p, mid, lo);
        if (RealTraits<Real>::lt(p[hi].w, p[mid].w)) swap_pairs(p, hi, mid);
        if (RealTraits<Real>::lt(p[mid].w, p[lo].w)) swap_pairs(p, mid, lo);
        swap_pairs(p, mid, hi - 1);
    }
    __syncwarp();
    const Real pivot = p[hi - 1].w;
    // Pass 1: stopper totals.
    int total_a = 0, total_b = 0;
    for (int base = lo; base <= hi - 1; base += 32) {
        const int pos = base + lane;
        bool fa = false, fb = false;
        if (pos <= hi - 1) {
            const Real w = p[pos].w;
            fa = pos >= lo + 1 && !RealTraits<Real>::lt(w, pivot);
            fb = pos <= hi - 2 && !RealTraits<Real>::lt(pivot, w);
        }
        total_a += __popc(__ballot_sync(0xffffffffu, fa));
        total_b += __popc(__ballot_sync(0xffffffffu, fb));
    }
    // Pass 2: ranks, swap decisions, swap lists, first non-swapping A.
    int run_a = 0, run_b = 0, swaps = 0, first_stop = -1;
    const unsigned lt = lanemask_lt();
    for (int base = lo; base <= hi - 1; base += 32) {
        const int pos = base + lane;
        bool fa = false, fb = false;
        if (pos <= hi - 1) {
            const Real w = p[pos].w;
            fa = pos >= lo + 1 && !RealTraits<Real>::lt(w, pivot);
            fb = pos <= hi - 2 && !RealTraits<Real>::lt(pivot, w);
        }
        const unsigned ba = __ballot_sync(0xffffffffu, fa);
        const unsigned bb = __ballot_sync(0xffffffffu, fb);
        const int a_before = run_a + __popc(ba & lt);          // A-stoppers left of pos
        const int b_upto = run_b + __popc(bb & (lt | (1u << lane)));
        const int b_after = total_b - b_upto;                   // B-stoppers right of pos
        const bool swap_a = fa && b_after > a_before;
        const bool swap_b = fb && a_before > b_after;
        if (swap_a) list_a[lo + a_before] = (int16_t)pos;
        if (swap_b) list_b[lo + b_after] = (int16_t)pos;
        swaps += __popc(__ballot_sync(0xffffffffu, swap_a));
        const unsigned stop = __ballot_sync(0xffffffffu, fa && !swap_a);
        if (first_stop < 0 && stop) first_stop = base + __ffs(stop) - 1;
        run_a += __popc(ba);
        run_b += __popc(bb);
    }
    __syncwarp();
    for (int k = lane; k < swaps; k += 32) swap_pairs(p, list_a[lo + k], list_b[lo + k]);
    __syncwarp();
    int i = first_stop;
    if (swaps > 0) {
        const int last_b = list_b[lo + swaps - 1];
        i = last_b < i ? last_b : i;
    }
    if (lane == 0) swap_pairs(p, i, hi - 1);
    __syncwarp();
    return i;
}

// Lanes holding the same 8-bit digit (bit 8 marks an invalid lane, whose
// mask is never used): one ballot per digit bit, each lane keeping the lanes
// that agree with it on every bit (the warp multisplit form of match.any,
// which is far slower on this GPU).
__device__ __forceinline__ unsigned same_digit_lanes(int d) {
    unsigned same = 0xffffffffu;
#pragma unroll
    for (int b = 0; b < 9; ++b) {
        const unsigned bits = __ballot_sync(0xffffffffu, (d >> b) & 1);
        same &= ((d >> b) & 1) ? bits : ~bits;
    }
    return same;
}

__device__ __forceinline__ int radix_digit(uint32_t k, int shift) { return (int)((k >> shift) & 0xffu); }
__device__ __forceinline__ int radix_digit(unsigned long long k, int shift) {
    const uint32_t w = shift < 32 ? (uint32_t)k : (uint32_t)(k >> 32);
    return (int)((w >> (shift & 31)) & 0xffu);
}

// Stable LSD radix sort (8-bit digits) of the order-preserving keys of
// r0[0..m) with their indices, by one warp.  Returns false, leaving r0 intact,
// when two keys are equal; otherwise writes the order to s2 and the sorted
// weights to r0.  Needs m >= 256 (the digit histogram lives in s5..s6).
template <typename Real>
__device__ bool radix_sort_distinct_warp(const Arena<Real>& a, int m) {
    using T = RealTraits<Real>;
    using Key = typename T::Bits;
    constexpr int kPasses = (int)sizeof(Key);
    const int lane = threadIdx.x & 31;
    const unsigned lt = lanemask_lt();
    Key* kin = reinterpret_cast<Key*>(a.r1);
    Key* kout = reinterpret_cast<Key*>(a.r2);
    int16_t* iin = a.s3;
    int16_t* iout = a.s4;
    int* hist = reinterpret_cast<int*>(a.s5);
    for (int i = lane; i < m; i += 32) { kin[i] = T::key(a.r0[i]); iin[i] = (int16_t)i; }
    __syncwarp();
    for (int pass = 0; pass < kPasses; ++pass) {
        const int shift = 8 * pass;
#pragma unroll
        for (int b = 0; b < 8; ++b) hist[8 * lane + b] = 0;
        __syncwarp();
        for (int i = lane; i < m; i += 32) atomicAdd(&hist[radix_digit(kin[i], shift)], 1);
        __syncwarp();
        // Exclusive scan; each lane owns 8 consecutive digits.
        int local[8], sum = 0, full = 0;
#pragma unroll
        for (int b = 0; b < 8; ++b) { local[b] = hist[8 * lane + b]; full |= local[b] == m; sum += local[b]; }
        int incl = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        if (__any_sync(0xffffffffu, full)) continue;  // one digit holds every key: this pass keeps the order
        int run = incl - sum;
#pragma unroll
        for (int b = 0; b < 8; ++b) { hist[8 * lane + b] = run; run += local[b]; }
        __syncwarp();
        for (int base = 0; base < m; base += 32) {
            const int i = base + lane;
            const bool valid = i < m;
            const Key k = valid ? kin[i] : Key(0);
            const int d = valid ? radix_digit(k, shift) : 256;
            const unsigned same = same_digit_lanes(d);
            int pos = 0;
            if (valid) pos = hist[d] + __popc(same & lt);
            __syncwarp();
            if (valid) {
                kout[pos] = k;
                iout[pos] = iin[i];
                if ((same & lt) == 0) hist[d] += __popc(same);
            }
            __syncwarp();
        }
        Key* kt = kin; kin = kout; kout = kt;
        int16_t* it = iin; iin = iout; iout = it;
        __syncwarp();
    }
    bool dup = false;
    for (int i = lane; i + 1 < m; i += 32) dup |= key_eq(kin[i], kin[i + 1]);
    if (__any_sync(0xffffffffu, dup)) return false;
    for (int i = lane; i < m; i += 32) {
        a.s2[i] = iin[i];
        a.r0[i] = T::from_key(kin[i]);
    }
    __syncwarp();
    return true;
}

// Sorts r0[0..m) with NumPy's quicksort order; leaves the order in s2 and the
// sorted weights in r0.  Whole-warp call.  try_distinct: attempt the
// tie-free radix path first (worth it where ties are rare: min_samples <= 2).
template <typename Real>
__device__ void sort_edges_warp(const Arena<Real>& a, int m, bool try_distinct) {
    const int lane = threadIdx.x & 31;
    if (try_distinct && m >= 256 && radix_sort_distinct_warp<Real>(a, m)) return;
    SortPair<Real>* p = reinterpret_cast<SortPair<Real>*>(a.r1);
    for (int i = lane; i < m; i += 32) { p[i].w = a.r0[i]; p[i].idx = i; }
    int16_t *task_lo = a.s5, *task_hi = a.s6, *task_depth = a.s7;  // depth*2 + checked
    int16_t *leaf_lo = a.s8, *leaf_hi = a.s9, *leaf_code = a.s2;     // segments finished by lanes
    // Warp partitions down to about m/16 elements leave some 16-32 segments
    // for the lanes.
    const int lane_max = min(kLaneSortMax, max(32, m >> 4));
    int top = 0, leaves = 0;
    if (m > 1) {
        int depth = 0;
        for (int c = m; c > 1; c >>= 1) depth += 2;  // 2*floor(log2(m)), _kernels.py:429-431
        if (lane == 0) { task_lo[0] = 0; task_hi[0] = (int16_t)(m - 1); task_depth[0] = (int16_t)(depth * 2 + 1); }
        top = 1;
    }
    __syncwarp();
    while (top > 0) {
        --top;
        const int lo = task_lo[top], hi = task_hi[top], code = task_depth[top];
        const int depth = code >> 1;  // arithmetic shift keeps negative depths
        const bool checked = code & 1;
        __syncwarp();
        if ((checked && depth < 0) || hi - lo + 1 < lane_max) {
            // Exhausted depth (heapsort, reference :442-443) or a short segment.
            if (lane == 0) { leaf_lo[leaves] = (int16_t)lo; leaf_hi[leaves] = (int16_t)hi; leaf_code[leaves] = (int16_t)code; }
            ++leaves;
        } else {
            const int i = partition_warp(p, lo, hi, a.s3, a.s4);
            const int d = depth - 1;
            // The larger side is deferred (checked on pop); the smaller side
            // continues in place without a depth check (_kernels.py:449-462).
            int big_lo, big_hi, small_lo, small_hi;
            if (i - lo < hi - i) { big_lo = i + 1; big_hi = hi; small_lo = lo; small_hi = i - 1; }
            else { big_lo = lo; big_hi = i - 1; small_lo = i + 1; small_hi = hi; }
            if (lane == 0) {
                task_lo[top] = (int16_t)big_lo; task_hi[top] = (int16_t)big_hi; task_depth[top] = (int16_t)(d * 2 + 1);
                task_lo[top + 1] = (int16_t)small_lo; task_hi[top + 1] = (int16_t)small_hi;
                task_depth[top + 1] = (int16_t)(d * 2);
            }
            top += 2;
        }
        __syncwarp();
    }
    for (int t = lane; t < leaves; t += 32) introsort_lane(p, leaf_lo[t], leaf_hi[t], leaf_code[t]);
    __syncwarp();
    for (int i = lane; i < m; i += 32) {
        a.s2[i] = (int16_t)p[i].idx;
        a.r0[i] = p[i].w;
    }
    __syncwarp();
}

// The same sort by every warp of the CTA (`nthreads` threads, all of which
// must call; the named barrier `bar` spans them): the partition tasks go in
// rounds, each warp taking every nw-th task of the round, and the lane
// segments are shared by all threads.  Segments are disjoint and each one's
// partition depends only on its own bounds and depth code, so the result
// equals the one-warp form's.  ctr: four ints of shared memory.
template <typename Real>
__device__ __forceinline__ void sort_edges_cta(const Arena<Real>& a, int m, int nthreads, int bar, int* ctr) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = nthreads >> 5;
    SortPair<Real>* p = reinterpret_cast<SortPair<Real>*>(a.r1);
    for (int i = tid; i < m; i += nthreads) { p[i].w = a.r0[i]; p[i].idx = i; }
    int16_t *task_lo = a.s5, *task_hi = a.s6, *task_depth = a.s7;  // two halves: this round, next round
    int16_t *leaf_lo = a.s8, *leaf_hi = a.s9, *leaf_code = a.s2;
    const int half = Arena<Real>::round_cap(m + 1) / 2;
    const int lane_max = 33;
    if (tid == 0) {
        int depth = 0;
        for (int c = m; c > 1; c >>= 1) depth += 2;  // 2*floor(log2(m)), _kernels.py:429-431
        task_lo[0] = 0;
        task_hi[0] = (int16_t)(m - 1);
        task_depth[0] = (int16_t)(depth * 2 + 1);
        ctr[0] = 0; ctr[1] = 0; ctr[2] = 0; ctr[3] = 0;  // pushes of rounds r % 3; leaves
    }
    asm volatile("bar.sync %0, %1;" ::"r"(bar), "r"(nthreads) : "memory");
    int count = m > 1 ? 1 : 0;
    for (int round = 0; count > 0; ++round) {
        const int cur = (round & 1) * half, nxt = half - cur;
        int* pushes = ctr + round % 3;
        if (tid == 0) ctr[(round + 1) % 3] = 0;  // last read two barriers ago
        for (int t = warp; t < count; t += nw) {
            const int lo = task_lo[cur + t], hi = task_hi[cur + t], code = task_depth[cur + t];
            const int depth = code >> 1;  // arithmetic shift keeps negative depths
            const bool checked = code & 1;
            if ((checked && depth < 0) || hi - lo + 1 < lane_max) {
                if (lane == 0) {
                    const int k = atomicAdd(ctr + 3, 1);
                    leaf_lo[k] = (int16_t)lo; leaf_hi[k] = (int16_t)hi; leaf_code[k] = (int16_t)code;
                }
            } else {
                const int i = partition_warp(p, lo, hi, a.s3, a.s4);
                const int d = depth - 1;
                int big_lo, big_hi, small_lo, small_hi;
                if (i - lo < hi - i) { big_lo = i + 1; big_hi = hi; small_lo = lo; small_hi = i - 1; }
                else { big_lo = lo; big_hi = i - 1; small_lo = i + 1; small_hi = hi; }
                if (lane == 0) {
                    const int k = nxt + atomicAdd(pushes, 2);
                    task_lo[k] = (int16_t)big_lo; task_hi[k] = (int16_t)big_hi; task_depth[k] = (int16_t)(d * 2 + 1);
                    task_lo[k + 1] = (int16_t)small_lo; task_hi[k + 1] = (int16_t)small_hi;
                    task_depth[k + 1] = (int16_t)(d * 2);
                }
            }
            __syncwarp();
        }
        asm volatile("bar.sync %0, %1;" ::"r"(bar), "r"(nthreads) : "memory");
        count = *pushes;
    }
    const int leaves = ctr[3];
    for (int t = tid; t < leaves; t += nthreads) introsort_lane(p, leaf_lo[t], leaf_hi[t], leaf_code[t]);
    asm volatile("bar.sync %0, %1;" ::"r"(bar), "r"(nthreads) : "memory");
    for (int i = tid; i < m; i += nthreads) {
        a.s2[i] = (int16_t)p[i].idx;
        a.r0[i] = p[i].w;
    }
    asm volatile("bar.sync %0, %1;" ::"r"(bar), "r"(nthreads) : "memory");
}

// ---------------------------------------------------------------------------
// Single linkage (reference: _kernels.py:518-556).  Node n+i merges the
// components of the i-th sorted edge (source side first).  Inputs: s2 sorted
// sources, s3 sorted targets.  Outputs: s4 left, s5 right, s6 size of node n+i
// at index i.  The union-find words live in r1/r2.
//
// Edges go in batches of 32: first every lane walks its edge's two endpoints
// to their roots in the state before the batch (in parallel), then the
// batch's unions are replayed in order in registers (one shuffle broadcast of
// the edge's two roots per step; lanes holding either root take the merged
// one), and finally every lane writes its edge's row and its part of the
// forest update.  The roots, sizes, orientations and node ids are those of
// the serial union-find.
// ---------------------------------------------------------------------------
template <typename Real>
__device__ void linkage_warp(const Arena<Real>& a, int n) {
    const int lane = threadIdx.x & 31;
    const int m = n - 1;
    uint2* U = reinterpret_cast<uint2*>(a.r1);  // {parent | node << 16, size}; node and size valid at roots
    for (int x = lane; x < n; x += 32) U[x] = make_uint2((uint32_t)x | ((uint32_t)x << 16), 1u);
    __syncwarp();
    for (int base = 0; base < m; base += 32) {
        const int e = base + lane;
        const int count = min(32, m - base);
        // 1. Each lane finds the roots of its edge's endpoints in the forest
        //    as it stood before this batch, with their {root | node, size}.
        uint2 wx = make_uint2(0u, 0u), wy = make_uint2(0u, 0u);
        if (e < m) {
            int x = a.s2[e], y = a.s3[e];
            wx = U[x];
            wy = U[y];
            while ((int)(wx.x & 0xffffu) != x || (int)(wy.x & 0xffffu) != y) {
                x = (int)(wx.x & 0xffffu);
                y = (int)(wy.x & 0xffffu);
                wx = U[x];
                wy = U[y];
            }
        }
        uint32_t kx = wx.x, sx = wx.y, ky = wy.x, sy = wy.y;
        // 2. The batch's merges in edge order, resolved in registers: step l
        //    broadcasts edge l's current roots, and every lane whose root is
        //    one of them takes the merged root, node and size.  A tree edge
        //    never joins a component to itself, so the two roots differ.
        uint32_t left = 0, right = 0, size = 0, winner = 0, loser = 0;
        bool superseded = false;  // this lane's root was merged again later in the batch
        for (int l = 0; l < count; ++l) {
            const uint32_t KX = __shfl_sync(0xffffffffu, kx, l), KY = __shfl_sync(0xffffffffu, ky, l);
            const uint32_t SX = __shfl_sync(0xffffffffu, sx, l), SY = __shfl_sync(0xffffffffu, sy, l);
            const uint32_t X = KX & 0xffffu, Y = KY & 0xffffu, S = SX + SY;
            const uint32_t W = SX < SY ? Y : X;  // union by size, ties keep x's root
            const uint32_t merged = W | ((uint32_t)(n + base + l) << 16);
            if (lane == l) {
                left = KX >> 16;
                right = KY >> 16;
                size = S;
                winner = W;
                loser = SX < SY ? X : Y;
            }
            if (lane < l && (winner == X || winner == Y)) superseded = true;
            const uint32_t rx = kx & 0xffffu, ry = ky & 0xffffu;
            if (rx == X || rx == Y) { kx = merged; sx = S; }
            if (ry == X || ry == Y) { ky = merged; sy = S; }
        }
        // 3. Outputs and the forest update, one lane per edge.  Every loser
        //    is merged once, and a winner's word is written only by the last
        //    edge of the batch that merged it, so no two lanes store to the
        //    same word.
        if (e < m) {
            a.s4[e] = (int16_t)left;
            a.s5[e] = (int16_t)right;
            a.s6[e] = (int16_t)size;
            U[loser].x = winner;
            if (!superseded) U[winner] = make_uint2(winner | ((uint32_t)(n + e) << 16), size);
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// Breadth-first condensation (reference: _kernels.py:558-643), one queue
// level per warp round.  Linkage node ids n..2n-2 (index id-n); cluster ids
// n.. (index id-n).  Inputs: s4 left, s5 right, s6 size, r0 merge weights
// (turned into lambda = 1/weight in place).  Outputs: s2 cluster parent, r1
// birth, r2 stability, sel, s9 point parent, s8 the linkage node each point
// was pruned at (its lambda is lambda[s8 - n]), s3 the deepest linkage node of
// each cluster (index id - n; lambda there is the largest lambda leaving the
// cluster, as lambda never decreases down a cluster's path).  Returns
// next_label (warp-uniform).
// ---------------------------------------------------------------------------
template <typename Real>
__device__ int condense_warp(const Arena<Real>& a, int n, int mcs, int32_t* cl_size = nullptr) {
    using T = RealTraits<Real>;
    const int lane = threadIdx.x & 31;
    const unsigned lt = lanemask_lt();
    int16_t* relabel = a.s7;   // cluster of each large linkage node
    int16_t* queue = a.s8;     // large linkage nodes in breadth-first order
    int16_t* dparent = a.s0;   // dendrogram parent of node ids 0..2n-3 (spans s0, s1)
    int16_t* parent = a.s2;
    Real* birth = a.r1;
    Real* stab = a.r2;
    Real* lam = a.r0;
    const int16_t* left = a.s4;
    const int16_t* right = a.s5;
    const int16_t* size = a.s6;
    const Real inf = T::inf();
    for (int c = lane; c < n; c += 32) { parent[c] = -1; birth[c] = 0; stab[c] = 0; a.sel[c] = 0; }
    for (int i = lane; i < n - 1; i += 32) {
        const Real d = lam[i];
        lam[i] = d > Real(0) ? T::recip(d) : inf;
        dparent[left[i]] = (int16_t)(n + i);
        dparent[right[i]] = (int16_t)(n + i);
    }
    const int root = 2 * n - 2;
    if (lane == 0) {
        queue[0] = (int16_t)root;
        relabel[root - n] = (int16_t)n;
        if (cl_size) cl_size[0] = n;
    }
    __syncwarp();
    int head = 0, tail = 1, next_label = n + 1;
    while (head < tail) {  // tail <= n - 1 (every node is queued at most once)
        const int level_end = tail;
        for (int base = head; base < level_end; base += 32) {
            const int q = base + lane;
            const bool valid = q < level_end;
            int l = 0, r = 0, cluster = n, size_l = 0, size_r = 0;
            Real lambda = Real(0);
            if (valid) {
                const int ni = queue[q] - n;
                l = left[ni];
                r = right[ni];
                cluster = relabel[ni];
                lambda = lam[ni];
                size_l = l < n ? 1 : size[l - n];
                size_r = r < n ? 1 : size[r - n];
            }
            const bool large_l = valid && size_l >= mcs, large_r = valid && size_r >= mcs;
            const bool split = large_l && large_r;
            const unsigned b1 = __ballot_sync(0xffffffffu, large_l || large_r);
            const unsigned b2 = __ballot_sync(0xffffffffu, split);
            const int pos = tail + __popc(b1 & lt) + __popc(b2 & lt);
            const int label0 = next_label + 2 * __popc(b2 & lt);
            if (valid) {
                const int ci = cluster - n;
                a.s3[ci] = (int16_t)(queue[q] - n);  // deeper levels overwrite: the cluster's last node
                const Real cb = birth[ci];
                Real st = stab[ci];
                if (split) {
                    // Both children: new consecutive ids (_kernels.py:603-613).
#pragma unroll
                    for (int k = 0; k < 2; ++k) {
                        const int child = k == 0 ? l : r;
                        const int csize = k == 0 ? size_l : size_r;
                        const int label = label0 + k;
                        relabel[child - n] = (int16_t)label;
                        parent[label - n] = (int16_t)cluster;
                        birth[label - n] = lambda;
                        a.sel[label - n] = 1;
                        if (cl_size) cl_size[label - n] = csize;
                        st = T::add(st, T::mul(T::sub(lambda, cb), (Real)csize));
                        queue[pos + k] = (int16_t)child;
                    }
                } else {
                    // A large child continues the cluster; a small one is
                    // pruned leaf by leaf, each leaf adding the same term
                    // (_kernels.py:614-637).
                    const Real term = T::sub(lambda, cb);
#pragma unroll
                    for (int k = 0; k < 2; ++k) {
                        const int child = k == 0 ? l : r;
                        if (k == 0 ? large_l : large_r) {
                            relabel[child - n] = (int16_t)cluster;
                            queue[pos] = (int16_t)child;
                        } else {
                            const int csize = k == 0 ? size_l : size_r;
                            for (int t = 0; t < csize; ++t) st = T::add(st, term);
                        }
                    }
                }
                stab[ci] = st;
            }
            tail += __popc(b1) + __popc(b2);
            next_label += 2 * __popc(b2);
        }
        __syncwarp();
        head = level_end;
    }
    // Every point was pruned at its lowest large ancestor (or the root).
    for (int i = lane; i < n; i += 32) {
        int v = dparent[i];
        while (v != root && size[v - n] < mcs) v = dparent[v];
        a.s9[i] = relabel[v - n];
        a.s8[i] = (int16_t)v;
    }
    __syncwarp();
    return next_label;
}

// ---------------------------------------------------------------------------
// Cluster selection and labels.  method 0: excess of mass (reference:
// _kernels.py:672-710, binary form :648-669), 1: leaf clusters; allow_single
// lets the root compete; epsilon merge and labels (reference:
// _kernels.py:712-760).  The leaf and allow_single options and the
// probabilities restate scikit-learn's selection (sklearn/cluster/_hdbscan/
// _tree.pyx:433-554, 644-799); with method 0 and allow_single false this is
// exactly the reference's path.  Writes labels[0..n) and, when non-null,
// probabilities[0..n) (global memory).
// ---------------------------------------------------------------------------
template <typename Real>
__device__ void select_and_label_warp(const Arena<Real>& a, int n, int next_label, Real epsilon, int method,
                                      bool allow_single, int32_t* labels, Real* probabilities) {
    using T = RealTraits<Real>;
    const int lane = threadIdx.x & 31;
    const int clusters = next_label - n;
    const bool splits = clusters > 1;
    const bool eps_on = epsilon > Real(0) && splits;
    const int16_t* parent = a.s2;
    const Real* birth = a.r1;
    const Real* lam = a.r0;
    Real* stab = a.r2;
    int16_t* first = a.s0;             // first child cluster (children come in consecutive pairs)
    int16_t* resolved = a.s1;          // nearest selected cluster at or above each cluster, -1 none
    const int16_t* last_node = a.s3;   // deepest linkage node of each cluster
    int16_t* blocked = a.s4;
    int16_t* stop = a.s5;
    int16_t* label_map = a.s6;
    int16_t* eps_side = a.s7;          // bit 0: 1/birth > epsilon, bit 1: 1/birth < epsilon
    for (int c = lane; c < clusters; c += 32) {
        first[c] = -1;
        if (eps_on) {
            const Real inv = T::recip(birth[c]);
            eps_side[c] = (int16_t)((inv > epsilon ? 1 : 0) | (inv < epsilon ? 2 : 0));
        }
    }
    __syncwarp();
    for (int child = n + 1 + 2 * lane; child < next_label; child += 64) first[parent[child - n] - n] = (int16_t)child;
    __syncwarp();
    // The three passes below restate the reference's serial loops over the
    // clusters in chunks of 32 consecutive ids, one lane per cluster.  A
    // cluster depends only on final values of its children (pass 1) or its
    // parent (passes 2, 3); parent ids are smaller than child ids, so a lane
    // computes once every dependency lies in an earlier chunk or belongs to a
    // lane of this chunk that is done (a ballot per round), and the results
    // equal the serial order's.
    constexpr unsigned kFull = 0xffffffffu;
    // 1. Candidates: excess of mass, children (larger ids) before parents;
    //    or the leaves of the cluster tree (none if the root never splits).
    if (method == 0) {
        if (lane == 0) a.sel[0] = allow_single ? 1 : 0;
        const int lo_node = allow_single ? n : n + 1;
        for (int hi = next_label - 1; hi >= lo_node; hi -= 32) {
            const int node = hi - lane;
            bool done = node < lo_node;
            const int f = done ? -1 : first[node - n];
            unsigned done_mask = __ballot_sync(kFull, done);
            // Each round finishes at least one lane of a valid tree: at most 32 rounds.
        for (int round = 0; done_mask != kFull && round < 32; ++round) {
                if (!done) {
                    const bool c0 = f < 0 || f > hi || ((done_mask >> (hi - f)) & 1u);
                    const bool c1 = f < 0 || f + 1 > hi || ((done_mask >> (hi - f - 1)) & 1u);
                    if (c0 && c1) {
                        const Real subtree = f < 0 ? Real(0) : T::add(T::add(Real(0), stab[f - n]), stab[f + 1 - n]);
                        if (T::lt(stab[node - n], subtree)) {
                            a.sel[node - n] = 0;
                            stab[node - n] = subtree;
                        }
                        done = true;
                    }
                }
                __syncwarp();
                done_mask = __ballot_sync(kFull, done);
            }
        }
    } else {
        if (lane == 0) a.sel[0] = 0;
        for (int node = n + 1 + lane; node < next_label; node += 32) a.sel[node - n] = first[node - n] < 0 ? 1 : 0;
    }
    __syncwarp();
    // 2. Parents first (ascending ids): suppress the descendants of a selected
    //    cluster; with epsilon, find each cluster's epsilon stop ancestor (the
    //    climb ends below the root, at the root with allow_single), then mark
    //    the cluster every surviving selection resolves to (itself or its stop).
    if (lane == 0) {
        blocked[0] = a.sel[0];
        label_map[0] = (eps_on && a.sel[0]) ? 1 : -1;  // 1/birth(root) = inf: the root never climbs
    }
    __syncwarp();
    for (int lo = n + 1; lo < next_label; lo += 32) {
        const int node = lo + lane;
        bool done = node >= next_label;
        const int anc = done ? n : parent[node - n];
        if (!done) label_map[node - n] = -1;
        unsigned done_mask = __ballot_sync(kFull, done);
        // Each round finishes at least one lane of a valid tree: at most 32 rounds.
        for (int round = 0; done_mask != kFull && round < 32; ++round) {
            if (!done && (anc < lo || ((done_mask >> (anc - lo)) & 1u))) {
                const int inherited = blocked[anc - n];
                int selected = a.sel[node - n];
                blocked[node - n] = (int16_t)(inherited || selected);
                if (inherited) selected = 0;
                a.sel[node - n] = (uint8_t)selected;
                if (eps_on)
                    stop[node - n] = (int16_t)(anc == n ? (allow_single ? n : node)
                                                        : ((eps_side[anc - n] & 1) ? anc : stop[anc - n]));
                done = true;
            }
            __syncwarp();
            done_mask = __ballot_sync(kFull, done);
        }
    }
    __syncwarp();
    if (eps_on) {
        for (int node = n + 1 + lane; node < next_label; node += 32)
            if (a.sel[node - n]) label_map[((eps_side[node - n] & 2) ? stop[node - n] : node) - n] = 1;
        __syncwarp();
    }
    // 3. Ascending: final selection, label numbers (a ballot prefix; the root
    //    first when selected), nearest selected cluster of every cluster.
    int label = 0;  // warp-uniform
    for (int lo = n; lo < next_label; lo += 32) {
        const int node = lo + lane;
        const bool valid = node < next_label;
        int selected = 0;
        if (valid) selected = eps_on ? (label_map[node - n] == 1) : a.sel[node - n];
        const unsigned sel_mask = __ballot_sync(kFull, valid && selected);
        if (valid) {
            a.sel[node - n] = (uint8_t)selected;
            label_map[node - n] = (int16_t)(selected ? label + __popc(sel_mask & lanemask_lt()) : -1);
        }
        label += __popc(sel_mask);
        bool done = !valid;
        const int par = (valid && node != n) ? parent[node - n] : n;
        if (valid && (selected || node == n)) {
            resolved[node - n] = (int16_t)(selected ? node : -1);
            done = true;
        }
        __syncwarp();
        unsigned done_mask = __ballot_sync(kFull, done);
        // Each round finishes at least one lane of a valid tree: at most 32 rounds.
        for (int round = 0; done_mask != kFull && round < 32; ++round) {
            if (!done && (par < lo || ((done_mask >> (par - lo)) & 1u))) {
                resolved[node - n] = resolved[par - n];
                done = true;
            }
            __syncwarp();
            done_mask = __ballot_sync(kFull, done);
        }
    }
    const int single_root = allow_single && label == 1 && a.sel[0];
    __syncwarp();
    // Points: the nearest selected cluster's label; below a lone selected root
    // (allow_single) a point joins at lambda >= 1/eps, or >= the largest
    // lambda leaving the root when eps = 0 (_tree.pyx:491-508); else noise.
    const Real threshold = epsilon != Real(0) ? T::recip(epsilon) : lam[last_node[0]];
    for (int i = lane; i < n; i += 32) {
        const int c = resolved[a.s9[i] - n];
        const Real lambda_i = lam[a.s8[i] - n];
        int lab = -1;
        if (c > n) lab = label_map[c - n];
        else if (c == n && single_root && lambda_i >= threshold) lab = label_map[0];
        labels[i] = lab;
        if (probabilities) {
            // Membership strength (_tree.pyx:515-554): the point's lambda over
            // the largest lambda leaving its cluster, capped at 1.
            Real prob = Real(0);
            if (lab >= 0) {
                const Real max_lambda = lam[last_node[c - n]];
                if (max_lambda == Real(0) || isinf(lambda_i)) prob = Real(1);
                else prob = T::div(lambda_i < max_lambda ? lambda_i : max_lambda, max_lambda);
            }
            probabilities[i] = prob;
        }
    }
    __syncwarp();
}

}  // namespace hdb
