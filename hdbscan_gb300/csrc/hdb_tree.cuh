// Hierarchy stages of one window, run by one CTA on a shared-memory arena:
// indirect introsort -> union-find single linkage -> breadth-first
// condensation -> excess-of-mass selection -> epsilon merge -> labels.
//
// Semantics follow the reference kernels (hdbscan_gpu/_kernels.py) stage by
// stage; each function cites the lines it reproduces.  The arena layout and
// the lifetime aliasing below are this project's own (16-bit indices, sort on
// (weight, index) pairs so each compare is one shared-memory load, endpoints
// gathered into sorted order before linkage).
#pragma once
#include "hdb_common.cuh"

namespace hdb {

// Element of the sort: the weight and the Prim edge index travel together.
template <typename Real> struct SortPair;
template <> struct __align__(8) SortPair<float> { float w; int32_t idx; };
template <> struct __align__(16) SortPair<double> { double w; int64_t idx; };

// Shared-memory arena for one window of capacity `cap` points (cap >= n).
//  r0  Real[cap]  edge weights in Prim order -> weights in sorted order
//  r1  Real[cap]  cluster birth lambda        (r1+r2 = SortPair[cap] during the sort)
//  r2  Real[cap]  cluster stability
//  s0  i16[cap]   Prim edge source            -> prune queue [0, cap)
//  s1  i16[cap]   Prim edge new vertex        -> prune queue [cap, 2cap)
//  s2  i16[cap]   sorted edge order           -> sorted sources
//  s3  i16[cap]   sort tasks | linkage left   -> first child
//  s4  i16[cap]   sort tasks | linkage right  -> next sibling
//  s5  i16[cap]   sort tasks | linkage size   -> EOM blocked -> epsilon stop
//  s6  i16[cap]   sort tasks | union-find     -> relabel -> resolved label
//  s7  i16[cap]   sort tasks | component node -> BFS queue -> label map
//  s8  i16[cap]   sort tasks | sorted targets -> cluster parent
//  s9  i16[cap]   point parent
//  sel u8[cap]    cluster selected flag
template <typename Real> struct Arena {
    Real *r0, *r1, *r2;
    int16_t *s0, *s1, *s2, *s3, *s4, *s5, *s6, *s7, *s8, *s9;
    uint8_t* sel;

    __host__ __device__ static int round_cap(int n) { return (n + 7) & ~7; }
    __host__ __device__ static size_t bytes(int n) {
        const size_t cap = (size_t)round_cap(n);
        return 3 * cap * sizeof(Real) + 10 * cap * sizeof(int16_t) + cap;
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

// ---------------------------------------------------------------------------
// Indirect introsort (reference: _kernels.py:358-516; NumPy 2.3.5 scalar
// aquicksort semantics).  Tie order depends on the exact sequence of
// median-of-3 swaps, Hoare partition swaps, insertion shifts and heapsort
// moves, so each task runs them serially; independent tasks run in parallel
// threads exactly as the reference's PARALLEL_SORT rounds (:441-480).
// ---------------------------------------------------------------------------
template <typename Real>
__device__ void heap_sort_pairs(SortPair<Real>* p, int lo, int hi) {
    const int count = hi - lo + 1;
    SortPair<Real>* a = p + lo - 1;  // 1-based
    for (int root = count / 2; root >= 1; --root) {
        SortPair<Real> value = a[root];
        int pos = root, child = 2 * root;
        while (child <= count) {
            if (child < count && a[child].w < a[child + 1].w) ++child;
            if (value.w < a[child].w) { a[pos] = a[child]; pos = child; child *= 2; } else break;
        }
        a[pos] = value;
    }
    for (int end = count; end > 1;) {
        SortPair<Real> value = a[end];
        a[end] = a[1];
        --end;
        int pos = 1, child = 2;
        while (child <= end) {
            if (child < end && a[child].w < a[child + 1].w) ++child;
            if (value.w < a[child].w) { a[pos] = a[child]; pos = child; child *= 2; } else break;
        }
        a[pos] = value;
    }
}

template <typename Real>
__device__ __forceinline__ void swap_pairs(SortPair<Real>* p, int i, int j) {
    SortPair<Real> t = p[i]; p[i] = p[j]; p[j] = t;
}

// Runs one task: heapsort if its (checked) depth is exhausted, else partition
// until <= 16 elements, deferring the larger side into `next_*`.
template <typename Real>
__device__ void sort_task(SortPair<Real>* p, int lo, int hi, int depth,
                          int16_t* next_lo, int16_t* next_hi, int16_t* next_depth, int* pending) {
    if (depth < 0) { heap_sort_pairs(p, lo, hi); return; }
    while (hi - lo > 15) {
        const int mid = lo + ((hi - lo) >> 1);
        if (p[mid].w < p[lo].w) swap_pairs(p, mid, lo);
        if (p[hi].w < p[mid].w) swap_pairs(p, hi, mid);
        if (p[mid].w < p[lo].w) swap_pairs(p, mid, lo);
        const Real pivot = p[mid].w;
        int i = lo, j = hi - 1;
        swap_pairs(p, mid, j);
        for (;;) {
            do { ++i; } while (p[i].w < pivot);
            do { --j; } while (pivot < p[j].w);
            if (i >= j) break;
            swap_pairs(p, i, j);
        }
        swap_pairs(p, i, hi - 1);
        --depth;
        const int slot = atomicAdd(pending, 1);
        if (i - lo < hi - i) {
            next_lo[slot] = (int16_t)(i + 1); next_hi[slot] = (int16_t)hi;
            hi = i - 1;
        } else {
            next_lo[slot] = (int16_t)lo; next_hi[slot] = (int16_t)(i - 1);
            lo = i + 1;
        }
        next_depth[slot] = (int16_t)depth;
    }
    for (int i = lo + 1; i <= hi; ++i) {
        SortPair<Real> value = p[i];
        int j = i;
        while (j > lo && value.w < p[j - 1].w) { p[j] = p[j - 1]; --j; }
        p[j] = value;
    }
}

// Sorts r0[0..m) (m = n-1 edge weights) into pairs; leaves the order in s2
// and the sorted weights in r0.  Whole-CTA call.
template <typename Real>
__device__ void sort_edges(const Arena<Real>& a, int m, int* s_counter) {
    SortPair<Real>* p = reinterpret_cast<SortPair<Real>*>(a.r1);
    for (int i = threadIdx.x; i < m; i += blockDim.x) { p[i].w = a.r0[i]; p[i].idx = i; }
    int16_t *cur_lo = a.s3, *cur_hi = a.s4, *cur_depth = a.s5;
    int16_t *nxt_lo = a.s6, *nxt_hi = a.s7, *nxt_depth = a.s8;
    __shared__ int s_tasks;
    if (threadIdx.x == 0) {
        int depth = 0;
        for (int c = m; c > 1; c >>= 1) depth += 2;  // 2*floor(log2(m)), _kernels.py:429-431
        s_tasks = m > 1 ? 1 : 0;
        cur_lo[0] = 0; cur_hi[0] = (int16_t)(m - 1); cur_depth[0] = (int16_t)depth;
        *s_counter = 0;
    }
    __syncthreads();
    int rounds = 0;
    while (s_tasks > 0 && rounds < 4 * 32768) {
        const int tasks = s_tasks;
        for (int t = threadIdx.x; t < tasks; t += blockDim.x)
            sort_task(p, cur_lo[t], cur_hi[t], cur_depth[t], nxt_lo, nxt_hi, nxt_depth, s_counter);
        __syncthreads();
        if (threadIdx.x == 0) { s_tasks = *s_counter; *s_counter = 0; }
        __syncthreads();
        int16_t* t0 = cur_lo; cur_lo = nxt_lo; nxt_lo = t0;
        t0 = cur_hi; cur_hi = nxt_hi; nxt_hi = t0;
        t0 = cur_depth; cur_depth = nxt_depth; nxt_depth = t0;
        ++rounds;
    }
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
        a.s2[i] = (int16_t)p[i].idx;
        a.r0[i] = p[i].w;
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------
// Single linkage (reference: _kernels.py:518-556, scikit-learn
// make_single_linkage semantics).  Node n+i merges the components of the
// i-th sorted edge's (source, target), children oriented (source side,
// target side).  Balanced union-find over leaf representatives with path
// halving; the component's current dendrogram node is kept per representative.
// Serial (thread 0).  Inputs: s2 = sorted sources, s8 = sorted targets.
// Outputs: s3 left, s4 right, s5 size for node n+i at index i.
// ---------------------------------------------------------------------------
template <typename Real>
__device__ void linkage_serial(const Arena<Real>& a, int n) {
    int16_t* uf = a.s6;
    int16_t* comp = a.s7;
    for (int i = 0; i < n - 1; ++i) {
        int x = a.s2[i], y = a.s8[i];
        int px = uf[x];
        while (px != x) { const int g = uf[px]; uf[x] = (int16_t)g; x = g; px = uf[x]; }
        int py = uf[y];
        while (py != y) { const int g = uf[py]; uf[y] = (int16_t)g; y = g; py = uf[y]; }
        const int ca = comp[x], cc = comp[y];
        const int sa = ca < n ? 1 : a.s5[ca - n];
        const int sc = cc < n ? 1 : a.s5[cc - n];
        a.s3[i] = (int16_t)ca;
        a.s4[i] = (int16_t)cc;
        a.s5[i] = (int16_t)(sa + sc);
        if (sa < sc) { uf[x] = (int16_t)y; comp[y] = (int16_t)(n + i); }
        else { uf[y] = (int16_t)x; comp[x] = (int16_t)(n + i); }
    }
}

// ---------------------------------------------------------------------------
// Breadth-first condensation (reference: _kernels.py:558-643).  Serial.
// Linkage node ids are n..2n-2 (index id-n); cluster ids are n.. (index id-n).
// Returns next_label.
// ---------------------------------------------------------------------------
template <typename Real>
__device__ int condense_serial(const Arena<Real>& a, int n, int mcs) {
    int16_t* relabel = a.s6;   // per linkage node
    int16_t* queue = a.s7;     // linkage nodes (ids)
    int16_t* prune = a.s0;     // 2*cap entries across s0,s1
    int16_t* parent = a.s8;    // per cluster
    Real* birth = a.r1;
    Real* stab = a.r2;
    const Real inf = RealTraits<Real>::inf();
    for (int c = 0; c < n; ++c) { parent[c] = -1; birth[c] = 0; stab[c] = 0; a.sel[c] = 0; }
    const int root = 2 * n - 2;
    int head = 0, tail = 1, next_label = n + 1;
    queue[0] = (int16_t)root;
    relabel[root - n] = (int16_t)n;
    while (head < tail) {
        const int node = queue[head++];
        const int ni = node - n;
        const int left = a.s3[ni], right = a.s4[ni];
        const int cluster = relabel[ni];
        const int ci = cluster - n;
        const Real cluster_birth = birth[ci];
        Real cluster_stability = stab[ci];
        const Real dist = a.r0[ni];
        const Real lambda = dist > Real(0) ? RealTraits<Real>::recip(dist) : inf;
        const int size_l = left < n ? 1 : a.s5[left - n];
        const int size_r = right < n ? 1 : a.s5[right - n];
        const bool large_l = size_l >= mcs, large_r = size_r >= mcs;
        if (large_l && large_r) {
            // Both children: new consecutive ids (_kernels.py:603-613).
            for (int k = 0; k < 2; ++k) {
                const int child = k == 0 ? left : right;
                const int size = k == 0 ? size_l : size_r;
                const int label = next_label++;
                relabel[child - n] = (int16_t)label;
                parent[label - n] = (int16_t)cluster;
                birth[label - n] = lambda;
                a.sel[label - n] = 1;
                cluster_stability = RealTraits<Real>::add(
                    cluster_stability,
                    RealTraits<Real>::mul(RealTraits<Real>::sub(lambda, cluster_birth), (Real)size));
                queue[tail++] = (int16_t)child;
            }
        } else {
            for (int k = 0; k < 2; ++k) {
                const int child = k == 0 ? left : right;
                if (k == 0 ? large_l : large_r) {
                    relabel[child - n] = (int16_t)cluster;
                    queue[tail++] = (int16_t)child;
                } else {
                    // Prune the whole subtree leaf by leaf (_kernels.py:626-637).
                    const Real term = RealTraits<Real>::sub(lambda, cluster_birth);
                    int ph = 0, pt = 0, leaf = child;
                    for (;;) {
                        if (leaf < n) {
                            a.s9[leaf] = (int16_t)cluster;
                            cluster_stability = RealTraits<Real>::add(cluster_stability, term);
                        } else {
                            prune[pt++] = a.s3[leaf - n];
                            prune[pt++] = a.s4[leaf - n];
                        }
                        if (ph == pt) break;
                        leaf = prune[ph++];
                    }
                }
            }
        }
        stab[ci] = cluster_stability;
    }
    return next_label;
}

// ---------------------------------------------------------------------------
// Excess of mass (reference: _kernels.py:672-710) + epsilon and labels
// (reference: _kernels.py:712-760).  Serial; writes labels[0..n).
// ---------------------------------------------------------------------------
template <typename Real>
__device__ void select_and_label(const Arena<Real>& a, int n, int next_label, Real epsilon, int32_t* labels) {
    const int clusters = next_label - n;
    int16_t* parent = a.s8;
    Real* birth = a.r1;
    Real* stab = a.r2;
    int16_t* first_child = a.s3;
    int16_t* next_sibling = a.s4;
    for (int c = 0; c < clusters; ++c) { first_child[c] = -1; next_sibling[c] = -1; }
    // Descending insertion keeps children in ascending id order.
    for (int child = next_label - 1; child > n; --child) {
        const int anc = parent[child - n] - n;
        next_sibling[child - n] = first_child[anc];
        first_child[anc] = (int16_t)child;
    }
    for (int node = next_label - 1; node > n; --node) {
        Real subtree = 0;
        for (int child = first_child[node - n]; child != -1; child = next_sibling[child - n])
            subtree = RealTraits<Real>::add(subtree, stab[child - n]);
        if (subtree > stab[node - n]) {
            a.sel[node - n] = 0;
            stab[node - n] = subtree;
        }
    }
    int16_t* blocked = a.s5;
    blocked[0] = 0;
    for (int node = n + 1; node < next_label; ++node) {
        const int inherited = blocked[parent[node - n] - n];
        blocked[node - n] = (int16_t)(inherited || a.sel[node - n]);
        if (inherited) a.sel[node - n] = 0;
    }
    int16_t* label_map = a.s7;
    for (int c = 0; c < clusters; ++c) label_map[c] = -1;
    if (epsilon > Real(0)) {
        int16_t* stop = a.s5;  // blocked is dead
        for (int node = n + 1; node < next_label; ++node) {
            const int anc = parent[node - n];
            stop[node - n] = (int16_t)(anc == n ? node
                                                : (RealTraits<Real>::recip(birth[anc - n]) > epsilon ? anc : stop[anc - n]));
            if (!a.sel[node - n]) continue;
            const int chosen = RealTraits<Real>::recip(birth[node - n]) < epsilon ? stop[node - n] : node;
            label_map[chosen - n] = 1;
        }
        for (int node = n + 1; node < next_label; ++node) a.sel[node - n] = label_map[node - n] == 1;
    }
    int label = 0;
    for (int node = n + 1; node < next_label; ++node)
        if (a.sel[node - n]) label_map[node - n] = (int16_t)label++;
    int16_t* resolved = a.s6;
    resolved[0] = -1;
    for (int node = n + 1; node < next_label; ++node)
        resolved[node - n] = a.sel[node - n] ? label_map[node - n] : resolved[parent[node - n] - n];
    (void)labels;
}

}  // namespace hdb
