/*
 * CPU restatement of the reference HDBSCAN path, one precision per inclusion.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: the tests, the
 * smoke check and the CPU-baseline leg of bench.py compare the CUDA kernels
 * against it.  No product code path may call it.
 *
 * hdb_oracle.c includes this body twice, with REAL = float / double and
 * SUF = f32 / f64.  Every stage restates the reference CUDA path of
 * CosineAI/hdbscan (hdbscan_gpu/_kernels.py, as compiled by
 * hdbscan_gpu/_cuda.py) in plain serial C; the cited lines are the ones whose
 * semantics each block reproduces.  Arithmetic is plain IEEE add/sub/mul/div/
 * sqrt in the order the reference performs it; compile with
 * -ffp-contract=off so that no multiply-add is fused.
 */

#define HDB_CAT2(a, b) a##_##b
#define HDB_CAT(a, b) HDB_CAT2(a, b)
#define FN(name) HDB_CAT(name, SUF)

/* Pairwise Euclidean distances, triangle computed once and mirrored.
 * hdbscan_gpu/_kernels.py:45-88 (DISTANCE_SOURCE): coordinate-order
 * accumulation total = total + delta*delta, no FMA (--fmad=false at
 * _cuda.py:24), correctly rounded sqrt, d(i,j) written for j >= i and mirrored. */
void FN(hdb_oracle_distances)(const REAL* x, int n, int d, REAL* out) {
    for (int i = 0; i < n; ++i) {
        for (int j = i; j < n; ++j) {
            REAL total = 0;
            for (int k = 0; k < d; ++k) {
                REAL delta = x[(size_t)i * d + k] - x[(size_t)j * d + k];
                total = total + delta * delta;
            }
            REAL dist = SQRT(total);
            out[(size_t)i * n + j] = dist;
            out[(size_t)j * n + i] = dist;
        }
    }
}

static int FN(cmp_real)(const void* a, const void* b) {
    REAL x = *(const REAL*)a, y = *(const REAL*)b;
    return (x > y) - (x < y);
}

/* Self-inclusive core distance: the (ms-1)-th smallest value (0-based) of
 * each distance row, diagonal zero included.  hdbscan_gpu/_cuda.py:114-118
 * (cp.partition(distances, ms-1)[..., ms-1]).  The k-th order statistic is a
 * unique value, so a full sort of a row copy gives the same number. */
void FN(hdb_oracle_core)(const REAL* dist, int n, int ms, REAL* core, REAL* scratch) {
    for (int i = 0; i < n; ++i) {
        memcpy(scratch, dist + (size_t)i * n, sizeof(REAL) * (size_t)n);
        qsort(scratch, (size_t)n, sizeof(REAL), FN(cmp_real));
        core[i] = scratch[ms - 1];
    }
}

/* Indirect introsort with NumPy's scalar tie order.
 * hdbscan_gpu/_kernels.py:358-516 (heapsort :358-387, median-of-3 Hoare
 * partition :389-405, insertion sort :407-415, serial driver :481-515):
 * depth limit 2*floor(log2(count)), partitions stop at 16 elements, the larger
 * side is deferred with the decremented depth and the smaller side continues in
 * place without re-checking the depth. */
static void FN(heap_sort)(const REAL* w, int32_t* order, int lo, int hi) {
    int count = hi - lo + 1;
    int32_t* a = order + lo - 1; /* 1-based view */
    for (int root = count / 2; root >= 1; --root) {
        int32_t value = a[root];
        int pos = root, child = 2 * root;
        while (child <= count) {
            if (child < count && w[a[child]] < w[a[child + 1]]) ++child;
            if (w[value] < w[a[child]]) {
                a[pos] = a[child];
                pos = child;
                child *= 2;
            } else {
                break;
            }
        }
        a[pos] = value;
    }
    for (int end = count; end > 1;) {
        int32_t value = a[end];
        a[end] = a[1];
        --end;
        int pos = 1, child = 2;
        while (child <= end) {
            if (child < end && w[a[child]] < w[a[child + 1]]) ++child;
            if (w[value] < w[a[child]]) {
                a[pos] = a[child];
                pos = child;
                child *= 2;
            } else {
                break;
            }
        }
        a[pos] = value;
    }
}

#define HDB_SWAP(p, q) do { int32_t t_ = (p); (p) = (q); (q) = t_; } while (0)

void FN(hdb_oracle_argsort)(const REAL* w, int m, int32_t* order, int depth_override, int use_override) {
    for (int i = 0; i < m; ++i) order[i] = i;
    if (m < 2) return;
    int stack_lo[64], stack_hi[64], stack_depth[64];
    int top = 0;
    int lo = 0, hi = m - 1, depth = 0;
    for (int c = m; c > 1; c >>= 1) depth += 2;
    if (use_override) depth = depth_override;
    for (;;) {
        if (depth < 0) {
            FN(heap_sort)(w, order, lo, hi);
        } else {
            while (hi - lo > 15) {
                int mid = lo + ((hi - lo) >> 1);
                if (w[order[mid]] < w[order[lo]]) HDB_SWAP(order[mid], order[lo]);
                if (w[order[hi]] < w[order[mid]]) HDB_SWAP(order[hi], order[mid]);
                if (w[order[mid]] < w[order[lo]]) HDB_SWAP(order[mid], order[lo]);
                REAL pivot = w[order[mid]];
                int i = lo, j = hi - 1;
                HDB_SWAP(order[mid], order[j]);
                for (;;) {
                    do { ++i; } while (w[order[i]] < pivot);
                    do { --j; } while (pivot < w[order[j]]);
                    if (i >= j) break;
                    HDB_SWAP(order[i], order[j]);
                }
                HDB_SWAP(order[i], order[hi - 1]);
                --depth;
                if (i - lo < hi - i) {
                    stack_lo[top] = i + 1; stack_hi[top] = hi;
                    hi = i - 1;
                } else {
                    stack_lo[top] = lo; stack_hi[top] = i - 1;
                    lo = i + 1;
                }
                stack_depth[top++] = depth;
            }
            for (int i = lo + 1; i <= hi; ++i) {
                int32_t value = order[i];
                int j = i;
                while (j > lo && w[value] < w[order[j - 1]]) {
                    order[j] = order[j - 1];
                    --j;
                }
                order[j] = value;
            }
        }
        if (top == 0) break;
        --top;
        lo = stack_lo[top]; hi = stack_hi[top]; depth = stack_depth[top];
    }
}

/* Optional outputs of one window (any pointer may be NULL).
 *   labels[n]                       final labels, -1 noise
 *   edges_uv[2*(n-1)], edge_w[n-1]  Prim edges (source, new vertex, weight) in Prim order
 *   order[n-1]                      argsort of edge_w
 *   link_lr[2*(n-1)], link_w, link_size   single-linkage rows for nodes n..2n-2
 *   n_clusters[1]                   condensed clusters including the root (ids n..)
 *   cl_parent/cl_birth/cl_stability/cl_selected/cl_size[n]   indexed by id - n
 *   point_parent[n], point_lambda[n]  condensed id each point falls out of, and at which lambda
 *   core[n]                         self-inclusive core distances (k = ms-1)
 *   core_nbr[n]                     lowest index j != i with d(i,j) == core (or -1)
 *   probabilities[n]                membership strength of each point (0 for noise) */
typedef struct {
    int32_t* labels;
    int32_t* edges_uv;
    REAL* edge_w;
    int32_t* order;
    int32_t* link_lr;
    REAL* link_w;
    int32_t* link_size;
    int32_t* n_clusters;
    int32_t* cl_parent;
    REAL* cl_birth;
    REAL* cl_stability;
    uint8_t* cl_selected;
    int32_t* cl_size;
    int32_t* point_parent;
    REAL* point_lambda;
    REAL* core;
    int32_t* core_nbr;
    REAL* probabilities;
} FN(hdb_oracle_out);

/* Graph stage: dense distance matrix + core distances -> hierarchy and labels.
 * core == NULL means the unit-core case (ms <= 2) where the mutual
 * reachability weight is the distance itself.
 * method 0 = excess of mass (the reference's only method), 1 = leaf;
 * allow_single != 0 lets the root be selected.  Both extensions restate
 * scikit-learn's cluster selection (sklearn/cluster/_hdbscan/_tree.pyx:644-799,
 * _do_labelling :433-512); with method 0 and allow_single 0 this is exactly
 * the reference's path. */
void FN(hdb_oracle_graph_ex)(const REAL* dist, const REAL* core, int n, int mcs, double eps_in, int method,
                             int allow_single, const FN(hdb_oracle_out)* out) {
    const REAL epsilon = (REAL)eps_in; /* options array is cast to the precision, _cuda.py:105 */
    const int unit_core = core == NULL;
    int m = n - 1;
    int32_t* eu = (int32_t*)malloc(sizeof(int32_t) * (size_t)(m > 0 ? m : 1));
    int32_t* ev = (int32_t*)malloc(sizeof(int32_t) * (size_t)(m > 0 ? m : 1));
    REAL* ew = (REAL*)malloc(sizeof(REAL) * (size_t)(m > 0 ? m : 1));
    int32_t* order = (int32_t*)malloc(sizeof(int32_t) * (size_t)(m > 0 ? m : 1));

    /* Prim over the dense mutual-reachability graph from vertex 0.
     * _kernels.py:164-320: strict '<' keeps the previous source on equal
     * weights (:236-240); argmin ties go to the lowest vertex index (:241-246,
     * :255-259); sources start at 1 and best at +inf (:166-169). */
    {
        uint8_t* in_tree = (uint8_t*)calloc((size_t)n, 1);
        REAL* best = (REAL*)malloc(sizeof(REAL) * (size_t)n);
        int32_t* src = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
        for (int j = 0; j < n; ++j) { best[j] = (REAL)INFINITY; src[j] = 1; }
        int current = 0;
        for (int i = 0; i < m; ++i) {
            in_tree[current] = 1;
            REAL candidate = REAL_MAX_VALUE;
            int next = 0, source = 0;
            for (int j = 0; j < n; ++j) {
                if (in_tree[j]) continue;
                REAL dcj = dist[(size_t)current * n + j];
                REAL weight = dcj;
                if (!unit_core) {
                    weight = FMAX(core[current], core[j]);
                    weight = FMAX(weight, dcj);
                }
                if (weight < best[j]) {
                    best[j] = weight;
                    src[j] = current;
                }
                weight = best[j];
                if (weight < candidate || (weight == candidate && j < next)) {
                    candidate = weight;
                    next = j;
                    source = src[j];
                }
            }
            eu[i] = candidate < REAL_MAX_VALUE ? source : 0;
            ev[i] = next;
            ew[i] = candidate;
            current = next;
        }
        free(in_tree); free(best); free(src);
    }

    FN(hdb_oracle_argsort)(ew, m, order, 0, 0);

    /* Single linkage over the sorted MST edges with scikit-learn's union-find
     * (sklearn/cluster/_hdbscan/_linkage.pyx make_single_linkage): each merge
     * creates node n+i whose children are the current roots of (edge_u,
     * edge_v), in that orientation.  Same tree as the balanced union-find of
     * _kernels.py:518-556. */
    int nodes = 2 * n - 1;
    int32_t* left = (int32_t*)malloc(sizeof(int32_t) * (size_t)nodes);
    int32_t* right = (int32_t*)malloc(sizeof(int32_t) * (size_t)nodes);
    int32_t* sizes = (int32_t*)malloc(sizeof(int32_t) * (size_t)nodes);
    REAL* ldist = (REAL*)malloc(sizeof(REAL) * (size_t)nodes);
    {
        int32_t* uf = (int32_t*)malloc(sizeof(int32_t) * (size_t)nodes);
        for (int i = 0; i < nodes; ++i) { uf[i] = -1; sizes[i] = i < n ? 1 : 0; left[i] = right[i] = -1; ldist[i] = 0; }
        for (int i = 0; i < m; ++i) {
            int e = order[i];
            int a = eu[e], c = ev[e];
            int ra = a; while (uf[ra] != -1) ra = uf[ra];
            while (a != ra) { int nx = uf[a]; uf[a] = ra; a = nx; }
            int rc = c; while (uf[rc] != -1) rc = uf[rc];
            while (c != rc) { int nx = uf[c]; uf[c] = rc; c = nx; }
            int node = n + i;
            left[node] = ra;
            right[node] = rc;
            sizes[node] = sizes[ra] + sizes[rc];
            ldist[node] = ew[e];
            uf[ra] = node;
            uf[rc] = node;
        }
        free(uf);
    }

    /* Breadth-first condensation from the root.  _kernels.py:558-643:
     * lambda = 1/d (+inf at d == 0); a split with both children >= mcs gives
     * two new consecutive cluster ids in queue order (:603-613); other children
     * either continue the parent cluster or are pruned leaf by leaf in BFS order
     * (:614-638), each leaf adding (lambda - birth) to the parent's stability. */
    int32_t* relabel = (int32_t*)malloc(sizeof(int32_t) * (size_t)nodes);
    int32_t* queue = (int32_t*)malloc(sizeof(int32_t) * (size_t)nodes);
    int32_t* prune = (int32_t*)malloc(sizeof(int32_t) * (size_t)nodes);
    int32_t* parent = (int32_t*)malloc(sizeof(int32_t) * (size_t)nodes);
    int32_t* csize = (int32_t*)malloc(sizeof(int32_t) * (size_t)nodes);
    REAL* birth = (REAL*)malloc(sizeof(REAL) * (size_t)nodes);
    REAL* stability = (REAL*)malloc(sizeof(REAL) * (size_t)nodes);
    uint8_t* selected = (uint8_t*)calloc((size_t)nodes, 1);
    int32_t* pparent = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    REAL* plambda = (REAL*)malloc(sizeof(REAL) * (size_t)n);
    int32_t* label_map = (int32_t*)malloc(sizeof(int32_t) * (size_t)nodes);
    for (int i = 0; i < nodes; ++i) {
        relabel[i] = -1; parent[i] = -1; csize[i] = 0; birth[i] = 0; stability[i] = 0; label_map[i] = -1;
    }
    int next_label = n + 1;
    {
        int root = 2 * n - 2, head = 0, tail = 1;
        queue[0] = root;
        relabel[root] = n;
        csize[n] = n;
        while (head < tail) {
            int node = queue[head++];
            int a = left[node], c = right[node];
            int cluster = relabel[node];
            REAL cluster_birth = birth[cluster];
            REAL cluster_stability = stability[cluster];
            REAL lambda = ldist[node] > 0 ? (REAL)1 / ldist[node] : (REAL)INFINITY;
            int large_a = sizes[a] >= mcs, large_c = sizes[c] >= mcs;
            int children[2] = {a, c};
            if (large_a && large_c) {
                for (int k = 0; k < 2; ++k) {
                    int child = children[k], label = next_label++;
                    relabel[child] = label;
                    parent[label] = cluster;
                    birth[label] = lambda;
                    csize[label] = sizes[child];
                    selected[label] = 1;
                    cluster_stability += (lambda - cluster_birth) * (REAL)sizes[child];
                    queue[tail++] = child;
                }
            } else {
                for (int k = 0; k < 2; ++k) {
                    int child = children[k];
                    if (k == 0 ? large_a : large_c) {
                        relabel[child] = cluster;
                        queue[tail++] = child;
                    } else {
                        int ph = 0, pt = 0, leaf = child;
                        for (;;) {
                            if (leaf < n) {
                                pparent[leaf] = cluster;
                                plambda[leaf] = lambda;
                                cluster_stability += lambda - cluster_birth;
                            } else {
                                prune[pt++] = left[leaf];
                                prune[pt++] = right[leaf];
                            }
                            if (ph == pt) break;
                            leaf = prune[ph++];
                        }
                    }
                }
            }
            stability[cluster] = cluster_stability;
        }
    }

    /* Cluster selection.
     * Excess of mass, _kernels.py:672-710: children are summed in ascending id
     * order, a node whose children's sum is strictly larger is deselected and
     * inherits the sum; then every descendant of a selected node is suppressed
     * in one forward pass (parents have smaller ids).  With allow_single the
     * root takes part like any other cluster (_tree.pyx:704-708, 727-739).
     * Leaf, _tree.pyx:761-781: the clusters without child clusters; none when
     * the root never splits. */
    const int root = n;
    const int splits = next_label > root + 1;
    {
        if (method == 0) {
            if (allow_single) selected[root] = 1;
            for (int node = next_label - 1; node >= (allow_single ? root : root + 1); --node) {
                REAL subtree = 0;
                for (int child = node + 1; child < next_label; ++child)
                    if (parent[child] == node) subtree += stability[child];
                if (subtree > stability[node]) {
                    selected[node] = 0;
                    stability[node] = subtree;
                }
            }
            uint8_t* blocked = (uint8_t*)calloc((size_t)nodes, 1);
            blocked[root] = selected[root];
            for (int node = n + 1; node < next_label; ++node) {
                int inherited = blocked[parent[node]];
                blocked[node] = (uint8_t)(inherited || selected[node]);
                if (inherited) selected[node] = 0;
            }
            free(blocked);
        } else {
            uint8_t* has_child = (uint8_t*)calloc((size_t)nodes, 1);
            for (int node = n + 1; node < next_label; ++node) has_child[parent[node]] = 1;
            selected[root] = 0;
            for (int node = n + 1; node < next_label; ++node) selected[node] = !has_child[node];
            free(has_child);
        }
    }

    /* Epsilon merge, _kernels.py:712-760: a selected cluster with 1/birth <
     * eps climbs to its first ancestor with 1/birth > eps; the climb stops
     * below the root (at the root with allow_single, _tree.pyx:578-603).
     * Skipped when the root never splits (_tree.pyx:741).  Every selected
     * cluster marks the cluster it resolves to (the reference's rule). */
    int32_t* resolved_cluster = (int32_t*)malloc(sizeof(int32_t) * (size_t)nodes);
    {
        if (epsilon > 0 && splits) {
            int32_t* stop = (int32_t*)malloc(sizeof(int32_t) * (size_t)nodes);
            uint8_t* chosen_mark = (uint8_t*)calloc((size_t)nodes, 1);
            stop[root] = root;
            if (selected[root]) chosen_mark[root] = 1;  /* 1/birth(root) = inf: never climbs */
            for (int node = n + 1; node < next_label; ++node) {
                int ancestor = parent[node];
                stop[node] = ancestor == root ? (allow_single ? root : node)
                           : ((REAL)1 / birth[ancestor] > epsilon ? ancestor : stop[ancestor]);
                if (!selected[node]) continue;
                int chosen = (REAL)1 / birth[node] < epsilon ? stop[node] : node;
                chosen_mark[chosen] = 1;
            }
            for (int node = root; node < next_label; ++node) selected[node] = chosen_mark[node];
            free(stop);
            free(chosen_mark);
        }
        /* Labels number the selected clusters by ascending id (the root first
         * when selected, _tree.pyx:785); every point takes its nearest selected
         * ancestor; a point whose nearest one is the root is noise unless the
         * root is the only cluster (allow_single), when it joins at lambda >=
         * 1/eps, or >= the largest lambda leaving the root when eps = 0
         * (_tree.pyx:491-508). */
        int label = 0, count = 0;
        for (int node = root; node < next_label; ++node) {
            label_map[node] = selected[node] ? label++ : -1;
            count += selected[node];
        }
        resolved_cluster[root] = selected[root] ? root : -1;
        for (int node = n + 1; node < next_label; ++node)
            resolved_cluster[node] = selected[node] ? node : resolved_cluster[parent[node]];
        REAL* deaths = (REAL*)calloc((size_t)nodes, sizeof(REAL));  /* largest lambda leaving each cluster */
        for (int i = 0; i < n; ++i) deaths[pparent[i]] = deaths[pparent[i]] > plambda[i] ? deaths[pparent[i]] : plambda[i];
        for (int node = n + 1; node < next_label; ++node)
            deaths[parent[node]] = deaths[parent[node]] > birth[node] ? deaths[parent[node]] : birth[node];
        const int single_root = allow_single && count == 1 && selected[root];
        const REAL threshold = epsilon != 0 ? (REAL)1 / epsilon : deaths[root];
        for (int i = 0; i < n; ++i) {
            int c = resolved_cluster[pparent[i]];
            int lab = -1;
            if (c > root) lab = label_map[c];
            else if (c == root && single_root && plambda[i] >= threshold) lab = label_map[root];
            if (out->labels) out->labels[i] = lab;
            /* Membership strength, _tree.pyx:515-554. */
            if (out->probabilities) {
                REAL prob = 0;
                if (lab >= 0) {
                    const REAL max_lambda = deaths[c];
                    if (max_lambda == 0 || isinf((double)plambda[i])) prob = 1;
                    else prob = (plambda[i] < max_lambda ? plambda[i] : max_lambda) / max_lambda;
                }
                out->probabilities[i] = prob;
            }
        }
        free(deaths);
    }
    free(resolved_cluster);

    if (out->edges_uv) for (int i = 0; i < m; ++i) { out->edges_uv[2 * i] = eu[i]; out->edges_uv[2 * i + 1] = ev[i]; }
    if (out->edge_w) for (int i = 0; i < m; ++i) out->edge_w[i] = ew[i];
    if (out->order) for (int i = 0; i < m; ++i) out->order[i] = order[i];
    if (out->link_lr) for (int i = 0; i < m; ++i) { out->link_lr[2 * i] = left[n + i]; out->link_lr[2 * i + 1] = right[n + i]; }
    if (out->link_w) for (int i = 0; i < m; ++i) out->link_w[i] = ldist[n + i];
    if (out->link_size) for (int i = 0; i < m; ++i) out->link_size[i] = sizes[n + i];
    if (out->n_clusters) *out->n_clusters = next_label - n;
    for (int c = 0; c < next_label - n; ++c) {
        if (out->cl_parent) out->cl_parent[c] = parent[n + c];
        if (out->cl_birth) out->cl_birth[c] = birth[n + c];
        if (out->cl_stability) out->cl_stability[c] = stability[n + c];
        if (out->cl_selected) out->cl_selected[c] = selected[n + c];
        if (out->cl_size) out->cl_size[c] = csize[n + c];
    }
    if (out->point_parent) for (int i = 0; i < n; ++i) out->point_parent[i] = pparent[i];
    if (out->point_lambda) for (int i = 0; i < n; ++i) out->point_lambda[i] = plambda[i];

    free(eu); free(ev); free(ew); free(order);
    free(left); free(right); free(sizes); free(ldist);
    free(relabel); free(queue); free(prune); free(parent); free(csize); free(birth); free(stability);
    free(selected); free(pparent); free(plambda); free(label_map);
}

void FN(hdb_oracle_graph)(const REAL* dist, const REAL* core, int n, int mcs, double eps_in,
                          const FN(hdb_oracle_out)* out) {
    FN(hdb_oracle_graph_ex)(dist, core, n, mcs, eps_in, 0, 0, out);
}

/* Full per-window pipeline from points.  Returns the window status (0 ok,
 * 1 distance overflow, 2 non-finite input; 2 outranks 1 as the host checks at
 * _cuda.py:98-99 run before those at :112-113).  out may be NULL. */
int FN(hdb_oracle_cluster_ex)(const REAL* x, int n, int d, int mcs, int ms, double eps, int method,
                              int allow_single, const FN(hdb_oracle_out)* out) {
    FN(hdb_oracle_out) none;
    memset(&none, 0, sizeof(none));
    if (!out) out = &none;
    for (size_t t = 0; t < (size_t)n * d; ++t)
        if (!isfinite((double)x[t])) return 2;
    REAL* dist = (REAL*)malloc(sizeof(REAL) * (size_t)n * n);
    REAL* core = (REAL*)malloc(sizeof(REAL) * (size_t)n);
    REAL* rowbuf = (REAL*)malloc(sizeof(REAL) * (size_t)n);
    FN(hdb_oracle_distances)(x, n, d, dist);
    int status = 0;
    for (size_t t = 0; t < (size_t)n * n; ++t)
        if (!isfinite((double)dist[t])) status = 1;
    if (!status) {
        const int unit_core = ms <= 2; /* _cuda.py:85, UNIT_CORE at _kernels.py:230-235 */
        if (!unit_core || out->core || out->core_nbr) FN(hdb_oracle_core)(dist, n, ms, core, rowbuf);
        if (out->core)
            for (int i = 0; i < n; ++i) out->core[i] = core[i];
        if (out->core_nbr) {
            for (int i = 0; i < n; ++i) {
                out->core_nbr[i] = -1;
                for (int j = 0; j < n; ++j)
                    if (j != i && dist[(size_t)i * n + j] == core[i]) { out->core_nbr[i] = j; break; }
            }
        }
        FN(hdb_oracle_graph_ex)(dist, unit_core ? NULL : core, n, mcs, eps, method, allow_single, out);
    }
    free(dist); free(core); free(rowbuf);
    return status;
}

int FN(hdb_oracle_cluster)(const REAL* x, int n, int d, int mcs, int ms, double eps,
                           const FN(hdb_oracle_out)* out) {
    return FN(hdb_oracle_cluster_ex)(x, n, d, mcs, ms, eps, 0, 0, out);
}

typedef struct {
    const REAL* x;
    const int64_t* offsets;
    int windows, d, mcs, ms;
    double eps;
    int32_t* labels;
    int32_t* status;
    int next; /* shared ticket */
} FN(hdb_batch_job);

static void* FN(hdb_batch_worker)(void* arg) {
    FN(hdb_batch_job)* job = (FN(hdb_batch_job)*)arg;
    for (;;) {
        int w = __atomic_fetch_add(&job->next, 1, __ATOMIC_RELAXED);
        if (w >= job->windows) break;
        int64_t lo = job->offsets[w], hi = job->offsets[w + 1];
        FN(hdb_oracle_out) out;
        memset(&out, 0, sizeof(out));
        out.labels = job->labels + lo;
        int s = FN(hdb_oracle_cluster)(job->x + lo * job->d, (int)(hi - lo), job->d, job->mcs, job->ms, job->eps,
                                       &out);
        if (job->status) job->status[w] = s;
    }
    return NULL;
}

/* Ragged batch over host threads (CPU baseline): windows are independent, so
 * worker threads take them from a shared ticket. */
int FN(hdb_oracle_batch)(const REAL* x, const int64_t* offsets, int windows, int d, int mcs, int ms,
                         double eps, int32_t* labels, int32_t* status, int threads) {
    FN(hdb_batch_job) job = {x, offsets, windows, d, mcs, ms, eps, labels, status, 0};
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    pthread_t tid[256];
    for (int t = 1; t < threads; ++t) pthread_create(&tid[t], NULL, FN(hdb_batch_worker), &job);
    FN(hdb_batch_worker)(&job);
    for (int t = 1; t < threads; ++t) pthread_join(tid[t], NULL);
    return 0;
}

/* Ragged batch with every stage's state, over host threads (parity tests).
 * `out` members point at packed arrays laid out as the GPU exports are: edge
 * rows of window w at offsets[w] - w, point and cluster rows at offsets[w],
 * n_clusters at w; NULL members are skipped. */
typedef struct {
    const REAL* x;
    const int64_t* offsets;
    int windows, d, mcs, ms;
    double eps;
    const FN(hdb_oracle_out)* out;
    int32_t* status;
    int next; /* shared ticket */
} FN(hdb_batch_ex_job);

#define HDB_AT(ptr, at) ((ptr) ? (ptr) + (at) : NULL)

static void* FN(hdb_batch_ex_worker)(void* arg) {
    FN(hdb_batch_ex_job)* job = (FN(hdb_batch_ex_job)*)arg;
    const FN(hdb_oracle_out)* o = job->out;
    for (;;) {
        int w = __atomic_fetch_add(&job->next, 1, __ATOMIC_RELAXED);
        if (w >= job->windows) break;
        int64_t lo = job->offsets[w], hi = job->offsets[w + 1], e = lo - w;
        FN(hdb_oracle_out) out;
        out.labels = HDB_AT(o->labels, lo);
        out.edges_uv = HDB_AT(o->edges_uv, 2 * e);
        out.edge_w = HDB_AT(o->edge_w, e);
        out.order = HDB_AT(o->order, e);
        out.link_lr = HDB_AT(o->link_lr, 2 * e);
        out.link_w = HDB_AT(o->link_w, e);
        out.link_size = HDB_AT(o->link_size, e);
        out.n_clusters = HDB_AT(o->n_clusters, w);
        out.cl_parent = HDB_AT(o->cl_parent, lo);
        out.cl_birth = HDB_AT(o->cl_birth, lo);
        out.cl_stability = HDB_AT(o->cl_stability, lo);
        out.cl_selected = HDB_AT(o->cl_selected, lo);
        out.cl_size = HDB_AT(o->cl_size, lo);
        out.point_parent = HDB_AT(o->point_parent, lo);
        out.point_lambda = HDB_AT(o->point_lambda, lo);
        out.core = HDB_AT(o->core, lo);
        out.core_nbr = HDB_AT(o->core_nbr, lo);
        out.probabilities = HDB_AT(o->probabilities, lo);
        int s = FN(hdb_oracle_cluster)(job->x + lo * job->d, (int)(hi - lo), job->d, job->mcs, job->ms, job->eps,
                                       &out);
        if (job->status) job->status[w] = s;
    }
    return NULL;
}

#undef HDB_AT

int FN(hdb_oracle_batch_ex)(const REAL* x, const int64_t* offsets, int windows, int d, int mcs, int ms,
                            double eps, const FN(hdb_oracle_out)* out, int32_t* status, int threads) {
    FN(hdb_batch_ex_job) job = {x, offsets, windows, d, mcs, ms, eps, out, status, 0};
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    pthread_t tid[256];
    for (int t = 1; t < threads; ++t) pthread_create(&tid[t], NULL, FN(hdb_batch_ex_worker), &job);
    FN(hdb_batch_ex_worker)(&job);
    for (int t = 1; t < threads; ++t) pthread_join(tid[t], NULL);
    return 0;
}

#undef FN
#undef HDB_CAT
#undef HDB_CAT2
#undef HDB_SWAP
