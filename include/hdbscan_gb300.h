/*
 * hdbscan_gb300 — C ABI of the GB300 (sm_103a) batched HDBSCAN library.
 *
 * Drop-in for the CUDA path of CosineAI/hdbscan's
 *   hdbscan_gpu.hdbscan(X, backend="cuda", precision=..., min_cluster_size,
 *                       min_samples, cluster_selection_epsilon) -> int32 labels
 * whose backend seam is `cluster(x, min_cluster_size, min_samples, epsilon,
 * precision)` (hdbscan_gpu/_api.py:92-102, implemented by
 * hdbscan_gpu/_cuda.py:91-128).
 *
 * Conventions
 *  - Every entry point returns 0 on success or a negative HDB_E_* code; the
 *    message of the calling thread's last failure is hdb_last_error().  No C++
 *    exception crosses this boundary.
 *  - Device pointers are plain addresses on the device that was current when
 *    the plan was created; `stream` is a cudaStream_t (NULL = legacy default).
 *    All device work is ordered on `stream`; nothing synchronizes the host.
 *  - The library allocates no device memory per call: the caller passes a
 *    workspace of hdb_plan_workspace_bytes() bytes (256-byte aligned).
 *  - Results are bit-exact with the reference CUDA path: Prim edges, NumPy
 *    tie order of the edge sort, linkage ids/orientation/weights/sizes,
 *    condensed clusters and labels.
 *  - The device status word is a bit-or of HDB_STATUS_*; it is zeroed by each
 *    forward call and read by the caller after synchronizing (the reference
 *    raises at its two host syncs, _cuda.py:98-99 and :112-113).
 *  - Threading: every entry point may be called from any host thread and any
 *    stream.  Calls on one plan (forward, capture, replay, backward) enqueue
 *    one at a time under the plan's lock; each call waits only for its own
 *    work.  The dense entry points share plans from a cache of 16 shapes and
 *    hold a reference while they enqueue, so eviction never frees a plan in
 *    use.  Concurrent calls must not share a workspace, labels or status.
 *    While a caller's own stream capture holds a plan's forward (not
 *    hdb_plan_capture), other threads must not use that plan until the
 *    capture ends.
 *  - Window sizes (offsets) are host data given at plan creation: the plan
 *    chooses kernels and sorts windows into its work queues from them.  A
 *    caller whose offsets live on the device copies them to the host once
 *    per batch shape, then reuses the plan (or its captured graph).
 */
#ifndef HDBSCAN_GB300_H
#define HDBSCAN_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HDB_VERSION 1

#define HDB_F32 0
#define HDB_F64 1

#define HDB_MAX_SAMPLES 4096 /* points per window, as MAX_SAMPLES at hdbscan_gpu/_api.py:7 */

/* Return codes. */
#define HDB_OK 0
#define HDB_E_INVALID (-1)   /* bad argument (message says which) */
#define HDB_E_CUDA (-2)      /* a CUDA runtime call failed */
#define HDB_E_WORKSPACE (-3) /* workspace missing, too small or misaligned */
#define HDB_E_DEVICE (-4)    /* called with a different current device than the plan's */

/* Device status bits (bit-or). */
#define HDB_STATUS_OVERFLOW 1  /* a pairwise distance overflowed the precision */
#define HDB_STATUS_NONFINITE 2 /* an input coordinate is NaN or infinite (outranks overflow) */
#define HDB_STATUS_INTERNAL 4  /* a device-side consistency check failed */

/* Plan flags. */
#define HDB_FLAG_FORCE_MATRIX 1u /* materialize every window's distance block (matrix Prim) */
#define HDB_FLAG_NO_GRAPH_STREAMS 2u /* run all window classes on the caller's stream */
#define HDB_FLAG_ONE_PERSISTENT 4u /* one persistent CTA (or cluster) per window class: every window of a
                                      class passes through the same CTAs (queue and hand-off tests) */
/* Cluster selection beyond the reference's fixed contract (excess of mass, no
 * single cluster), as scikit-learn's HDBSCAN(cluster_selection_method=,
 * allow_single_cluster=) defines them (sklearn/cluster/_hdbscan/_tree.pyx). */
#define HDB_FLAG_LEAF 8u           /* cluster_selection_method="leaf" */
#define HDB_FLAG_ALLOW_SINGLE 16u  /* allow_single_cluster=True */
/* Producer stage (no reference counterpart): X holds bfloat16 / float16
 * values (converted exactly to the compute precision), and/or every point is
 * L2-normalised first (s = sum of x_k*x_k in k order, x_k / sqrt(s), both
 * round-to-nearest; zero vectors unchanged).  One pass into the workspace;
 * hdb_plan_backward refuses such plans. */
#define HDB_FLAG_INPUT_BF16 32u
#define HDB_FLAG_INPUT_F16 64u
#define HDB_FLAG_L2_NORMALIZE 128u
/* Test only (no reference counterpart): in windows run on a thread-block
 * cluster the first window ticket is never broadcast, so every CTA's first
 * bounded wait runs out after 1 ms; the kernel then ends with
 * HDB_STATUS_INTERNAL and writes no labels.  It exercises the give-up path of
 * the cluster waits without any transfer in flight. */
#define HDB_FLAG_TEST_STALL 256u

typedef struct hdb_plan hdb_plan_t;

/* Optional device outputs of a forward call; NULL members are skipped.
 * E = sum over windows of (n_w - 1) edges; T = sum of n_w points; B windows.
 * Edge rows of window w start at offsets[w] - w, per-point and per-cluster
 * rows at offsets[w] (clusters are indexed by condensed id - n_w). */
typedef struct hdb_exports {
    int32_t* edges_uv;     /* [E,2] Prim edges (source, new vertex), window-local ids */
    void* edge_w;          /* [E]   Prim edge weights (Real) */
    int32_t* order;        /* [E]   NumPy-quicksort order of edge_w (window-local) */
    int32_t* link_lr;      /* [E,2] single-linkage children of node n_w + i */
    void* link_w;          /* [E]   merge weights (Real), sklearn single_linkage_tree_ 'value' */
    int32_t* link_size;    /* [E]   merged cluster sizes */
    int32_t* n_clusters;   /* [B]   condensed clusters incl. the root */
    int32_t* cl_parent;    /* [T]   condensed parent id (-1 for the root) */
    void* cl_birth;        /* [T]   lambda at which the cluster was born (Real) */
    void* cl_stability;    /* [T]   stability after excess-of-mass selection (Real) */
    uint8_t* cl_selected;  /* [T]   final selection flag */
    int32_t* point_parent; /* [T]   condensed cluster each point falls out of */
    void* core;            /* [T]   core distances (Real); written when min_samples > 2 */
    int32_t* core_nbr;     /* [T]   ms-th nearest neighbour in (distance, index) order */
    int64_t* stage_ns;     /* [B,8] device timestamps (ns) per window: start, Prim start, Prim end,
                                    hierarchy start, sort end, linkage end, condensation end, labels end */
    void* probabilities;   /* [T]   membership strength in [0, 1] (Real), scikit-learn's probabilities_ */
    /* Condensed-tree rows as scikit-learn's condensed_tree_ holds them
     * (sklearn/cluster/_hdbscan/_tree.pyx:122-237): cluster c > n_w is the row
     * (cl_parent, c, cl_birth, cl_size); point i is (point_parent, i,
     * point_lambda, 1). */
    int32_t* cl_size;      /* [T]   points in each condensed cluster when it is born (root: n_w) */
    void* point_lambda;    /* [T]   lambda at which each point falls out of its cluster (Real) */
} hdb_exports_t;

/* Library version (HDB_VERSION). */
int hdb_version(void);

/* Message of the calling thread's most recent failure ("" if none). */
const char* hdb_last_error(void);

/* Autotune table used by later hdb_plan_create calls (process-wide).  Each
 * rule is 9 int32: {precision (HDB_F32/HDB_F64/-1 any), unit core (1 =
 * min_samples <= 2, 0 = core distances, -1 any), n_max, d_max, Prim threads,
 * slots per thread, register dims (0 = matrix variant), CTAs per window (1 =
 * one CTA, 2..8 = a thread-block cluster), CTAs per SM (1..4)}; the first rule
 * that matches a window and names a compiled variant wins, built-in defaults
 * back it up.
 * n_rules = 0 restores the defaults.  Replaces the fixed launch choice of
 * hdbscan_gpu/_cuda.py:82-88 (block width, register Prim, shared arena). */
int hdb_set_tuning(const int32_t* rules, int n_rules);

/* Copies up to `capacity` rules of the current table; returns their count. */
int hdb_get_tuning(int32_t* rules, int capacity);

/* Compiled forward variants of a precision as {Prim threads, slots, register
 * dims (0 = matrix), CTAs per window, CTAs per SM} 5-tuples; returns their
 * count (the autotuner's candidates). */
int hdb_list_variants(int precision, int32_t* out, int capacity);

/* Build a plan for a ragged batch: `windows` windows whose points are rows
 * offsets_host[w] .. offsets_host[w+1]-1 of a packed [T, dims] array.
 * Validation and messages follow hdbscan_gpu/_api.py:32-87: min_cluster_size
 * >= 2, 1 <= min_samples <= every n_w, 2 <= n_w <= HDB_MAX_SAMPLES.  The plan
 * chooses per-window kernel variants (autotune table), sorts windows by size
 * into a persistent work queue and owns a pinned copy of its device tables.
 * Replaces the per-call kernel selection of hdbscan_gpu/_cuda.py:66-88. */
int hdb_plan_create(hdb_plan_t** plan, int precision, int windows, const int64_t* offsets_host, int dims,
                    int min_cluster_size, int min_samples, double epsilon, unsigned flags);

int hdb_plan_destroy(hdb_plan_t* plan);

/* Bytes of device workspace a forward/backward call of this plan needs. */
size_t hdb_plan_workspace_bytes(const hdb_plan_t* plan);

/* JSON description of the plan's window classes and kernel choices. */
int hdb_plan_describe(const hdb_plan_t* plan, char* buffer, size_t size);

/* Cluster the batch: X is the packed [T, dims] Real array, labels [T] int32
 * (-1 noise), status one int32.  Replaces hdbscan_gpu/_cuda.py:91-128. */
int hdb_plan_forward(hdb_plan_t* plan, const void* X, int32_t* labels, void* workspace, size_t workspace_bytes,
                     int32_t* status, const hdb_exports_t* exports, void* stream);

/* Phases of the forward, for hdb_plan_profile. */
#define HDB_PHASE_PREPARE 0  /* producer stage (bfloat16/float16 input, L2 normalisation) */
#define HDB_PHASE_DISTANCE 1 /* distance blocks of matrix-variant windows */
#define HDB_PHASE_CORE 2     /* core distances */
#define HDB_PHASE_FORWARD 3  /* persistent Prim + hierarchy kernels */
#define HDB_PHASES 4

/* hdb_plan_forward with every launch serialized on `stream` and timed by CUDA
 * events (no reference counterpart: the reference's stage profiler times its
 * stages with host synchronizations, scripts/profile_cuda.py:49-90).  Writes
 * the summed milliseconds per phase into phase_ms[HDB_PHASES] and, when not
 * NULL, the launches per phase into phase_launches[HDB_PHASES]; synchronizes
 * the stream.  Results equal hdb_plan_forward's. */
int hdb_plan_profile(hdb_plan_t* plan, const void* X, int32_t* labels, void* workspace, size_t workspace_bytes,
                     int32_t* status, const hdb_exports_t* exports, void* stream, double* phase_ms,
                     int32_t* phase_launches);

/* Capture hdb_plan_forward with these exact pointers into a CUDA graph owned
 * by the plan (replacing any previous one), then hdb_plan_replay() launches
 * it.  The pointers must stay valid while the graph is used. */
int hdb_plan_capture(hdb_plan_t* plan, const void* X, int32_t* labels, void* workspace, size_t workspace_bytes,
                     int32_t* status, const hdb_exports_t* exports, void* stream);
int hdb_plan_replay(hdb_plan_t* plan, void* stream);

/* Gradient of the merge weights with respect to X (no reference
 * counterpart: the reference has no gradients).  `exports` must hold the
 * edges_uv, order and link_w of the forward call on the same X (and core,
 * core_nbr when min_samples > 2); grad is [E] Real in linkage order; dX is
 * [T, dims] Real and is accumulated into (zero it first). */
int hdb_plan_backward(hdb_plan_t* plan, const void* X, const hdb_exports_t* exports, const void* grad, void* dX,
                      void* workspace, size_t workspace_bytes, void* stream);

/* Dense uniform batch, the reference seam itself: X [batch, n, dims]
 * contiguous, labels [batch, n].  Plans are cached per shape/parameters. */
size_t hdb_cluster_workspace_bytes(int precision, int batch, int n, int dims, int min_cluster_size,
                                   int min_samples);
int hdb_cluster_f32(const float* X, int batch, int n, int dims, int min_cluster_size, int min_samples,
                    double epsilon, int32_t* labels, void* workspace, size_t workspace_bytes, int32_t* status,
                    void* stream);
int hdb_cluster_f64(const double* X, int batch, int n, int dims, int min_cluster_size, int min_samples,
                    double epsilon, int32_t* labels, void* workspace, size_t workspace_bytes, int32_t* status,
                    void* stream);

/* Dense batch without any device allocation.  This entry point has no
 * counterpart in the reference.  It serves callers that may not allocate
 * device memory where they cluster: a serving process that gives all device
 * memory to its own pool at start-up and treats any other allocation as an
 * error, or a plugin whose host framework owns the device allocator.  They
 * pass X and labels (and status) as usual; the scratch the kernels need
 * (window tables, work queue, core distances) is one array of
 * HDB_NOALLOC_SCRATCH_BYTES compiled into this library, which stays resident
 * on every device that loads the library until the process exits.
 *  - Limits: batch <= HDB_NOALLOC_MAX_WINDOWS, batch*n <= HDB_NOALLOC_MAX_POINTS,
 *    and dims by window size (every window's coordinates stay in registers):
 *      float32: n <= 1024: dims <= 32; n <= 2048: dims <= 16; n <= 4096: dims <= 8
 *      float64: n <= 1024: dims <= 16; n <= 2048: dims <= 8; larger windows: none
 *    Larger requests fail with HDB_E_INVALID and a message naming the limit.
 *  - The first call in a CUDA context (normally the device's primary context)
 *    looks up the array's device address with that context current and caches
 *    it per context; make that first call before any stream capture.
 *  - All calls share the one array and overwrite it: calls that overlap on the
 *    GPU (other streams or host threads) race; order them on one stream.
 *  - Calls no cudaMalloc/cudaFree and no allocating library routine. */
#define HDB_NOALLOC_MAX_WINDOWS 16384
#define HDB_NOALLOC_MAX_POINTS 262144
#define HDB_NOALLOC_SCRATCH_BYTES (5u << 20)
int hdb_cluster_noalloc(int precision, const void* X, int batch, int n, int dims, int min_cluster_size,
                        int min_samples, double epsilon, int32_t* labels, int32_t* status, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* HDBSCAN_GB300_H */
