// C ABI and host plan layer (include/hdbscan_gb300.h).
//
// A plan turns a ragged batch description into: per-window kernel variants
// (the autotune table in choose_variant), window classes launched as
// persistent grids over size-sorted queues, the tile and row work lists of
// the distance/core kernels, and one pinned host image of every device table,
// uploaded by a single cudaMemcpyAsync per call so the whole forward is
// capturable in a CUDA graph.  The distance tiles and core distances run as
// one chain on the caller's stream, class by class from the largest windows
// down; each class's persistent forward is forked onto its own stream (higher
// priority for larger windows) as soon as its own inputs are ready, so the
// longest Prim loops start first and the remaining pre-work and smaller
// classes fill the other SMs.  The order is explicit in the dependencies, so
// a captured graph schedules exactly like the stream launch.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <list>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/hdbscan_gb300.h"
#include "hdb_args.h"
#include "hdb_registry.h"

namespace {

thread_local std::string g_error;

int fail(int code, const std::string& message) {
    g_error = message;
    return code;
}

#define HDB_CUDA(call)                                                                        \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) return fail(HDB_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

struct CoreLaunch {
    const hdb::CoreVariant* cv = nullptr;  // null = select kernel
    bool matrix = false;
    std::vector<int32_t> items;             // (window, row) pairs
    size_t items_off = 0;                   // byte offset in tables
    size_t select_smem = 0;
};

struct WindowClass {
    const hdb::ForwardVariant* fv = nullptr;
    int x_in_smem = 0;
    int n_arenas = 1;
    hdb::ForwardLayout layout{};
    std::vector<int> windows;  // descending n
    int nmax = 0;
    size_t smem = 0;
    int grid = 0;
    size_t queue_off = 0;      // element offset into the queue table
    int ticket = 0;            // index into the ticket table
    int priority = 0;          // launch priority (largest windows highest)
    size_t tiles_first = 0;    // first distance tile (triple) of this class
    size_t n_tiles = 0;
    int tile = 64;             // distance tile edge
    std::vector<CoreLaunch> cores;
};

}  // namespace

struct hdb_plan {
    int precision = 0;
    int B = 0;
    int D = 0;
    int mcs = 2;
    int ms = 1;
    double eps = 0;
    unsigned flags = 0;
    int device = 0;
    int sms = 0;
    int64_t T = 0;
    std::vector<int64_t> offsets;
    const hdb::PrecisionKernels* k = nullptr;
    std::vector<WindowClass> classes;
    std::vector<int32_t> tiles;             // (window, ti, tj), grouped by class
    std::vector<int64_t> dist_offsets;      // per window (elements), -1 if not materialized
    int64_t dist_elems = 0;
    // Table layout (byte offsets within the workspace).
    size_t t_offsets = 0, t_dist_off = 0, t_queue = 0, t_tickets = 0, t_tiles = 0, t_edge_window = 0;
    size_t tables_bytes = 0;
    size_t w_core = 0, w_core_nbr = 0, w_dist = 0, w_prep = 0, ws_bytes = 0;
    int input_type = 0;     // hdb::InputType of X
    int normalize = 0;      // L2-normalise every point first
    bool prepared = false;  // X passes through the producer stage into the workspace
    unsigned char* h_tables = nullptr;      // pinned
    std::vector<cudaStream_t> aux;          // one per class (empty: everything on the caller's stream)
    std::vector<cudaEvent_t> events;        // [2i] class i inputs ready, [2i+1] class i done
    cudaEvent_t uploaded = nullptr;         // after the latest (uncaptured) upload of h_tables
    cudaGraphExec_t graph = nullptr;
    // Serializes the host-side enqueue of forward, capture and backward calls:
    // the fork/join events and class streams above are shared by every call,
    // and cudaStreamWaitEvent waits on an event's latest record at the time of
    // the call, so each call's record/wait pairs must not interleave with
    // another thread's.  Work of concurrent calls then orders on the class
    // streams; each call still joins only its own forwards.
    std::mutex enqueue;
};

namespace hdb {

void set_last_error(const char* message) { g_error = message; }

// The dynamic shared-memory limit is a per-function attribute shared by every
// caller in the process, so it only ever grows: lowering it to one plan's need
// would break launches of an earlier plan with larger windows.
static std::mutex g_attr_mutex;
cudaError_t raise_dynamic_smem(const void* func, size_t bytes) {
    std::lock_guard<std::mutex> lock(g_attr_mutex);
    cudaFuncAttributes attr;
    cudaError_t e = cudaFuncGetAttributes(&attr, func);
    if (e != cudaSuccess) return e;
    if ((size_t)attr.maxDynamicSharedSizeBytes >= bytes) return cudaSuccess;
    return cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

}  // namespace hdb

namespace {

int real_bytes(int precision) { return precision == HDB_F32 ? 4 : 8; }

constexpr size_t kChunks = 4;     // pipeline depth for large matrix-variant classes
constexpr size_t kMinChunk = 8;   // windows per chunk at least
constexpr int kTile128MinN = 384;  // float32 matrix classes from this size use 128x128 distance tiles

cudaError_t raise_smem_limit(const void* func, size_t bytes) { return hdb::raise_dynamic_smem(func, bytes); }

// Autotune rules: the first rule whose (precision, core mode, n, D) bounds
// match a window picks its variant (Prim threads, slots per thread, register
// dimensions; dims 0 = matrix variant; CTAs per window, 1 = single CTA; CTAs
// per SM).  The compiled-in defaults below are
// replaced at run time by hdb_set_tuning (the package loads the table that
// hdbscan_gb300/autotune.py measured).  A rule naming a variant that is not
// compiled falls through to the next rule, and the shape heuristic backs up
// the whole table.
struct TuningRule {
    int precision;  // HDB_F32 / HDB_F64 / -1 any
    int unit;       // 1 = min_samples <= 2, 0 = core distances, -1 any
    int n_max;
    int d_max;
    int threads;
    int slots;
    int dims;       // register dimensions; 0 = matrix variant
    int cluster;    // CTAs per window (thread-block cluster size); 1 = single CTA
    int per_sm;     // CTAs per SM of a single-CTA variant (1 or 2)
};
constexpr int kRuleFields = 9;

std::mutex g_tuning_mutex;
std::vector<TuningRule> g_tuning;  // empty = defaults

void class_shape(int n, int* threads, int* v) {
    if (n <= 64) { *threads = 32; *v = 2; }
    else if (n <= 128) { *threads = 64; *v = 2; }
    else if (n <= 256) { *threads = 128; *v = 2; }
    else if (n <= 512) { *threads = 256; *v = 2; }
    else if (n <= 1024) { *threads = 512; *v = 2; }
    else if (n <= 2048) { *threads = 512; *v = 4; }
    else { *threads = 512; *v = 8; }
}

const hdb::ForwardVariant* find_variant(const hdb::PrecisionKernels& k, int threads, int v, int dp, int cluster = 1,
                                        int per_sm = 1) {
    const hdb::ForwardVariant* list = cluster > 1 ? k.cluster : k.forward;
    const int count = cluster > 1 ? k.n_cluster : k.n_forward;
    for (int i = 0; i < count; ++i) {
        const hdb::ForwardVariant& f = list[i];
        if (f.threads == threads && f.v == v && f.dp == dp && f.cluster == cluster && f.per_sm == per_sm) return &f;
    }
    return nullptr;
}

const hdb::ForwardVariant* choose_variant(const hdb::PrecisionKernels& k, int precision, int n, int D,
                                          bool unit, bool force_matrix, bool allow_cluster = true) {
    int threads, v;
    class_shape(n, &threads, &v);
    if (force_matrix) return find_variant(k, threads, v, 0);
    {
        std::lock_guard<std::mutex> lock(g_tuning_mutex);
        for (const TuningRule& r : g_tuning) {
            if ((r.precision >= 0 && r.precision != precision) || (r.unit >= 0 && r.unit != (unit ? 1 : 0)) ||
                n > r.n_max || D > r.d_max || r.threads * r.slots * r.cluster < n || (r.dims > 0 && D > r.dims) ||
                (!allow_cluster && r.cluster > 1))
                continue;
            const hdb::ForwardVariant* f = find_variant(k, r.threads, r.slots, r.dims, r.cluster, r.per_sm);
            if (f) return f;
        }
    }
    // Defaults.  float32 windows above 1024 points with D <= 32 spread their
    // Prim over a cluster of 2 or 4 CTAs (1024 register-resident vertices per
    // CTA).  float64 SIMT is a small fraction of float32 on GB300, so float64
    // windows use the matrix variant: the distance block is computed once per
    // pair by a grid spread over every SM, and Prim only reads rows.
    if (allow_cluster && precision == HDB_F32 && n > 1024 && D <= 32) {
        const int cluster = n <= 2048 ? 2 : 4;
        for (int option : {8, 16, 32})
            if (D <= option) {
                const hdb::ForwardVariant* f = find_variant(k, 512, 2, option, cluster);
                if (f) return f;
                break;
            }
    }
    int dp = 0;
    if (precision == HDB_F32) {
        for (int option : {8, 16, 32})
            if (D <= option && v * option <= 64) { dp = option; break; }
    }
    const hdb::ForwardVariant* f = find_variant(k, threads, v, dp);
    return f ? f : find_variant(k, threads, v, 0);
}

// Dynamic shared memory available to one CTA of a forward variant next to its
// static use, when `per_sm` CTAs share an SM (each also reserves 1 KB).
int smem_budget(const hdb::ForwardVariant* fv, int optin, int per_sm_total, size_t* budget) {
    cudaFuncAttributes attr;
    cudaError_t e = cudaFuncGetAttributes(&attr, fv->func);
    if (e != cudaSuccess) return fail(HDB_E_CUDA, std::string("cudaFuncGetAttributes: ") + cudaGetErrorString(e));
    size_t limit = (size_t)optin;
    if (fv->per_sm > 1) limit = std::min(limit, (size_t)per_sm_total / (size_t)fv->per_sm);
    *budget = limit > attr.sharedSizeBytes + 1024 ? limit - attr.sharedSizeBytes - 1024 : 0;
    return HDB_OK;
}

const hdb::CoreVariant* choose_core(const hdb::PrecisionKernels& k, int precision, int ms, int D, bool matrix) {
    int K = 0;
    for (int c : {8, 16, 32, 64})
        if (ms <= c) { K = c; break; }
    if (!K) return nullptr;
    int dp = 0;
    if (!matrix) {
        const int limit = precision == HDB_F32 ? 64 : 32;
        for (int c : {8, 16, 32, 64})
            if (D <= c && c <= limit) { dp = c; break; }
        if (!dp) return nullptr;
    }
    for (int i = 0; i < k.n_core; ++i)
        if (k.core[i].k == K && k.core[i].dp == dp) return &k.core[i];
    return nullptr;
}

template <typename T>
size_t put(std::vector<unsigned char>& image, size_t& cursor, const std::vector<T>& values) {
    cursor = align_up(cursor, 256);
    const size_t at = cursor;
    const size_t bytes = values.size() * sizeof(T);
    if (image.size() < at + bytes) image.resize(at + bytes);
    if (bytes) std::memcpy(image.data() + at, values.data(), bytes);
    cursor = at + bytes;
    return at;
}

int build_plan(hdb_plan* p) {
    const hdb::PrecisionKernels& k = *p->k;
    const bool unit = p->ms <= 2;
    const bool force_matrix = (p->flags & HDB_FLAG_FORCE_MATRIX) != 0;
    int optin = 0, per_sm_smem = 0;
    HDB_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, p->device));
    HDB_CUDA(cudaDeviceGetAttribute(&per_sm_smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, p->device));
    HDB_CUDA(cudaDeviceGetAttribute(&p->sms, cudaDevAttrMultiProcessorCount, p->device));

    // ---- classes ------------------------------------------------------------
    std::vector<int> order(p->B);
    for (int w = 0; w < p->B; ++w) order[w] = w;
    auto size_of = [&](int w) { return (int)(p->offsets[w + 1] - p->offsets[w]); };
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return size_of(a) > size_of(b); });
    std::vector<const hdb::ForwardVariant*> chosen(p->B, nullptr);
    int ctas = 0;  // CTAs the batch occupies at once: one per window, CS per clustered window
    for (int w : order) {
        chosen[w] = choose_variant(k, p->precision, size_of(w), p->D, unit, force_matrix);
        if (!chosen[w]) return fail(HDB_E_INVALID, "no kernel variant for a window of " + std::to_string(size_of(w)) + " points");
        ctas += chosen[w]->cluster;
    }
    // A cluster shortens one window's Prim but holds CS SMs; once the batch
    // needs more than one wave, the smallest clustered windows run on one CTA
    // each, until the batch fits the SMs again.
    for (auto it = order.rbegin(); it != order.rend() && ctas > p->sms; ++it) {
        const int w = *it;
        if (chosen[w]->cluster <= 1) continue;
        const hdb::ForwardVariant* single = choose_variant(k, p->precision, size_of(w), p->D, unit, force_matrix, false);
        if (!single) continue;
        ctas -= chosen[w]->cluster - 1;
        chosen[w] = single;
    }
    for (int w : order) {
        const int n = size_of(w);
        const hdb::ForwardVariant* fv = chosen[w];
        size_t budget = 0;
        int rc = smem_budget(fv, optin, per_sm_smem, &budget);
        if (rc) return rc;
        hdb::ForwardLayout layout{};
        if (!fv->layout(n, unit, budget, &layout))
            return fail(HDB_E_INVALID, "window of " + std::to_string(n) + " points exceeds shared memory");
        WindowClass* cls = nullptr;
        for (auto& c : p->classes)
            if (c.fv == fv && c.x_in_smem == layout.x_in_smem && c.n_arenas == layout.n_arenas) { cls = &c; break; }
        if (!cls) {
            p->classes.emplace_back();
            cls = &p->classes.back();
            cls->fv = fv;
            cls->x_in_smem = layout.x_in_smem;
            cls->n_arenas = layout.n_arenas;
        }
        cls->windows.push_back(w);
        cls->nmax = std::max(cls->nmax, n);
    }
    // Matrix-variant classes with many windows are cut into chunks of the
    // size-sorted queue: each chunk's Prim loops start once its own distance
    // blocks exist and overlap the distance work of the next chunk.
    {
        std::vector<WindowClass> chunked;
        for (auto& c : p->classes) {
            const size_t W = c.windows.size();
            const size_t parts = (c.fv->dp == 0 && W >= 2 * kMinChunk) ? std::min<size_t>(kChunks, W / kMinChunk) : 1;
            for (size_t part = 0; part < parts; ++part) {
                WindowClass piece = c;
                const size_t lo = W * part / parts, hi = W * (part + 1) / parts;
                piece.windows.assign(c.windows.begin() + lo, c.windows.begin() + hi);
                piece.nmax = 0;
                for (int w : piece.windows) piece.nmax = std::max(piece.nmax, size_of(w));
                chunked.push_back(std::move(piece));
            }
        }
        p->classes.swap(chunked);
    }
    std::stable_sort(p->classes.begin(), p->classes.end(),
                     [](const WindowClass& a, const WindowClass& b) { return a.nmax > b.nmax; });

    // ---- distance blocks and tiles for matrix-variant windows --------------
    p->dist_offsets.assign(p->B, -1);
    p->dist_elems = 0;
    for (auto& c : p->classes) {
        c.tiles_first = p->tiles.size() / 3;
        if (c.fv->dp != 0) continue;
        // Float32 classes of larger windows take the 128x128 tile kernel.
        c.tile = (p->precision == HDB_F32 && c.nmax >= kTile128MinN) ? 128 : 64;
        for (int w : c.windows) {
            const int n = size_of(w);
            const int64_t ld = (n + 3) & ~3;
            p->dist_offsets[w] = p->dist_elems;
            p->dist_elems += align_up((size_t)(n * ld), 64);
            const int t = (n + c.tile - 1) / c.tile;
            for (int ti = 0; ti < t; ++ti)
                for (int tj = ti; tj < t; ++tj) {
                    p->tiles.push_back(w);
                    p->tiles.push_back(ti);
                    p->tiles.push_back(tj);
                }
        }
        c.n_tiles = p->tiles.size() / 3 - c.tiles_first;
    }

    // ---- core distances -----------------------------------------------------
    if (!unit) {
        for (auto& c : p->classes) {
            const bool matrix = c.fv->dp == 0;
            CoreLaunch launch;
            launch.matrix = matrix;
            launch.cv = choose_core(k, p->precision, p->ms, p->D, matrix);
            CoreLaunch select;
            select.matrix = matrix;
            for (int w : c.windows) {
                const int n = size_of(w);
                if (launch.cv) {
                    for (int r = 0; r < n; r += launch.cv->rows) { launch.items.push_back(w); launch.items.push_back(r); }
                } else {
                    for (int r = 0; r < n; ++r) { select.items.push_back(w); select.items.push_back(r); }
                }
            }
            if (!launch.items.empty()) c.cores.push_back(launch);
            if (!select.items.empty()) {
                select.select_smem = (size_t)c.nmax * (size_t)real_bytes(p->precision);
                c.cores.push_back(select);
            }
        }
    }

    // ---- grids --------------------------------------------------------------
    for (auto& c : p->classes) {
        size_t budget = 0;
        int rc = smem_budget(c.fv, optin, per_sm_smem, &budget);
        if (rc) return rc;
        if (!c.fv->layout(c.nmax, unit, budget, &c.layout) || c.layout.n_arenas != c.n_arenas ||
            c.layout.x_in_smem != c.x_in_smem)
            return fail(HDB_E_INVALID, "inconsistent shared-memory layout for a window class");
        c.smem = c.layout.bytes;
        HDB_CUDA(raise_smem_limit(c.fv->func, c.smem));
        if (c.fv->cluster > 1) {
            // Persistent clusters: as many as can be co-resident, at most one per window.
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3((unsigned)(c.fv->cluster * std::max<size_t>(c.windows.size(), 1)));
            cfg.blockDim = dim3((unsigned)(c.fv->threads + 32));
            cfg.dynamicSmemBytes = c.smem;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeClusterDimension;
            attr[0].val.clusterDim.x = (unsigned)c.fv->cluster;
            attr[0].val.clusterDim.y = 1;
            attr[0].val.clusterDim.z = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            int clusters = 0;
            HDB_CUDA(cudaOccupancyMaxActiveClusters(&clusters, c.fv->func, &cfg));
            if (clusters < 1) return fail(HDB_E_INVALID, "cluster forward kernel variant cannot be resident");
            if (p->flags & HDB_FLAG_ONE_PERSISTENT) clusters = 1;
            c.grid = c.fv->cluster * (int)std::min<size_t>(c.windows.size(), (size_t)clusters);
        } else {
            int per_sm = 0;
            HDB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, c.fv->func, c.fv->threads + 32, c.smem));
            if (per_sm < 1) return fail(HDB_E_INVALID, "forward kernel variant cannot be resident");
            c.grid = (p->flags & HDB_FLAG_ONE_PERSISTENT) ? 1
                                                          : (int)std::min<size_t>(c.windows.size(), (size_t)per_sm * p->sms);
        }
    }
    for (auto& cls : p->classes)
        for (auto& c : cls.cores)
            if (!c.cv && c.select_smem > 48 * 1024) HDB_CUDA(raise_smem_limit(k.select_func, c.select_smem));

    // ---- table image --------------------------------------------------------
    std::vector<unsigned char> image;
    size_t cursor = 0;
    p->t_offsets = put(image, cursor, p->offsets);
    p->t_dist_off = put(image, cursor, p->dist_offsets);
    std::vector<int32_t> queue;
    std::vector<int32_t> tickets(p->classes.size(), 0);
    for (size_t i = 0; i < p->classes.size(); ++i) {
        auto& c = p->classes[i];
        c.queue_off = queue.size();
        c.ticket = (int)i;
        queue.insert(queue.end(), c.windows.begin(), c.windows.end());
    }
    p->t_queue = put(image, cursor, queue);
    p->t_tickets = put(image, cursor, tickets);
    p->t_tiles = put(image, cursor, p->tiles);
    for (auto& cls : p->classes)
        for (auto& c : cls.cores) c.items_off = put(image, cursor, c.items);
    std::vector<int32_t> edge_window;
    edge_window.reserve((size_t)(p->T - p->B));
    for (int w = 0; w < p->B; ++w)
        for (int i = 0; i < size_of(w) - 1; ++i) edge_window.push_back(w);
    p->t_edge_window = put(image, cursor, edge_window);
    p->tables_bytes = align_up(std::max<size_t>(cursor, 256), 256);
    image.resize(p->tables_bytes, 0);
    HDB_CUDA(cudaMallocHost((void**)&p->h_tables, p->tables_bytes));
    std::memcpy(p->h_tables, image.data(), p->tables_bytes);

    // ---- workspace layout ---------------------------------------------------
    size_t ws = p->tables_bytes;
    const size_t rb = (size_t)real_bytes(p->precision);
    p->w_core = ws = align_up(ws, 256);
    if (!unit) ws += (size_t)p->T * rb;
    p->w_core_nbr = ws = align_up(ws, 256);
    if (!unit) ws += (size_t)p->T * sizeof(int32_t);
    p->w_dist = ws = align_up(ws, 256);
    ws += (size_t)p->dist_elems * rb;
    p->w_prep = ws = align_up(ws, 256);
    if (p->prepared) ws += (size_t)p->T * (size_t)p->D * rb;
    p->ws_bytes = align_up(std::max<size_t>(ws, 256), 256);

    HDB_CUDA(cudaEventCreateWithFlags(&p->uploaded, cudaEventDisableTiming));

    // ---- streams for concurrent classes ------------------------------------
    const bool fork = !(p->flags & HDB_FLAG_NO_GRAPH_STREAMS) && p->classes.size() > 1;
    if (fork) {
        int least = 0, greatest = 0;  // numerically: greatest <= least
        HDB_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        for (size_t i = 0; i < p->classes.size(); ++i) {
            cudaStream_t s;
            const int priority = std::min(least, greatest + (int)i);
            p->classes[i].priority = priority;
            HDB_CUDA(cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, priority));
            p->aux.push_back(s);
        }
        for (size_t i = 0; i < 2 * p->classes.size(); ++i) {
            cudaEvent_t e;
            HDB_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            p->events.push_back(e);
        }
    }
    return HDB_OK;
}

int check_device(const hdb_plan* p) {
    int device = -1;
    HDB_CUDA(cudaGetDevice(&device));
    if (device != p->device)
        return fail(HDB_E_DEVICE, "plan was created on device " + std::to_string(p->device) + " but device " +
                                      std::to_string(device) + " is current");
    return HDB_OK;
}

int check_workspace(const hdb_plan* p, void* ws, size_t bytes) {
    if (!ws) return fail(HDB_E_WORKSPACE, "workspace is NULL");
    if (bytes < p->ws_bytes)
        return fail(HDB_E_WORKSPACE, "workspace of " + std::to_string(bytes) + " bytes is smaller than the " +
                                         std::to_string(p->ws_bytes) + " bytes the plan needs");
    if (reinterpret_cast<uintptr_t>(ws) % 256)
        return fail(HDB_E_WORKSPACE, "workspace must be 256-byte aligned");
    return HDB_OK;
}

// Records p->uploaded after an upload from the pinned table image, so that
// destroying the plan can wait for copies still reading it.  Skipped while the
// stream is being captured (the graph's copy runs at replay time, and the
// graph belongs to the plan).
cudaError_t note_upload(hdb_plan* p, cudaStream_t stream) {
    cudaStreamCaptureStatus capturing = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing(stream, &capturing);
    if (e != cudaSuccess || capturing != cudaStreamCaptureStatusNone) return e;
    return cudaEventRecord(p->uploaded, stream);
}

// Optional per-launch timing of run_forward (hdb_plan_profile): each kernel
// launch is bracketed by two events on the caller's stream and tagged with its
// phase (HDB_PHASE_*).
struct Spans {
    std::vector<int> phase;
    std::vector<cudaEvent_t> events;  // start, stop per launch
    cudaError_t begin(int ph, cudaStream_t s) {
        cudaEvent_t e[2];
        for (auto& x : e) {
            cudaError_t r = cudaEventCreate(&x);
            if (r != cudaSuccess) return r;
            events.push_back(x);
        }
        phase.push_back(ph);
        return cudaEventRecord(e[0], s);
    }
    cudaError_t end(cudaStream_t s) { return cudaEventRecord(events.back(), s); }
    ~Spans() {
        for (auto e : events) cudaEventDestroy(e);
    }
};

int run_forward(hdb_plan* p, const void* X, int32_t* labels, void* ws_v, int32_t* status,
                const hdb_exports_t* ex, cudaStream_t stream, Spans* spans = nullptr) {
    const hdb::PrecisionKernels& k = *p->k;
    unsigned char* ws = static_cast<unsigned char*>(ws_v);
    const bool unit = p->ms <= 2;
    hdb_exports_t none;
    std::memset(&none, 0, sizeof(none));
    if (!ex) ex = &none;
    HDB_CUDA(cudaMemcpyAsync(ws, p->h_tables, p->tables_bytes, cudaMemcpyHostToDevice, stream));
    HDB_CUDA(note_upload(p, stream));
    if (status) HDB_CUDA(cudaMemsetAsync(status, 0, sizeof(int32_t), stream));
    if (p->prepared) {  // producer stage: every later kernel reads the converted / normalised copy
        if (spans) HDB_CUDA(spans->begin(HDB_PHASE_PREPARE, stream));
        HDB_CUDA(k.launch_prepare(X, p->input_type, ws + p->w_prep, p->T, p->D, p->normalize, stream,
                                  p->classes.empty() ? 0 : p->classes[0].priority));
        if (spans) HDB_CUDA(spans->end(stream));
        X = ws + p->w_prep;
    }
    const int64_t* d_offsets = reinterpret_cast<const int64_t*>(ws + p->t_offsets);
    const int64_t* d_dist_off = reinterpret_cast<const int64_t*>(ws + p->t_dist_off);
    void* dist = ws + p->w_dist;
    void* core = ex->core ? ex->core : (void*)(ws + p->w_core);
    int32_t* core_nbr = ex->core_nbr ? ex->core_nbr : reinterpret_cast<int32_t*>(ws + p->w_core_nbr);

    if (ex->link_lr && (!ex->link_w || !ex->link_size)) return fail(HDB_E_INVALID, "link_lr needs link_w and link_size");
    if (ex->edges_uv && !ex->edge_w) return fail(HDB_E_INVALID, "edges_uv needs edge_w");
    if (ex->cl_parent && (!ex->cl_birth || !ex->cl_stability || !ex->cl_selected || !ex->point_parent || !ex->n_clusters))
        return fail(HDB_E_INVALID, "cl_parent needs cl_birth, cl_stability, cl_selected, point_parent, n_clusters");

    const bool fork = !p->aux.empty() && !spans;
    for (size_t i = 0; i < p->classes.size(); ++i) {
        const WindowClass& c = p->classes[i];
        // 1. distance blocks of this class's matrix-variant windows (caller's stream)
        if (c.n_tiles) {
            hdb::DistanceArgs a{};
            a.X = X;
            a.offsets = d_offsets;
            a.tiles = reinterpret_cast<const int32_t*>(ws + p->t_tiles) + 3 * c.tiles_first;
            a.n_tiles = (int)c.n_tiles;
            a.tile = c.tile;
            a.D = p->D;
            a.dist = dist;
            a.dist_offsets = d_dist_off;
            a.status = status;
            if (spans) HDB_CUDA(spans->begin(HDB_PHASE_DISTANCE, stream));
            HDB_CUDA(k.launch_distance(a, a.n_tiles, stream, c.priority));
            if (spans) HDB_CUDA(spans->end(stream));
        }
        // 2. core distances of its windows (caller's stream)
        for (const auto& cl : c.cores) {
            hdb::CoreArgs a{};
            a.X = X;
            a.offsets = d_offsets;
            a.items = reinterpret_cast<const int32_t*>(ws + cl.items_off);
            a.n_items = (int)(cl.items.size() / 2);
            a.D = p->D;
            a.ms = p->ms;
            a.dist = cl.matrix ? dist : nullptr;
            a.dist_offsets = d_dist_off;
            a.core = core;
            a.core_nbr = core_nbr;
            a.status = status;
            if (spans) HDB_CUDA(spans->begin(HDB_PHASE_CORE, stream));
            if (cl.cv) HDB_CUDA(cl.cv->launch(a, a.n_items, stream, c.priority));
            else HDB_CUDA(k.launch_select(a, a.n_items, cl.select_smem, stream, c.priority));
            if (spans) HDB_CUDA(spans->end(stream));
        }
        cudaStream_t s = stream;
        if (fork) {
            s = p->aux[i];
            HDB_CUDA(cudaEventRecord(p->events[2 * i], stream));
            HDB_CUDA(cudaStreamWaitEvent(s, p->events[2 * i], 0));
        }
        // 3. the persistent forward over its queue
        hdb::ForwardArgs a{};
        a.X = X;
        a.offsets = d_offsets;
        a.queue = reinterpret_cast<const int32_t*>(ws + p->t_queue) + c.queue_off;
        a.queue_len = (int)c.windows.size();
        a.ticket = reinterpret_cast<int32_t*>(ws + p->t_tickets) + c.ticket;
        a.D = p->D;
        a.mcs = p->mcs;
        a.unit_core = unit ? 1 : 0;
        a.x_in_smem = c.x_in_smem;
        a.n_arenas = c.layout.n_arenas;
        a.arena_stride = (int)c.layout.arena_stride;
        a.x_off = (int)c.layout.x_off;
        a.core_off = (int)c.layout.core_off;
        a.eps = p->eps;
        a.core = unit ? nullptr : core;
        a.dist = dist;
        a.dist_offsets = d_dist_off;
        a.labels = labels;
        a.status = status;
        a.edges_uv = ex->edges_uv;
        a.edge_w = ex->edge_w;
        a.order = ex->order;
        a.link_lr = ex->link_lr;
        a.link_w = ex->link_w;
        a.link_size = ex->link_size;
        a.n_clusters = ex->n_clusters;
        a.cl_parent = ex->cl_parent;
        a.cl_birth = ex->cl_birth;
        a.cl_stability = ex->cl_stability;
        a.cl_selected = ex->cl_selected;
        a.point_parent = ex->point_parent;
        a.stage_ns = ex->stage_ns;
        a.probabilities = ex->probabilities;
        a.cl_size = ex->cl_size;
        a.point_lambda = ex->point_lambda;
        if (p->flags & HDB_FLAG_TEST_STALL) {
            a.stall_first_ticket = 1;
            a.wait_limit_ns = 1000000;  // 1 ms
        }
        a.method = (p->flags & HDB_FLAG_LEAF) ? 1 : 0;
        a.allow_single = (p->flags & HDB_FLAG_ALLOW_SINGLE) ? 1 : 0;
        if (spans) HDB_CUDA(spans->begin(HDB_PHASE_FORWARD, s));
        HDB_CUDA(c.fv->launch(a, c.grid, c.smem, s, c.priority));
        if (spans) HDB_CUDA(spans->end(s));
        if (fork) HDB_CUDA(cudaEventRecord(p->events[2 * i + 1], s));
    }
    if (fork)
        for (size_t i = 0; i < p->classes.size(); ++i) HDB_CUDA(cudaStreamWaitEvent(stream, p->events[2 * i + 1], 0));
    return HDB_OK;
}

// ---- plan cache of the dense seam -----------------------------------------
// Plans are shared: a call holds its own reference while it enqueues, so
// evicting the least recently used entry only drops the cache's reference and
// never frees a plan another thread is still using.
struct CacheKey {
    int precision, batch, n, dims, mcs, ms, device;
    uint64_t eps_bits;
    bool operator==(const CacheKey& o) const {
        return precision == o.precision && batch == o.batch && n == o.n && dims == o.dims && mcs == o.mcs &&
               ms == o.ms && device == o.device && eps_bits == o.eps_bits;
    }
};
using PlanRef = std::shared_ptr<hdb_plan>;
constexpr size_t kCachedPlans = 16;
std::mutex g_cache_mutex;
std::list<std::pair<CacheKey, PlanRef>> g_cache;

int cached_plan(int precision, int batch, int n, int dims, int mcs, int ms, double eps, PlanRef* out) {
    int device = 0;
    HDB_CUDA(cudaGetDevice(&device));
    CacheKey key{precision, batch, n, dims, mcs, ms, device, 0};
    std::memcpy(&key.eps_bits, &eps, sizeof(eps));
    {
        std::lock_guard<std::mutex> lock(g_cache_mutex);
        for (auto it = g_cache.begin(); it != g_cache.end(); ++it) {
            if (it->first == key) {
                g_cache.splice(g_cache.begin(), g_cache, it);
                *out = it->second;
                return HDB_OK;
            }
        }
    }
    if ((int64_t)batch * n > INT32_MAX) return fail(HDB_E_INVALID, "batch * n exceeds int32");
    std::vector<int64_t> offsets((size_t)batch + 1);
    for (int b = 0; b <= batch; ++b) offsets[b] = (int64_t)b * n;
    hdb_plan* raw = nullptr;
    int rc = hdb_plan_create(&raw, precision, batch, offsets.data(), dims, mcs, ms, eps, 0);
    if (rc) return rc;
    PlanRef plan(raw, hdb_plan_destroy);
    PlanRef evicted;  // released after the cache lock
    {
        std::lock_guard<std::mutex> lock(g_cache_mutex);
        for (auto it = g_cache.begin(); it != g_cache.end(); ++it) {
            if (it->first == key) {  // another thread built the same plan meanwhile
                g_cache.splice(g_cache.begin(), g_cache, it);
                *out = it->second;
                return HDB_OK;  // `plan` is destroyed on return
            }
        }
        g_cache.emplace_front(key, plan);
        if (g_cache.size() > kCachedPlans) {
            evicted = std::move(g_cache.back().second);
            g_cache.pop_back();
        }
    }
    *out = std::move(plan);
    return HDB_OK;
}

int cluster_dense(int precision, const void* X, int batch, int n, int dims, int mcs, int ms, double eps,
                  int32_t* labels, void* ws, size_t ws_bytes, int32_t* status, void* stream) {
    PlanRef p;
    int rc = cached_plan(precision, batch, n, dims, mcs, ms, eps, &p);
    if (rc) return rc;
    return hdb_plan_forward(p.get(), X, labels, ws, ws_bytes, status, nullptr, stream);
}

}  // namespace

extern "C" {

int hdb_version(void) { return HDB_VERSION; }

int hdb_set_tuning(const int32_t* rules, int n_rules) {
    if (n_rules < 0 || (n_rules > 0 && !rules)) return fail(HDB_E_INVALID, "tuning rules must be a [n, 9] int32 array");
    std::vector<TuningRule> table;
    for (int i = 0; i < n_rules; ++i) {
        const int32_t* r = rules + kRuleFields * i;
        TuningRule t{r[0], r[1], r[2], r[3], r[4], r[5], r[6], r[7], r[8]};
        if (t.precision < -1 || t.precision > 1 || t.unit < -1 || t.unit > 1 || t.n_max < 2 || t.d_max < 1 ||
            t.threads < 32 || t.threads % 32 || t.threads > 992 || t.slots < 1 || t.dims < 0 || t.cluster < 1 ||
            t.cluster > 8 || t.per_sm < 1 || t.per_sm > 4)
            return fail(HDB_E_INVALID, "tuning rule " + std::to_string(i) + " is out of range");
        table.push_back(t);
    }
    std::lock_guard<std::mutex> lock(g_tuning_mutex);
    g_tuning = std::move(table);
    return HDB_OK;
}

int hdb_list_variants(int precision, int32_t* out, int capacity) {
    if (precision != HDB_F32 && precision != HDB_F64) return fail(HDB_E_INVALID, "precision must be 'float32' or 'float64'");
    const hdb::PrecisionKernels& k = precision == HDB_F32 ? hdb::kernels_f32() : hdb::kernels_f64();
    const int total = k.n_forward + k.n_cluster;
    for (int i = 0; i < total && i < capacity && out; ++i) {
        const hdb::ForwardVariant& f = i < k.n_forward ? k.forward[i] : k.cluster[i - k.n_forward];
        out[5 * i] = f.threads;
        out[5 * i + 1] = f.v;
        out[5 * i + 2] = f.dp;
        out[5 * i + 3] = f.cluster;
        out[5 * i + 4] = f.per_sm;
    }
    return total;
}

int hdb_get_tuning(int32_t* rules, int capacity) {
    std::lock_guard<std::mutex> lock(g_tuning_mutex);
    const int count = (int)g_tuning.size();
    for (int i = 0; i < count && i < capacity && rules; ++i) {
        const TuningRule& t = g_tuning[i];
        const int32_t v[kRuleFields] = {t.precision, t.unit, t.n_max, t.d_max, t.threads, t.slots,
                                        t.dims,      t.cluster, t.per_sm};
        for (int j = 0; j < kRuleFields; ++j) rules[kRuleFields * i + j] = v[j];
    }
    return count;
}

const char* hdb_last_error(void) { return g_error.c_str(); }

int hdb_plan_create(hdb_plan_t** out, int precision, int windows, const int64_t* offsets_host, int dims,
                    int min_cluster_size, int min_samples, double epsilon, unsigned flags) {
    if (!out) return fail(HDB_E_INVALID, "plan output pointer is NULL");
    *out = nullptr;
    if (precision != HDB_F32 && precision != HDB_F64)
        return fail(HDB_E_INVALID, "precision must be 'float32' or 'float64'");
    if (windows < 1 || dims < 1 || !offsets_host)
        return fail(HDB_E_INVALID, "X requires nonempty batches/features and at least 2 samples");
    if (min_cluster_size < 2) return fail(HDB_E_INVALID, "min_cluster_size must be >= 2");
    if (min_samples < 1) return fail(HDB_E_INVALID, "min_samples must be >= 1");
    if (!(epsilon >= 0) || epsilon > 1.7976931348623157e308)
        return fail(HDB_E_INVALID, "cluster_selection_epsilon must be finite and >= 0");
    if (precision == HDB_F32 && epsilon > 3.4028234663852886e38)
        return fail(HDB_E_INVALID, "cluster_selection_epsilon is not representable in the requested precision");
    if (offsets_host[0] != 0) return fail(HDB_E_INVALID, "offsets must start at 0");
    for (int w = 0; w < windows; ++w) {
        const int64_t n = offsets_host[w + 1] - offsets_host[w];
        if (n < 2) return fail(HDB_E_INVALID, "X requires nonempty batches/features and at least 2 samples");
        if (n > HDB_MAX_SAMPLES)
            return fail(HDB_E_INVALID, "at most " + std::to_string(HDB_MAX_SAMPLES) + " samples per window are supported");
        if (min_samples > n) return fail(HDB_E_INVALID, "min_samples must not exceed the number of samples");
    }
    if (offsets_host[windows] > INT32_MAX) return fail(HDB_E_INVALID, "more than 2^31-1 points in one batch");
    hdb_plan* p = new hdb_plan();
    p->precision = precision;
    p->B = windows;
    p->D = dims;
    p->mcs = min_cluster_size;
    p->ms = min_samples;
    p->eps = epsilon;
    p->flags = flags;
    p->offsets.assign(offsets_host, offsets_host + windows + 1);
    if ((flags & HDB_FLAG_INPUT_BF16) && (flags & HDB_FLAG_INPUT_F16)) {
        delete p;
        return fail(HDB_E_INVALID, "X can be bfloat16 or float16, not both");
    }
    p->input_type = (flags & HDB_FLAG_INPUT_BF16) ? 1 : ((flags & HDB_FLAG_INPUT_F16) ? 2 : 0);
    p->normalize = (flags & HDB_FLAG_L2_NORMALIZE) ? 1 : 0;
    p->prepared = p->input_type != 0 || p->normalize != 0;
    p->T = offsets_host[windows];
    p->k = precision == HDB_F32 ? &hdb::kernels_f32() : &hdb::kernels_f64();
    cudaError_t e = cudaGetDevice(&p->device);
    if (e != cudaSuccess) {
        delete p;
        return fail(HDB_E_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    }
    int rc = build_plan(p);
    if (rc) {
        hdb_plan_destroy(p);
        return rc;
    }
    *out = p;
    return HDB_OK;
}

int hdb_plan_destroy(hdb_plan_t* p) {
    if (!p) return HDB_OK;
    // A copy from the pinned table image may still be queued on some stream.
    if (p->uploaded) {
        cudaEventSynchronize(p->uploaded);
        cudaEventDestroy(p->uploaded);
    }
    if (p->graph) cudaGraphExecDestroy(p->graph);
    for (auto s : p->aux) cudaStreamDestroy(s);
    for (auto e : p->events) cudaEventDestroy(e);
    if (p->h_tables) cudaFreeHost(p->h_tables);
    delete p;
    return HDB_OK;
}

size_t hdb_plan_workspace_bytes(const hdb_plan_t* p) { return p ? p->ws_bytes : 0; }

// Sum over a class's windows of n (power 1) or n^2 (power 2).
static int64_t class_points(const hdb_plan* p, const WindowClass& c, int power) {
    int64_t total = 0;
    for (int w : c.windows) {
        const int64_t n = p->offsets[w + 1] - p->offsets[w];
        total += power == 2 ? n * n : n;
    }
    return total;
}

int hdb_plan_describe(const hdb_plan_t* p, char* buffer, size_t size) {
    if (!p || !buffer || !size) return fail(HDB_E_INVALID, "describe needs a plan and a buffer");
    std::string s = "{\"precision\":\"" + std::string(p->precision == HDB_F32 ? "float32" : "float64") +
                    "\",\"windows\":" + std::to_string(p->B) + ",\"points\":" + std::to_string(p->T) +
                    ",\"dims\":" + std::to_string(p->D) + ",\"workspace_bytes\":" + std::to_string(p->ws_bytes) +
                    ",\"distance_tiles\":" + std::to_string(p->tiles.size() / 3) + ",\"classes\":[";
    for (size_t i = 0; i < p->classes.size(); ++i) {
        const auto& c = p->classes[i];
        s += (i ? "," : "") + std::string("{\"threads\":") + std::to_string(c.fv->threads) +
             ",\"vertices_per_thread\":" + std::to_string(c.fv->v) + ",\"register_dims\":" +
             std::to_string(c.fv->dp) + ",\"cluster\":" + std::to_string(c.fv->cluster) +
             ",\"per_sm\":" + std::to_string(c.fv->per_sm) +
             ",\"variant\":\"" + (c.fv->dp ? "recompute" : "matrix") +
             "\",\"x_in_smem\":" + std::to_string(c.x_in_smem) + ",\"arenas\":" + std::to_string(c.n_arenas) +
             ",\"distance_tiles\":" + std::to_string(c.n_tiles) + ",\"tile\":" + std::to_string(c.tile) +
             ",\"priority\":" + std::to_string(c.priority) +
             ",\"windows\":" + std::to_string(c.windows.size()) + ",\"points\":" +
             std::to_string(class_points(p, c, 1)) + ",\"sum_n2\":" + std::to_string(class_points(p, c, 2)) +
             ",\"nmax\":" + std::to_string(c.nmax) + ",\"smem\":" +
             std::to_string(c.smem) + ",\"grid\":" + std::to_string(c.grid) + "}";
    }
    s += "],\"core\":[";
    bool first = true;
    for (const auto& cls : p->classes)
        for (const auto& c : cls.cores) {
            s += (first ? "" : ",") + std::string("{\"kernel\":\"") +
                 (c.cv ? (c.matrix ? "core_matrix" : "core_points") : "core_select") + "\",\"k\":" +
                 std::to_string(c.cv ? c.cv->k : 0) + ",\"register_dims\":" + std::to_string(c.cv ? c.cv->dp : 0) +
                 ",\"items\":" + std::to_string(c.items.size() / 2) + "}";
            first = false;
        }
    s += "]}";
    if (s.size() + 1 > size) return fail(HDB_E_INVALID, "describe buffer too small");
    std::memcpy(buffer, s.c_str(), s.size() + 1);
    return HDB_OK;
}

int hdb_plan_forward(hdb_plan_t* p, const void* X, int32_t* labels, void* ws, size_t ws_bytes, int32_t* status,
                     const hdb_exports_t* exports, void* stream) {
    if (!p || !X || !labels) return fail(HDB_E_INVALID, "plan, X and labels are required");
    int rc = check_device(p);
    if (rc) return rc;
    rc = check_workspace(p, ws, ws_bytes);
    if (rc) return rc;
    std::lock_guard<std::mutex> lock(p->enqueue);
    return run_forward(p, X, labels, ws, status, exports, static_cast<cudaStream_t>(stream));
}

int hdb_plan_profile(hdb_plan_t* p, const void* X, int32_t* labels, void* ws, size_t ws_bytes, int32_t* status,
                     const hdb_exports_t* exports, void* stream_v, double* phase_ms, int32_t* phase_launches) {
    if (!p || !X || !labels || !phase_ms) return fail(HDB_E_INVALID, "plan, X, labels and phase_ms are required");
    int rc = check_device(p);
    if (rc) return rc;
    rc = check_workspace(p, ws, ws_bytes);
    if (rc) return rc;
    cudaStream_t stream = static_cast<cudaStream_t>(stream_v);
    Spans spans;
    {
        std::lock_guard<std::mutex> lock(p->enqueue);
        rc = run_forward(p, X, labels, ws, status, exports, stream, &spans);
    }
    if (rc) return rc;
    HDB_CUDA(cudaStreamSynchronize(stream));
    for (int i = 0; i < HDB_PHASES; ++i) {
        phase_ms[i] = 0;
        if (phase_launches) phase_launches[i] = 0;
    }
    for (size_t i = 0; i < spans.phase.size(); ++i) {
        float ms = 0;
        HDB_CUDA(cudaEventElapsedTime(&ms, spans.events[2 * i], spans.events[2 * i + 1]));
        phase_ms[spans.phase[i]] += ms;
        if (phase_launches) ++phase_launches[spans.phase[i]];
    }
    return HDB_OK;
}

int hdb_plan_capture(hdb_plan_t* p, const void* X, int32_t* labels, void* ws, size_t ws_bytes, int32_t* status,
                     const hdb_exports_t* exports, void* stream_v) {
    if (!p || !X || !labels) return fail(HDB_E_INVALID, "plan, X and labels are required");
    int rc = check_device(p);
    if (rc) return rc;
    rc = check_workspace(p, ws, ws_bytes);
    if (rc) return rc;
    cudaStream_t stream = static_cast<cudaStream_t>(stream_v);
    cudaStream_t capture = stream;
    bool own = false;
    // The class streams join the capture until it ends: no other call may
    // enqueue on them meanwhile.
    std::lock_guard<std::mutex> lock(p->enqueue);
    if (!capture) {  // the legacy stream cannot be captured
        HDB_CUDA(cudaStreamCreateWithFlags(&capture, cudaStreamNonBlocking));
        own = true;
    }
    HDB_CUDA(cudaStreamBeginCapture(capture, cudaStreamCaptureModeThreadLocal));
    rc = run_forward(p, X, labels, ws, status, exports, capture);
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(capture, &graph);
    if (own) cudaStreamDestroy(capture);
    if (rc) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    if (e != cudaSuccess) return fail(HDB_E_CUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e));
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return fail(HDB_E_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
    if (p->graph) cudaGraphExecDestroy(p->graph);
    p->graph = exec;
    return HDB_OK;
}

int hdb_plan_replay(hdb_plan_t* p, void* stream) {
    if (!p || !p->graph) return fail(HDB_E_INVALID, "plan has no captured graph");
    int rc = check_device(p);
    if (rc) return rc;
    std::lock_guard<std::mutex> lock(p->enqueue);
    HDB_CUDA(cudaGraphLaunch(p->graph, static_cast<cudaStream_t>(stream)));
    return HDB_OK;
}

int hdb_plan_backward(hdb_plan_t* p, const void* X, const hdb_exports_t* ex, const void* grad, void* dX, void* ws_v,
                      size_t ws_bytes, void* stream) {
    if (!p || !X || !ex || !grad || !dX) return fail(HDB_E_INVALID, "plan, X, exports, grad and dX are required");
    if (!ex->edges_uv || !ex->order || !ex->link_w)
        return fail(HDB_E_INVALID, "backward needs the forward's edges_uv, order and link_w");
    const bool unit = p->ms <= 2;
    if (!unit && (!ex->core || !ex->core_nbr))
        return fail(HDB_E_INVALID, "backward with min_samples > 2 needs the forward's core and core_nbr");
    if (p->prepared)
        return fail(HDB_E_INVALID, "backward needs input in the compute precision without normalisation");
    int rc = check_device(p);
    if (rc) return rc;
    rc = check_workspace(p, ws_v, ws_bytes);
    if (rc) return rc;
    unsigned char* ws = static_cast<unsigned char*>(ws_v);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    std::lock_guard<std::mutex> lock(p->enqueue);
    HDB_CUDA(cudaMemcpyAsync(ws, p->h_tables, p->tables_bytes, cudaMemcpyHostToDevice, s));
    HDB_CUDA(note_upload(p, s));
    hdb::BackwardArgs a{};
    a.X = X;
    a.offsets = reinterpret_cast<const int64_t*>(ws + p->t_offsets);
    a.edge_window = reinterpret_cast<const int32_t*>(ws + p->t_edge_window);
    a.n_edges = (int)(p->T - p->B);
    a.D = p->D;
    a.unit_core = unit ? 1 : 0;
    a.edges_uv = ex->edges_uv;
    a.order = ex->order;
    a.link_w = ex->link_w;
    a.grad = grad;
    a.core = ex->core;
    a.core_nbr = ex->core_nbr;
    a.dX = dX;
    if (a.n_edges > 0)
        HDB_CUDA(p->k->launch_backward(a, (a.n_edges + 32 * hdb::kBackwardWarps - 1) / (32 * hdb::kBackwardWarps), s, 0));
    return HDB_OK;
}

size_t hdb_cluster_workspace_bytes(int precision, int batch, int n, int dims, int mcs, int ms) {
    PlanRef p;
    if (cached_plan(precision, batch, n, dims, mcs, ms, 0.0, &p)) return 0;
    return p->ws_bytes;
}

int hdb_cluster_f32(const float* X, int batch, int n, int dims, int mcs, int ms, double eps, int32_t* labels,
                    void* ws, size_t ws_bytes, int32_t* status, void* stream) {
    return cluster_dense(HDB_F32, X, batch, n, dims, mcs, ms, eps, labels, ws, ws_bytes, status, stream);
}

int hdb_cluster_f64(const double* X, int batch, int n, int dims, int mcs, int ms, double eps, int32_t* labels,
                    void* ws, size_t ws_bytes, int32_t* status, void* stream) {
    return cluster_dense(HDB_F64, X, batch, n, dims, mcs, ms, eps, labels, ws, ws_bytes, status, stream);
}

}  // extern "C"
