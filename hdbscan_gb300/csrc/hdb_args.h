// Plain-C++ argument blocks shared by the host plan layer and the kernels.
#pragma once
#include <cstdint>

namespace hdb {

enum Status : int32_t {
    kOk = 0,
    kOverflow = 1,     // a pairwise distance is not finite (reference: _cuda.py:112-113)
    kNonFinite = 2,    // an input coordinate is not finite (reference: _cuda.py:98-99)
    kInternal = 4,     // device-side bounds check tripped (a bug, never expected)
};

struct ForwardArgs {
    const void* X;             // packed [T, D] Real
    const int64_t* offsets;    // [B+1] device
    const int32_t* queue;      // windows of this launch, size-sorted
    int queue_len;
    int32_t* ticket;           // persistent work counter (zeroed before launch)
    int D;
    int mcs;
    int unit_core;             // ms <= 2
    int x_in_smem;             // stage the window's coordinates in shared memory
    int n_arenas;              // 1 or 2 hierarchy arenas (2 = Prim/tree overlap)
    int arena_stride;          // bytes per arena in dynamic shared memory
    int x_off;                 // byte offset of the staged coordinates
    int core_off;              // byte offset of the staged core distances
    double eps;
    const void* core;          // [T] Real, or null when unit_core
    const void* dist;          // matrix variant: packed per-window [n, n] Real blocks
    const int64_t* dist_offsets;  // [B] element offset of each window's block
    int32_t* labels;           // [T]
    int32_t* status;           // bit-or of Status codes
    // Optional exports (null = skip).  Edge arrays are packed per window at
    // offsets[w] - w (n-1 entries each); cluster arrays at offsets[w].
    int32_t* edges_uv;         // [T-B, 2] Prim order
    void* edge_w;              // [T-B]   Prim order
    int32_t* order;            // [T-B]   argsort of edge_w (window-local indices)
    int32_t* link_lr;          // [T-B, 2] children of node n+i
    void* link_w;              // [T-B]
    int32_t* link_size;        // [T-B]
    int32_t* n_clusters;       // [B]
    int32_t* cl_parent;        // [T]
    void* cl_birth;            // [T]
    void* cl_stability;        // [T]
    uint8_t* cl_selected;      // [T]
    int32_t* point_parent;     // [T]
    int64_t* stage_ns;         // [B, 8] globaltimer at stage boundaries (diagnostics)
    void* probabilities;       // [T] membership strengths (Real)
    int32_t* cl_size;          // [T] cluster sizes at birth
    void* point_lambda;        // [T] lambda at which each point falls out (Real)
    int method;                // cluster selection: 0 excess of mass, 1 leaf
    int allow_single;          // the root may be selected
    // Cluster form only: limit of every bounded mbarrier wait (0 = the 2 s
    // default), and a test switch under which the first window ticket is never
    // broadcast, so every CTA's first wait runs out (nothing is in flight then).
    int64_t wait_limit_ns;
    int stall_first_ticket;
};

struct DistanceArgs {
    const void* X;
    const int64_t* offsets;
    const int32_t* tiles;        // [n_tiles, 3] = (window, tile row, tile col), col >= row
    int n_tiles;
    int tile;                    // tile edge: 64, or 128 (float32 only)
    int D;
    void* dist;                  // packed blocks
    const int64_t* dist_offsets; // [B]
    int32_t* status;
};

struct CoreArgs {
    const void* X;
    const int64_t* offsets;
    const int32_t* items;        // [n_items, 2] = (window, first row)
    int n_items;
    int D;
    int ms;                      // order statistic k = ms-1 (0-based), self included
    const void* dist;            // matrix variant only
    const int64_t* dist_offsets;
    void* core;                  // [T]
    int32_t* core_nbr;           // [T] or null
    int32_t* status;
};

constexpr int kBackwardWarps = 8;  // backward kernel: warps (32 linkage rows each) per CTA

struct BackwardArgs {
    const void* X;               // [T, D]
    const int64_t* offsets;      // [B+1]
    const int32_t* edge_window;  // [T-B] window of each packed edge row
    int n_edges;                 // T - B
    int D;
    int unit_core;
    const int32_t* edges_uv;     // [T-B, 2] Prim order (window-local vertex ids)
    const int32_t* order;        // [T-B] Prim-edge index (window-local) of linkage row i
    const void* link_w;          // [T-B] merge weights in linkage order
    const void* grad;            // [T-B] dL/dmerge_weight in linkage order
    const void* core;            // [T] or null
    const int32_t* core_nbr;     // [T] or null
    void* dX;                    // [T, D] accumulated (caller zeroes)
};

}  // namespace hdb
