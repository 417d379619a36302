// Dense-batch forward that allocates nothing (hdb_cluster_noalloc).
//
// Who needs it: a caller that may not call cudaMalloc at the point where it
// clusters -- for example a serving process that hands all device memory to
// its own pool at start-up and treats any other allocation as a failure, or a
// plugin living inside a host framework whose allocator owns the device.  Such
// a caller can still pass its input and output buffers, but cannot provide the
// workspace the planned entry points ask for.
//
// How: the forward kernel's scratch (window offsets, work queue, queue ticket,
// core-distance work items, core distances) lives in one file-scope
// __device__ array of kScratchBytes, resident on every device that loads this
// library until the process exits.  Host code must not use the array's name as
// a device address (in host code it names a host-side stand-in), so the first
// call in each CUDA context resolves the real address with
// cudaGetSymbolAddress, with that context's device current, and caches it
// under the context's unique id (a context created later, for instance after
// cudaDeviceReset, gets its own lookup).  That first call should therefore
// come before any stream capture.  A small kernel rebuilds the tables in the
// scratch on every call (nothing is copied from host memory), so no pinned
// buffer is needed either.
//
// Limits: the Prim kernels this entry point can use keep every window's
// coordinates in registers (no distance-block workspace), so the dims a window
// may have shrink as its point count grows (noalloc_max_dims below).
//
// Every call shares the array and overwrites what the previous call left:
// calls that overlap on the GPU (other streams, other host threads) race with
// each other; keep them ordered on one stream.
#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include <cuda.h>  // CUcontext / CUresult types only; the driver calls are resolved at run time
#include <cuda_runtime.h>

#include "../../include/hdbscan_gb300.h"
#include "hdb_args.h"
#include "hdb_registry.h"

namespace {

constexpr size_t kScratchBytes = HDB_NOALLOC_SCRATCH_BYTES;

// Byte layout of the scratch array.
constexpr size_t kOffOffsets = 0;                                                     // int64 [windows+1]
constexpr size_t kOffQueue = (((size_t)(HDB_NOALLOC_MAX_WINDOWS + 1) * 8 + 255) / 256) * 256;  // int32 [windows]
constexpr size_t kOffTicket = kOffQueue + (((size_t)HDB_NOALLOC_MAX_WINDOWS * 4 + 255) / 256) * 256;
constexpr size_t kOffItems = kOffTicket + 256;                                        // int32 [2*points]
constexpr size_t kOffCore = kOffItems + (size_t)HDB_NOALLOC_MAX_POINTS * 8;          // Real [points]
constexpr size_t kScratchUsed = kOffCore + (size_t)HDB_NOALLOC_MAX_POINTS * 8;
static_assert(kScratchUsed <= kScratchBytes, "no-allocation scratch layout exceeds its array");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_scratch_mutex;
struct ScratchEntry {
    unsigned long long context;  // unique id of the CUDA context (cuCtxGetId), or the device ordinal
    unsigned char* address;
};
std::vector<ScratchEntry> g_scratch_device;

// Failures are reported through the library's hdb_last_error().
int fail(int code, const std::string& message) {
    hdb::set_last_error(message);
    return code;
}

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

// Unique id of the current context, through driver entry points looked up by
// the runtime (no link-time dependency on the driver library).  False when the
// driver offers no such query or no context is current yet.
bool current_context_id(unsigned long long* id) {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult found;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &found) == cudaSuccess &&
            found == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<CtxGetCurrentFn>(fn);
        fn = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &fn, 12000, cudaEnableDefault, &found) == cudaSuccess &&
            found == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<CtxGetIdFn>(fn);
    });
    if (!get_current || !get_id) return false;
    CUcontext ctx = nullptr;
    if (get_current(&ctx) != CUDA_SUCCESS || !ctx) return false;
    return get_id(ctx, id) == CUDA_SUCCESS;
}

// Device address of the scratch array in the current context (on `device`).
int scratch_address(int device, unsigned char** out) {
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    unsigned long long key = 0;
    const bool by_context = current_context_id(&key);
    if (by_context) key |= 1ull << 63;  // context ids and device ordinals never collide
    else key = (unsigned long long)device;
    for (const ScratchEntry& e : g_scratch_device)
        if (e.context == key) {
            *out = e.address;
            return HDB_OK;
        }
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess)
        return fail(HDB_E_CUDA, std::string("cudaGetSymbolAddress(no-allocation scratch): ") + cudaGetErrorString(e));
    // The lookup above may have created the context; key the entry on it.
    unsigned long long now = 0;
    if (current_context_id(&now)) key = now | (1ull << 63);
    g_scratch_device.push_back({key, static_cast<unsigned char*>(ptr)});
    *out = static_cast<unsigned char*>(ptr);
    return HDB_OK;
}

// Largest dims a window of n points may have in this precision (0: none): the
// register-resident Prim variants hold slots x register dims <= 64 words.
int noalloc_max_dims(int precision, int n) {
    if (precision == HDB_F32) return n <= 1024 ? 32 : (n <= 2048 ? 16 : 8);
    return n <= 1024 ? 16 : (n <= 2048 ? 8 : 0);
}

// Rebuilds the uniform-batch tables; also zeroes the ticket and the status.
__global__ void noalloc_tables_kernel(int64_t* offsets, int32_t* queue, int32_t* ticket, int32_t* items, int batch,
                                      int n, int rows_per_item, int n_items, int32_t* status) {
    const int stride = gridDim.x * blockDim.x;
    const int per_window = (n + rows_per_item - 1) / rows_per_item;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < batch + 1 || t < n_items; t += stride) {
        if (t <= batch) offsets[t] = (int64_t)t * n;
        if (t < batch) queue[t] = t;
        if (t < n_items) {
            const int w = t / per_window;
            items[2 * t] = w;
            items[2 * t + 1] = (t - w * per_window) * rows_per_item;
        }
        if (t == 0) {
            ticket[0] = 0;
            if (status) status[0] = 0;
        }
    }
}

const hdb::ForwardVariant* pick_forward(const hdb::PrecisionKernels& k, int precision, int n, int dims) {
    int threads, v;
    if (n <= 64) { threads = 32; v = 2; }
    else if (n <= 128) { threads = 64; v = 2; }
    else if (n <= 256) { threads = 128; v = 2; }
    else if (n <= 512) { threads = 256; v = 2; }
    else if (n <= 1024) { threads = 512; v = 2; }
    else if (n <= 2048) { threads = 512; v = 4; }
    else { threads = 512; v = 8; }
    const int words = precision == HDB_F32 ? 1 : 2;
    for (int dp : {8, 16, 32}) {
        if (dims > dp || v * dp * words > 64) continue;
        for (int i = 0; i < k.n_forward; ++i)
            if (k.forward[i].threads == threads && k.forward[i].v == v && k.forward[i].dp == dp &&
                k.forward[i].per_sm == 1)
                return &k.forward[i];
    }
    return nullptr;
}

const hdb::CoreVariant* pick_core(const hdb::PrecisionKernels& k, int precision, int ms, int dims) {
    for (int K : {8, 16, 32, 64}) {
        if (ms > K) continue;
        for (int dp : {8, 16, 32, 64}) {
            if (dims > dp || (precision == HDB_F64 && dp > 32)) continue;
            for (int i = 0; i < k.n_core; ++i)
                if (k.core[i].k == K && k.core[i].dp == dp) return &k.core[i];
        }
        return nullptr;
    }
    return nullptr;
}

}  // namespace

extern "C" int hdb_cluster_noalloc(int precision, const void* X, int batch, int n, int dims, int min_cluster_size,
                                   int min_samples, double epsilon, int32_t* labels, int32_t* status, void* stream_v) {
    if (precision != HDB_F32 && precision != HDB_F64)
        return fail(HDB_E_INVALID, "precision must be 'float32' or 'float64'");
    if (!X || !labels) return fail(HDB_E_INVALID, "X and labels are required");
    if (batch < 1 || dims < 1 || n < 2)
        return fail(HDB_E_INVALID, "X requires nonempty batches/features and at least 2 samples");
    if (n > HDB_MAX_SAMPLES) return fail(HDB_E_INVALID, "at most 4096 samples per window are supported");
    if (min_cluster_size < 2) return fail(HDB_E_INVALID, "min_cluster_size must be >= 2");
    if (min_samples < 1) return fail(HDB_E_INVALID, "min_samples must be >= 1");
    if (min_samples > n) return fail(HDB_E_INVALID, "min_samples must not exceed the number of samples");
    if (!(epsilon >= 0) || epsilon > 1.7976931348623157e308)
        return fail(HDB_E_INVALID, "cluster_selection_epsilon must be finite and >= 0");
    if (precision == HDB_F32 && epsilon > 3.4028234663852886e38)
        return fail(HDB_E_INVALID, "cluster_selection_epsilon is not representable in the requested precision");
    if (batch > HDB_NOALLOC_MAX_WINDOWS || (int64_t)batch * n > HDB_NOALLOC_MAX_POINTS)
        return fail(HDB_E_INVALID, "batch of " + std::to_string(batch) + " x " + std::to_string(n) +
                                       " points exceeds the no-allocation limit (at most " +
                                       std::to_string(HDB_NOALLOC_MAX_WINDOWS) + " windows and " +
                                       std::to_string(HDB_NOALLOC_MAX_POINTS) + " points)");
    const int max_dims = noalloc_max_dims(precision, n);
    if (dims > max_dims)
        return fail(HDB_E_INVALID,
                    std::string("dims of ") + std::to_string(dims) + " exceed the no-allocation limit for " +
                        (precision == HDB_F32 ? "float32" : "float64") + " windows of " + std::to_string(n) +
                        " points (" + (max_dims ? "at most " + std::to_string(max_dims) + " dims" : "not supported") +
                        "; larger windows or dims need the distance-block workspace of hdb_plan_*)");

    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) return fail(HDB_E_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    unsigned char* scratch = nullptr;
    int rc = scratch_address(device, &scratch);
    if (rc) return rc;

    const hdb::PrecisionKernels& k = precision == HDB_F32 ? hdb::kernels_f32() : hdb::kernels_f64();
    const bool unit = min_samples <= 2;
    const hdb::ForwardVariant* fv = pick_forward(k, precision, n, dims);
    if (!fv) return fail(HDB_E_INVALID, "no register variant for this window size and dims");
    const hdb::CoreVariant* cv = unit ? nullptr : pick_core(k, precision, min_samples, dims);

    int optin = 0, sms = 0;
    e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) return fail(HDB_E_CUDA, std::string("cudaDeviceGetAttribute: ") + cudaGetErrorString(e));
    cudaFuncAttributes attr;
    e = cudaFuncGetAttributes(&attr, fv->func);
    if (e != cudaSuccess) return fail(HDB_E_CUDA, std::string("cudaFuncGetAttributes: ") + cudaGetErrorString(e));
    const size_t budget = (size_t)optin > attr.sharedSizeBytes + 1024 ? (size_t)optin - attr.sharedSizeBytes - 1024 : 0;
    hdb::ForwardLayout layout{};
    if (!k.forward_layout(n, fv->dp, unit, budget, 2, &layout))
        return fail(HDB_E_INVALID, "window exceeds shared memory");
    const size_t smem = layout.bytes;
    e = hdb::raise_dynamic_smem(fv->func, smem);
    int per_sm = 0;
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fv->func, fv->threads + 32, smem);
    if (e != cudaSuccess) return fail(HDB_E_CUDA, std::string("forward kernel set-up: ") + cudaGetErrorString(e));
    if (per_sm < 1) return fail(HDB_E_INVALID, "forward kernel variant cannot be resident");
    const size_t select_smem = (size_t)n * (precision == HDB_F32 ? 4 : 8);
    if (!unit && !cv && select_smem > 48 * 1024) {
        e = hdb::raise_dynamic_smem(k.select_func, select_smem);
        if (e != cudaSuccess) return fail(HDB_E_CUDA, std::string("select kernel set-up: ") + cudaGetErrorString(e));
    }

    cudaStream_t stream = static_cast<cudaStream_t>(stream_v);
    int64_t* offsets = reinterpret_cast<int64_t*>(scratch + kOffOffsets);
    int32_t* queue = reinterpret_cast<int32_t*>(scratch + kOffQueue);
    int32_t* ticket = reinterpret_cast<int32_t*>(scratch + kOffTicket);
    int32_t* items = reinterpret_cast<int32_t*>(scratch + kOffItems);
    void* core = scratch + kOffCore;
    const int rows_per_item = unit ? 1 : (cv ? cv->rows : 1);
    const int n_items = unit ? 0 : batch * ((n + rows_per_item - 1) / rows_per_item);
    const int work = (batch + 1 > n_items ? batch + 1 : n_items);
    noalloc_tables_kernel<<<(work + 255) / 256, 256, 0, stream>>>(offsets, queue, ticket, items, batch, n,
                                                                   rows_per_item, n_items, status);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(HDB_E_CUDA, std::string("tables kernel: ") + cudaGetErrorString(e));

    if (!unit) {
        hdb::CoreArgs a{};
        a.X = X;
        a.offsets = offsets;
        a.items = items;
        a.n_items = n_items;
        a.D = dims;
        a.ms = min_samples;
        a.core = core;
        a.status = status;
        if (cv) e = cv->launch(a, n_items, stream, 0);
        else e = k.launch_select(a, n_items, select_smem, stream, 0);
        if (e != cudaSuccess) return fail(HDB_E_CUDA, std::string("core kernel: ") + cudaGetErrorString(e));
    }

    hdb::ForwardArgs a{};
    a.X = X;
    a.offsets = offsets;
    a.queue = queue;
    a.queue_len = batch;
    a.ticket = ticket;
    a.D = dims;
    a.mcs = min_cluster_size;
    a.unit_core = unit ? 1 : 0;
    a.x_in_smem = layout.x_in_smem;
    a.n_arenas = layout.n_arenas;
    a.arena_stride = (int)layout.arena_stride;
    a.x_off = (int)layout.x_off;
    a.core_off = (int)layout.core_off;
    a.eps = epsilon;
    a.core = unit ? nullptr : core;
    a.labels = labels;
    a.status = status;
    const int grid = batch < per_sm * sms ? batch : per_sm * sms;
    e = fv->launch(a, grid, smem, stream, 0);
    if (e != cudaSuccess) return fail(HDB_E_CUDA, std::string("forward kernel: ") + cudaGetErrorString(e));
    return HDB_OK;
}
