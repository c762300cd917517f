#include <algorithm>
// Context, scratch management, launch geometry and representation builders.
#include <cstdio>
#include <cstring>
#include <new>

#include "bw_internal.cuh"

#ifndef BW_VERSION_STRING
#define BW_VERSION_STRING "belewitte-gb300-unknown"
#endif

namespace bw {

static thread_local char g_last_error[512] = "";

void set_last_error(cudaError_t e, const char *what)
{
    std::snprintf(g_last_error, sizeof g_last_error, "%s: %s (%s)", what,
                  cudaGetErrorString(e), cudaGetErrorName(e));
}

void compute_division(uint64_t count, uint32_t sm, uint32_t max_tpb,
                      uint32_t *block, uint32_t *grid)
{
    // result.first = ceil(count / (i * SMs)) for the smallest i with
    // result.first <= maxThreadsPerBlock, rounded up to a multiple of 32;
    // result.second = min(i * SMs, ceil(count / result.first)).
    if (sm == 0) sm = 1;
    if (max_tpb == 0) max_tpb = 1024;
    auto ceil_div = [](uint64_t x, uint64_t y) { return (x + y - 1) / y; };
    uint64_t i = 1;
    uint64_t b = ceil_div(count, sm);
    while (b > max_tpb) { i++; b = ceil_div(count, i * sm); }
    uint64_t adjust = b % 32;
    b += adjust ? 32 - adjust : 0;
    if (b == 0) b = 32;
    uint64_t g = i * sm;
    uint64_t need = ceil_div(count, b);
    if (need < g) g = need;
    if (g == 0) g = 1;
    *block = static_cast<uint32_t>(b);
    *grid = static_cast<uint32_t>(g);
}

template<typename T>
static int grow(T **ptr, uint64_t count)
{
    if (*ptr) { cudaFree(*ptr); *ptr = nullptr; }
    if (count == 0) count = 1;
    BW_CUDA(cudaMalloc(reinterpret_cast<void **>(ptr), count * sizeof(T)));
    return BW_OK;
}

int ensure_bfs_scratch(bw_context *ctx, uint64_t n, uint64_t m)
{
    if (!ctx->bfs_ctl) {
        BW_CUDA(cudaMalloc(reinterpret_cast<void **>(&ctx->bfs_ctl), sizeof(BfsCtl)));
        BW_CUDA(cudaMemset(ctx->bfs_ctl, 0, sizeof(BfsCtl)));
        BW_CUDA(cudaMallocHost(reinterpret_cast<void **>(&ctx->bfs_ctl_host), sizeof(BfsCtl)));
    }
    if (n > ctx->bfs_n_cap) {
        BW_TRY(grow(&ctx->queue[0], n));
        BW_TRY(grow(&ctx->queue[1], n));
        ctx->bfs_n_cap = n;
    }
    // Hub chunks: every queued vertex has degree > 256 and yields at most
    // 2*deg/256 chunks of 256 edges, so 2M/256 + N/256 bounds a level.
    uint64_t hcap = 2 * m / 256 + n / 256 + 1024;
    if (hcap > ctx->heavy_cap) {
        BW_TRY(grow(&ctx->heavy, hcap));
        ctx->heavy_cap = hcap;
    }
    return BW_OK;
}

__global__ void k_row_lengths(const uint32_t *__restrict__ off, uint64_t n,
                              uint32_t *__restrict__ deg)
{
    for (uint64_t v = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; v < n;
         v += uint64_t(gridDim.x) * blockDim.x)
        deg[v] = off[v + 1] - off[v];
}

// Out-degrees of the view's graph, recomputed for every run (one pass over
// N): a cache keyed on the offsets pointer went stale when a freed graph's
// memory was reused by another graph of the same size.
int ensure_outdeg(bw_context *ctx, const bw_graph_view *g, cudaStream_t s)
{
    if (!g->fwd_vertices) return BW_ERR_MISSING_REPRESENTATION;
    if (g->vertex_count > ctx->outdeg_cap) {
        BW_TRY(grow(&ctx->outdeg, g->vertex_count));
        ctx->outdeg_cap = g->vertex_count;
    }
    k_row_lengths<<<default_grid(ctx, 4), 256, 0, s>>>(g->fwd_vertices, g->vertex_count, ctx->outdeg);
    BW_CUDA(cudaGetLastError());
    return BW_OK;
}

int ensure_pr_scratch(bw_context *ctx, uint64_t n, uint32_t iterations)
{
    if (n > ctx->pr_n_cap) {
        BW_TRY(grow(&ctx->pr_acc, n));
        // both contribution buffers in one allocation, so one L2
        // access-policy window covers the vector every iteration gathers;
        // the second starts on a 256-byte boundary (the kernels read both
        // with 16-byte vector loads)
        const uint64_t stride = (n + 63) & ~uint64_t(63);
        BW_TRY(grow(&ctx->pr_buf[0], 2 * stride));
        ctx->pr_buf[1] = ctx->pr_buf[0] + stride;
        BW_TRY(grow(&ctx->pr_deg, n));
        ctx->pr_n_cap = n;
    }
    uint32_t need = iterations + 1;
    if (need > ctx->pr_diff_cap) {
        BW_TRY(grow(&ctx->pr_diffs, need));
        ctx->pr_diff_cap = need;
    }
    return BW_OK;
}

int ensure_level_events(bw_context *ctx, uint32_t count)
{
    if (count <= ctx->level_event_cap) return BW_OK;
    for (uint32_t i = 0; i < ctx->level_event_cap; i++) cudaEventDestroy(ctx->level_events[i]);
    delete[] ctx->level_events;
    ctx->level_events = new (std::nothrow) cudaEvent_t[count];
    ctx->level_event_cap = 0;
    if (!ctx->level_events) return BW_ERR_OUT_OF_MEMORY;
    for (uint32_t i = 0; i < count; i++) {
        BW_CUDA(cudaEventCreate(&ctx->level_events[i]));
        ctx->level_event_cap = i + 1;
    }
    return BW_OK;
}

// In-edge (row id) expansion of a CSR: one warp per row range, coalesced
// stores of the row id over each row.
__global__ void k_expand_rows(const uint32_t *__restrict__ off, uint64_t n,
                              uint32_t *__restrict__ in_edges)
{
    const uint64_t warp = (blockIdx.x * uint64_t(blockDim.x) + threadIdx.x) >> 5;
    const uint64_t warps = (uint64_t(gridDim.x) * blockDim.x) >> 5;
    const unsigned lane = threadIdx.x & 31;
    for (uint64_t v = warp; v < n; v += warps) {
        const uint32_t s = off[v], e = off[v + 1];
        for (uint32_t i = s + lane; i < e; i += 32) in_edges[i] = static_cast<uint32_t>(v);
    }
}

__global__ void k_struct_edges(const uint32_t *__restrict__ in, const uint32_t *__restrict__ out,
                               uint64_t m, uint2 *__restrict__ s)
{
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < m;
         i += uint64_t(gridDim.x) * blockDim.x)
        s[i] = make_uint2(in[i], out[i]);
}

}  // namespace bw

using namespace bw;

extern "C" {

const char *bw_status_string(int status)
{
    switch (status) {
      case BW_OK: return "ok";
      case BW_ERR_INVALID_ARGUMENT: return "invalid argument";
      case BW_ERR_MISSING_REPRESENTATION: return "graph view lacks a representation the variant needs";
      case BW_ERR_UNKNOWN_VARIANT: return "unknown variant";
      case BW_ERR_CUDA: return "CUDA error";
      case BW_ERR_OUT_OF_MEMORY: return "out of memory";
      case BW_ERR_LEVEL_LIMIT: return "level limit reached";
      case BW_ERR_TOO_LARGE: return "size beyond the supported range";
      case BW_ERR_IO: return "I/O error";
      case BW_ERR_FORMAT: return "malformed graph file";
      case BW_ERR_NO_DEVICE: return "no CUDA device";
      default: return "unknown status";
    }
}

const char *bw_last_error(void) { return g_last_error; }

const char *bw_version(void) { return BW_VERSION_STRING; }

int bw_context_create(int device, bw_context **out)
{
    if (!out) return BW_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        if (e != cudaSuccess) set_last_error(e, "cudaGetDeviceCount");
        return BW_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= count) return BW_ERR_INVALID_ARGUMENT;
    BW_CUDA(cudaSetDevice(device));
    cudaDeviceProp prop;
    BW_CUDA(cudaGetDeviceProperties(&prop, device));
    bw_context *ctx = new (std::nothrow) bw_context();
    if (!ctx) return BW_ERR_OUT_OF_MEMORY;
    ctx->device = device;
    ctx->sm_count = prop.multiProcessorCount;
    ctx->max_threads_per_block = prop.maxThreadsPerBlock;
    ctx->max_smem_per_block = prop.sharedMemPerBlock;
    ctx->max_smem_optin = prop.sharedMemPerBlockOptin;
    ctx->max_smem_per_sm = prop.sharedMemPerMultiprocessor;
    if (cudaEventCreate(&ctx->ev_start) != cudaSuccess ||
        cudaEventCreate(&ctx->ev_stop) != cudaSuccess) {
        bw_context_destroy(ctx);
        return BW_ERR_CUDA;
    }
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    if (cudaMemPoolCreate(&ctx->pool, &props) == cudaSuccess) {
        uint64_t keep = ~uint64_t(0);
        cudaMemPoolSetAttribute(ctx->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    } else {
        ctx->pool = nullptr;                 // fall back to the device's default pool
        cudaGetLastError();
    }
    *out = ctx;
    return BW_OK;
}

int bw_context_destroy(bw_context *ctx)
{
    if (!ctx) return BW_OK;
    cudaSetDevice(ctx->device);
    if (ctx->pool) {
        cudaDeviceSynchronize();             // scratch frees still queued on streams
        cudaMemPoolDestroy(ctx->pool);
    }
    cudaFree(ctx->bfs_ctl);
    if (ctx->bfs_ctl_host) cudaFreeHost(ctx->bfs_ctl_host);
    cudaFree(ctx->queue[0]);
    cudaFree(ctx->queue[1]);
    cudaFree(ctx->heavy);
    cudaFree(ctx->outdeg);
    cudaFree(ctx->pr_acc);
    cudaFree(ctx->pr_buf[0]);                 // pr_buf[1] lies inside it
    cudaFree(ctx->pr_deg);
    cudaFree(ctx->pr_diffs);
    if (ctx->ev_start) cudaEventDestroy(ctx->ev_start);
    if (ctx->ev_stop) cudaEventDestroy(ctx->ev_stop);
    for (uint32_t i = 0; i < ctx->level_event_cap; i++) cudaEventDestroy(ctx->level_events[i]);
    delete[] ctx->level_events;
    delete ctx;
    return BW_OK;
}

int bw_context_sm_count(const bw_context *ctx) { return ctx ? ctx->sm_count : 0; }

void bw_compute_division(uint64_t count, uint32_t sm_count,
                         uint32_t max_threads_per_block,
                         uint32_t *block_out, uint32_t *grid_out)
{
    uint32_t b = 0, g = 0;
    compute_division(count, sm_count, max_threads_per_block, &b, &g);
    if (block_out) *block_out = b;
    if (grid_out) *grid_out = g;
}

int bw_expand_edge_list(const uint32_t *vertices, uint64_t vertex_count,
                        uint64_t edge_count, uint32_t *in_edges, void *stream)
{
    if (!vertices || (edge_count && !in_edges)) return BW_ERR_INVALID_ARGUMENT;
    if (vertex_count == 0 || edge_count == 0) return BW_OK;
    int dev = 0, sm = 0;
    BW_CUDA(cudaGetDevice(&dev));
    BW_CUDA(cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev));
    k_expand_rows<<<sm * 8, 256, 0, as_stream(stream)>>>(vertices, vertex_count, in_edges);
    BW_CUDA(cudaGetLastError());
    return BW_OK;
}

int bw_build_struct_edges(const uint32_t *in_edges, const uint32_t *out_edges,
                          uint64_t edge_count, uint32_t *struct_edges, void *stream)
{
    if (edge_count && (!in_edges || !out_edges || !struct_edges)) return BW_ERR_INVALID_ARGUMENT;
    if (edge_count == 0) return BW_OK;
    int dev = 0, sm = 0;
    BW_CUDA(cudaGetDevice(&dev));
    BW_CUDA(cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev));
    k_struct_edges<<<sm * 8, 256, 0, as_stream(stream)>>>(in_edges, out_edges, edge_count,
                                                         reinterpret_cast<uint2 *>(struct_edges));
    BW_CUDA(cudaGetLastError());
    return BW_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// L2 access-policy window (BW_LAUNCH_L2_WINDOW)
// ---------------------------------------------------------------------------
namespace bw {

L2Window::~L2Window() { l2_window_end(*this); }

int l2_window_begin(bw_context *ctx, cudaStream_t s, const void *base, size_t bytes, L2Window &w, bool carve_out)
{
    l2_window_end(w);
    if (!base || bytes == 0) return BW_OK;
    // a window is a stream attribute: the legacy default stream (and the
    // per-thread one) carries none
    if (s == nullptr || s == cudaStreamLegacy || s == cudaStreamPerThread) {
        set_last_error(cudaErrorInvalidResourceHandle, "BW_LAUNCH_L2_WINDOW needs a created stream");
        return BW_ERR_INVALID_ARGUMENT;
    }
    int persist_max = 0, window_max = 0;
    BW_CUDA(cudaDeviceGetAttribute(&persist_max, cudaDevAttrMaxPersistingL2CacheSize, ctx->device));
    BW_CUDA(cudaDeviceGetAttribute(&window_max, cudaDevAttrMaxAccessPolicyWindowSize, ctx->device));
    if (persist_max <= 0 || window_max <= 0) return BW_OK;      // not supported: nothing to do
    const size_t span = std::min<size_t>(bytes, static_cast<size_t>(window_max));
    const size_t carve = std::min<size_t>(span, static_cast<size_t>(persist_max));
    if (carve_out) BW_CUDA(cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, carve));
    w.carved = carve_out;
    cudaStreamAttrValue v{};
    v.accessPolicyWindow.base_ptr = const_cast<void *>(base);
    v.accessPolicyWindow.num_bytes = span;
    v.accessPolicyWindow.hitRatio = static_cast<float>(std::min(1.0, static_cast<double>(carve) / span));
    v.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
    v.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
    BW_CUDA(cudaStreamSetAttribute(s, cudaStreamAttributeAccessPolicyWindow, &v));
    w.stream = s;
    w.on = true;
    w.bytes = span;
    return BW_OK;
}

void l2_window_end(L2Window &w)
{
    if (!w.on) return;
    cudaStreamAttrValue v{};                       // an empty window
    v.accessPolicyWindow.num_bytes = 0;
    cudaStreamSetAttribute(w.stream, cudaStreamAttributeAccessPolicyWindow, &v);
    if (w.carved) {
        cudaCtxResetPersistingL2Cache();           // the lines go back to normal
        cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, 0);
    }
    w.on = false;
    w.carved = false;
}

}  // namespace bw
