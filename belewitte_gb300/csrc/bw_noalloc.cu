// Allocation-free BFS entry point: frontier-push with its scratch (control
// block, two frontier queues, hub-chunk queue) in a file-scope device array
// instead of a bw_context.
//
// Some callers cannot allocate device memory once they are running: a
// serving process that reserves its HBM budget at start-up and forbids
// allocation on the request path (cudaMalloc can synchronise the device and
// can fail under fragmentation), or a host application that loads this
// library as a plugin under an allocator policy it does not own.  This entry
// point lets them run BFS with caller-owned inputs and outputs only.
#include <mutex>

#include "bw_internal.cuh"

namespace bw {

__global__ void k_bfs_init_side(int32_t *levels, uint64_t n, uint32_t root, uint32_t *q0, BfsCtl *ctl,
                                uint32_t max_levels, const uint32_t *outdeg);

namespace {

constexpr uint64_t NOALLOC_MAX_VERTICES = uint64_t(1) << 20;
constexpr uint64_t NOALLOC_MAX_EDGES = uint64_t(1) << 24;
// frontier-push queues hub rows (> 256 edges) as 256-edge chunks: at most
// 2M/256 chunks per level (see ensure_bfs_scratch).
constexpr uint64_t NOALLOC_HEAVY = 2 * NOALLOC_MAX_EDGES / 256 + NOALLOC_MAX_VERTICES / 256 + 1024;

struct NoAllocScratch {
    BfsCtl ctl;
    uint32_t q0[NOALLOC_MAX_VERTICES];
    uint32_t q1[NOALLOC_MAX_VERTICES];
    uint2 heavy[NOALLOC_HEAVY];
};

// About 9.2 MB on every GPU that loads this library, held until exit.
static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

// Device addresses of g_noalloc_scratch per device (the host-side symbol is
// only a stand-in; kernels must be given these).
constexpr int MAX_DEVICES = 64;
NoAllocScratch *g_scratch_ptr[MAX_DEVICES] = {};
std::mutex g_scratch_mutex;

int scratch_for_current_device(NoAllocScratch **out)
{
    int dev = 0;
    BW_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= MAX_DEVICES) return BW_ERR_NO_DEVICE;
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        BW_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_scratch_ptr[dev] = static_cast<NoAllocScratch *>(p);
    }
    *out = g_scratch_ptr[dev];
    return BW_OK;
}

}  // namespace
}  // namespace bw

using namespace bw;

extern "C" int bw_bfs_run_noalloc(const bw_graph_view *g, uint32_t root, int32_t *levels, uint32_t max_levels,
                                  uint32_t *level_count, void *stream)
{
    if (!g || !levels || !g->fwd_vertices || (g->edge_count && !g->fwd_edges)) return BW_ERR_INVALID_ARGUMENT;
    if (g->vertex_count == 0 || root >= g->vertex_count) return BW_ERR_INVALID_ARGUMENT;
    if (g->vertex_count > NOALLOC_MAX_VERTICES || g->edge_count > NOALLOC_MAX_EDGES) return BW_ERR_TOO_LARGE;
    NoAllocScratch *sc = nullptr;
    BW_TRY(scratch_for_current_device(&sc));
    int dev = 0, sm = 0;
    BW_CUDA(cudaGetDevice(&dev));
    BW_CUDA(cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev));
    cudaStream_t s = as_stream(stream);
    const uint64_t n = g->vertex_count;
    if (max_levels == 0) max_levels = static_cast<uint32_t>(n + 1);

    BfsArgs a{};
    a.fwd_v = g->fwd_vertices;
    a.fwd_e = g->fwd_edges;
    a.n = n;
    a.m = g->edge_count;
    a.levels = levels;
    a.ctl = &sc->ctl;
    a.q0 = sc->q0;
    a.q1 = sc->q1;
    a.heavy = sc->heavy;
    a.warp_size = 32;
    a.chunk_size = 32;
    const BfsKernelFn push = bfs_frontier_push_kernel(false);
    const BfsKernelFn hubs = bfs_hub_kernel(false);

    // The init kernel clears the control block left by the previous call and
    // sets the first queue to {root}; the queues need no clearing.
    k_bfs_init_side<<<sm * 4, 256, 0, s>>>(levels, n, root, sc->q0, &sc->ctl, max_levels, nullptr);
    BW_CUDA(cudaGetLastError());
    if (g->edge_count == 0) {          // level 0 finds nothing (the edge array may be null)
        BW_CUDA(cudaStreamSynchronize(s));
        if (level_count) *level_count = 1;
        return BW_OK;
    }
    uint32_t level = 0;
    for (;;) {
        if (level >= max_levels) {
            if (level_count) *level_count = level;
            return BW_ERR_LEVEL_LIMIT;
        }
        a.depth = static_cast<int32_t>(level);
        push<<<sm * 8, 256, 0, s>>>(a);
        hubs<<<sm * 8, 256, 0, s>>>(a);
        BW_CUDA(cudaGetLastError());
        uint32_t frontier = 0;
        BW_CUDA(cudaMemcpyAsync(&frontier, &sc->ctl.slot[level % 3].frontier, sizeof frontier,
                                cudaMemcpyDeviceToHost, s));
        BW_CUDA(cudaStreamSynchronize(s));
        level++;
        if (frontier == 0) break;
    }
    if (level_count) *level_count = level;
    return BW_OK;
}
