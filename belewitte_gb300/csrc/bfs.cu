// BFS half of the C ABI: variant registry, level launch, host-loop and
// CUDA-graph (device-side conditional loop) traversals.
//
// Reference: BFS::runImplementation (bfs/bfs.cpp:51-118) and the variant
// registration of bfs/bfs.cpp:121-224.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>

#include "bw_internal.cuh"

namespace bw {
namespace {

constexpr int FAMILIES = 8;
constexpr int V_FRONTIER_PUSH = 32;
constexpr int V_FRONTIER_PULL = 33;
constexpr int VARIANT_COUNT = 34;

const char *const kFamily[FAMILIES] = {
    "edge-list", "rev-edge-list", "struct-edge-list", "rev-struct-edge-list",
    "vertex-push", "vertex-pull", "vertex-push-warp", "vertex-pull-warp"};
const char *const kSuffix[4] = {"", "-bulk", "-warpreduce", "-blockreduce"};

constexpr int REP_FWD_CSR = 1, REP_REV_CSR = 2, REP_FWD_EL = 4, REP_REV_EL = 8,
              REP_FWD_ST = 16, REP_REV_ST = 32;
const int kFamilyReps[FAMILIES] = {REP_FWD_EL, REP_REV_EL, REP_FWD_ST, REP_REV_ST,
                                   REP_FWD_CSR, REP_REV_CSR, REP_FWD_CSR, REP_REV_CSR};

struct NameTable {
    std::string names[VARIANT_COUNT];
    NameTable()
    {
        for (int f = 0; f < FAMILIES; f++)
            for (int r = 0; r < 4; r++) names[f * 4 + r] = std::string(kFamily[f]) + kSuffix[r];
        names[V_FRONTIER_PUSH] = "frontier-push";
        names[V_FRONTIER_PULL] = "frontier-pull";
    }
};
const NameTable &names()
{
    static NameTable t;
    return t;
}

int variant_reps(int v)
{
    if (v >= 0 && v < 32) return kFamilyReps[v / 4];
    if (v == V_FRONTIER_PUSH) return REP_FWD_CSR;
    if (v == V_FRONTIER_PULL) return REP_REV_CSR;
    return 0;
}

int check_reps(const bw_graph_view *g, int reps)
{
    if ((reps & REP_FWD_CSR) && (!g->fwd_vertices || !g->fwd_edges)) return BW_ERR_MISSING_REPRESENTATION;
    if ((reps & REP_REV_CSR) && (!g->rev_vertices || !g->rev_edges)) return BW_ERR_MISSING_REPRESENTATION;
    if ((reps & REP_FWD_EL) && (!g->fwd_in_edges || !g->fwd_edges)) return BW_ERR_MISSING_REPRESENTATION;
    if ((reps & REP_REV_EL) && (!g->rev_in_edges || !g->rev_edges)) return BW_ERR_MISSING_REPRESENTATION;
    if ((reps & REP_FWD_ST) && !g->fwd_struct_edges) return BW_ERR_MISSING_REPRESENTATION;
    if ((reps & REP_REV_ST) && !g->rev_struct_edges) return BW_ERR_MISSING_REPRESENTATION;
    return BW_OK;
}

}  // namespace

// Depth initialisation (bfs/bfs.cpp:69-76) plus the control block; with
// `outdeg` the root's degree statistics seed the frontier features.
__global__ void k_bfs_init_side(int32_t *levels, uint64_t n, uint32_t root, uint32_t *q0, BfsCtl *ctl,
                                uint32_t max_levels, const uint32_t *outdeg)
{
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t v = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; v < n; v += stride)
        levels[v] = v == root ? 0 : INF;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        q0[0] = root;
        for (int i = 0; i < 3; i++) ctl->slot[i] = LevelSlot{};
        ctl->slot[2].frontier = 1;
        ctl->slot[2].qlen = 1;     // input queue of level 0 = {root}
        ctl->depth = 0;
        ctl->levels_done = 0;
        ctl->variant = 0;
        ctl->status = 0;
        ctl->visited = 1;
        ctl->traversed = 0;
        ctl->max_levels = max_levels;
        ctl->skip = 0;
        if (outdeg) {
            const uint32_t d = outdeg[root];
            const float l = __log2f(1.0f + static_cast<float>(d));
            ctl->slot[2].fedges = d;
            ctl->slot[2].lsum = lsum_fx(l);
            ctl->slot[2].lsq = lsq_fx(l);
            ctl->slot[2].lmax_bits = __float_as_uint(l);
            ctl->traversed = d;
        }
    }
}

namespace {

// Device-loop step: runs after every level inside the conditional body.
// Logs the level, advances the depth and ends the loop when the level
// visited nothing or the level cap is reached (status = LEVEL_LIMIT).
__global__ void k_bfs_step(BfsCtl *ctl, LevelSlot *log, uint32_t log_cap,
                           cudaGraphConditionalHandle loop)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int32_t L = ctl->depth;
    const LevelSlot s = ctl->slot[L % 3];
    if (log && static_cast<uint32_t>(L) < log_cap) log[L] = s;
    ctl->visited += s.frontier;
    ctl->traversed += s.fedges;
    ctl->levels_done = static_cast<uint32_t>(L) + 1;
    ctl->depth = L + 1;
    ctl->skip = 0;
    bool stop = s.frontier == 0;
    if (!stop && ctl->levels_done >= ctl->max_levels) {
        ctl->status = BW_ERR_LEVEL_LIMIT;
        stop = true;
    }
    if (stop) cudaGraphSetConditional(loop, 0);
}

// Sum of out-degrees of reached vertices (TEPS numerator).
__global__ void k_traversed(const int32_t *levels, const uint32_t *off, uint64_t n,
                            unsigned long long *out)
{
    unsigned long long acc = 0;
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t v = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; v < n; v += stride)
        if (levels[v] != INF) acc += off[v + 1] - off[v];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(FULL_MASK, acc, o);
    if ((threadIdx.x & 31) == 0 && acc) atomicAdd(out, acc);
}

struct Launch {
    BfsKernelFn k;
    BfsKernelFn k2;    // hub kernel after frontier-push
    unsigned block, grid;
    size_t smem;
};

int plan_launch(const bw_context *ctx, int variant, bool side, const bw_launch_config *cfg,
                Launch *out)
{
    Launch l{nullptr, nullptr, 256, static_cast<unsigned>(ctx->sm_count) * 8, 0};
    const uint32_t W = (cfg && cfg->warp_size) ? cfg->warp_size : 32;
    const uint32_t C = (cfg && cfg->chunk_size) ? cfg->chunk_size : 32;
    if (variant >= 0 && variant < 16) {
        // edge-list families (0..3 rev/struct via variant / 4)
        const int fam = variant / 4;
        const int layout = fam == 0 ? 0 : fam == 1 ? 1 : fam == 2 ? 2 : 3;
        l.k = bfs_edge_kernel(layout, variant % 4, side);
        l.block = 512;
        l.grid = static_cast<unsigned>(ctx->sm_count) * 4;
    } else if (variant >= 16 && variant < 32) {
        l.k = bfs_vertex_kernel(variant / 4, variant % 4, side);
        const int fam = variant / 4;
        if (fam == 4 || fam == 6) l.k2 = bfs_hub_kernel(side);   // vertex-push(-warp): hub rows in chunks
        if (fam == 6 || fam == 7) {
            // ImplementationTemplate.hpp:463-471: power-of-two W <= 32, C % W == 0
            if (W == 0 || W > 32 || (W & (W - 1)) || C == 0 || C % W) return BW_ERR_INVALID_ARGUMENT;
        }
    } else if (variant == V_FRONTIER_PUSH) {
        l.k = bfs_frontier_push_kernel(side);
        l.k2 = bfs_hub_kernel(side);
    } else if (variant == V_FRONTIER_PULL) {
        l.k = bfs_frontier_pull_kernel(side);
    } else {
        return BW_ERR_UNKNOWN_VARIANT;
    }
    if (cfg && cfg->block_size) {
        if (cfg->block_size % 32 || cfg->block_size > 1024) return BW_ERR_INVALID_ARGUMENT;
        if ((variant == V_FRONTIER_PUSH || variant == V_FRONTIER_PULL) && cfg->block_size != 256)
            return BW_ERR_INVALID_ARGUMENT;
        if (cfg->block_size > 512) return BW_ERR_INVALID_ARGUMENT;   // __launch_bounds__(512)
        l.block = cfg->block_size;
    }
    if (cfg && cfg->grid_size) l.grid = cfg->grid_size;
    if (variant >= 24 && variant < 32) {
        if (l.block % W) return BW_ERR_INVALID_ARGUMENT;
        l.smem = (l.block / W) * (C * 4 + (C + 1) * 4);
        if (l.smem > ctx->max_smem_per_block) return BW_ERR_INVALID_ARGUMENT;
    }
    *out = l;
    return BW_OK;
}

BfsArgs make_args(bw_context *ctx, const bw_graph_view *g, int32_t *levels, int32_t depth,
                  const bw_launch_config *cfg)
{
    BfsArgs a{};
    a.fwd_v = g->fwd_vertices; a.fwd_e = g->fwd_edges;
    a.rev_v = g->rev_vertices; a.rev_e = g->rev_edges;
    a.fwd_in = g->fwd_in_edges; a.rev_in = g->rev_in_edges;
    a.fwd_s = reinterpret_cast<const uint2 *>(g->fwd_struct_edges);
    a.rev_s = reinterpret_cast<const uint2 *>(g->rev_struct_edges);
    a.outdeg = ctx->outdeg;
    a.n = g->vertex_count; a.m = g->edge_count;
    a.levels = levels;
    a.ctl = ctx->bfs_ctl;
    a.q0 = ctx->queue[0]; a.q1 = ctx->queue[1];
    a.heavy = ctx->heavy;
    a.depth = depth;
    a.warp_size = (cfg && cfg->warp_size) ? cfg->warp_size : 32;
    a.chunk_size = (cfg && cfg->chunk_size) ? cfg->chunk_size : 32;
    return a;
}

int launch(const Launch &l, const BfsArgs &a, cudaStream_t s)
{
    l.k<<<l.grid, l.block, l.smem, s>>>(a);
    // the hub-chunk kernel is built for 256-thread blocks: the same threads
    if (l.k2) l.k2<<<hub_grid(l.grid, l.block), 256, 0, s>>>(a);
    BW_CUDA(cudaGetLastError());
    return BW_OK;
}

int validate_graph(const bw_graph_view *g)
{
    if (!g) return BW_ERR_INVALID_ARGUMENT;
    if (g->vertex_count == 0 || g->vertex_count >= 0x7fffffffULL || g->edge_count > 0xffffffffULL)
        return BW_ERR_INVALID_ARGUMENT;
    return BW_OK;
}

void fill_stats(const LevelSlot &s, int variant, bw_bfs_level_stats *out)
{
    out->frontier_vertices = s.frontier;
    out->variant = static_cast<uint32_t>(variant);
    out->frontier_edges = s.fedges;
    out->log_degree_sum = static_cast<float>(lsum_value(s.lsum));
    out->log_degree_sq_sum = static_cast<float>(lsq_value(s.lsq));
    uint32_t bits = s.lmax_bits;
    float f;
    std::memcpy(&f, &bits, sizeof f);
    out->log_degree_max = f;
    out->device_ms = 0.0f;
}

int traversed_edges(bw_context *ctx, const bw_graph_view *g, int32_t *levels, cudaStream_t s,
                    uint64_t *out)
{
    *out = 0;
    if (!g->fwd_vertices) return BW_OK;
    unsigned long long *d = nullptr;
    BW_CUDA(ctx_malloc_async(ctx, reinterpret_cast<void **>(&d), sizeof *d, s));
    BW_CUDA(cudaMemsetAsync(d, 0, sizeof *d, s));
    k_traversed<<<ctx->sm_count * 4, 256, 0, s>>>(levels, g->fwd_vertices, g->vertex_count, d);
    unsigned long long h = 0;
    BW_CUDA(cudaMemcpyAsync(&h, d, sizeof h, cudaMemcpyDeviceToHost, s));
    BW_CUDA(cudaFreeAsync(d, s));
    BW_CUDA(cudaStreamSynchronize(s));
    *out = h;
    return BW_OK;
}

// Host-loop traversal with a per-level variant schedule.
int run_host(bw_context *ctx, const bw_graph_view *g, const int32_t *schedule, uint32_t sched_len,
             uint32_t root, int32_t *levels, const bw_launch_config *cfg, uint32_t max_levels,
             int time_levels, bool side, bw_bfs_result *result, bw_bfs_level_stats *stats,
             uint32_t stats_cap, cudaStream_t s)
{
    const uint64_t n = g->vertex_count;
    if (max_levels == 0) max_levels = static_cast<uint32_t>(std::min<uint64_t>(n + 1, 0xffffffffULL));
    Launch plans[VARIANT_COUNT];
    bool planned[VARIANT_COUNT] = {};
    for (uint32_t i = 0; i < sched_len; i++) {
        const int v = schedule[i];
        if (v < 0 || v >= VARIANT_COUNT) return BW_ERR_UNKNOWN_VARIANT;
        if (!planned[v]) {
            BW_TRY(plan_launch(ctx, v, side, cfg, &plans[v]));
            planned[v] = true;
        }
    }
    if (time_levels) BW_TRY(ensure_level_events(ctx, 2));
    k_bfs_init_side<<<ctx->sm_count * 4, 256, 0, s>>>(levels, n, root, ctx->queue[0], ctx->bfs_ctl, max_levels,
                                                     side ? ctx->outdeg : nullptr);
    BW_CUDA(cudaGetLastError());
    BW_CUDA(cudaEventRecord(ctx->ev_start, s));
    float total_ms = 0.0f;
    uint32_t level = 0;
    uint64_t visited = 1;
    int status = BW_OK;
    for (;;) {
        if (level >= max_levels) { status = BW_ERR_LEVEL_LIMIT; break; }
        const int v = schedule[std::min(level, sched_len - 1)];
        BfsArgs a = make_args(ctx, g, levels, static_cast<int32_t>(level), cfg);
        if (time_levels) BW_CUDA(cudaEventRecord(ctx->level_events[0], s));
        BW_TRY(launch(plans[v], a, s));
        if (time_levels) BW_CUDA(cudaEventRecord(ctx->level_events[1], s));
        // getFrontier() (bfs/bfs.cu:13-18): read this level's slot back.
        BW_CUDA(cudaMemcpyAsync(&ctx->bfs_ctl_host->slot[level % 3], &ctx->bfs_ctl->slot[level % 3],
                                sizeof(LevelSlot), cudaMemcpyDeviceToHost, s));
        BW_CUDA(cudaStreamSynchronize(s));
        const LevelSlot sl = ctx->bfs_ctl_host->slot[level % 3];
        if (stats && level < stats_cap) {
            fill_stats(sl, v, &stats[level]);
            if (time_levels)
                BW_CUDA(cudaEventElapsedTime(&stats[level].device_ms, ctx->level_events[0], ctx->level_events[1]));
        }
        visited += sl.frontier;
        level++;
        if (sl.frontier == 0) break;
    }
    BW_CUDA(cudaEventRecord(ctx->ev_stop, s));
    BW_CUDA(cudaEventSynchronize(ctx->ev_stop));
    BW_CUDA(cudaEventElapsedTime(&total_ms, ctx->ev_start, ctx->ev_stop));
    if (result) {
        result->level_count = level;
        result->visited = visited;
        result->device_ms = total_ms;
        BW_TRY(traversed_edges(ctx, g, levels, s, &result->traversed_edges));
    }
    return status;
}

// Device-loop traversal: one CUDA graph whose conditional WHILE node runs
// [level kernel(s) -> step kernel] until the step kernel clears the loop
// condition.  No host round trip per level.
int run_graph(bw_context *ctx, const bw_graph_view *g, int variant, uint32_t root,
              int32_t *levels, const bw_launch_config *cfg, uint32_t max_levels, bool side,
              bw_bfs_result *result, bw_bfs_level_stats *stats, uint32_t stats_cap,
              cudaStream_t s)
{
    const uint64_t n = g->vertex_count;
    if (max_levels == 0) max_levels = static_cast<uint32_t>(std::min<uint64_t>(n + 1, 0xffffffffULL));
    Launch plan;
    BW_TRY(plan_launch(ctx, variant, side, cfg, &plan));
    const bool cluster_path = variant == V_FRONTIER_PUSH;
    if (cluster_path) {
        BW_TRY(ensure_outdeg(ctx, g, s));   // frontier edge volumes gate the cluster path
        BW_TRY(bfs_cluster_prepare());
    }
    LevelSlot *log = nullptr;
    const uint32_t log_cap = stats ? std::min(stats_cap, max_levels) : 0;
    if (log_cap) BW_CUDA(ctx_malloc_async(ctx, reinterpret_cast<void **>(&log), log_cap * sizeof(LevelSlot), s));

    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int rc = BW_OK;
    auto fail = [&](cudaError_t e, const char *what) {
        set_last_error(e, what);
        rc = e == cudaErrorMemoryAllocation ? BW_ERR_OUT_OF_MEMORY : BW_ERR_CUDA;
    };
    do {
        cudaError_t e = cudaGraphCreate(&graph, 0);
        if (e != cudaSuccess) { fail(e, "cudaGraphCreate"); break; }
        cudaGraphConditionalHandle handle;
        e = cudaGraphConditionalHandleCreate(&handle, graph, 1, cudaGraphCondAssignDefault);
        if (e != cudaSuccess) { fail(e, "cudaGraphConditionalHandleCreate"); break; }
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = handle;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t cnode;
        e = cudaGraphAddNode(&cnode, graph, nullptr, nullptr, 0, &cp);
        if (e != cudaSuccess) { fail(e, "cudaGraphAddNode(conditional)"); break; }
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        // Capture the body on a private stream.
        cudaStream_t cap;
        e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
        if (e != cudaSuccess) { fail(e, "cudaStreamCreate"); break; }
        // BW_LAUNCH_L2_WINDOW: the captured kernels keep the depth array persisting in L2
        L2Window win_cap;
        if (cfg && (cfg->flags & BW_LAUNCH_L2_WINDOW) &&
            l2_window_begin(ctx, cap, levels, n * sizeof(int32_t), win_cap, false) != BW_OK) {
            cudaStreamDestroy(cap);
            rc = BW_ERR_CUDA;
            break;
        }
        e = cudaStreamBeginCaptureToGraph(cap, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
        if (e == cudaSuccess) {
            BfsArgs a = make_args(ctx, g, levels, -1, cfg);
            if (cluster_path) {
                // small frontiers: the cluster kernel runs many levels per launch
                a.skip_check = 1;
                a.log = log;
                a.log_cap = log_cap;
                bfs_cluster_kernel(side ? 1 : 0)<<<CLUSTER_CTAS, CLUSTER_THREADS, bfs_cluster_smem(), cap>>>(a);
            }
            plan.k<<<plan.grid, plan.block, plan.smem, cap>>>(a);
            if (plan.k2) plan.k2<<<hub_grid(plan.grid, plan.block), 256, 0, cap>>>(a);
            k_bfs_step<<<1, 32, 0, cap>>>(ctx->bfs_ctl, log, log_cap, handle);
            cudaGraph_t captured = body;
            e = cudaStreamEndCapture(cap, &captured);
            if (e != cudaSuccess) fail(e, "cudaStreamEndCapture");
        } else {
            fail(e, "cudaStreamBeginCaptureToGraph");
        }
        l2_window_end(win_cap);                 // before its stream goes
        cudaStreamDestroy(cap);
        if (rc) break;
        e = cudaGraphInstantiate(&exec, graph, 0);
        if (e != cudaSuccess) { fail(e, "cudaGraphInstantiate"); break; }
    } while (0);
    if (rc) {
        if (graph) cudaGraphDestroy(graph);
        if (log) cudaFreeAsync(log, s);
        return rc;
    }

    k_bfs_init_side<<<ctx->sm_count * 4, 256, 0, s>>>(levels, n, root, ctx->queue[0], ctx->bfs_ctl, max_levels,
                                                     (side || cluster_path) ? ctx->outdeg : nullptr);
    BW_CUDA(cudaGetLastError());
    BW_CUDA(cudaEventRecord(ctx->ev_start, s));
    BW_CUDA(cudaGraphLaunch(exec, s));
    BW_CUDA(cudaEventRecord(ctx->ev_stop, s));
    BW_CUDA(cudaMemcpyAsync(ctx->bfs_ctl_host, ctx->bfs_ctl, sizeof(BfsCtl), cudaMemcpyDeviceToHost, s));
    BW_CUDA(cudaStreamSynchronize(s));
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    const BfsCtl c = *ctx->bfs_ctl_host;
    if (log_cap) {
        const uint32_t got = std::min(c.levels_done, log_cap);
        LevelSlot *tmp = new LevelSlot[got ? got : 1];
        BW_CUDA(cudaMemcpy(tmp, log, got * sizeof(LevelSlot), cudaMemcpyDeviceToHost));
        for (uint32_t i = 0; i < got; i++) fill_stats(tmp[i], variant, &stats[i]);
        delete[] tmp;
        BW_CUDA(cudaFreeAsync(log, s));
    }
    if (result) {
        float ms = 0.0f;
        BW_CUDA(cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop));
        result->level_count = c.levels_done;
        result->visited = c.visited;
        result->device_ms = ms;
        BW_TRY(traversed_edges(ctx, g, levels, s, &result->traversed_edges));
    }
    return c.status ? static_cast<int>(c.status) : BW_OK;
}

int prepare(bw_context *ctx, const bw_graph_view *g, int reps, bool side, int32_t *levels,
            uint32_t root, cudaStream_t s)
{
    if (!ctx || !levels) return BW_ERR_INVALID_ARGUMENT;
    BW_TRY(validate_graph(g));
    if (root >= g->vertex_count) return BW_ERR_INVALID_ARGUMENT;
    BW_TRY(check_reps(g, reps));
    BW_TRY(ensure_bfs_scratch(ctx, g->vertex_count, g->edge_count));
    if (side) BW_TRY(ensure_outdeg(ctx, g, s));
    return BW_OK;
}

}  // namespace

// A graph without edges (the edge arrays may then be null): level 0 expands
// {root} and finds nothing, so the root gets depth 0 and every other vertex
// INT_MAX after one level (bfs/bfs.cpp:80-107); no level kernel runs.
int bfs_edgeless(bw_context *ctx, const bw_graph_view *g, int variant, uint32_t root, int32_t *levels,
                 bw_bfs_result *result, bw_bfs_level_stats *stats, uint32_t stats_capacity, cudaStream_t s)
{
    if (!ctx || !levels) return BW_ERR_INVALID_ARGUMENT;
    BW_TRY(validate_graph(g));
    if (root >= g->vertex_count) return BW_ERR_INVALID_ARGUMENT;
    if (!g->fwd_vertices && !g->rev_vertices) return BW_ERR_MISSING_REPRESENTATION;
    BW_TRY(ensure_bfs_scratch(ctx, g->vertex_count, 0));
    k_bfs_init_side<<<ctx->sm_count * 4, 256, 0, s>>>(levels, g->vertex_count, root, ctx->queue[0], ctx->bfs_ctl,
                                                     0, nullptr);
    BW_CUDA(cudaGetLastError());
    BW_CUDA(cudaStreamSynchronize(s));
    if (stats && stats_capacity) {
        stats[0] = bw_bfs_level_stats{};
        stats[0].variant = static_cast<uint32_t>(variant);
    }
    if (result) {
        result->level_count = 1;
        result->visited = 1;
        result->traversed_edges = 0;
        result->device_ms = 0.0;
    }
    return BW_OK;
}

// Shared with bw_learn.cu.
int bfs_prepare(bw_context *ctx, const bw_graph_view *g, int reps, bool side, int32_t *levels, uint32_t root,
                cudaStream_t s)
{ return prepare(ctx, g, reps, side, levels, root, s); }

int bfs_plan(const bw_context *ctx, int variant, bool side, const bw_launch_config *cfg, BfsKernelFn *k,
             BfsKernelFn *k2, unsigned *block, unsigned *grid, size_t *smem)
{
    Launch l;
    BW_TRY(plan_launch(ctx, variant, side, cfg, &l));
    *k = l.k; *k2 = l.k2; *block = l.block; *grid = l.grid; *smem = l.smem;
    return BW_OK;
}

BfsArgs bfs_args(bw_context *ctx, const bw_graph_view *g, int32_t *levels, int32_t depth,
                 const bw_launch_config *cfg)
{ return make_args(ctx, g, levels, depth, cfg); }

int bfs_variant_reps(int v) { return variant_reps(v); }

int bfs_traversed(bw_context *ctx, const bw_graph_view *g, int32_t *levels, cudaStream_t s, uint64_t *out)
{ return traversed_edges(ctx, g, levels, s, out); }

}  // namespace bw

using namespace bw;

extern "C" {

int bw_bfs_variant_count(void) { return VARIANT_COUNT; }

const char *bw_bfs_variant_name(int variant)
{
    return (variant >= 0 && variant < VARIANT_COUNT) ? names().names[variant].c_str() : nullptr;
}

int bw_bfs_variant_lookup(const char *name)
{
    if (!name) return -1;
    for (int i = 0; i < VARIANT_COUNT; i++)
        if (names().names[i] == name) return i;
    return -1;
}

int bw_bfs_variant_reps(int variant) { return variant_reps(variant); }

int bw_bfs_init(bw_context *ctx, uint64_t vertex_count, uint32_t root, int32_t *levels, void *stream)
{
    if (!ctx || !levels || vertex_count == 0 || root >= vertex_count) return BW_ERR_INVALID_ARGUMENT;
    BW_TRY(ensure_bfs_scratch(ctx, vertex_count, 0));
    k_bfs_init_side<<<ctx->sm_count * 4, 256, 0, as_stream(stream)>>>(levels, vertex_count, root, ctx->queue[0],
                                                                      ctx->bfs_ctl, 0, nullptr);
    BW_CUDA(cudaGetLastError());
    return BW_OK;
}

int bw_bfs_level(bw_context *ctx, const bw_graph_view *g, int variant, int32_t *levels, int32_t depth,
                 const bw_launch_config *cfg, uint32_t *frontier, void *stream)
{
    if (!ctx || !levels || depth < 0) return BW_ERR_INVALID_ARGUMENT;
    BW_TRY(validate_graph(g));
    if (variant < 0 || variant >= VARIANT_COUNT) return BW_ERR_UNKNOWN_VARIANT;
    if (!ctx->bfs_ctl || ctx->bfs_n_cap < g->vertex_count) return BW_ERR_INVALID_ARGUMENT;  // bw_bfs_init first
    if (g->edge_count == 0) {
        // no edges: the level visits nothing; its counts read as zero
        cudaStream_t s = as_stream(stream);
        BW_CUDA(cudaMemsetAsync(&ctx->bfs_ctl->slot[depth % 3], 0, sizeof(LevelSlot), s));
        BW_CUDA(cudaStreamSynchronize(s));
        if (frontier) *frontier = 0;
        return BW_OK;
    }
    BW_TRY(check_reps(g, variant_reps(variant)));
    BW_TRY(ensure_bfs_scratch(ctx, g->vertex_count, g->edge_count));
    Launch plan;
    // Queue-driven variants need the queue kept by every level: levels run
    // through this entry point always emit it.
    const bool side = g->fwd_vertices != nullptr;
    if (side) BW_TRY(ensure_outdeg(ctx, g, as_stream(stream)));
    if (!side && (variant == V_FRONTIER_PUSH)) return BW_ERR_MISSING_REPRESENTATION;
    BW_TRY(plan_launch(ctx, variant, side, cfg, &plan));
    cudaStream_t s = as_stream(stream);
    BfsArgs a = make_args(ctx, g, levels, depth, cfg);
    BW_TRY(launch(plan, a, s));
    BW_CUDA(cudaMemcpyAsync(&ctx->bfs_ctl_host->slot[depth % 3], &ctx->bfs_ctl->slot[depth % 3],
                            sizeof(LevelSlot), cudaMemcpyDeviceToHost, s));
    BW_CUDA(cudaStreamSynchronize(s));
    if (frontier) *frontier = ctx->bfs_ctl_host->slot[depth % 3].frontier;
    return BW_OK;
}

int bw_bfs_run(bw_context *ctx, const bw_graph_view *g, int variant, uint32_t root, int32_t *levels,
               const bw_launch_config *cfg, int loop_mode, uint32_t max_levels,
               bw_bfs_result *result, bw_bfs_level_stats *stats, uint32_t stats_capacity,
               void *stream)
{
    if (variant < 0 || variant >= VARIANT_COUNT) return BW_ERR_UNKNOWN_VARIANT;
    // frontier-push needs the queue of the level before it, which only it
    // (or a side-output level) writes; a fixed frontier-push run keeps it.
    const bool side = stats != nullptr && stats_capacity > 0;
    int reps = variant_reps(variant) | (side ? REP_FWD_CSR : 0);
    cudaStream_t s = as_stream(stream);
    if (loop_mode != BW_LOOP_GRAPH && loop_mode != BW_LOOP_HOST) return BW_ERR_INVALID_ARGUMENT;
    if (g && g->edge_count == 0) return bfs_edgeless(ctx, g, variant, root, levels, result, stats, stats_capacity, s);
    BW_TRY(prepare(ctx, g, reps, side, levels, root, s));
    L2Window win;                  // BW_LAUNCH_L2_WINDOW: the depth array persisting in L2
    if (cfg && (cfg->flags & BW_LAUNCH_L2_WINDOW))
        BW_TRY(l2_window_begin(ctx, s, levels, g->vertex_count * sizeof(int32_t), win));
    if (loop_mode == BW_LOOP_GRAPH)
        return run_graph(ctx, g, variant, root, levels, cfg, max_levels, side, result, stats, stats_capacity, s);
    if (loop_mode != BW_LOOP_HOST) return BW_ERR_INVALID_ARGUMENT;
    int32_t sched = variant;
    return run_host(ctx, g, &sched, 1, root, levels, cfg, max_levels, 0, side, result, stats,
                    stats_capacity, s);
}

int bw_bfs_run_schedule(bw_context *ctx, const bw_graph_view *g, const int32_t *schedule,
                        uint32_t schedule_len, uint32_t root, int32_t *levels,
                        const bw_launch_config *cfg, uint32_t max_levels, int time_levels,
                        bw_bfs_result *result, bw_bfs_level_stats *stats, uint32_t stats_capacity,
                        void *stream)
{
    if (!schedule || schedule_len == 0) return BW_ERR_INVALID_ARGUMENT;
    // Mixed schedules hand the frontier from one variant to the next, so
    // every level emits the queue and statistics (needs the forward CSR).
    int reps = REP_FWD_CSR;
    for (uint32_t i = 0; i < schedule_len; i++) {
        if (schedule[i] < 0 || schedule[i] >= VARIANT_COUNT) return BW_ERR_UNKNOWN_VARIANT;
        reps |= variant_reps(schedule[i]);
    }
    cudaStream_t s = as_stream(stream);
    if (g && g->edge_count == 0)
        return bfs_edgeless(ctx, g, schedule[0], root, levels, result, stats, stats_capacity, s);
    BW_TRY(prepare(ctx, g, reps, true, levels, root, s));
    return run_host(ctx, g, schedule, schedule_len, root, levels, cfg, max_levels, time_levels, true,
                    result, stats, stats_capacity, s);
}

}  // extern "C"
