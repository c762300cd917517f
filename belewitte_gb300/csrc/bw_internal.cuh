// Internal declarations shared by the CUDA translation units of
// libbelewitte_gb300.so.  Not part of the C ABI.
#pragma once
#include <cmath>

#include <cstdint>
#include <climits>
#include <cuda_runtime.h>

#include "belewitte_gb300.h"

namespace bw {

constexpr int32_t INF = INT32_MAX;
constexpr unsigned FULL_MASK = 0xffffffffu;

// ---------------------------------------------------------------------------
// Error handling: every CUDA call is checked, the message is kept per thread
// and the C ABI returns BW_ERR_CUDA (the reference prints and exits instead,
// CUDA.cpp:7-26).
// ---------------------------------------------------------------------------
void set_last_error(cudaError_t e, const char *what);

#define BW_CUDA(call)                                                       \
    do {                                                                    \
        cudaError_t bw_err_ = (call);                                       \
        if (bw_err_ != cudaSuccess) {                                       \
            ::bw::set_last_error(bw_err_, #call);                           \
            return bw_err_ == cudaErrorMemoryAllocation                     \
                       ? BW_ERR_OUT_OF_MEMORY : BW_ERR_CUDA;                \
        }                                                                   \
    } while (0)

#define BW_TRY(expr)                                                        \
    do {                                                                    \
        int bw_rc_ = (expr);                                                \
        if (bw_rc_ != BW_OK) return bw_rc_;                                 \
    } while (0)

// ---------------------------------------------------------------------------
// BFS device control block.  A level L accumulates into slot[L % 3], reads
// the length of its input frontier queue from slot[(L + 2) % 3] and block 0
// zeroes slot[(L + 1) % 3] for the next level, so no separate reset launch
// (the reference's resetFrontier(), bfs/bfs.cu:7-11) is needed per level.
// ---------------------------------------------------------------------------
struct LevelSlot {
    uint32_t frontier;            // reference `frontier` counter
    uint32_t qlen;                // next frontier queue length
    unsigned long long fedges;    // sum of out-degrees of new vertices
    unsigned long long lsum;      // sum log2(1+deg), fixed point (lsum_fx)
    unsigned long long lsq;       // sum log2(1+deg)^2, fixed point (lsq_fx)
    uint32_t lmax_bits;           // max log2(1+deg) as float bits
    uint32_t heavy;               // hub chunks queued (frontier-push)
};

// The level statistics of log2(1 + out-degree) are summed in fixed point,
// in units of 2^-24 (sum) and 2^-20 (sum of squares): integer additions are
// associative, so a level's sums -- and the learned switch's decisions that
// read them -- are the same whatever order threads, warps and blocks add in.
// log2(1 + d) <= 32 for 32-bit degrees, so a term is below 2^30 and 2^32
// terms stay below 2^62.
constexpr float LSUM_UNIT = 16777216.0f;   // 2^24
constexpr float LSQ_UNIT = 1048576.0f;     // 2^20
__host__ __device__ __forceinline__ unsigned long long lsum_fx(float l)
{
#if defined(__CUDA_ARCH__)
    return __float2ull_rn(l * LSUM_UNIT);
#else
    return static_cast<unsigned long long>(std::nearbyint(l * LSUM_UNIT));
#endif
}
__host__ __device__ __forceinline__ unsigned long long lsq_fx(float l)
{
#if defined(__CUDA_ARCH__)
    return __float2ull_rn(__fmul_rn(l, l) * LSQ_UNIT);
#else
    return static_cast<unsigned long long>(std::nearbyint((l * l) * LSQ_UNIT));
#endif
}
__host__ __device__ __forceinline__ double lsum_value(unsigned long long v) { return static_cast<double>(v) / LSUM_UNIT; }
__host__ __device__ __forceinline__ double lsq_value(unsigned long long v) { return static_cast<double>(v) / LSQ_UNIT; }
// The moments as the features read them: rounded to IEEE single, the
// precision the level statistics report them in (bw_bfs_level_stats), so
// the device switch, the host loop, the training samples and a predictor
// library fed the reported statistics all form identical features.
__host__ __device__ __forceinline__ double lsum_feature(unsigned long long v)
{ return static_cast<double>(static_cast<float>(lsum_value(v))); }
__host__ __device__ __forceinline__ double lsq_feature(unsigned long long v)
{ return static_cast<double>(static_cast<float>(lsq_value(v))); }

struct BfsCtl {
    LevelSlot slot[3];
    int32_t depth;                // level being run (device-loop mode)
    uint32_t levels_done;
    int32_t variant;              // variant of the next level (device loop)
    uint32_t status;              // 0 ok, BW_ERR_LEVEL_LIMIT
    unsigned long long visited;   // running totals (device loop)
    unsigned long long traversed;
    uint32_t max_levels;
    uint32_t skip;                // the cluster kernel already ran this level
    uint32_t pad[2];
};

struct BfsArgs {
    const uint32_t *fwd_v, *fwd_e, *rev_v, *rev_e;
    const uint32_t *fwd_in, *rev_in;
    const uint2 *fwd_s, *rev_s;
    const uint32_t *outdeg;       // out-degree per vertex (side statistics)
    uint64_t n, m;
    int32_t *levels;
    BfsCtl *ctl;
    uint32_t *q0, *q1;            // frontier queues, parity = depth & 1
    uint2 *heavy;                 // hub chunk queue {vertex, first edge}
    int32_t depth;                // >= 0: this level; < 0: read ctl->depth
    uint32_t warp_size, chunk_size;
    uint32_t skip_check;          // device loop with the cluster path: honour ctl->skip
    LevelSlot *log;               // device-loop level log (cluster path)
    uint32_t log_cap;
};

// ---------------------------------------------------------------------------
// PageRank scratch
// ---------------------------------------------------------------------------
struct PrCtl {
    float diff;                   // reference `diff` (pagerank/pagerank.cu:4)
    uint32_t pad[7];
};

}  // namespace bw

// The opaque context of the C ABI.
struct bw_context {
    int device = 0;
    int sm_count = 0;
    int max_threads_per_block = 1024;
    size_t max_smem_per_block = 0;
    size_t max_smem_optin = 0;
    size_t max_smem_per_sm = 0;
    // Stream-ordered pool for per-run scratch.  Its release threshold is
    // unbounded, so memory freed at the end of a run is reused by the next
    // one instead of going back to the driver at every synchronisation.
    cudaMemPool_t pool = nullptr;
    uint32_t launches = 0;                // own kernels launched by the current run

    // BFS scratch
    bw::BfsCtl *bfs_ctl = nullptr;        // device
    bw::BfsCtl *bfs_ctl_host = nullptr;   // pinned mirror for read-back
    uint32_t *queue[2] = {nullptr, nullptr};
    uint2 *heavy = nullptr;
    uint64_t bfs_n_cap = 0, heavy_cap = 0;
    uint32_t *outdeg = nullptr;
    uint64_t outdeg_cap = 0;

    // PageRank scratch
    float *pr_acc = nullptr, *pr_buf[2] = {nullptr, nullptr};
    uint32_t *pr_deg = nullptr;
    float *pr_diffs = nullptr;            // per-iteration diff (device)
    uint64_t pr_n_cap = 0;
    uint32_t pr_diff_cap = 0;

    cudaEvent_t ev_start = nullptr, ev_stop = nullptr;
    cudaEvent_t *level_events = nullptr;
    uint32_t level_event_cap = 0;
};

namespace bw {

int ensure_bfs_scratch(bw_context *ctx, uint64_t n, uint64_t m);
int ensure_outdeg(bw_context *ctx, const bw_graph_view *g, cudaStream_t s);
int pagerank_run_schedule_loop(bw_context *ctx, const bw_graph_view *g, const int32_t *schedule,
                               uint32_t schedule_len, uint32_t iterations, float *ranks, int loop_mode,
                               bw_pagerank_result *result, float *diffs, cudaStream_t stream);
int pagerank_moments(bw_context *ctx, const bw_graph_view *g, float *ls, float *lq, float *lm, cudaStream_t s);
void pagerank_feature_vector(const bw_graph_view *g, float ls, float lq, float lm, uint32_t iteration, float *x);
int bfs_edgeless(bw_context *ctx, const bw_graph_view *g, int variant, uint32_t root, int32_t *levels,
                 bw_bfs_result *result, bw_bfs_level_stats *stats, uint32_t stats_capacity, cudaStream_t s);
int ensure_pr_scratch(bw_context *ctx, uint64_t n, uint32_t iterations);
int ensure_level_events(bw_context *ctx, uint32_t count);

inline cudaStream_t as_stream(void *s) { return static_cast<cudaStream_t>(s); }

// BW_LAUNCH_L2_WINDOW: an access-policy window that keeps [base, base +
// bytes) persisting in L2 for the kernels of `s` (and of graphs captured
// from it), with a persisting carve-out of the same size (at most the
// device's maximum); l2_window_end removes the window, resets the
// persisting lines and the carve-out to 0.  A context-level setting: it
// ends with the process.
struct L2Window {
    cudaStream_t stream = nullptr;
    bool on = false;
    bool carved = false;                           // this window set the carve-out
    size_t bytes = 0;
    L2Window() = default;
    L2Window(const L2Window &) = delete;
    L2Window &operator=(const L2Window &) = delete;
    ~L2Window();                                   // l2_window_end
};
// carve_out false: the window only (a stream whose kernels run under a
// carve-out another window holds, e.g. one that captures a graph).
int l2_window_begin(bw_context *ctx, cudaStream_t s, const void *base, size_t bytes, L2Window &w,
                    bool carve_out = true);
void l2_window_end(L2Window &w);

// Persistent-style default grid: `per_sm` blocks per SM.
inline unsigned default_grid(const bw_context *ctx, unsigned per_sm)
{ return static_cast<unsigned>(ctx->sm_count) * per_sm; }

// deg[v] = off[v+1] - off[v]
__global__ void k_row_lengths(const uint32_t *__restrict__ off, uint64_t n,
                              uint32_t *__restrict__ deg);

using BfsKernelFn = void (*)(BfsArgs);
// Instantiation tables (bfs_edge.cu, bfs_vertex.cu).
BfsKernelFn bfs_edge_kernel(int layout, int reduction, bool side);
BfsKernelFn bfs_vertex_kernel(int family, int reduction, bool side);
BfsKernelFn bfs_frontier_push_kernel(bool side);
BfsKernelFn bfs_hub_kernel(bool side);
// The hub-chunk kernel runs 256-thread blocks: the grid that gives it the
// same number of threads as a level kernel of `grid` x `block`.
inline unsigned hub_grid(unsigned grid, unsigned block)
{ return static_cast<unsigned>((static_cast<unsigned long long>(grid) * block + 255) / 256); }
BfsKernelFn bfs_frontier_pull_kernel(bool side);
// the 8-block cluster kernel (CLUSTER_CTAS blocks of 1024 threads); stats:
// 0 none, 1 every level's, 2 only a handed-over level's
BfsKernelFn bfs_cluster_kernel(int stats);
size_t bfs_cluster_smem();                    // its dynamic shared memory
int bfs_cluster_prepare();                    // allows that much on the current device
constexpr unsigned CLUSTER_CTAS = 8;
constexpr unsigned CLUSTER_THREADS = 1024;
constexpr uint32_t CLUSTER_LIST = 4096;            // frontier entries per block list
constexpr uint32_t CLUSTER_CAP = CLUSTER_LIST * CLUSTER_CTAS;   // frontier vertices the cluster kernel takes
constexpr unsigned long long CLUSTER_EDGE_CAP = 65536;        // and their out-edges

// Reference Backend::computeDivision (Backend.cpp:52-70).
void compute_division(uint64_t count, uint32_t sm, uint32_t max_tpb,
                      uint32_t *block, uint32_t *grid);

}  // namespace bw

// Stream-ordered scratch from the context's pool.
inline cudaError_t ctx_malloc_async(bw_context *ctx, void **p, size_t bytes, cudaStream_t s)
{
    return ctx && ctx->pool ? cudaMallocFromPoolAsync(p, bytes, ctx->pool, s) : cudaMallocAsync(p, bytes, s);
}
