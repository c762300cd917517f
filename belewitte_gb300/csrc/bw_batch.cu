// Batched persistent traversal: many graphs, or many BFS sources, in one
// launch.  Each CTA takes units from a device work queue (an atomic cursor
// over a largest-first order) and runs each unit to completion with
// CTA-level barriers between BFS levels and PageRank iterations.
//
// Per unit: BFS with CTA-wide frontier queues in global scratch (private to
// the CTA), warp-cooperative row expansion (32 frontier rows concatenated per
// warp step) and CTA-cooperative expansion of rows above BATCH_HEAVY edges;
// for whole-graph units, then `pr_iterations` PageRank iterations of that
// graph alone, each vertex summing its reverse row in row order with the
// reference's consolidation (pagerank/vertex_pull.cu:23-29,
// pagerank/pagerank.cu:131-136), so ranks are bit-identical to a
// single-graph vertex-pull run.
#include <algorithm>
#include <climits>

#include <cooperative_groups.h>

#include "bw_consolidate.h"
#include "bw_internal.cuh"
#include "bw_seqsum_warp.cuh"

namespace bw {
namespace {
namespace cg = cooperative_groups;

constexpr int BATCH_THREADS = 512;
constexpr int BATCH_WARPS = BATCH_THREADS / 32;
constexpr uint32_t BATCH_HEAVY = 1024;    // rows above this are expanded by the whole CTA
constexpr uint32_t HEAVY_SLOTS = 256;
constexpr uint32_t NO_UNIT = 0xffffffffu;
constexpr float DAMPING = 0.85f;
constexpr uint32_t BATCH_PR_LIGHT = 256;  // PageRank rows above this are summed by a whole warp
constexpr int BATCH_PR_UNROLL = 8;
constexpr int BATCH_BFS_UNROLL = 4;
constexpr uint32_t BATCH_BU_DIV = 24;     // default push/pull divisor: bottom-up above 1/24 of the unit
constexpr uint32_t BATCH_PR_L = 8;        // warp sums: windows of 32 x 8 terms

struct BatchArgs {
    const uint32_t *fwd_v, *fwd_e, *rev_v, *rev_e;
    uint64_t n;
    int mode;
    const uint32_t *goff;
    const uint32_t *roots, *order;
    uint32_t units;
    uint32_t *cursor;
    uint32_t *queues;         // per CTA: 2 * qcap
    float *contrib;           // per CTA: 2 * qcap
    uint32_t qcap;
    int32_t *levels;
    float *ranks;
    uint32_t pr_iters;
    uint32_t vis_words;       // > 0: the unit's visited set is a shared-memory bitmap of this many words
    uint32_t bu_div;          // a level whose frontier holds more than 1/bu_div of the unit runs bottom-up
    unsigned long long *traversed;
};

__device__ __forceinline__ bool relax_local(int32_t *lv, uint32_t v, int32_t nd)
{ return lv[v] > nd && atomicMin(&lv[v], nd) > nd; }

__global__ void __launch_bounds__(BATCH_THREADS, 2) k_batch(BatchArgs a)
{
    __shared__ uint32_t s_unit, s_qlen[2], s_heavy_n;
    __shared__ uint32_t s_heavy[HEAVY_SLOTS];
    __shared__ uint32_t s_excl[BATCH_WARPS][32], s_start[BATCH_WARPS][32];
    __shared__ double s_base;
    __shared__ uint32_t s_long_n, s_job;
    __shared__ float s_stage[BATCH_WARPS][33 * BATCH_PR_L];
    extern __shared__ uint32_t s_vis[];
    __shared__ unsigned long long s_trav;
    const unsigned tid = threadIdx.x, lane = tid & 31, wib = tid >> 5;
    uint32_t *q[2] = {a.queues + static_cast<size_t>(blockIdx.x) * 2 * a.qcap,
                      a.queues + static_cast<size_t>(blockIdx.x) * 2 * a.qcap + a.qcap};
    float *cbuf[2] = {a.contrib + static_cast<size_t>(blockIdx.x) * 2 * a.qcap,
                      a.contrib + static_cast<size_t>(blockIdx.x) * 2 * a.qcap + a.qcap};
    for (;;) {
        if (tid == 0) {
            const uint32_t t = atomicAdd(a.cursor, 1u);
            s_unit = t < a.units ? (a.order ? a.order[t] : t) : NO_UNIT;
            s_trav = 0;
        }
        __syncthreads();
        const uint32_t unit = s_unit;
        if (unit == NO_UNIT) break;
        uint32_t vb, ve;
        int32_t *lv;
        if (a.mode == BW_BATCH_GRAPHS) {
            vb = a.goff[unit];
            ve = a.goff[unit + 1];
            lv = a.levels;
        } else {
            vb = 0;
            ve = static_cast<uint32_t>(a.n);
            lv = a.levels + static_cast<size_t>(unit) * a.n;
        }
        const uint32_t root = a.roots[unit];
        for (uint32_t v = vb + tid; v < ve; v += BATCH_THREADS) lv[v] = v == root ? 0 : INF;
        const bool bitmap = a.vis_words != 0;
        if (bitmap) {
            for (uint32_t w = tid; w < (ve - vb + 31) / 32; w += BATCH_THREADS) s_vis[w] = 0u;
            __syncthreads();
        }
        if (tid == 0) {
            if (bitmap) s_vis[(root - vb) >> 5] = 1u << ((root - vb) & 31);
            q[0][0] = root;
            s_qlen[0] = 1;
            s_qlen[1] = 0;
            s_heavy_n = 0;
        }
        __syncthreads();
        // ------------------------------ BFS ------------------------------
        for (int32_t depth = 0;; depth++) {
            const uint32_t len = s_qlen[depth & 1];
            if (len == 0) break;
            const int32_t nd = depth + 1;
            const uint32_t *qin = q[depth & 1];
            uint32_t *qout = q[(depth + 1) & 1];
            uint32_t *olen = &s_qlen[(depth + 1) & 1];
            // first visit of u: the shared-memory bitmap answers without a
            // global access (and its atomic is a shared one); the depth is
            // then stored once
            auto relax = [&](uint32_t u) -> bool {
                if (!bitmap) return relax_local(lv, u, nd);
                const uint32_t w = (u - vb) >> 5, bit = 1u << ((u - vb) & 31);
                if (s_vis[w] & bit) return false;
                if (atomicOr(&s_vis[w], bit) & bit) return false;
                lv[u] = nd;
                return true;
            };
            auto visit = [&](uint32_t u) {
                if (relax(u)) {
                    cg::coalesced_group g = cg::coalesced_threads();
                    uint32_t base = 0;
                    if (g.thread_rank() == 0) base = atomicAdd(olen, g.size());
                    base = g.shfl(base, 0);
                    qout[base + g.thread_rank()] = u;
                }
            };
            // A frontier above 1/bu_div of the unit's vertices: bottom-up.
            // Every vertex not yet reached looks for an in-neighbour reached
            // before this level, which is then at `depth` (one at a smaller
            // depth would have reached it already); the bitmap answers, and
            // is updated only once the level is done, so that it reads as of
            // the level's start.
            const uint32_t nunit = ve - vb;
            const bool bottom_up = bitmap && a.rev_v && len > nunit / a.bu_div;
            if (bottom_up) {
                const uint32_t words = (nunit + 31) / 32;
                for (uint32_t w = tid; w < words; w += BATCH_THREADS) {
                    uint32_t todo = ~s_vis[w];
                    if (w == words - 1 && (nunit & 31)) todo &= (1u << (nunit & 31)) - 1u;
                    while (todo) {
                        const uint32_t v = vb + w * 32 + (__ffs(todo) - 1);
                        todo &= todo - 1;
                        const uint32_t s = a.rev_v[v], e = a.rev_v[v + 1];
                        bool found = false;
                        for (uint32_t i = s; i < e && !found; i += BATCH_BFS_UNROLL) {
                            uint32_t pu[BATCH_BFS_UNROLL];
#pragma unroll
                            for (int j = 0; j < BATCH_BFS_UNROLL; j++)
                                pu[j] = i + j < e ? __ldg(a.rev_e + i + j) - vb : NO_UNIT;
#pragma unroll
                            for (int j = 0; j < BATCH_BFS_UNROLL; j++)
                                if (pu[j] != NO_UNIT) found |= ((s_vis[pu[j] >> 5] >> (pu[j] & 31)) & 1u) != 0u;
                        }
                        if (found) {
                            lv[v] = nd;
                            cg::coalesced_group g = cg::coalesced_threads();
                            uint32_t base = 0;
                            if (g.thread_rank() == 0) base = atomicAdd(olen, g.size());
                            base = g.shfl(base, 0);
                            qout[base + g.thread_rank()] = v;
                        }
                    }
                }
                __syncthreads();
                for (uint32_t i = tid; i < *olen; i += BATCH_THREADS) {
                    const uint32_t u = qout[i] - vb;
                    atomicOr(&s_vis[u >> 5], 1u << (u & 31));
                }
            }
            for (uint32_t t = wib * 32; !bottom_up && t < len; t += BATCH_THREADS) {
                const uint32_t i = t + lane;
                uint32_t v = 0, s = 0, d = 0;
                if (i < len) {
                    v = qin[i];
                    s = a.fwd_v[v];
                    d = a.fwd_v[v + 1] - s;
                }
                if (d > BATCH_HEAVY) {
                    const uint32_t slot = atomicAdd(&s_heavy_n, 1u);
                    if (slot < HEAVY_SLOTS) { s_heavy[slot] = v; d = 0; }   // else: this warp expands it
                }
                uint32_t incl = d;
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t y = __shfl_up_sync(FULL_MASK, incl, o);
                    if (lane >= static_cast<unsigned>(o)) incl += y;
                }
                const uint32_t total = __shfl_sync(FULL_MASK, incl, 31);
                s_excl[wib][lane] = incl - d;
                s_start[wib][lane] = s;
                __syncwarp();
                // edge k of the 32 concatenated rows: a per-lane cursor over
                // the rows' exclusive offsets (k grows), BATCH_BFS_UNROLL
                // neighbours' indices in flight before their visits
                uint32_t seg = 0;
                for (uint32_t k0 = 0; k0 < total; k0 += 32 * BATCH_BFS_UNROLL) {
                    uint32_t u[BATCH_BFS_UNROLL];
#pragma unroll
                    for (int j = 0; j < BATCH_BFS_UNROLL; j++) {
                        const uint32_t k = k0 + j * 32 + lane;
                        u[j] = NO_UNIT;
                        if (k < total) {
                            while (seg < 31 && s_excl[wib][seg + 1] <= k) seg++;
                            u[j] = __ldg(a.fwd_e + s_start[wib][seg] + (k - s_excl[wib][seg]));
                        }
                    }
#pragma unroll
                    for (int j = 0; j < BATCH_BFS_UNROLL; j++)
                        if (u[j] != NO_UNIT) visit(u[j]);
                }
                __syncwarp();
            }
            __syncthreads();
            const uint32_t heavy = bottom_up ? 0u : min(s_heavy_n, HEAVY_SLOTS);
            for (uint32_t h = 0; h < heavy; h++) {
                const uint32_t v = s_heavy[h];
                const uint32_t s = a.fwd_v[v], e = a.fwd_v[v + 1];
                for (uint32_t i0 = s; i0 < e; i0 += BATCH_THREADS * BATCH_BFS_UNROLL) {
                    uint32_t u[BATCH_BFS_UNROLL];
#pragma unroll
                    for (int j = 0; j < BATCH_BFS_UNROLL; j++) {
                        const uint32_t i = i0 + j * BATCH_THREADS + tid;
                        u[j] = i < e ? __ldg(a.fwd_e + i) : NO_UNIT;
                    }
#pragma unroll
                    for (int j = 0; j < BATCH_BFS_UNROLL; j++)
                        if (u[j] != NO_UNIT) visit(u[j]);
                }
            }
            __syncthreads();
            if (tid == 0) {
                s_qlen[depth & 1] = 0;
                s_heavy_n = 0;
            }
            __syncthreads();
        }
        // traversed edges: out-degrees of reached vertices
        unsigned long long trav = 0;
        for (uint32_t v = vb + tid; v < ve; v += BATCH_THREADS)
            if (lv[v] != INF) trav += a.fwd_v[v + 1] - a.fwd_v[v];
        for (int o = 16; o > 0; o >>= 1) trav += __shfl_xor_sync(FULL_MASK, trav, o);
        if (lane == 0 && trav) atomicAdd(&s_trav, trav);
        // --------------------------- PageRank -----------------------------
        // Every row is summed in row order from +0 (bit-identical to the
        // reference's loop).  Rows of at most BATCH_PR_LIGHT terms: one lane
        // each, BATCH_PR_UNROLL gathers in flight.  Longer rows: one warp
        // each (warp_sequential_continue_load: coalesced gathers staged in
        // shared memory, a serial start by one lane, then binade-map scans),
        // so that a hub's row no longer holds the CTA's iteration.  Warps take
        // jobs -- the long rows, then chunks of 32 vertices -- from a
        // shared-memory counter.
        if (a.mode == BW_BATCH_GRAPHS && a.pr_iters) {
            const uint32_t ng = ve - vb;
            if (tid == 0) {
                s_base = (1.0 - static_cast<double>(DAMPING)) / static_cast<double>(ng);
                s_long_n = 0;
                s_job = 0;
            }
            __syncthreads();
            const double base = s_base;
            const float init = __fdiv_rn(1.0f, static_cast<float>(ng));
            uint32_t *long_rows = q[0];                  // the BFS queues are free now
            for (uint32_t v = vb + tid; v < ve; v += BATCH_THREADS) {
                const uint32_t d = a.fwd_v[v + 1] - a.fwd_v[v];
                a.ranks[v] = init;
                cbuf[0][v - vb] = d ? __fdiv_rn(init, static_cast<float>(d)) : 0.0f;
                if (a.rev_v[v + 1] - a.rev_v[v] > BATCH_PR_LIGHT) long_rows[atomicAdd(&s_long_n, 1u)] = v;
            }
            __syncthreads();
            const uint32_t n_long = s_long_n, jobs = n_long + (ng + 31) / 32;
            auto finish = [&](uint32_t v, float sum, float *cout) {
                const float scaled = __fmul_rn(DAMPING, sum);
                bool ok;
                const uint32_t rb = bwcons::add_round_bits(static_cast<uint64_t>(__double_as_longlong(base)),
                                                           __float_as_uint(scaled), ok);
                const float nr = ok ? __uint_as_float(rb) : __double2float_rn(__dadd_rn(base, static_cast<double>(scaled)));
                a.ranks[v] = nr;
                const uint32_t d = a.fwd_v[v + 1] - a.fwd_v[v];
                cout[v - vb] = d ? __fdiv_rn(nr, static_cast<float>(d)) : 0.0f;
            };
            for (uint32_t it = 1; it <= a.pr_iters; it++) {
                const float *cin = cbuf[(it - 1) & 1];
                float *cout = cbuf[it & 1];
                for (;;) {
                    uint32_t job = 0;
                    if (lane == 0) job = atomicAdd(&s_job, 1u);
                    job = __shfl_sync(FULL_MASK, job, 0);
                    if (job >= jobs) break;
                    if (job < n_long) {
                        const uint32_t v = long_rows[job];
                        const uint32_t s = a.rev_v[v], len = a.rev_v[v + 1] - s;
                        auto load = [&](uint32_t i) { return cin[__ldg(a.rev_e + s + i) - vb]; };
                        uint32_t sb = 0;
                        float sum;
                        if (warp_sequential_continue_load<BATCH_PR_L>(load, 0, len, sb, s_stage[wib], lane)) {
                            sum = __uint_as_float(sb);
                        } else {                         // terms outside the maps' domain: the plain loop
                            sum = 0.0f;
                            if (lane == 0)
                                for (uint32_t i = 0; i < len; i++) sum = __fadd_rn(sum, load(i));
                        }
                        if (lane == 0) finish(v, sum, cout);
                    } else {
                        const uint32_t v = vb + (job - n_long) * 32 + lane;
                        if (v < ve) {
                            const uint32_t s = a.rev_v[v], e = a.rev_v[v + 1];
                            if (e - s <= BATCH_PR_LIGHT) {
                                float sum = 0.0f;
                                for (uint32_t i = s; i < e; i += BATCH_PR_UNROLL) {
                                    float t[BATCH_PR_UNROLL];
#pragma unroll
                                    for (int k = 0; k < BATCH_PR_UNROLL; k++)
                                        t[k] = i + k < e ? cin[__ldg(a.rev_e + i + k) - vb] : 0.0f;
#pragma unroll
                                    for (int k = 0; k < BATCH_PR_UNROLL; k++)
                                        if (i + k < e) sum = __fadd_rn(sum, t[k]);
                                }
                                finish(v, sum, cout);
                            }
                        }
                    }
                }
                __syncthreads();
                if (tid == 0) s_job = 0;
                __syncthreads();
            }
        }
        __syncthreads();
        if (tid == 0 && s_trav) atomicAdd(a.traversed, s_trav);
    }
}

}  // namespace
}  // namespace bw

using namespace bw;

extern "C" int bw_batch_run(bw_context *ctx, const bw_graph_view *g, int mode, const uint32_t *graph_offsets,
                            uint32_t graph_count, const uint32_t *roots, const uint32_t *order, uint32_t unit_count,
                            uint32_t max_unit_vertices, uint32_t pr_iterations, int32_t *levels, float *ranks,
                            const bw_launch_config *cfg, bw_batch_result *result, void *stream)
{
    if (!ctx || !g || !roots || !levels || !g->fwd_vertices || !g->fwd_edges) return BW_ERR_INVALID_ARGUMENT;
    if (mode != BW_BATCH_GRAPHS && mode != BW_BATCH_SOURCES) return BW_ERR_INVALID_ARGUMENT;
    if (mode == BW_BATCH_GRAPHS) {
        if (!graph_offsets || graph_count == 0 || unit_count != graph_count) return BW_ERR_INVALID_ARGUMENT;
        if (pr_iterations && (!ranks || !g->rev_vertices || !g->rev_edges)) return BW_ERR_MISSING_REPRESENTATION;
    } else if (graph_count != 1 || g->vertex_count > max_unit_vertices) {
        return BW_ERR_INVALID_ARGUMENT;
    }
    if (max_unit_vertices == 0 || g->vertex_count > 0xffffffffULL) return BW_ERR_INVALID_ARGUMENT;
    if (unit_count == 0) {
        if (result) *result = bw_batch_result{};
        return BW_OK;
    }
    cudaStream_t s = as_stream(stream);
    // the visited bitmap of the largest unit in shared memory when it fits
    // beside the kernel's static shared memory; CTAs per SM as it allows
    cudaFuncAttributes fa{};
    BW_CUDA(cudaFuncGetAttributes(&fa, k_batch));
    const uint64_t words = (static_cast<uint64_t>(max_unit_vertices) + 31) / 32;
    const bool bitmap = fa.sharedSizeBytes + words * 4 + 1024 <= static_cast<uint64_t>(ctx->max_smem_optin);
    const size_t dyn = bitmap ? words * 4 : 0;
    BW_CUDA(cudaFuncSetAttribute(k_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(dyn)));
    int per_sm = 0;
    BW_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch, BATCH_THREADS, dyn));
    unsigned grid = static_cast<unsigned>(ctx->sm_count) * static_cast<unsigned>(std::max(1, std::min(per_sm, 2)));
    if (cfg && cfg->grid_size) grid = cfg->grid_size;
    if (cfg && cfg->block_size && cfg->block_size != BATCH_THREADS) return BW_ERR_INVALID_ARGUMENT;
    BatchArgs a{};
    a.fwd_v = g->fwd_vertices; a.fwd_e = g->fwd_edges; a.rev_v = g->rev_vertices; a.rev_e = g->rev_edges;
    a.n = g->vertex_count;
    a.mode = mode;
    a.goff = graph_offsets;
    a.roots = roots;
    a.order = order;
    a.units = unit_count;
    a.qcap = max_unit_vertices;
    a.levels = levels;
    a.ranks = ranks;
    a.pr_iters = mode == BW_BATCH_GRAPHS ? pr_iterations : 0;
    a.vis_words = bitmap ? static_cast<uint32_t>(words) : 0u;
    a.bu_div = (cfg && cfg->chunk_size) ? cfg->chunk_size : BATCH_BU_DIV;
    const size_t per_cta = static_cast<size_t>(2) * max_unit_vertices;
    char *scratch = nullptr;
    const size_t bytes = 64 + grid * per_cta * sizeof(uint32_t) + (a.pr_iters ? grid * per_cta * sizeof(float) : 0);
    BW_CUDA(ctx_malloc_async(ctx, reinterpret_cast<void **>(&scratch), bytes, s));
    BW_CUDA(cudaMemsetAsync(scratch, 0, 64, s));
    a.cursor = reinterpret_cast<uint32_t *>(scratch);
    a.traversed = reinterpret_cast<unsigned long long *>(scratch + 8);
    a.queues = reinterpret_cast<uint32_t *>(scratch + 64);
    a.contrib = a.pr_iters ? reinterpret_cast<float *>(scratch + 64 + grid * per_cta * sizeof(uint32_t)) : nullptr;
    BW_CUDA(cudaEventRecord(ctx->ev_start, s));
    k_batch<<<grid, BATCH_THREADS, dyn, s>>>(a);
    BW_CUDA(cudaGetLastError());
    BW_CUDA(cudaEventRecord(ctx->ev_stop, s));
    unsigned long long trav = 0;
    BW_CUDA(cudaMemcpyAsync(&trav, a.traversed, sizeof trav, cudaMemcpyDeviceToHost, s));
    BW_CUDA(cudaFreeAsync(scratch, s));
    BW_CUDA(cudaStreamSynchronize(s));
    if (result) {
        float ms = 0.0f;
        BW_CUDA(cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop));
        result->units = unit_count;
        result->traversed_edges = trav;
        result->device_ms = ms;
    }
    return BW_OK;
}
