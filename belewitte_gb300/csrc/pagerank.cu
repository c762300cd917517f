// PageRank kernels and the PageRank half of the C ABI.
//
// Reference: pagerank/pagerank.cu (degrees, consolidateRank,
// consolidateRankNoDiv), pagerank/{edgelist,rev_edgelist,struct_edgelist,
// rev_struct_edgelist,vertex_push,vertex_pull,vertex_pull_nodiv,
// vertex_push_warp,vertex_pull_warp,vertex_pull_warp_nodiv}.cu and the
// host loop PageRank::runImplementation (pagerank/pagerank.cpp:74-171).
//
// Arithmetic kept bit-for-bit:
//   contribution of u      pr[u] / (float) deg[u]   (IEEE division)
//   consolidateRank        (float)((1.0 - 0.85f) / N + (double)(0.85f * acc))
//   consolidateRankNoDiv   fmaf(0.85f, acc, (1 - 0.85f) / (float) N), then
//                          / (float) deg when deg != 0 and not the last
//                          iteration
// The division is precomputed once per vertex per iteration (contrib[]),
// which gives the same float as dividing per edge.  Accumulation order:
// vertex-pull and vertex-pull-nodiv sum each reverse row sequentially, as
// the reference does (bit-exact); the atomic variants and the warp /
// segmented reductions sum in another order (the reference's own float
// atomics make its order arbitrary too).
#include <algorithm>
#include <cstring>
#include <cooperative_groups.h>

#include "bw_consolidate.h"
#include "bw_internal.cuh"

namespace bw {
namespace {

constexpr float DAMPING = 0.85f;

enum PrVariant {
    PR_EDGE_LIST = 0, PR_REV_EDGE_LIST, PR_STRUCT_EDGE_LIST, PR_REV_STRUCT_EDGE_LIST,
    PR_VERTEX_PUSH, PR_VERTEX_PULL, PR_VERTEX_PUSH_WARP, PR_VERTEX_PULL_WARP,
    PR_VERTEX_PULL_NODIV, PR_VERTEX_PULL_WARP_NODIV, PR_PULL_SEGMENTED, PR_VARIANT_COUNT
};

const char *const kPrNames[PR_VARIANT_COUNT] = {
    "edge-list", "rev-edge-list", "struct-edge-list", "rev-struct-edge-list",
    "vertex-push", "vertex-pull", "vertex-push-warp", "vertex-pull-warp",
    "vertex-pull-nodiv", "vertex-pull-warp-nodiv", "pull-segmented"};

// Representation bits (bw_pagerank_variant_reps).
constexpr int REP_FWD_CSR = 1, REP_REV_CSR = 2, REP_FWD_EL = 4, REP_REV_EL = 8,
              REP_FWD_ST = 16, REP_REV_ST = 32;
const int kPrReps[PR_VARIANT_COUNT] = {
    REP_FWD_EL, REP_REV_EL, REP_FWD_ST, REP_REV_ST, REP_FWD_CSR, REP_REV_CSR,
    REP_FWD_CSR, REP_REV_CSR, REP_REV_CSR, REP_REV_CSR, REP_REV_CSR};

inline bool is_nodiv(int v) { return v == PR_VERTEX_PULL_NODIV || v == PR_VERTEX_PULL_WARP_NODIV; }
inline bool is_fused(int v)
{
    return v == PR_VERTEX_PULL || v == PR_VERTEX_PULL_WARP || v == PR_VERTEX_PULL_NODIV ||
           v == PR_VERTEX_PULL_WARP_NODIV || v == PR_PULL_SEGMENTED;
}
inline bool uses_rowlen(int v) { return v == PR_VERTEX_PUSH || v == PR_VERTEX_PUSH_WARP; }

struct PrArgs {
    const uint32_t *fwd_v, *fwd_e, *rev_v, *rev_e, *fwd_in, *rev_in;
    const uint2 *fwd_s, *rev_s;
    uint64_t n, m;
    const uint32_t *deg;
    const float *pr_in;        // previous ranks (nodiv: previous, pre-divided)
    const float *contrib_in;   // pr/deg of the previous iteration (div)
    float *acc;                // accumulator of the atomic variants
    float *pr_out;
    float *contrib_out;
    float *diff;               // this iteration's diff slot
    int not_last;
    uint32_t warp_size, chunk_size;
    const uint4 *work;         // pull-segmented work items
    uint32_t work_count;
    uint32_t *long_count;      // arrival counters of split rows
    double base_div;           // (1.0 - 0.85f) / N, computed once on the host
};

__device__ __forceinline__ uint64_t gtid() { return blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; }
__device__ __forceinline__ uint64_t gthreads() { return uint64_t(gridDim.x) * blockDim.x; }

// pagerank/pagerank.cu:132: new_rank = (float)(((1.0 - d) / N) + (double)(d * acc))
// -- a double base term (computed once: IEEE division is correctly rounded,
// so the host value is the one the reference computes per vertex), a float
// product, one double addition and the rounding to float.
// The double addition and the rounding to float are done in integer
// arithmetic (bw_consolidate.h): bit-identical to the FP64 instructions,
// which GB300 issues at a small fraction of the FP32 rate.
__device__ __forceinline__ float consolidate_div(float acc, double base)
{
    const float scaled = __fmul_rn(DAMPING, acc);
    bool ok;
    const uint32_t r = bwcons::add_round_bits(static_cast<uint64_t>(__double_as_longlong(base)),
                                              __float_as_uint(scaled), ok);
    if (ok) return __uint_as_float(r);
    return __double2float_rn(__dadd_rn(base, static_cast<double>(scaled)));   // outside the emulated domain
}

__device__ __forceinline__ float nodiv_base(uint64_t n)
{ return __fdiv_rn(__fsub_rn(1.0f, DAMPING), static_cast<float>(n)); }

__device__ __forceinline__ void add_diff(float *slot, float d)
{
    for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(FULL_MASK, d, o);
    if ((threadIdx.x & 31) == 0 && d != 0.0f) atomicAdd(slot, d);
}

// ----------------------------- degrees ------------------------------------
// Histogram of a source-id stream with warp aggregation of equal ids
// (one atomic per distinct id per warp step).  Counting inEdges of the
// forward edge list, outEdges of the reverse one, or every reverse-CSR
// entry all give out-degrees (pagerank/pagerank.cu:40-123).
__global__ void __launch_bounds__(256) k_count_ids(const uint32_t *__restrict__ ids,
                                                   uint64_t count, uint32_t stride_words,
                                                   uint32_t *__restrict__ deg)
{
    const unsigned lane = threadIdx.x & 31;
    const uint64_t warp = gtid() >> 5, warps = gthreads() >> 5;
    for (uint64_t base = warp * 32; base < count; base += warps * 32) {
        const uint64_t i = base + lane;
        const uint32_t id = i < count ? ids[i * stride_words] : 0xffffffffu;
        const unsigned peers = __match_any_sync(FULL_MASK, id);
        if (id != 0xffffffffu && (__ffs(peers) - 1) == static_cast<int>(lane))
            atomicAdd(&deg[id], static_cast<uint32_t>(__popc(peers)));
    }
}

// Initial ranks 1/N (pagerank/pagerank.cpp:88) and contributions.
__global__ void k_pr_init(PrArgs a, float *pr, float *contrib, int rowlen)
{
    const float init = __fdiv_rn(1.0f, static_cast<float>(a.n));
    for (uint64_t v = gtid(); v < a.n; v += gthreads()) {
        pr[v] = init;
        if (a.acc) a.acc[v] = 0.0f;
        if (contrib) {
            const uint32_t d = rowlen ? a.fwd_v[v + 1] - a.fwd_v[v] : a.deg[v];
            contrib[v] = d ? __fdiv_rn(init, static_cast<float>(d)) : 0.0f;
        }
    }
}

// consolidateRank (div) for the atomic variants; also produces the next
// contributions and clears the accumulator (pagerank/pagerank.cu:125-140).
__global__ void __launch_bounds__(256) k_consolidate_div(PrArgs a, int rowlen)
{
    float dsum = 0.0f;
    const uint64_t n = a.n;
    for (uint64_t base = (gtid() >> 5) * 32; base < n; base += (gthreads() >> 5) * 32) {
        const uint64_t v = base + (threadIdx.x & 31);
        if (v < n) {
            const float nr = consolidate_div(a.acc[v], a.base_div);
            dsum += fabsf(nr - a.pr_out[v]);
            a.pr_out[v] = nr;
            a.acc[v] = 0.0f;
            const uint32_t d = rowlen ? a.fwd_v[v + 1] - a.fwd_v[v] : a.deg[v];
            a.contrib_out[v] = d ? __fdiv_rn(nr, static_cast<float>(d)) : 0.0f;
        }
    }
    add_diff(a.diff, dsum);
}

// ----------------------- edge-list families -------------------------------
// acc[dst] += contrib[src] per edge (pagerank/edgelist.cu:14-22 and the
// rev/struct forms).  Forward layouts (source-sorted) scatter with one
// float atomic per edge.  The reverse SoA layout is destination-sorted:
// each warp step reduces runs of equal destinations with a segmented
// shuffle scan and issues one atomic per run.
template<int LAYOUT>  // 0 fwd SoA, 1 rev SoA, 2 fwd AoS, 3 rev AoS
__global__ void __launch_bounds__(256) k_pr_edge(PrArgs a)
{
    const unsigned lane = threadIdx.x & 31;
    const uint64_t warp = gtid() >> 5, warps = gthreads() >> 5;
    const uint64_t m = a.m;
    for (uint64_t base = warp * 32; base < m; base += warps * 32) {
        const uint64_t e = base + lane;
        uint32_t src = 0, dst = 0xffffffffu;
        if (e < m) {
            if constexpr (LAYOUT == 0) { src = __ldcs(a.fwd_in + e); dst = __ldcs(a.fwd_e + e); }
            else if constexpr (LAYOUT == 1) { dst = __ldcs(a.rev_in + e); src = __ldcs(a.rev_e + e); }
            else if constexpr (LAYOUT == 2) { const uint2 p = __ldcs(a.fwd_s + e); src = p.x; dst = p.y; }
            else { const uint2 p = __ldcs(a.rev_s + e); dst = p.x; src = p.y; }
        }
        float val = e < m ? __ldg(a.contrib_in + src) : 0.0f;
        if constexpr (LAYOUT == 1 || LAYOUT == 3) {
            // segmented suffix sums over runs of equal dst (sorted)
            for (int o = 1; o < 32; o <<= 1) {
                const float y = __shfl_down_sync(FULL_MASK, val, o);
                const uint32_t k = __shfl_down_sync(FULL_MASK, dst, o);
                if (lane + o < 32 && k == dst) val += y;
            }
            const uint32_t prev = __shfl_up_sync(FULL_MASK, dst, 1);
            const bool head = lane == 0 || prev != dst;
            if (e < m && head) atomicAdd(&a.acc[dst], val);
        } else {
            if (e < m) atomicAdd(&a.acc[dst], val);
        }
    }
}

// ----------------------------- vertex-push --------------------------------
// Thread per vertex; each owner scatters pr[v] / rowlen to its out-row
// (pagerank/vertex_push.cu:3-31).
__global__ void __launch_bounds__(256) k_pr_vertex_push(PrArgs a)
{
    for (uint64_t v = gtid(); v < a.n; v += gthreads()) {
        const uint32_t s = a.fwd_v[v], e = a.fwd_v[v + 1];
        if (s == e) continue;
        const float out = a.contrib_in[v];
        for (uint32_t i = s; i < e; i++) atomicAdd(&a.acc[__ldg(a.fwd_e + i)], out);
    }
}

// vertex-push-warp (pagerank/vertex_push_warp.cu:4-49): virtual warp of W
// lanes per chunk of C vertices, ranks and offsets staged in shared memory.
__global__ void __launch_bounds__(512) k_pr_vertex_push_warp(PrArgs a)
{
    extern __shared__ uint32_t smem[];
    const uint32_t W = a.warp_size, C = a.chunk_size;
    const uint32_t per_block = blockDim.x / W, vw = threadIdx.x / W, lane = threadIdx.x % W;
    const unsigned mask = W >= 32 ? FULL_MASK : (((1u << W) - 1u) << ((threadIdx.x & 31) & ~(W - 1u)));
    float *my_c = reinterpret_cast<float *>(smem) + vw * C;
    uint32_t *my_off = smem + per_block * C + vw * (C + 1);
    const uint64_t n = a.n, total = uint64_t(gridDim.x) * per_block;
    for (uint64_t chunk = blockIdx.x * uint64_t(per_block) + vw; chunk * C < n; chunk += total) {
        const uint64_t v0 = chunk * C;
        const uint32_t cnt = static_cast<uint32_t>(min(uint64_t(C), n - v0));
        for (uint32_t i = lane; i < cnt; i += W) my_c[i] = a.contrib_in[v0 + i];
        for (uint32_t i = lane; i < cnt + 1; i += W) my_off[i] = a.fwd_v[v0 + i];
        __syncwarp(mask);
        for (uint32_t v = 0; v < cnt; v++) {
            const float out = my_c[v];
            for (uint32_t i = my_off[v] + lane; i < my_off[v + 1]; i += W)
                atomicAdd(&a.acc[__ldg(a.fwd_e + i)], out);
        }
        __syncwarp(mask);
    }
}

// ----------------------------- pull variants ------------------------------
// vertex-pull-warp / -nodiv (pagerank/vertex_pull_warp.cu:4-49,
// vertex_pull_warp_nodiv.cu:4-47): a virtual warp of W lanes per vertex
// of a C-vertex chunk; lane-strided partial sums are combined with a
// shuffle tree (the reference adds each lane's partial with a float
// atomic) and the vertex is consolidated in place.
template<bool NODIV>
__global__ void __launch_bounds__(512) k_pr_vertex_pull_warp(PrArgs a)
{
    extern __shared__ uint32_t smem[];
    const uint32_t W = a.warp_size, C = a.chunk_size;
    const uint32_t per_block = blockDim.x / W, vw = threadIdx.x / W, lane = threadIdx.x % W;
    const unsigned mask = W >= 32 ? FULL_MASK : (((1u << W) - 1u) << ((threadIdx.x & 31) & ~(W - 1u)));
    uint32_t *my_off = smem + vw * (C + 1);
    const uint64_t n = a.n, total = uint64_t(gridDim.x) * per_block;
    const float *src = NODIV ? a.pr_in : a.contrib_in;
    const float base_nd = nodiv_base(n);
    float dsum = 0.0f;
    for (uint64_t chunk = blockIdx.x * uint64_t(per_block) + vw; chunk * C < n; chunk += total) {
        const uint64_t v0 = chunk * C;
        const uint32_t cnt = static_cast<uint32_t>(min(uint64_t(C), n - v0));
        for (uint32_t i = lane; i < cnt + 1; i += W) my_off[i] = a.rev_v[v0 + i];
        __syncwarp(mask);
        for (uint32_t v = 0; v < cnt; v++) {
            float part = 0.0f;
            for (uint32_t i = my_off[v] + lane; i < my_off[v + 1]; i += W)
                part += __ldg(src + __ldg(a.rev_e + i));
            for (uint32_t o = W >> 1; o > 0; o >>= 1) part += __shfl_xor_sync(mask, part, o, W);
            if (lane == 0) {
                const uint64_t x = v0 + v;
                if constexpr (!NODIV) {
                    const float nr = consolidate_div(part, a.base_div);
                    dsum += fabsf(nr - a.pr_out[x]);
                    a.pr_out[x] = nr;
                    const uint32_t d = a.deg[x];
                    a.contrib_out[x] = d ? __fdiv_rn(nr, static_cast<float>(d)) : 0.0f;
                } else {
                    float nr = __fmaf_rn(DAMPING, part, base_nd);
                    dsum += fabsf(nr - a.pr_in[x]);
                    const uint32_t d = a.deg[x];
                    if (d != 0 && a.not_last) nr = __fdiv_rn(nr, static_cast<float>(d));
                    a.pr_out[x] = nr;
                }
            }
        }
        __syncwarp(mask);
    }
    add_diff(a.diff, dsum);
}

// ------------------------- work-list pull kernels ---------------------------
// vertex-pull, vertex-pull-nodiv and pull-segmented share one kernel over a
// work list cut once per run from the reverse CSR: an item is either at
// most 32 consecutive rows with at most SEG_EDGES edges (rows of at most
// SEG_LONG edges), or one long row.  Item: {row_begin, row_end | flags,
// edge_begin, edge_end}.
//
// Short rows: the warp loads the item's indices with unrolled coalesced
// loads, gathers all contributions at once (up to 1024 independent loads
// in flight per warp) into shared memory, and then each lane adds its own
// row's values one after the other in row order -- the reference's
// sequential summation (pagerank/vertex_pull.cu:23-27), so these rows are
// bit-identical to it.
// Long rows, EXACT (vertex-pull, vertex-pull-nodiv): one warp streams the
// row in 1024-edge chunks (parallel gathers into shared memory) and lane 0
// keeps the single sequential sum -- bit-identical, bounded by the add
// chain of the longest row.
// Long rows, split (pull-segmented): 1024-edge pieces summed by any warp
// (lane partials + shuffle tree), combined in acc[] by float atomics; the
// last piece to arrive (arrival counter) consolidates the row.
constexpr uint32_t SEG_EDGES = 512;
constexpr uint32_t SEG_LONG = 256;
constexpr uint32_t PIECE_FLAG = 0x80000000u;   // split piece of a long row
constexpr uint32_t LONG_FLAG = 0x40000000u;    // whole long row
constexpr uint32_t ROW_MASK = 0x3fffffffu;
constexpr int PULL_WARPS = 8;                  // warps per block
constexpr int GATHER_UNROLL = 16;   // 512 edges = one unrolled round

__global__ void k_seg_count(const uint32_t *__restrict__ off, uint64_t n, int split, uint32_t *__restrict__ counts)
{
    // one thread per 32-row window: number of work items it will emit
    const uint64_t windows = (n + 31) / 32;
    for (uint64_t w = gtid(); w < windows; w += gthreads()) {
        const uint64_t r0 = w * 32, r1 = min(n, r0 + 32);
        uint32_t items = 0, acc_edges = 0, acc_rows = 0;
        for (uint64_t r = r0; r < r1; r++) {
            const uint32_t d = off[r + 1] - off[r];
            if (d > SEG_LONG) {
                if (acc_rows) { items++; acc_rows = 0; acc_edges = 0; }
                items += split ? (d + SEG_EDGES - 1) / SEG_EDGES : 1;
                continue;
            }
            if (acc_rows && acc_edges + d > SEG_EDGES) { items++; acc_rows = 0; acc_edges = 0; }
            acc_rows++; acc_edges += d;
        }
        if (acc_rows) items++;
        counts[w] = items;
    }
}

__global__ void k_seg_emit(const uint32_t *__restrict__ off, uint64_t n, int split,
                           const uint32_t *__restrict__ first, uint4 *__restrict__ work,
                           uint32_t *__restrict__ long_count)
{
    const uint64_t windows = (n + 31) / 32;
    for (uint64_t w = gtid(); w < windows; w += gthreads()) {
        const uint64_t r0 = w * 32, r1 = min(n, r0 + 32);
        uint32_t out = first[w];
        uint64_t start_row = r0;
        uint32_t acc_edges = 0, acc_rows = 0;
        for (uint64_t r = r0; r < r1; r++) {
            const uint32_t d = off[r + 1] - off[r];
            if (d > SEG_LONG) {
                if (acc_rows) {
                    work[out++] = make_uint4(uint32_t(start_row), uint32_t(r), off[start_row], off[r]);
                    acc_rows = 0; acc_edges = 0;
                }
                if (split) {
                    for (uint32_t p = off[r]; p < off[r + 1]; p += SEG_EDGES)
                        work[out++] = make_uint4(uint32_t(r), uint32_t(r + 1) | PIECE_FLAG, p,
                                                 min(p + SEG_EDGES, off[r + 1]));
                    long_count[r] = 0;
                } else {
                    work[out++] = make_uint4(uint32_t(r), uint32_t(r + 1) | LONG_FLAG, off[r], off[r + 1]);
                }
                continue;
            }
            if (acc_rows && acc_edges + d > SEG_EDGES) {
                work[out++] = make_uint4(uint32_t(start_row), uint32_t(r), off[start_row], off[r]);
                acc_rows = 0; acc_edges = 0;
            }
            if (acc_rows == 0) start_row = r;
            acc_rows++; acc_edges += d;
        }
        if (acc_rows) work[out++] = make_uint4(uint32_t(start_row), uint32_t(r1), off[start_row], off[r1]);
    }
}

// Consolidate vertex v from its in-sum (div: consolidateRank plus the next
// contribution; nodiv: consolidateRankNoDiv).  Returns |pr_new - pr_old|.
template<bool NODIV>
__device__ __forceinline__ float finish_vertex(const PrArgs &a, uint64_t v, float sum, float base_nd)
{
    if constexpr (!NODIV) {
        const float nr = consolidate_div(sum, a.base_div);
        const float d = fabsf(nr - a.pr_out[v]);
        a.pr_out[v] = nr;
        const uint32_t dg = a.deg[v];
        a.contrib_out[v] = dg ? __fdiv_rn(nr, static_cast<float>(dg)) : 0.0f;
        return d;
    } else {
        float nr = __fmaf_rn(DAMPING, sum, base_nd);
        const float d = fabsf(nr - a.pr_in[v]);
        const uint32_t dg = a.deg[v];
        if (dg != 0 && a.not_last) nr = __fdiv_rn(nr, static_cast<float>(dg));
        a.pr_out[v] = nr;
        return d;
    }
}

// Gather src[rev_e[e0 + k]] for k in [0, len) (len <= SEG_EDGES) into buf.
__device__ __forceinline__ void gather_into(const uint32_t *__restrict__ rev_e, const float *__restrict__ src,
                                            uint32_t e0, uint32_t len, float *buf, unsigned lane)
{
    for (uint32_t base = 0; base < len; base += 32 * GATHER_UNROLL) {
        uint32_t idx[GATHER_UNROLL];
#pragma unroll
        for (int u = 0; u < GATHER_UNROLL; u++) {
            const uint32_t k = base + u * 32 + lane;
            idx[u] = k < len ? __ldcs(rev_e + e0 + k) : 0u;
        }
        float v[GATHER_UNROLL];
#pragma unroll
        for (int u = 0; u < GATHER_UNROLL; u++) {
            const uint32_t k = base + u * 32 + lane;
            v[u] = k < len ? __ldg(src + idx[u]) : 0.0f;
        }
#pragma unroll
        for (int u = 0; u < GATHER_UNROLL; u++) {
            const uint32_t k = base + u * 32 + lane;
            if (k < len) buf[k] = v[u];
        }
    }
}

template<bool NODIV, bool EXACT_LONG>
__global__ void __launch_bounds__(PULL_WARPS * 32, 5) k_pr_pull_items(PrArgs a)
{
    __shared__ __align__(16) float s_val[PULL_WARPS][SEG_EDGES];
    __shared__ uint32_t s_end[PULL_WARPS][33];
    const unsigned lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint64_t warp = gtid() >> 5, warps = gthreads() >> 5;
    const float *src = NODIV ? a.pr_in : a.contrib_in;
    const float base_nd = nodiv_base(a.n);
    float *buf = s_val[wib];
    float dsum = 0.0f;
    for (uint64_t it = warp; it < a.work_count; it += warps) {
        const uint4 w = a.work[it];
        const uint32_t r0 = w.x, r1 = w.y & ROW_MASK, e0 = w.z, e1 = w.w;
        if (w.y & PIECE_FLAG) {
            float part = 0.0f;
            for (uint32_t base = e0; base < e1; base += 32 * GATHER_UNROLL) {
                uint32_t idx[GATHER_UNROLL];
#pragma unroll
                for (int u = 0; u < GATHER_UNROLL; u++) {
                    const uint32_t i = base + u * 32 + lane;
                    idx[u] = i < e1 ? __ldcs(a.rev_e + i) : 0u;
                }
#pragma unroll
                for (int u = 0; u < GATHER_UNROLL; u++) {
                    const uint32_t i = base + u * 32 + lane;
                    part += i < e1 ? __ldg(src + idx[u]) : 0.0f;
                }
            }
            for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(FULL_MASK, part, o);
            if (lane == 0) {
                atomicAdd(&a.acc[r0], part);
                __threadfence();
                const uint32_t pieces = (a.rev_v[r0 + 1] - a.rev_v[r0] + SEG_EDGES - 1) / SEG_EDGES;
                if (atomicAdd(&a.long_count[r0], 1u) + 1 == pieces) {
                    __threadfence();
                    const float total = atomicExch(&a.acc[r0], 0.0f);
                    a.long_count[r0] = 0;
                    dsum += finish_vertex<NODIV>(a, r0, total, base_nd);
                }
            }
            continue;
        }
        if (w.y & LONG_FLAG) {
            // Lane 0 keeps the sequential sum of chunk c while lanes 1..31
            // gather chunk c + 1 into the other half of the warp's buffer.
            float *half[2] = {buf, buf + SEG_EDGES / 2};
            constexpr uint32_t CH = SEG_EDGES / 2;
            const uint32_t nch = (e1 - e0 + CH - 1) / CH;
            auto gather31 = [&](uint32_t c, float *dst) {
                const uint32_t b0 = e0 + c * CH, cnt = min(CH, e1 - b0);
                if (lane == 0) return;
                constexpr int U = (CH + 30) / 31;
                uint32_t idx[U];
#pragma unroll
                for (int u = 0; u < U; u++) {
                    const uint32_t k = (lane - 1) + 31 * u;
                    idx[u] = k < cnt ? __ldcs(a.rev_e + b0 + k) : 0u;
                }
#pragma unroll
                for (int u = 0; u < U; u++) {
                    const uint32_t k = (lane - 1) + 31 * u;
                    if (k < cnt) dst[k] = __ldg(src + idx[u]);
                }
            };
            gather31(0, half[0]);
            __syncwarp();
            float sum = 0.0f;
            for (uint32_t c = 0; c < nch; c++) {
                if (c + 1 < nch) gather31(c + 1, half[(c + 1) & 1]);
                if (lane == 0) {
                    const float *q = half[c & 1];
                    const uint32_t cnt = min(CH, e1 - (e0 + c * CH));
                    uint32_t i = 0;
                    for (; i + 4 <= cnt; i += 4) {
                        const float4 v = *reinterpret_cast<const float4 *>(q + i);
                        sum = __fadd_rn(sum, v.x); sum = __fadd_rn(sum, v.y);
                        sum = __fadd_rn(sum, v.z); sum = __fadd_rn(sum, v.w);
                    }
                    for (; i < cnt; i++) sum = __fadd_rn(sum, q[i]);
                }
                __syncwarp();
            }
            if (lane == 0) dsum += finish_vertex<NODIV>(a, r0, sum, base_nd);
            continue;
        }
        // up to 32 short rows
        const uint32_t rows = r1 - r0, len = e1 - e0;
        if (lane < rows) s_end[wib][lane] = a.rev_v[r0 + lane + 1] - e0;
        gather_into(a.rev_e, src, e0, len, buf, lane);
        __syncwarp();
        if (lane < rows) {
            const uint32_t b = lane ? s_end[wib][lane - 1] : 0u, e = s_end[wib][lane];
            float sum = 0.0f;
            for (uint32_t i = b; i < e; i++) sum = __fadd_rn(sum, buf[i]);
            dsum += finish_vertex<NODIV>(a, r0 + lane, sum, base_nd);
        }
        __syncwarp();
    }
    (void) EXACT_LONG;
    add_diff(a.diff, dsum);
}

__global__ void k_exclusive_scan_small(uint32_t *data, uint64_t count, uint32_t *total)
{
    // single block scan used for the work-item layout (count = N/32)
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (uint64_t base = 0; base < count; base += blockDim.x) {
        const uint64_t i = base + threadIdx.x;
        uint32_t x = i < count ? data[i] : 0;
        // block inclusive scan via warp scans
        __shared__ uint32_t warp_tot[32];
        const unsigned lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        uint32_t incl = x;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL_MASK, incl, o);
            if (lane >= static_cast<unsigned>(o)) incl += y;
        }
        if (lane == 31) warp_tot[wid] = incl;
        __syncthreads();
        if (wid == 0) {
            uint32_t t = lane < (blockDim.x >> 5) ? warp_tot[lane] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(FULL_MASK, t, o);
                if (lane >= static_cast<unsigned>(o)) t += y;
            }
            warp_tot[lane] = t;
        }
        __syncthreads();
        const uint32_t before = (wid ? warp_tot[wid - 1] : 0) + carry;
        if (i < count) data[i] = before + incl - x;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = before + incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

}  // namespace
}  // namespace bw

using namespace bw;

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
namespace {

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

// Per-run state of one PageRank execution.
struct PrRun {
    PrArgs a{};
    uint4 *work = nullptr;
    uint32_t work_count = 0;
    uint32_t *long_count = nullptr;
    uint32_t *win_counts = nullptr;
};

struct Geometry { unsigned block, grid; size_t smem; };

Geometry geometry(const bw_context *ctx, int variant, const bw_launch_config *cfg)
{
    Geometry g{256, static_cast<unsigned>(ctx->sm_count) * 8, 0};
    if (variant == PR_VERTEX_PULL || variant == PR_VERTEX_PULL_NODIV || variant == PR_PULL_SEGMENTED)
        g.grid = static_cast<unsigned>(ctx->sm_count) * 5;   // one resident wave (register bound)
    const uint32_t W = (cfg && cfg->warp_size) ? cfg->warp_size : 32;
    const uint32_t C = (cfg && cfg->chunk_size) ? cfg->chunk_size : 32;
    if (cfg && cfg->block_size) g.block = cfg->block_size;
    if (cfg && cfg->grid_size) g.grid = cfg->grid_size;
    if (variant == PR_VERTEX_PUSH_WARP) g.smem = (g.block / W) * (C * 4 + (C + 1) * 4);
    if (variant == PR_VERTEX_PULL_WARP || variant == PR_VERTEX_PULL_WARP_NODIV)
        g.smem = (g.block / W) * ((C + 1) * 4);
    return g;
}

int validate_cfg(const bw_context *ctx, int variant, const bw_launch_config *cfg)
{
    if (!cfg) return BW_OK;
    if (cfg->block_size && (cfg->block_size % 32 || cfg->block_size > 256)) {
        // every PageRank kernel is built for at most 256 threads, the warp
        // variants for 512
        const bool warp = variant == PR_VERTEX_PUSH_WARP || variant == PR_VERTEX_PULL_WARP ||
                          variant == PR_VERTEX_PULL_WARP_NODIV;
        if (cfg->block_size % 32 || cfg->block_size > (warp ? 512u : 256u)) return BW_ERR_INVALID_ARGUMENT;
    }
    if ((variant == PR_PULL_SEGMENTED || variant == PR_VERTEX_PULL || variant == PR_VERTEX_PULL_NODIV) &&
        cfg->block_size && cfg->block_size != PULL_WARPS * 32)
        return BW_ERR_INVALID_ARGUMENT;
    const uint32_t W = cfg->warp_size ? cfg->warp_size : 32;
    const uint32_t C = cfg->chunk_size ? cfg->chunk_size : 32;
    // ImplementationTemplate.hpp:463-471: power-of-two W <= 32, C % W == 0.
    if (W == 0 || W > 32 || (W & (W - 1)) || C % W) return BW_ERR_INVALID_ARGUMENT;
    Geometry g = geometry(ctx, variant, cfg);
    if (g.smem > ctx->max_smem_per_block) return BW_ERR_INVALID_ARGUMENT;
    return BW_OK;
}

int launch_degrees(bw_context *ctx, const bw_graph_view *g, int variant, uint32_t *deg, cudaStream_t s)
{
    if (uses_rowlen(variant)) return BW_OK;   // push variants use the row length
    BW_CUDA(cudaMemsetAsync(deg, 0, g->vertex_count * sizeof(uint32_t), s));  // zeroInitDegreesKernel
    if (g->edge_count == 0) return BW_OK;
    const unsigned grid = ctx->sm_count * 8;
    switch (variant) {
      case PR_EDGE_LIST:           // edgeListComputeDegrees: inEdges
        k_count_ids<<<grid, 256, 0, s>>>(g->fwd_in_edges, g->edge_count, 1, deg); break;
      case PR_REV_EDGE_LIST:       // reverseEdgeListComputeDegrees: outEdges
        k_count_ids<<<grid, 256, 0, s>>>(g->rev_edges, g->edge_count, 1, deg); break;
      case PR_STRUCT_EDGE_LIST:    // structEdgeListComputeDegrees: edges[].in
        k_count_ids<<<grid, 256, 0, s>>>(g->fwd_struct_edges, g->edge_count, 2, deg); break;
      case PR_REV_STRUCT_EDGE_LIST:// reverseStructEdgeListComputeDegrees: edges[].out
        k_count_ids<<<grid, 256, 0, s>>>(g->rev_struct_edges + 1, g->edge_count, 2, deg); break;
      default:                     // reverseCSRComputeDegrees
        k_count_ids<<<grid, 256, 0, s>>>(g->rev_edges, g->edge_count, 1, deg); break;
    }
    BW_CUDA(cudaGetLastError());
    return BW_OK;
}

int build_segments(bw_context *ctx, const bw_graph_view *g, int split, PrRun &run, cudaStream_t s)
{
    const uint64_t n = g->vertex_count;
    const uint64_t windows = (n + 31) / 32;
    // Row groups <= N; pieces <= M / SEG_EDGES + (rows longer than
    // SEG_LONG) <= M / SEG_EDGES + M / SEG_LONG.
    const uint64_t cap = windows + n + g->edge_count / SEG_EDGES + g->edge_count / SEG_LONG + 16;
    BW_CUDA(cudaMallocAsync(reinterpret_cast<void **>(&run.win_counts), (windows + 1) * sizeof(uint32_t), s));
    BW_CUDA(cudaMallocAsync(reinterpret_cast<void **>(&run.work), cap * sizeof(uint4), s));
    BW_CUDA(cudaMallocAsync(reinterpret_cast<void **>(&run.long_count), n * sizeof(uint32_t), s));
    k_seg_count<<<ctx->sm_count * 4, 256, 0, s>>>(g->rev_vertices, n, split, run.win_counts);
    k_exclusive_scan_small<<<1, 1024, 0, s>>>(run.win_counts, windows, run.win_counts + windows);
    k_seg_emit<<<ctx->sm_count * 4, 256, 0, s>>>(g->rev_vertices, n, split, run.win_counts, run.work, run.long_count);
    BW_CUDA(cudaGetLastError());
    uint32_t count = 0;
    BW_CUDA(cudaMemcpyAsync(&count, run.win_counts + windows, sizeof count, cudaMemcpyDeviceToHost, s));
    BW_CUDA(cudaStreamSynchronize(s));
    run.work_count = count;
    return BW_OK;
}

void free_run(PrRun &run, cudaStream_t s)
{
    if (run.work) cudaFreeAsync(run.work, s);
    if (run.long_count) cudaFreeAsync(run.long_count, s);
    if (run.win_counts) cudaFreeAsync(run.win_counts, s);
    run.work = nullptr; run.long_count = nullptr; run.win_counts = nullptr;
}

int launch_iteration(bw_context *ctx, int variant, PrArgs &a, const Geometry &geo, cudaStream_t s)
{
    switch (variant) {
      case PR_EDGE_LIST: k_pr_edge<0><<<geo.grid, geo.block, 0, s>>>(a); break;
      case PR_REV_EDGE_LIST: k_pr_edge<1><<<geo.grid, geo.block, 0, s>>>(a); break;
      case PR_STRUCT_EDGE_LIST: k_pr_edge<2><<<geo.grid, geo.block, 0, s>>>(a); break;
      case PR_REV_STRUCT_EDGE_LIST: k_pr_edge<3><<<geo.grid, geo.block, 0, s>>>(a); break;
      case PR_VERTEX_PUSH: k_pr_vertex_push<<<geo.grid, geo.block, 0, s>>>(a); break;
      case PR_VERTEX_PUSH_WARP: k_pr_vertex_push_warp<<<geo.grid, geo.block, geo.smem, s>>>(a); break;
      case PR_VERTEX_PULL: k_pr_pull_items<false, true><<<geo.grid, PULL_WARPS * 32, 0, s>>>(a); break;
      case PR_VERTEX_PULL_NODIV: k_pr_pull_items<true, true><<<geo.grid, PULL_WARPS * 32, 0, s>>>(a); break;
      case PR_VERTEX_PULL_WARP: k_pr_vertex_pull_warp<false><<<geo.grid, geo.block, geo.smem, s>>>(a); break;
      case PR_VERTEX_PULL_WARP_NODIV: k_pr_vertex_pull_warp<true><<<geo.grid, geo.block, geo.smem, s>>>(a); break;
      case PR_PULL_SEGMENTED: k_pr_pull_items<false, false><<<geo.grid, PULL_WARPS * 32, 0, s>>>(a); break;
      default: return BW_ERR_UNKNOWN_VARIANT;
    }
    if (!is_fused(variant)) {
        k_consolidate_div<<<ctx->sm_count * 8, 256, 0, s>>>(a, uses_rowlen(variant) ? 1 : 0);
    }
    BW_CUDA(cudaGetLastError());
    return BW_OK;
}

// Runs a (possibly switching) schedule of variants of one semantics class.
int run_pagerank(bw_context *ctx, const bw_graph_view *g, const int32_t *schedule,
                 uint32_t schedule_len, uint32_t iterations, float *ranks,
                 const bw_launch_config *cfg, int loop_mode, int time_iterations,
                 float *iteration_ms, bw_pagerank_result *result, float *diffs_host,
                 void *stream)
{
    if (!ctx || !g || !schedule || schedule_len == 0 || !ranks) return BW_ERR_INVALID_ARGUMENT;
    if (g->vertex_count == 0 || g->vertex_count > 0xffffffffULL || g->edge_count > 0xffffffffULL)
        return BW_ERR_INVALID_ARGUMENT;
    const bool nodiv = is_nodiv(schedule[0]);
    int reps = 0;
    bool need_split = false, need_exact = false, any_rowlen = false, any_deg = false;
    for (uint32_t i = 0; i < schedule_len; i++) {
        const int v = schedule[i];
        if (v < 0 || v >= PR_VARIANT_COUNT) return BW_ERR_UNKNOWN_VARIANT;
        if (is_nodiv(v) != nodiv) return BW_ERR_INVALID_ARGUMENT;
        BW_TRY(validate_cfg(ctx, v, cfg));
        reps |= kPrReps[v];
        if (v == PR_PULL_SEGMENTED) need_split = true;
        if (v == PR_VERTEX_PULL || v == PR_VERTEX_PULL_NODIV) need_exact = true;
        if (uses_rowlen(v)) any_rowlen = true; else any_deg = true;
    }
    BW_TRY(check_reps(g, reps));
    if (any_rowlen && any_deg && !g->fwd_vertices) return BW_ERR_MISSING_REPRESENTATION;
    cudaStream_t s = as_stream(stream);
    const uint64_t n = g->vertex_count;
    BW_TRY(ensure_pr_scratch(ctx, n, iterations));
    if (time_iterations) BW_TRY(ensure_level_events(ctx, iterations + 1));

    PrRun split_run, exact_run;
    if (need_split) BW_TRY(build_segments(ctx, g, 1, split_run, s));
    if (need_exact) BW_TRY(build_segments(ctx, g, 0, exact_run, s));

    PrArgs a{};
    a.fwd_v = g->fwd_vertices; a.fwd_e = g->fwd_edges; a.rev_v = g->rev_vertices; a.rev_e = g->rev_edges;
    a.fwd_in = g->fwd_in_edges; a.rev_in = g->rev_in_edges;
    a.fwd_s = reinterpret_cast<const uint2 *>(g->fwd_struct_edges);
    a.rev_s = reinterpret_cast<const uint2 *>(g->rev_struct_edges);
    a.n = n; a.m = g->edge_count;
    a.base_div = (1.0 - static_cast<double>(0.85f)) / static_cast<double>(n);
    a.deg = ctx->pr_deg;
    a.acc = ctx->pr_acc;
    a.warp_size = (cfg && cfg->warp_size) ? cfg->warp_size : 32;
    a.chunk_size = (cfg && cfg->chunk_size) ? cfg->chunk_size : 32;

    BW_CUDA(cudaEventRecord(ctx->ev_start, s));
    // Degrees inside the timed region, as pagerank/pagerank.cpp:102-112.
    BW_TRY(launch_degrees(ctx, g, schedule[0], ctx->pr_deg, s));
    if (any_rowlen && any_deg) {
        // mixed schedule: make the degree buffer valid for every variant
        k_row_lengths<<<ctx->sm_count * 4, 256, 0, s>>>(g->fwd_vertices, n, ctx->pr_deg);
    }
    BW_CUDA(cudaMemsetAsync(ctx->pr_diffs, 0, (iterations + 1) * sizeof(float), s));

    // Buffers: div -> ranks in place, contributions double-buffered in
    // pr_buf[0/1]; nodiv -> ranks double-buffered between `ranks` and
    // pr_buf[0] so the last iteration lands in `ranks`.
    float *contrib[2] = {ctx->pr_buf[0], ctx->pr_buf[1]};
    float *nb[2];
    if (nodiv) {
        nb[0] = (iterations % 2 == 0) ? ranks : ctx->pr_buf[0];
        nb[1] = (iterations % 2 == 0) ? ctx->pr_buf[0] : ranks;
    }
    const int first_rowlen = uses_rowlen(schedule[0]) && !any_deg ? 1 : 0;
    k_pr_init<<<ctx->sm_count * 4, 256, 0, s>>>(a, nodiv ? nb[0] : ranks, nodiv ? nullptr : contrib[0],
                                                 first_rowlen);
    BW_CUDA(cudaGetLastError());

    for (uint32_t j = 1; j <= iterations; j++) {
        const int v = schedule[std::min<uint32_t>(j - 1, schedule_len - 1)];
        if (time_iterations) BW_CUDA(cudaEventRecord(ctx->level_events[j - 1], s));
        a.not_last = iterations > j ? 1 : 0;
        a.diff = ctx->pr_diffs + (j - 1);
        if (nodiv) {
            a.pr_in = nb[(j - 1) & 1];
            a.pr_out = nb[j & 1];
        } else {
            a.pr_out = ranks;
            if (is_fused(v)) {
                a.contrib_in = contrib[(j - 1) & 1];
                a.contrib_out = contrib[j & 1];
            } else {
                // atomic variants consolidate into the buffer they read next
                a.contrib_in = contrib[(j - 1) & 1];
                a.contrib_out = contrib[j & 1];
            }
        }
        const PrRun &items = v == PR_PULL_SEGMENTED ? split_run : exact_run;
        a.work = items.work;
        a.work_count = items.work_count;
        a.long_count = items.long_count;
        Geometry geo = geometry(ctx, v, cfg);
        BW_TRY(launch_iteration(ctx, v, a, geo, s));
        (void) loop_mode;
    }
    if (time_iterations) BW_CUDA(cudaEventRecord(ctx->level_events[iterations], s));
    BW_CUDA(cudaEventRecord(ctx->ev_stop, s));
    float diffs_dev_last = 0.0f;
    if (diffs_host && iterations)
        BW_CUDA(cudaMemcpyAsync(diffs_host, ctx->pr_diffs, iterations * sizeof(float), cudaMemcpyDeviceToHost, s));
    if (iterations)
        BW_CUDA(cudaMemcpyAsync(&diffs_dev_last, ctx->pr_diffs + iterations - 1, sizeof(float),
                                cudaMemcpyDeviceToHost, s));
    BW_CUDA(cudaStreamSynchronize(s));
    free_run(split_run, s);
    free_run(exact_run, s);
    if (time_iterations && iteration_ms) {
        for (uint32_t j = 0; j < iterations; j++)
            BW_CUDA(cudaEventElapsedTime(&iteration_ms[j], ctx->level_events[j], ctx->level_events[j + 1]));
    }
    if (result) {
        float ms = 0.0f;
        BW_CUDA(cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop));
        result->iterations = iterations;
        result->last_diff = diffs_dev_last;
        result->device_ms = ms;
    }
    return BW_OK;
}

}  // namespace

extern "C" {

int bw_pagerank_variant_count(void) { return PR_VARIANT_COUNT; }

const char *bw_pagerank_variant_name(int variant)
{
    return (variant >= 0 && variant < PR_VARIANT_COUNT) ? kPrNames[variant] : nullptr;
}

int bw_pagerank_variant_lookup(const char *name)
{
    if (!name) return -1;
    for (int i = 0; i < PR_VARIANT_COUNT; i++)
        if (std::strcmp(name, kPrNames[i]) == 0) return i;
    return -1;
}

int bw_pagerank_variant_reps(int variant)
{
    return (variant >= 0 && variant < PR_VARIANT_COUNT) ? kPrReps[variant] : 0;
}

int bw_pagerank_run(bw_context *ctx, const bw_graph_view *g, int variant,
                    uint32_t iterations, float *ranks, const bw_launch_config *cfg,
                    int loop_mode, bw_pagerank_result *result, float *diffs, void *stream)
{
    int32_t sched = variant;
    return run_pagerank(ctx, g, &sched, 1, iterations, ranks, cfg, loop_mode, 0, nullptr,
                        result, diffs, stream);
}

int bw_pagerank_run_schedule(bw_context *ctx, const bw_graph_view *g, const int32_t *schedule,
                             uint32_t schedule_len, uint32_t iterations, float *ranks,
                             const bw_launch_config *cfg, int time_iterations,
                             float *iteration_ms, bw_pagerank_result *result, void *stream)
{
    return run_pagerank(ctx, g, schedule, schedule_len, iterations, ranks, cfg, BW_LOOP_HOST,
                        time_iterations, iteration_ms, result, nullptr, stream);
}

}  // extern "C"
