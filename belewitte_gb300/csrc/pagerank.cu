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
#include <cmath>
#include <cstring>
#include <cooperative_groups.h>

#include "bw_consolidate.h"
#include "bw_seqsum.h"
#include "bw_seqsum_warp.cuh"
#include "bw_internal.cuh"
#include "bw_sort.cuh"

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
    uint32_t *long_count;      // arrival counters of long rows (pieces)
    float *vals;               // exact long rows: gathered terms, indexed by edge
    // Hub-first source order (work-list kernels): the gathered array is
    // stored at slot[v] and gat_e holds the reverse-CSR sources translated to
    // slots (slot == nullptr: identity, gat_e == rev_e).  The nodiv family
    // keeps its ranks in vertex order and writes the gathered copy to
    // gat_out[slot[v]] (read as gat_in next iteration).
    const uint32_t *gat_e;
    const uint32_t *slot;
    uint32_t hub_count;        // work-list kernels: gathered entries cached in shared memory
    const uint32_t *rows;      // work-list kernels: rows with in-edges, then rows without
    const uint32_t *long_rows;    // exact variants: long rows by decreasing length
    const uint32_t *long_total;   // device: number of long rows
    const uint32_t *giant_total;  // device: long rows summed piece-parallel (the first ones)
    const uint32_t *giant_pieces; // device: their pieces (work items [0, giant_pieces))
    float *piece_sum;             // exact pieces: float sum of the piece's terms (any order)
    uint4 *piece_map;             // giant-row pieces: two-uint4 records (k_pr_long_sums)
    uint32_t *sum_ctr;            // k_pr_long_sums' job and finish counters
    // Heavy units of the push and warp-pull variants (rows or chunks with
    // too many edges for one warp), cut into tiles that every warp of a
    // second kernel shares:
    uint4 *heavy_q;               // {unit, first edge, end edge, 0}
    uint32_t *heavy_ctr;          // [0] tiles queued, [1] taken, [2] warps done, [3] chunks listed, [4] warps done
    uint32_t *heavy_chunks;       // warp-pull: heavy chunks, consolidated by k_pr_heavy_finish
    uint32_t heavy_cap;           // capacity of heavy_q
    // Decided on the device, so the host never waits inside a run:
    const uint32_t *relabel_on;   // != 0: the hub-first order was taken (nullptr: never)
    const uint32_t *count_dev;    // work-list length (nullptr: work_count)
    const float *gat_in;
    float *gat_out;
    // First iteration of a div work-list run in the hub-first order: the
    // sources are read as vertex ids (rev_e) and translated by that
    // iteration's kernel, which gathers {slot, first contribution} from
    // first_pk and writes the slots to gat_e_out (nullptr: gat_e is ready).
    const uint2 *first_pk;
    uint32_t *gat_e_out;
    // Forward edge lists: the destination stream with the hot destinations
    // (the most edges in) replaced by HOT_BIT | their slot, and the vertex
    // of each slot (k_pr_edge_hot); nullptr: not built.
    const uint32_t *hot_dst;      // edge-list: translated outEdges
    const uint2 *hot_pairs;       // struct-edge-list: translated {in, out}
    const uint32_t *hot_vertex;
    const uint32_t *hot_count;    // device: slots in use
    double base_div;           // (1.0 - 0.85f) / N, computed once on the host
};

__device__ __forceinline__ uint64_t gtid() { return blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; }
__device__ __forceinline__ uint64_t gthreads() { return uint64_t(gridDim.x) * blockDim.x; }

// Applies the decisions taken on the device to a kernel's copy of the args.
__device__ __forceinline__ void resolve_args(PrArgs &a)
{
    if (a.relabel_on && *a.relabel_on == 0) {
        a.slot = nullptr;
        a.gat_e = a.rev_e;
        a.gat_in = nullptr;
        a.gat_out = nullptr;
    }
    if (a.count_dev) a.work_count = *a.count_dev;
}

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

// The same histogram for a stream whose hot ids are low (R-MAT and
// preferential-attachment graphs number their hubs first): ids below
// COUNT_PRIVATE are counted in the block's shared memory and added to the
// global counts once per block; the rest as in k_count_ids.  Thousands of
// atomics on one hub's counter otherwise serialise at its L2 slice.
constexpr uint32_t COUNT_PRIVATE = 8192;

__global__ void __launch_bounds__(1024) k_count_ids_private(const uint32_t *__restrict__ ids, uint64_t count,
                                                            uint32_t stride_words, uint64_t n,
                                                            uint32_t *__restrict__ deg)
{
    __shared__ uint32_t local[COUNT_PRIVATE];
    const uint32_t priv = static_cast<uint32_t>(n < COUNT_PRIVATE ? n : COUNT_PRIVATE);
    for (uint32_t i = threadIdx.x; i < priv; i += blockDim.x) local[i] = 0;
    __syncthreads();
    const unsigned lane = threadIdx.x & 31;
    const uint64_t warp = gtid() >> 5, warps = gthreads() >> 5;
    for (uint64_t base = warp * 32; base < count; base += warps * 32) {
        const uint64_t i = base + lane;
        const uint32_t id = i < count ? ids[i * stride_words] : 0xffffffffu;
        if (id < priv) {
            atomicAdd(&local[id], 1u);
        } else {
            const unsigned peers = __match_any_sync(__activemask(), id);
            if (id != 0xffffffffu && (__ffs(peers) - 1) == static_cast<int>(lane))
                atomicAdd(&deg[id], static_cast<uint32_t>(__popc(peers)));
        }
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < priv; i += blockDim.x)
        if (local[i]) atomicAdd(&deg[i], local[i]);
}

// Initial ranks 1/N (pagerank/pagerank.cpp:88) and contributions (stored at
// the vertex's slot when sources are relabelled; `gat` is the nodiv family's
// relabelled copy of the ranks).
__global__ void k_pr_init(PrArgs a, float *pr, float *contrib, float *gat, int rowlen)
{
    resolve_args(a);
    if (!a.slot) gat = nullptr;                   // the relabelled copy is not used
    const float init = __fdiv_rn(1.0f, static_cast<float>(a.n));
    for (uint64_t v = gtid(); v < a.n; v += gthreads()) {
        pr[v] = init;
        if (a.acc) a.acc[v] = 0.0f;
        const uint64_t at = a.slot ? a.slot[v] : v;
        if (contrib) {
            const uint32_t d = rowlen ? a.fwd_v[v + 1] - a.fwd_v[v] : a.deg[v];
            contrib[at] = d ? __fdiv_rn(init, static_cast<float>(d)) : 0.0f;
        }
        if (gat) gat[at] = init;
    }
}

// ----------------------- hub-first source order -----------------------------
// Gathers dominate the pull kernels; a source is gathered once per out-edge.
// Storing the gathered array in decreasing out-degree order packs the hubs
// of skewed graphs into few cache lines, which then stay in L1.  Rows keep
// their order and their sources' order, so every sum is unchanged.
// The sort key of a vertex: floor(log2(deg)) classes, larger degrees first
// (32 for a vertex without out-edges).
struct RelabelDigit {
    const uint32_t *deg;
    __device__ __forceinline__ uint32_t digit(uint64_t v) const
    {
        const uint32_t d = deg[v];
        return d ? static_cast<uint32_t>(__clz(d)) : 32u;
    }
};
// The sort's output, written per vertex v (coalesced: the sort walks the
// vertices in order) and per position: order[pos] = v, slot[v] = pos and,
// for the div variants, pk[v] = {pos, first-iteration contribution} -- the
// value k_pr_init gives them, 1/N over the degree.  Written whether or not
// the order is taken: nothing reads them unless it is.
struct RelabelPut {
    uint32_t *order, *slot;
    uint2 *pk;
    const uint32_t *deg;
    float init;
    __device__ __forceinline__ void put(uint32_t pos, uint64_t v) const
    {
        order[pos] = static_cast<uint32_t>(v);
        slot[v] = pos;
        if (pk) {
            const uint32_t d = deg[v];
            pk[v] = make_uint2(pos, __float_as_uint(d ? __fdiv_rn(init, static_cast<float>(d)) : 0.0f));
        }
    }
};
constexpr int RELABEL_BINS = 64, RELABEL_WARPS = 8, RELABEL_BLOCKS_PER_SM = 8;

// Edges covered by the first `k` entries in degree order (cov[0]) and in
// vertex order (cov[1]), from counters the caller zeroed; the last block to
// finish (cov[2] counts them) decides whether the order is worth a pass over
// the edges (>= 5% more of them on the cached hubs) and writes *on.
__global__ void __launch_bounds__(1024) k_relabel_coverage(const uint32_t *__restrict__ deg,
                                                           const uint32_t *__restrict__ order, uint64_t k,
                                                           uint64_t m, unsigned long long *cov, uint32_t *on)
{
    __shared__ unsigned long long part[2][32];
    __shared__ bool last;
    unsigned long long sorted = 0, natural = 0;
    const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
    if (i < k) {
        sorted = deg[order[i]];
        natural = deg[i];
    }
    for (int o = 16; o > 0; o >>= 1) {
        sorted += __shfl_xor_sync(FULL_MASK, sorted, o);
        natural += __shfl_xor_sync(FULL_MASK, natural, o);
    }
    if ((threadIdx.x & 31) == 0) { part[0][threadIdx.x >> 5] = sorted; part[1][threadIdx.x >> 5] = natural; }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long a = 0, b = 0;
        for (unsigned w = 0; w < blockDim.x / 32; w++) { a += part[0][w]; b += part[1][w]; }
        atomicAdd(&cov[0], a);
        atomicAdd(&cov[1], b);
        __threadfence();
        last = atomicAdd(reinterpret_cast<unsigned int *>(&cov[2]), 1u) + 1 == gridDim.x;
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        const unsigned long long a = atomicAdd(&cov[0], 0ull), b = atomicAdd(&cov[1], 0ull);
        *on = (static_cast<double>(a) - static_cast<double>(b) >= 0.05 * static_cast<double>(m)) ? 1u : 0u;
    }
}

__global__ void __launch_bounds__(256) k_relabel_edges(const uint32_t *__restrict__ src, uint64_t m,
                                                       const uint32_t *on, const uint32_t *__restrict__ slot,
                                                       uint32_t *__restrict__ out)
{
    if (*on == 0) return;
    const uint64_t quads = m / 4;
    const uint4 *s4 = reinterpret_cast<const uint4 *>(src);
    uint4 *o4 = reinterpret_cast<uint4 *>(out);
    const bool aligned = (reinterpret_cast<uintptr_t>(src) & 15) == 0;
    if (aligned) {
        for (uint64_t q = gtid(); q < quads; q += gthreads()) {
            const uint4 x = __ldcs(s4 + q);
            __stcs(o4 + q, make_uint4(__ldg(slot + x.x), __ldg(slot + x.y), __ldg(slot + x.z), __ldg(slot + x.w)));
        }
    }
    for (uint64_t i = (aligned ? quads * 4 : 0) + gtid(); i < m; i += gthreads()) out[i] = __ldg(slot + src[i]);
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
            const float acc = a.acc[v], prev = a.pr_out[v];
            const uint32_t d = rowlen ? a.fwd_v[v + 1] - a.fwd_v[v] : a.deg[v];
            const float nr = consolidate_div(acc, a.base_div);
            dsum += fabsf(nr - prev);
            a.pr_out[v] = nr;
            a.acc[v] = 0.0f;
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

// -------------------- forward edge lists: hot destinations ------------------
// edgeListPageRank and structEdgeListPageRank (pagerank/edgelist.cu:3-23,
// struct_edgelist.cu) add every edge's contribution to its destination with
// one float atomic.  On a skewed graph a few thousand destinations take a
// third of the edges, and atomics on one address serialise in L2.  Once per
// run the destinations with the most in-edges (whole log2 classes of the
// in-degree, at most HOT_SLOTS of them) get a slot, and the destination
// stream is rewritten with HOT_BIT | slot in their place.  Each block then
// adds those edges into its own shared-memory copy of the hot accumulators
// and flushes each nonzero slot to acc[] with one atomic when its edges are
// done; every other edge is added as before.  Float-atomic order is the
// variants' own (the reference's is unspecified), so results stay within
// the order-changing variants' tolerance.
constexpr uint32_t HOT_SLOTS = 16384;          // 64 KB of accumulators per block
constexpr uint32_t HOT_BIT = 0x80000000u;
constexpr int HOT_THREADS = 1024;

// 33 counters: vertices by floor(log2(in-degree)) (class 32: in-degree 0)
__global__ void k_hot_classes(const uint32_t *__restrict__ indeg, uint64_t n, uint32_t *__restrict__ bins)
{
    __shared__ uint32_t b[33];
    if (threadIdx.x < 33) b[threadIdx.x] = 0;
    __syncthreads();
    for (uint64_t v = gtid(); v < n; v += gthreads()) {
        const uint32_t d = indeg[v];
        atomicAdd(&b[d ? 31 - __clz(d) : 32], 1u);
    }
    __syncthreads();
    if (threadIdx.x < 33 && b[threadIdx.x]) atomicAdd(&bins[threadIdx.x], b[threadIdx.x]);
}

// bins[33] = the lowest class taken: the top classes while they fit the
// slots (classes of in-degree below 2 are never taken)
__global__ void k_hot_pick(uint32_t *bins)
{
    if (blockIdx.x || threadIdx.x) return;
    uint32_t total = 0, lowest = 32;
    for (int c = 31; c >= 1; c--) {
        if (total + bins[c] > HOT_SLOTS) break;
        total += bins[c];
        lowest = static_cast<uint32_t>(c);
    }
    bins[33] = lowest;
    bins[34] = 0;                                  // slot counter
}

__global__ void k_hot_assign(const uint32_t *__restrict__ indeg, uint64_t n, uint32_t *__restrict__ bins,
                             uint32_t *__restrict__ slot_of, uint32_t *__restrict__ hot_vertex)
{
    const uint32_t lowest = bins[33];
    for (uint64_t v = gtid(); v < n; v += gthreads()) {
        const uint32_t d = indeg[v];
        uint32_t sl = 0xffffffffu;
        if (lowest < 32 && d && static_cast<uint32_t>(31 - __clz(d)) >= lowest) {
            sl = atomicAdd(&bins[34], 1u);
            hot_vertex[sl] = static_cast<uint32_t>(v);
        }
        slot_of[v] = sl;
    }
}

// PAIRS: {in, out} pairs (struct-edge-list), else the outEdges stream
template<bool PAIRS>
__global__ void __launch_bounds__(256) k_hot_translate(const uint32_t *__restrict__ dst, const uint2 *__restrict__ pairs,
                                                       uint64_t m, const uint32_t *__restrict__ slot_of,
                                                       uint32_t *__restrict__ out, uint2 *__restrict__ out_pairs)
{
    for (uint64_t e = gtid(); e < m; e += gthreads()) {
        if constexpr (PAIRS) {
            uint2 p = __ldcs(pairs + e);
            const uint32_t sl = slot_of[p.y];
            if (sl != 0xffffffffu) p.y = HOT_BIT | sl;
            __stcs(out_pairs + e, p);
        } else {
            const uint32_t d = __ldcs(dst + e), sl = slot_of[d];
            __stcs(out + e, sl != 0xffffffffu ? (HOT_BIT | sl) : d);
        }
    }
}

template<int LAYOUT>  // 0 fwd SoA, 2 fwd AoS
__global__ void __launch_bounds__(HOT_THREADS) k_pr_edge_hot(PrArgs a)
{
    extern __shared__ float hot[];                 // HOT_SLOTS floats
    const uint32_t slots = *a.hot_count;
    for (uint32_t i = threadIdx.x; i < slots; i += blockDim.x) hot[i] = 0.0f;
    __syncthreads();
    const unsigned lane = threadIdx.x & 31;
    const uint64_t warp = gtid() >> 5, warps = gthreads() >> 5;
    const uint64_t m = a.m;
    for (uint64_t base = warp * 32; base < m; base += warps * 32) {
        const uint64_t e = base + lane;
        if (e >= m) continue;
        uint32_t src, dst;
        if constexpr (LAYOUT == 0) { src = __ldcs(a.fwd_in + e); dst = __ldcs(a.hot_dst + e); }
        else { const uint2 p = __ldcs(a.hot_pairs + e); src = p.x; dst = p.y; }
        const float val = __ldg(a.contrib_in + src);
        if (dst & HOT_BIT) atomicAdd(&hot[dst & ~HOT_BIT], val);
        else atomicAdd(&a.acc[dst], val);
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < slots; i += blockDim.x)
        if (hot[i] != 0.0f) atomicAdd(&a.acc[a.hot_vertex[i]], hot[i]);
}

// ----------------------------- vertex-push --------------------------------
// Thread per vertex; each owner scatters pr[v] / rowlen to its out-row
// (pagerank/vertex_push.cu:3-31).  Rows longer than PUSH_HEAVY would keep
// one lane issuing its row's atomics one after the other while the rest of
// its warp idles: the warp expands those rows together instead (coalesced
// index loads, one row after the other, in lane order).
constexpr uint32_t PUSH_HEAVY = 32;
constexpr int PUSH_UNROLL = 8;

// A row (vertex-push) or a chunk (the virtual-warp variants) with more than
// HEAVY_UNIT edges would hold one warp for the whole iteration on a skewed
// graph -- R-MAT's hubs share the lowest ids.  Its edge range is queued
// instead, in HEAVY_TILE-edge tiles that every warp of k_pr_heavy_tiles
// takes from a counter.  The queue holds at most M / HEAVY_TILE +
// M / (the unit threshold) + 1 tiles.
constexpr uint32_t HEAVY_UNIT = 8192;
constexpr uint32_t HEAVY_TILE = 2048;
// vertex-push: a warp expands its rows of more than PUSH_HEAVY edges one
// after the other, so rows above PUSH_GIANT go to the tiles already
constexpr uint32_t PUSH_GIANT = 1024;

__device__ __forceinline__ void enqueue_tiles(const PrArgs &a, uint32_t unit, uint32_t t0, uint32_t t1)
{
    const uint32_t cnt = (t1 - t0 + HEAVY_TILE - 1) / HEAVY_TILE;
    const uint32_t base = atomicAdd(&a.heavy_ctr[0], cnt);
    for (uint32_t k = 0; k < cnt; k++)
        if (base + k < a.heavy_cap)
            a.heavy_q[base + k] = make_uint4(unit, t0 + k * HEAVY_TILE, min(t1, t0 + (k + 1) * HEAVY_TILE), 0u);
}

__global__ void __launch_bounds__(256) k_pr_vertex_push(PrArgs a)
{
    const unsigned lane = threadIdx.x & 31;
    for (uint64_t w0 = gtid() - lane; w0 < a.n; w0 += gthreads()) {
        const uint64_t v = w0 + lane;
        uint32_t s = 0, e = 0;
        if (v < a.n) {
            s = a.fwd_v[v];
            e = a.fwd_v[v + 1];
        }
        const float out = s < e ? a.contrib_in[v] : 0.0f;
        const bool giant = e - s > PUSH_GIANT;
        if (giant) enqueue_tiles(a, static_cast<uint32_t>(v), s, e);
        const bool heavy = !giant && e - s > PUSH_HEAVY;
        if (!heavy && !giant) {
#pragma unroll 4
            for (uint32_t i = s; i < e; i++) atomicAdd(&a.acc[__ldg(a.fwd_e + i)], out);
        }
        for (unsigned hv = __ballot_sync(FULL_MASK, heavy); hv; hv &= hv - 1) {
            const unsigned l = __ffs(hv) - 1;
            const uint32_t hs = __shfl_sync(FULL_MASK, s, l), he = __shfl_sync(FULL_MASK, e, l);
            const float ho = __shfl_sync(FULL_MASK, out, l);
            for (uint32_t base = hs; base < he; base += 32 * PUSH_UNROLL) {
                uint32_t d[PUSH_UNROLL];
#pragma unroll
                for (int u = 0; u < PUSH_UNROLL; u++) {
                    const uint32_t i = base + u * 32 + lane;
                    d[u] = i < he ? __ldcs(a.fwd_e + i) : 0u;
                }
#pragma unroll
                for (int u = 0; u < PUSH_UNROLL; u++)
                    if (base + u * 32 + lane < he) atomicAdd(&a.acc[d[u]], ho);
            }
        }
    }
}

// vertex-push-warp (pagerank/vertex_push_warp.cu:4-49): a virtual warp of W
// lanes per chunk of C vertices, contributions and offsets staged in shared
// memory.  The chunk's out-rows are contiguous in the forward CSR, so the
// virtual warp streams the chunk's whole edge range -- coalesced index
// loads, PUSH_UNROLL per lane in flight -- instead of one row at a time;
// each lane finds the row of its edge by a cursor over the staged offsets.
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
        const uint32_t e0 = my_off[0], e1 = my_off[cnt];
        const bool heavy = e1 - e0 > HEAVY_UNIT;       // tiles for k_pr_heavy_tiles
        if (heavy && lane == 0) enqueue_tiles(a, static_cast<uint32_t>(chunk), e0, e1);
        uint32_t r = 0;                              // this lane's row cursor
        for (uint32_t base = e0; base < (heavy ? e0 : e1); base += W * PUSH_UNROLL) {
            uint32_t d[PUSH_UNROLL];
#pragma unroll
            for (int u = 0; u < PUSH_UNROLL; u++) {
                const uint32_t p = base + u * W + lane;
                d[u] = p < e1 ? __ldcs(a.fwd_e + p) : 0u;
            }
#pragma unroll
            for (int u = 0; u < PUSH_UNROLL; u++) {
                const uint32_t p = base + u * W + lane;
                if (p < e1) {
                    while (my_off[r + 1] <= p) r++;      // ends: my_off[cnt] = e1 > p
                    atomicAdd(&a.acc[d[u]], my_c[r]);
                }
            }
        }
        __syncwarp(mask);
    }
}

// Consolidate vertex v from its in-sum (div: consolidateRank plus the next
// contribution; nodiv: consolidateRankNoDiv).  Returns |pr_new - pr_old|.
// The per-vertex inputs are loaded by finish_load, which the work-list
// kernel issues before its gathers so that their latency overlaps them
// (and before any store: the arrays are not restrict, so a load after a
// store would wait for it).
struct FinishIn {
    float prev;        // the rank the diff compares against
    uint32_t dg;       // out-degree
    uint32_t at;       // where the gathered copy goes (slot or vertex)
};

template<bool NODIV>
__device__ __forceinline__ FinishIn finish_load(const PrArgs &a, uint64_t v)
{
    FinishIn in;
    in.prev = NODIV ? a.pr_in[v] : a.pr_out[v];
    in.dg = a.deg[v];
    in.at = a.slot ? a.slot[v] : static_cast<uint32_t>(v);
    return in;
}

template<bool NODIV>
__device__ __forceinline__ float finish_store(const PrArgs &a, uint64_t v, float sum, float base_nd, FinishIn in)
{
    if constexpr (!NODIV) {
        const float nr = consolidate_div(sum, a.base_div);
        a.pr_out[v] = nr;
        a.contrib_out[in.at] = in.dg ? __fdiv_rn(nr, static_cast<float>(in.dg)) : 0.0f;
        return fabsf(nr - in.prev);
    } else {
        float nr = __fmaf_rn(DAMPING, sum, base_nd);
        const float d = fabsf(nr - in.prev);
        if (in.dg != 0 && a.not_last) nr = __fdiv_rn(nr, static_cast<float>(in.dg));
        a.pr_out[v] = nr;
        if (a.gat_out) a.gat_out[in.at] = nr;
        return d;
    }
}

template<bool NODIV>
__device__ __forceinline__ float finish_vertex(const PrArgs &a, uint64_t v, float sum, float base_nd)
{
    return finish_store<NODIV>(a, v, sum, base_nd, finish_load<NODIV>(a, v));
}

// ----------------------------- pull variants ------------------------------
// vertex-pull-warp / -nodiv (pagerank/vertex_pull_warp.cu:4-49,
// vertex_pull_warp_nodiv.cu:4-47): a virtual warp of W lanes per chunk of C
// vertices, each vertex consolidated in place.  The reference takes the
// chunk's vertices one after the other and adds each lane's partial with a
// float atomic, so its summation order is unspecified.  Here the chunk's
// in-rows, contiguous in the reverse CSR, are streamed as one edge range:
// coalesced index loads and PUSH_UNROLL independent gathers per lane in
// flight; each lane adds the terms of its run of one row in a register and
// flushes the run into the row's shared-memory accumulator; then the lanes
// consolidate the chunk's vertices together.
template<bool NODIV>
__global__ void __launch_bounds__(512) k_pr_vertex_pull_warp(PrArgs a)
{
    extern __shared__ uint32_t smem[];
    const uint32_t W = a.warp_size, C = a.chunk_size;
    const uint32_t per_block = blockDim.x / W, vw = threadIdx.x / W, lane = threadIdx.x % W;
    const unsigned mask = W >= 32 ? FULL_MASK : (((1u << W) - 1u) << ((threadIdx.x & 31) & ~(W - 1u)));
    float *my_acc = reinterpret_cast<float *>(smem) + vw * C;
    uint32_t *my_off = smem + per_block * C + vw * (C + 1);
    const uint64_t n = a.n, total = uint64_t(gridDim.x) * per_block;
    const float *src = NODIV ? a.pr_in : a.contrib_in;
    const float base_nd = nodiv_base(n);
    constexpr uint32_t NO_ROW = 0xffffffffu;
    float dsum = 0.0f;
    for (uint64_t chunk = blockIdx.x * uint64_t(per_block) + vw; chunk * C < n; chunk += total) {
        const uint64_t v0 = chunk * C;
        const uint32_t cnt = static_cast<uint32_t>(min(uint64_t(C), n - v0));
        for (uint32_t i = lane; i < cnt + 1; i += W) my_off[i] = a.rev_v[v0 + i];
        for (uint32_t i = lane; i < cnt; i += W) my_acc[i] = 0.0f;
        __syncwarp(mask);
        const uint32_t e0 = my_off[0], e1 = my_off[cnt];
        if (e1 - e0 > HEAVY_UNIT) {                  // summed by k_pr_heavy_tiles, finished by k_pr_heavy_finish
            if (lane == 0) {
                enqueue_tiles(a, static_cast<uint32_t>(chunk), e0, e1);
                a.heavy_chunks[atomicAdd(&a.heavy_ctr[3], 1u)] = static_cast<uint32_t>(chunk);
            }
            __syncwarp(mask);
            continue;
        }
        uint32_t r = 0, run_row = NO_ROW;            // row cursor; row of the open run
        float run = 0.0f;
        for (uint32_t base = e0; base < e1; base += W * PUSH_UNROLL) {
            uint32_t idx[PUSH_UNROLL];
#pragma unroll
            for (int u = 0; u < PUSH_UNROLL; u++) {
                const uint32_t p = base + u * W + lane;
                idx[u] = p < e1 ? __ldcs(a.rev_e + p) : 0u;
            }
            float val[PUSH_UNROLL];
#pragma unroll
            for (int u = 0; u < PUSH_UNROLL; u++) {
                const uint32_t p = base + u * W + lane;
                val[u] = p < e1 ? __ldcg(src + idx[u]) : 0.0f;
            }
#pragma unroll
            for (int u = 0; u < PUSH_UNROLL; u++) {
                const uint32_t p = base + u * W + lane;
                if (p < e1) {
                    while (my_off[r + 1] <= p) r++;      // ends: my_off[cnt] = e1 > p
                    if (r != run_row) {
                        if (run_row != NO_ROW) atomicAdd(&my_acc[run_row], run);
                        run_row = r;
                        run = 0.0f;
                    }
                    run += val[u];
                }
            }
        }
        if (run_row != NO_ROW) atomicAdd(&my_acc[run_row], run);
        __syncwarp(mask);
        for (uint32_t i = lane; i < cnt; i += W) dsum += finish_vertex<NODIV>(a, v0 + i, my_acc[i], base_nd);
        __syncwarp(mask);
    }
    add_diff(a.diff, dsum);
}

// Tiles of the heavy units queued by this iteration's first kernel
// (enqueue_tiles), taken by every warp from a counter; the last warp out
// resets the counters.  The push modes add each edge's contribution to its
// destination with a float atomic, as the first kernel does.  The pull
// modes add each lane's run of one row into acc[row] with a float atomic
// (the reference's warp kernels add lane partials with atomics too), and
// k_pr_heavy_finish consolidates the rows.
template<int MODE>   // 0 vertex-push, 1 vertex-push-warp, 2 vertex-pull-warp, 3 vertex-pull-warp-nodiv
__global__ void __launch_bounds__(256) k_pr_heavy_tiles(PrArgs a)
{
    constexpr uint32_t NO_ROW = 0xffffffffu;
    const unsigned lane = threadIdx.x & 31;
    const uint32_t tiles = min(a.heavy_ctr[0], a.heavy_cap);
    const uint32_t *V = MODE <= 1 ? a.fwd_v : a.rev_v;
    const uint32_t *E = MODE <= 1 ? a.fwd_e : a.rev_e;
    const float *src = MODE == 3 ? a.pr_in : a.contrib_in;
    for (;;) {
        uint32_t t = 0;
        if (lane == 0) t = atomicAdd(&a.heavy_ctr[1], 1u);
        t = __shfl_sync(FULL_MASK, t, 0);
        if (t >= tiles) break;
        const uint4 q = a.heavy_q[t];
        const uint32_t t0 = q.y, t1 = q.z;
        if constexpr (MODE == 0) {                   // one row: its contribution to every edge
            const float c = a.contrib_in[q.x];
            for (uint32_t base = t0; base < t1; base += 32 * PUSH_UNROLL) {
                uint32_t d[PUSH_UNROLL];
#pragma unroll
                for (int u = 0; u < PUSH_UNROLL; u++) {
                    const uint32_t i = base + u * 32 + lane;
                    d[u] = i < t1 ? __ldcs(E + i) : 0u;
                }
#pragma unroll
                for (int u = 0; u < PUSH_UNROLL; u++)
                    if (base + u * 32 + lane < t1) atomicAdd(&a.acc[d[u]], c);
            }
            continue;
        }
        // a chunk's rows v0 .. v0 + cnt - 1: the row of edge t0 by bisection,
        // then a cursor per lane
        const uint64_t v0 = uint64_t(q.x) * a.chunk_size;
        const uint32_t cnt = static_cast<uint32_t>(min(uint64_t(a.chunk_size), a.n - v0));
        uint32_t lo = 0, hi = cnt - 1;                // the last r with V[v0 + r] <= t0
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) / 2;
            if (V[v0 + mid] <= t0) lo = mid; else hi = mid - 1;
        }
        uint32_t r = lo, run_row = NO_ROW;
        float run = 0.0f;
        for (uint32_t base = t0; base < t1; base += 32 * PUSH_UNROLL) {
            uint32_t idx[PUSH_UNROLL];
#pragma unroll
            for (int u = 0; u < PUSH_UNROLL; u++) {
                const uint32_t p = base + u * 32 + lane;
                idx[u] = p < t1 ? __ldcs(E + p) : 0u;
            }
            float val[PUSH_UNROLL];
            if constexpr (MODE >= 2) {
#pragma unroll
                for (int u = 0; u < PUSH_UNROLL; u++) {
                    const uint32_t p = base + u * 32 + lane;
                    val[u] = p < t1 ? __ldcg(src + idx[u]) : 0.0f;
                }
            }
#pragma unroll
            for (int u = 0; u < PUSH_UNROLL; u++) {
                const uint32_t p = base + u * 32 + lane;
                if (p < t1) {
                    while (V[v0 + r + 1] <= p) r++;      // ends: V[v0 + cnt] >= t1 > p
                    if constexpr (MODE == 1) {
                        atomicAdd(&a.acc[idx[u]], a.contrib_in[v0 + r]);
                    } else {
                        if (r != run_row) {
                            if (run_row != NO_ROW) atomicAdd(&a.acc[v0 + run_row], run);
                            run_row = r;
                            run = 0.0f;
                        }
                        run += val[u];
                    }
                }
            }
        }
        if constexpr (MODE >= 2)
            if (run_row != NO_ROW) atomicAdd(&a.acc[v0 + run_row], run);
    }
    if (lane == 0) {
        const uint32_t warps = gridDim.x * (blockDim.x / 32);
        if (atomicAdd(&a.heavy_ctr[2], 1u) + 1 == warps) {
            a.heavy_ctr[0] = 0;
            a.heavy_ctr[1] = 0;
            a.heavy_ctr[2] = 0;
        }
    }
}

// Consolidates the rows of the heavy chunks of the warp-pull variants from
// acc[] (summed by k_pr_heavy_tiles) and clears acc[] for the next
// iteration; the last warp out resets the chunk list.
template<bool NODIV>
__global__ void __launch_bounds__(256) k_pr_heavy_finish(PrArgs a)
{
    const unsigned lane = threadIdx.x & 31;
    const uint64_t warp = gtid() >> 5, warps = gthreads() >> 5;
    const uint32_t chunks = a.heavy_ctr[3];
    const float base_nd = nodiv_base(a.n);
    float dsum = 0.0f;
    for (uint64_t k = warp; k < chunks; k += warps) {
        const uint64_t v0 = uint64_t(a.heavy_chunks[k]) * a.chunk_size;
        const uint32_t cnt = static_cast<uint32_t>(min(uint64_t(a.chunk_size), a.n - v0));
        for (uint32_t i = lane; i < cnt; i += 32) {
            const float sum = a.acc[v0 + i];
            a.acc[v0 + i] = 0.0f;
            dsum += finish_vertex<NODIV>(a, v0 + i, sum, base_nd);
        }
    }
    add_diff(a.diff, dsum);
    if (lane == 0 && atomicAdd(&a.heavy_ctr[4], 1u) + 1 == warps) {
        a.heavy_ctr[3] = 0;
        a.heavy_ctr[4] = 0;
    }
}

// ------------------------- work-list pull kernels ---------------------------
// vertex-pull, vertex-pull-nodiv and pull-segmented share one kernel over a
// work list cut once per run from the reverse CSR: an item is either at
// most 32 consecutive rows with at most SEG_EDGES edges (rows of at most
// the long-row threshold, SEG_LONG unless the launch gives another), or a
// piece of one long row.  Item: {row_begin, row_end | flags,
// edge_begin, edge_end}.
//
// Short rows: the warp loads the item's indices with unrolled coalesced
// loads, gathers all contributions at once (up to 1024 independent loads
// in flight per warp) into shared memory, and then each lane adds its own
// row's values one after the other in row order -- the reference's
// sequential summation (pagerank/vertex_pull.cu:23-27), so these rows are
// bit-identical to it.
// Long rows (more edges than the threshold) are cut into SEG_EDGES-edge pieces
// that any warp takes; the work list puts every piece, longest rows first,
// before the short-row items:
//   pieces store their gathered terms in vals[] (edge order);
//   k_pr_long_sums then evaluates every long row's sequential sum
//   (bit-identical to the reference's loop) and consolidates it.
constexpr uint32_t SEG_EDGES = 512;
constexpr uint32_t SEG_LONG = 256;             // default long-row threshold (at most SEG_EDGES)
constexpr uint32_t LONG_FLAG = 0x40000000u;    // piece of a long row
constexpr uint32_t CONST_FLAG = 0x20000000u;   // rows without in-edges
constexpr uint32_t ROW_MASK = 0x1fffffffu;     // work-list variants take N < 2^29
// Two block shapes: WIDE, one block of 32 warps per SM, and NARROW, blocks
// of 8 warps, several per SM (more warps in flight, fewer registers).
// Shared memory holds each warp's gather buffer and, after it, a cache of
// the first hub_count entries of the gathered array: with sources in
// hub-first order those are the most gathered values of the graph, read
// from shared memory instead of L2.  Every block holds its own copy, and
// what shared memory takes is lost to L1, which bounds the misses in flight.
constexpr int PULL_WIDE = 1024, PULL_NARROW = 256;
// Per warp: a gather buffer of SEG_EDGES terms, then 33 words of row ends.
constexpr uint32_t PULL_BUF = SEG_EDGES;
constexpr size_t pull_fixed_smem(int block) { return (block / 32) * (PULL_BUF + 33) * sizeof(float); }
constexpr int pull_min_blocks(int block) { return block == PULL_WIDE ? 1 : 4; }
// Default hub-cache entries per block.  WIDE's fixed buffers (69,760 bytes)
// with 16K entries already take the 164 KB shared-memory carveout; 24,288
// entries fill it (with the 1 KB the system reserves per block), so L1
// keeps the same 92 KB.  Measured on GB300 (vertex-pull, us per iteration):
// R-MAT-22 16K 323.0, 20K 320.0, 24,288 317.9, 28K 315.9, 32K 381.4;
// ER(4M, 67M) 276.9, 277.0, 277.0, 281.2, 505.3 -- from 32K the carveout
// grows to 228 KB and the 28 KB left to L1 cannot hold the gathers in flight.
constexpr uint32_t PULL_WIDE_HUBS = 24288, PULL_NARROW_HUBS = 0;
constexpr int GATHER_UNROLL = 16;   // 512 edges = one unrolled round

// Work-list construction.
//  * Rows are partitioned, stably, into the rows with in-edges and the rows
//    without (rows[0, ne) and rows[ne, N)).  Short items are cut over the
//    first part, so a warp's 32 rows all carry edges; the rows without
//    in-edges become CONST items at the end of the list (for the div
//    variants their rank and contribution are the same from the second
//    iteration on, so later iterations leave them out).
//  * Long rows (more edges than the threshold) are put in decreasing length
//    order (long_row_key) and cut into SEG_EDGES pieces in that order, at
//    the front of the list.
// Layout: [pieces | short items | CONST items]; the lengths stay on the
// device (tot[0] = items before the CONST ones, tot[1] = all items).
// Tile b of SCAN_TILE rows: part_e[b] rows with in-edges, part_l[b] long rows.
constexpr uint64_t ROW_TILE = sortk::SCAN_TILE;
__global__ void __launch_bounds__(sortk::SCAN_THREADS) k_rows_count(const uint32_t *__restrict__ off, uint64_t n,
                                                                    uint32_t seg_long, uint32_t *__restrict__ part_e,
                                                                    uint32_t *__restrict__ part_l)
{
    __shared__ uint32_t ws[sortk::SCAN_THREADS / 32];
    const uint64_t t0 = blockIdx.x * ROW_TILE;
    uint32_t e = 0, l = 0;
#pragma unroll
    for (int k = 0; k < sortk::SCAN_ITEMS; k++) {
        const uint64_t r = t0 + k * sortk::SCAN_THREADS + threadIdx.x;
        if (r < n) {
            const uint32_t d = off[r + 1] - off[r];
            e += d ? 1u : 0u;
            l += d > seg_long ? 1u : 0u;
        }
    }
    uint32_t te, tl;
    sortk::block_exclusive<sortk::SCAN_THREADS>(e, te, ws);
    sortk::block_exclusive<sortk::SCAN_THREADS>(l, tl, ws);
    if (threadIdx.x == 0) {
        part_e[blockIdx.x] = te;
        part_l[blockIdx.x] = tl;
    }
}

// The stable partition, from the scanned tile counts (part_e[tiles] = ne
// rows with in-edges, part_l[tiles] = long rows): rows with in-edges in row
// order at rows[0, ne), the rest at rows[ne, n); the long rows, in row
// order, with their lengths.  Each thread takes SCAN_ITEMS consecutive rows
// of its tile, whose lengths are staged in shared memory.
__global__ void __launch_bounds__(sortk::SCAN_THREADS) k_rows_partition(
    const uint32_t *__restrict__ off, uint64_t n, uint32_t seg_long, const uint32_t *__restrict__ part_e,
    const uint32_t *__restrict__ part_l, uint64_t tiles, uint32_t *__restrict__ rows,
    uint32_t *__restrict__ long_len, uint32_t *__restrict__ long_row)
{
    __shared__ uint32_t len[ROW_TILE + ROW_TILE / 32];
    __shared__ uint32_t ws[sortk::SCAN_THREADS / 32];
    const uint64_t t0 = blockIdx.x * ROW_TILE;
#pragma unroll
    for (int k = 0; k < sortk::SCAN_ITEMS; k++) {
        const uint32_t j = k * sortk::SCAN_THREADS + threadIdx.x;
        const uint64_t r = t0 + j;
        len[sortk::scan_pad(j)] = r < n ? off[r + 1] - off[r] : 0u;
    }
    __syncthreads();
    const uint32_t j0 = threadIdx.x * sortk::SCAN_ITEMS;
    uint32_t e = 0, l = 0;
#pragma unroll
    for (int k = 0; k < sortk::SCAN_ITEMS; k++) {
        const uint32_t d = len[sortk::scan_pad(j0 + k)];
        e += d ? 1u : 0u;
        l += d > seg_long ? 1u : 0u;
    }
    uint32_t te, tl;
    uint32_t pe = part_e[blockIdx.x] + sortk::block_exclusive<sortk::SCAN_THREADS>(e, te, ws);
    uint32_t pl = part_l[blockIdx.x] + sortk::block_exclusive<sortk::SCAN_THREADS>(l, tl, ws);
    const uint64_t ne = part_e[tiles];
    for (int k = 0; k < sortk::SCAN_ITEMS; k++) {
        const uint64_t r = t0 + j0 + k;
        if (r >= n) break;
        const uint32_t d = len[sortk::scan_pad(j0 + k)];
        // pe: rows with in-edges before r, so r - pe rows without
        if (d) rows[pe++] = static_cast<uint32_t>(r);
        else rows[ne + (r - pe)] = static_cast<uint32_t>(r);
        if (d > seg_long) {
            long_len[pl] = d;
            long_row[pl] = static_cast<uint32_t>(r);
            pl++;
        }
    }
}

// Piece counts of the sorted long rows (0 past the last one).
__global__ void k_piece_count(const uint32_t *__restrict__ long_len, const uint32_t *__restrict__ long_total,
                              uint64_t cap, uint32_t *__restrict__ pieces)
{
    const uint64_t L = *long_total;
    for (uint64_t i = gtid(); i < cap; i += gthreads())
        pieces[i] = i < L ? (long_len[i] + SEG_EDGES - 1) / SEG_EDGES : 0u;
}

// Exact long rows above GIANT_ROW terms are summed piece-parallel (binade
// maps per piece, combined by the row's last piece); shorter ones in
// batches of 32, one row per lane.  A lane's row is a chain of dependent
// additions with only a few dozen of its terms in flight (the warp's
// shared-memory ring): the longest batch rows set the kernel's critical
// path, which bounds their length.
constexpr uint32_t GIANT_ROW = 2048;

// Long rows are put in decreasing length order by one stable counting sort
// on this key (smaller key, earlier row).  Rows of at most GIANT_ROW terms
// (the batch rows) get one key per length, so their order is exact: rows of
// equal length in row order.  The giant rows come first, in 64 classes per
// octave of length (1.1% wide), each class in row order: their order only
// schedules their pieces.
constexpr uint32_t LONG_GIANT_KEYS = (32 - 11) * 64;                       // octaves 2^11 .. 2^31
constexpr int LONG_SORT_BINS = 4096, LONG_SORT_WARPS = 4, LONG_SORT_GRID = 64;
static_assert(LONG_GIANT_KEYS + GIANT_ROW <= LONG_SORT_BINS, "every key is a bin");
__device__ __forceinline__ uint32_t long_row_key(uint32_t len)
{
    if (len > GIANT_ROW) {
        const uint32_t b = 31u - static_cast<uint32_t>(__clz(len));              // 11 .. 31
        const uint32_t cls = (b - 11u) * 64u + ((len >> (b - 6u)) & 63u);      // grows with len
        return LONG_GIANT_KEYS - 1u - cls;
    }
    return LONG_GIANT_KEYS + (GIANT_ROW - len);
}
struct LongRowDigit {
    const uint32_t *len;
    __device__ __forceinline__ uint32_t digit(uint64_t i) const { return long_row_key(len[i]); }
};
struct LongRowPut {
    const uint32_t *len_in, *row_in;
    uint32_t *len_out, *row_out;
    __device__ __forceinline__ void put(uint32_t pos, uint64_t i) const
    {
        len_out[pos] = len_in[i];
        row_out[pos] = row_in[i];
    }
};

// Pieces of sorted long row i at [ppos[i], ppos[i + 1]); the arrival
// counters cleared; the number of rows above GIANT_ROW and of their pieces.
__global__ void k_piece_emit(const uint32_t *__restrict__ off, const uint32_t *__restrict__ long_row,
                             const uint32_t *__restrict__ long_len, const uint32_t *__restrict__ long_total,
                             const uint32_t *__restrict__ ppos, uint4 *__restrict__ work,
                             uint32_t *__restrict__ long_count, uint32_t *__restrict__ giant_total,
                             uint32_t *__restrict__ giant_pieces)
{
    const uint64_t L = *long_total;
    uint64_t lo = 0, hi = L;                       // giant rows come first (lengths decrease)
    while (lo < hi) {
        const uint64_t mid = (lo + hi) / 2;
        if (long_len[mid] > GIANT_ROW) lo = mid + 1; else hi = mid;
    }
    if (gtid() == 0) {
        *giant_total = static_cast<uint32_t>(lo);
        *giant_pieces = ppos[lo];
    }
    for (uint64_t i = gtid(); i < L; i += gthreads()) {
        const uint32_t r = long_row[i];
        uint32_t out = ppos[i], p = off[r];
        long_count[r] = 0;
        for (; p < off[r + 1]; p += SEG_EDGES)
            work[out++] = make_uint4(r, (r + 1) | LONG_FLAG, p, min(p + SEG_EDGES, off[r + 1]));
    }
}

// Short items are cut greedily over windows of 32 rows of rows[0, ne), in
// order: an item ends before a long row (more than seg_long edges) and
// before a row that would take it past SEG_EDGES edges.  A warp takes 32
// consecutive windows: its lanes first load the 1024 rows' lengths and
// first edges together into shared memory (row j of window i at i * 33 + j,
// so that the lanes' walks below hit distinct banks), then lane l walks
// window l from there.
constexpr int SEG_WARPS = 4;
constexpr uint32_t SEG_PAD = 33;
constexpr uint32_t SEG_STAGE = 32 * SEG_PAD;                // words per warp and array

__device__ __forceinline__ void stage_windows(const uint32_t *__restrict__ off, const uint32_t *__restrict__ rows,
                                              uint64_t k0, uint64_t ne, uint32_t *s_d, uint32_t *s_o,
                                              unsigned lane)
{
#pragma unroll 4
    for (uint32_t i = 0; i < 32; i++) {
        const uint64_t k = k0 + i * 32 + lane;
        uint32_t d = 0, o = 0;
        if (k < ne) {
            const uint32_t r = rows[k];
            o = off[r];
            d = off[r + 1] - o;
        }
        s_d[i * SEG_PAD + lane] = d;
        s_o[i * SEG_PAD + lane] = o;
    }
    __syncwarp();
}

// counts[w]: the short items of window w; counts[W + w]: the CONST item of
// window w of rows[ne, N).
__global__ void __launch_bounds__(SEG_WARPS * 32) k_seg_count(const uint32_t *__restrict__ off,
                                                              const uint32_t *__restrict__ rows,
                                                              const uint32_t *__restrict__ ne_dev, uint64_t n,
                                                              uint32_t seg_long, uint32_t *__restrict__ counts)
{
    __shared__ uint32_t s_d[SEG_WARPS * SEG_STAGE], s_o[SEG_WARPS * SEG_STAGE];
    const uint64_t windows = (n + 31) / 32, ne = *ne_dev;
    const unsigned lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    uint32_t *d_w = s_d + wib * SEG_STAGE, *o_w = s_o + wib * SEG_STAGE;
    const uint64_t groups = (windows + 31) / 32, warps = gthreads() >> 5;
    for (uint64_t gi = gtid() >> 5; gi < groups; gi += warps) {
        stage_windows(off, rows, gi * 1024, ne, d_w, o_w, lane);
        const uint64_t w = gi * 32 + lane;
        if (w < windows) {
            const uint64_t k0 = w * 32;
            const uint32_t cnt = k0 < ne ? static_cast<uint32_t>(ne - k0 < 32 ? ne - k0 : 32) : 0u;
            uint32_t items = 0, acc_e = 0, acc_r = 0;
            for (uint32_t j = 0; j < cnt; j++) {
                const uint32_t d = d_w[lane * SEG_PAD + j];
                if (d > seg_long) {                     // long rows go to pieces
                    if (acc_r) { items++; acc_r = 0; acc_e = 0; }
                    continue;
                }
                if (acc_r && acc_e + d > SEG_EDGES) { items++; acc_r = 0; acc_e = 0; }
                acc_r++;
                acc_e += d;
            }
            if (acc_r) items++;
            counts[w] = items;
            counts[windows + w] = k0 < n - ne ? 1u : 0u;
        }
        __syncwarp();
    }
}

// Short items {k0, k1, e0, e1} over rows[k0, k1) (their edges are
// contiguous: rows in between have none); CONST items
// {ne + k0, ne + k1 | CONST, 0, 0}; both after the P pieces.
__global__ void __launch_bounds__(SEG_WARPS * 32) k_seg_emit(const uint32_t *__restrict__ off,
                                                             const uint32_t *__restrict__ rows,
                                                             const uint32_t *__restrict__ ne_dev, uint64_t n,
                                                             uint32_t seg_long, const uint32_t *__restrict__ first,
                                                             const uint32_t *__restrict__ piece_total,
                                                             uint4 *__restrict__ work, uint32_t *__restrict__ tot)
{
    __shared__ uint32_t s_d[SEG_WARPS * SEG_STAGE], s_o[SEG_WARPS * SEG_STAGE];
    const uint64_t windows = (n + 31) / 32, ne = *ne_dev;
    const uint32_t P = *piece_total;
    const unsigned lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    if (gtid() == 0) {
        tot[0] = P + first[windows];
        tot[1] = P + first[2 * windows];
    }
    uint32_t *d_w = s_d + wib * SEG_STAGE, *o_w = s_o + wib * SEG_STAGE;
    const uint64_t groups = (windows + 31) / 32, warps = gthreads() >> 5;
    for (uint64_t gi = gtid() >> 5; gi < groups; gi += warps) {
        stage_windows(off, rows, gi * 1024, ne, d_w, o_w, lane);
        const uint64_t w = gi * 32 + lane;
        if (w < windows) {
            const uint64_t k0 = w * 32;
            const uint32_t cnt = k0 < ne ? static_cast<uint32_t>(ne - k0 < 32 ? ne - k0 : 32) : 0u;
            const uint32_t *dr = d_w + lane * SEG_PAD, *orow = o_w + lane * SEG_PAD;
            uint32_t out = P + first[w];
            uint32_t start = 0, acc_e = 0, acc_r = 0;
            for (uint32_t j = 0; j < cnt; j++) {
                const uint32_t d = dr[j];
                if (d > seg_long) {
                    if (acc_r) {
                        work[out++] = make_uint4(uint32_t(k0 + start), uint32_t(k0 + j), orow[start], orow[j]);
                        acc_r = 0; acc_e = 0;
                    }
                    continue;
                }
                if (acc_r && acc_e + d > SEG_EDGES) {
                    work[out++] = make_uint4(uint32_t(k0 + start), uint32_t(k0 + j), orow[start], orow[j]);
                    acc_r = 0; acc_e = 0;
                }
                if (acc_r == 0) start = j;
                acc_r++;
                acc_e += d;
            }
            if (acc_r)
                work[out++] = make_uint4(uint32_t(k0 + start), uint32_t(k0 + cnt), orow[start],
                                         orow[cnt - 1] + dr[cnt - 1]);
            if (k0 < n - ne) {
                const uint64_t c0 = ne + k0, c1 = min(n, c0 + 32);
                work[P + first[windows + w]] = make_uint4(uint32_t(c0), uint32_t(c1) | CONST_FLAG, 0u, 0u);
            }
        }
        __syncwarp();
    }
}

// The batch rows of k_pr_long_sums: lane l returns the sequential float sum
// of its row's terms vals[beg, beg + len), in row order.  A lane that reads
// its own row strided from the others (one 16-byte load per lane and
// instruction) keeps L1TEX on 32 lines per load: measured on GB300, about
// 88 cycles a term.  Instead the warp stages its 32 rows through a ring of
// BATCH_STAGES stages in shared memory with coalesced 16-byte cp.async
// copies, issued BATCH_STAGES - 1 stages ahead.  Stage c of a row is the
// 16-byte aligned window of BATCH_TERMS floats at (beg & ~3) + c *
// BATCH_TERMS; window positions before beg or past the row's end add +0,
// which leaves the running sum unchanged (it starts at +0 and is never -0:
// x + -x rounds to +0), so the result is the plain loop's, bit for bit.
// Chunks wholly past the row's end are zero-filled without a read; vals[]
// holds 4 floats past the edges, the most a chunk that starts inside the
// row reads beyond it.
constexpr uint32_t BATCH_TERMS = 16;
constexpr uint32_t BATCH_CHUNKS = BATCH_TERMS / 4;          // 16-byte chunks of a row per stage
constexpr uint32_t BATCH_SLOT = BATCH_TERMS + 4;            // padded: conflict-free 16-byte reads
constexpr uint32_t BATCH_STAGES = 3;
constexpr uint32_t BATCH_RING = BATCH_STAGES * 32 * BATCH_SLOT;   // floats per warp
static_assert(BATCH_TERMS % 4 == 0 && 32 % BATCH_CHUNKS == 0, "whole chunks; whole rows per copy");

__device__ __forceinline__ void cp_async16(float *dst, const float *src, uint32_t bytes)
{
    const uint32_t d = static_cast<uint32_t>(__cvta_generic_to_shared(dst));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(src), "r"(bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template<int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Out of line: its registers are allocated apart from the giant-row path's.
__device__ __noinline__ float batch_sequential_sum(const float *vals, uint32_t beg, uint32_t len, float *ring,
                                                   unsigned lane)
{
    constexpr uint32_t ROWS_PER_COPY = 32 / BATCH_CHUNKS;    // rows one copy instruction covers
    constexpr uint32_t COPIES = 32 / ROWS_PER_COPY;          // copy instructions per stage
    const uint32_t end = beg + len, a0 = beg & ~3u;
    const uint32_t stages = (__reduce_max_sync(FULL_MASK, end - a0) + BATCH_TERMS - 1) / BATCH_TERMS;
    // this lane copies chunk `k` of rows i * ROWS_PER_COPY + lane / BATCH_CHUNKS
    const uint32_t k = lane % BATCH_CHUNKS;
    uint32_t cg[COPIES], ce[COPIES];
#pragma unroll
    for (uint32_t i = 0; i < COPIES; i++) {
        const uint32_t r = i * ROWS_PER_COPY + lane / BATCH_CHUNKS;
        cg[i] = (__shfl_sync(FULL_MASK, beg, r) & ~3u) + 4 * k;
        ce[i] = __shfl_sync(FULL_MASK, end, r);
    }
    auto issue = [&](uint32_t c) {
        float *st = ring + (c % BATCH_STAGES) * (32 * BATCH_SLOT);
#pragma unroll
        for (uint32_t i = 0; i < COPIES; i++) {
            const uint32_t r = i * ROWS_PER_COPY + lane / BATCH_CHUNKS, g = cg[i] + c * BATCH_TERMS;
            const bool want = g < ce[i];
            cp_async16(st + r * BATCH_SLOT + 4 * k, want ? vals + g : vals, want ? 16u : 0u);
        }
    };
#pragma unroll 1
    for (uint32_t c = 0; c + 1 < BATCH_STAGES; c++) {
        if (c < stages) issue(c);
        cp_async_commit();
    }
    float acc = 0.0f;
#pragma unroll 1
    for (uint32_t c = 0; c < stages; c++) {
        if (c + BATCH_STAGES - 1 < stages) issue(c + BATCH_STAGES - 1);
        cp_async_commit();
        cp_async_wait<BATCH_STAGES - 1>();           // this lane's copies of stage c are done
        __syncwarp();                                // ... and every lane's
        const float4 *mine = reinterpret_cast<const float4 *>(ring + (c % BATCH_STAGES) * (32 * BATCH_SLOT) +
                                                              lane * BATCH_SLOT);
        float x[BATCH_TERMS];
#pragma unroll
        for (uint32_t q = 0; q < BATCH_CHUNKS; q++) {
            const float4 v = mine[q];
            x[4 * q] = v.x; x[4 * q + 1] = v.y; x[4 * q + 2] = v.z; x[4 * q + 3] = v.w;
        }
        const uint32_t first = a0 + c * BATCH_TERMS;  // row position of the window's first float
        if (first >= beg && first + BATCH_TERMS <= end) {
#pragma unroll
            for (uint32_t t = 0; t < BATCH_TERMS; t++) acc = __fadd_rn(acc, x[t]);
        } else {
#pragma unroll
            for (uint32_t t = 0; t < BATCH_TERMS; t++)
                acc = __fadd_rn(acc, first + t >= beg && first + t < end ? x[t] : 0.0f);
        }
        __syncwarp();                                // the slot is free for stage c + BATCH_STAGES
    }
    cp_async_wait<0>();
    return acc;
}

// One gathered value: from the shared-memory hub cache when the source is
// among the first `hubs` entries, else from global memory.
__device__ __forceinline__ float gather1(const float *__restrict__ src, const float *hub, uint32_t hubs, uint32_t i)
{
    // L2 only: random lines would only evict one another from L1 (measured
    // on GB300: ER(4M, 67M) 278 -> 268 us per iteration; reading the next
    // tier of hubs through L1 instead gained nothing on R-MAT-22)
    return i < hubs ? hub[i] : __ldcg(src + i);
}

// The first iteration's value of source vertex i at edge e, whose slot it
// writes to gat_out[e] (the translated source stream of later iterations).
__device__ __forceinline__ float gather_first(const uint2 *__restrict__ pk, uint32_t *__restrict__ gat_out,
                                              uint32_t i, uint32_t e)
{
    const uint2 p = __ldcg(pk + i);
    __stcs(gat_out + e, p.x);
    return __uint_as_float(p.y);
}

// Gather src[rev_e[e0 + k]] for k in [0, len) (len <= SEG_EDGES) into buf
// (FIRST with pk: the first iteration's values and translation).
template<bool FIRST>
__device__ __forceinline__ void gather_into(const uint32_t *__restrict__ rev_e, const float *__restrict__ src,
                                            const float *hub, uint32_t hubs,
                                            uint32_t e0, uint32_t len, float *buf, unsigned lane,
                                            const uint2 *pk, uint32_t *gat_out)
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
            if (FIRST && pk) v[u] = k < len ? gather_first(pk, gat_out, idx[u], e0 + k) : 0.0f;
            else v[u] = k < len ? gather1(src, hub, hubs, idx[u]) : 0.0f;
        }
#pragma unroll
        for (int u = 0; u < GATHER_UNROLL; u++) {
            const uint32_t k = base + u * 32 + lane;
            if (k < len) buf[k] = v[u];
        }
    }
}

// The sequential sum of vals[b, e) continued from the running sum `sb`
// (warp_sequential_continue_load, bw_seqsum_warp.cuh); `vals` was written by
// the previous kernel, so it is read through L2.
template<uint32_t L>
__device__ __forceinline__ bool warp_sequential_continue(const float *vals, uint32_t b, uint32_t e, uint32_t &sb,
                                                         float *stage, unsigned lane)
{
    return warp_sequential_continue_load<L>([vals](uint32_t i) { return __ldcg(vals + i); }, b, e, sb, stage, lane);
}

// One lane's plain loop over the row (terms outside the maps' domain);
// every lane returns the sum.
__device__ __noinline__ float warp_plain_sum(const float *vals, uint32_t n, unsigned lane)
{
    float s = 0.0f;
    if (lane == 0)
        for (uint32_t i = 0; i < n; i++) s = __fadd_rn(s, __ldcg(vals + i));
    return __shfl_sync(FULL_MASK, s, 0);
}

// --------------- binade-map records of long-row pieces -------------------
// Shared by k_pr_long_sums (vertex-pull, vertex-pull-nodiv: terms staged in
// vals[]) and the fused pull-segmented kernel (terms gathered into the
// warp's shared-memory buffer).
constexpr uint32_t PIECE_L = SEG_EDGES / 32;        // terms per lane: one window per piece
constexpr uint32_t SERIAL_PIECES = SERIAL_TERMS / SEG_EDGES;
static_assert(SERIAL_TERMS % SEG_EDGES == 0, "the serial start covers whole pieces");
static_assert(GIANT_ROW >= SERIAL_TERMS, "giant rows go past the serial start");
// Piece records, two uint4 per piece: r0 = {kind | tg << 8, K | K2 << 8, M1.e, M1.o},
// r1 = {bits of term tg, M2.e, M2.o, 0}
constexpr uint32_t REC_NONE = 0;      // evaluated exactly by the combination
constexpr uint32_t REC_BINADE = 1;    // M1: the piece's terms in binade K
constexpr uint32_t REC_STATE = 2;     // r0.y: the running sum after the serial start
constexpr uint32_t REC_CROSS = 3;     // M1: terms before tg in K; tg crosses into K2; M2: the rest in K2

__device__ __forceinline__ uint32_t atomic_add_acq_rel(uint32_t *p, uint32_t v)
{
    uint32_t old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

// The sum of rv[0, SERIAL_TERMS) in row order: coalesced loads of the whole
// range, then lane 0 adds the terms from shared memory (four per load).
// `stage` is 16-byte aligned and holds 32 x PIECE_L floats.
__device__ __forceinline__ uint32_t warp_serial_start(const float *rv, float *stage, unsigned lane)
{
    constexpr uint32_t HALF = 32 * PIECE_L;
    static_assert(SERIAL_TERMS == 2 * HALF, "the serial start is two stages");
    float v[2][PIECE_L];
#pragma unroll
    for (uint32_t h = 0; h < 2; h++)
#pragma unroll
        for (uint32_t u = 0; u < PIECE_L; u++) v[h][u] = __ldcg(rv + h * HALF + u * 32 + lane);
    float acc = 0.0f;
#pragma unroll
    for (uint32_t h = 0; h < 2; h++) {
#pragma unroll
        for (uint32_t u = 0; u < PIECE_L; u++) stage[u * 32 + lane] = v[h][u];
        __syncwarp();
        if (lane == 0) {
            const float4 *s4 = reinterpret_cast<const float4 *>(stage);
#pragma unroll 8
            for (uint32_t i = 0; i < HALF / 4; i++) {
                const float4 q = s4[i];
                acc = __fadd_rn(acc, q.x); acc = __fadd_rn(acc, q.y);
                acc = __fadd_rn(acc, q.z); acc = __fadd_rn(acc, q.w);
            }
        }
        __syncwarp();
    }
    return __shfl_sync(FULL_MASK, __float_as_uint(acc), 0);
}

// Ordered composition of the lanes' maps; lane 0 ends with all of them.
__device__ __forceinline__ bwseq::Map warp_compose(bwseq::Map m, unsigned lane)
{
#pragma unroll
    for (uint32_t o = 1; o < 32; o <<= 1) {
        const bwseq::Map y{__shfl_down_sync(FULL_MASK, m.e, o), __shfl_down_sync(FULL_MASK, m.o, o)};
        if ((lane & (2 * o - 1)) == 0) m = bwseq::compose(m, y);
    }
    return m;
}

// A lane's PIECE_L maps of terms x in binade K composed as a tree (with
// skip != ~0, the terms at positions first + u <= skip are replaced by +0,
// the identity).
__device__ __forceinline__ bwseq::Map lane_maps(const uint32_t (&x)[PIECE_L], uint32_t K, uint32_t first,
                                                uint32_t skip, bool &good)
{
    using namespace bwseq;
    Map t[PIECE_L];
#pragma unroll
    for (uint32_t u = 0; u < PIECE_L; u++)
        t[u] = step_select(skip == 0xffffffffu || first + u > skip ? x[u] : 0u, K, good);
#pragma unroll
    for (uint32_t st = 1; st < PIECE_L; st <<= 1) {
#pragma unroll
        for (uint32_t u = 0; u + st < PIECE_L; u += 2 * st) t[u] = compose_short(t[u], t[u + st]);
    }
    return saturated(t[0]);
}

// The record of a piece's terms under the guessed running sum `guess` at
// its start (valid in lane 0): lane l holds the piece's terms l * PIECE_L
// .. l * PIECE_L + PIECE_L - 1 (past the piece's end: +0, the identity).
// REC_NONE when the guess or a term is outside the maps' domain.
__device__ __forceinline__ void record_of_terms(const uint32_t (&x)[PIECE_L], uint32_t guess, unsigned lane,
                                                uint4 &r0, uint4 &r1)
{
    using namespace bwseq;
    r0 = make_uint4(REC_NONE, 0u, 0u, 0u);
    r1 = make_uint4(0u, 0u, 0u, 0u);
    if (!in_domain(guess)) return;
    const uint32_t K = exponent_of(guess), first = lane * PIECE_L;
    bool good = true;
    const Map m = lane_maps(x, K, first, 0xffffffffu, good);
    if (__any_sync(FULL_MASK, !good)) return;
    Map incl = m;                                     // lanes' maps scanned
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const Map y{__shfl_up_sync(FULL_MASK, incl.e, o), __shfl_up_sync(FULL_MASK, incl.o, o)};
        if (lane >= static_cast<unsigned>(o)) incl = compose(y, incl);
    }
    Map excl{__shfl_up_sync(FULL_MASK, incl.e, 1), __shfl_up_sync(FULL_MASK, incl.o, 1)};
    if (lane == 0) excl = identity();
    const uint32_t a0 = apply(excl, significand_of(guess)), a1 = apply(m, a0);
    const unsigned cross = __ballot_sync(FULL_MASK, a1 >= TOP);
    if (!cross) {
        r0 = make_uint4(REC_BINADE, K, __shfl_sync(FULL_MASK, incl.e, 31), __shfl_sync(FULL_MASK, incl.o, 31));
        return;
    }
    // the guessed crossing: the first lane whose run leaves the binade finds the term
    const unsigned f = __ffs(cross) - 1;
    uint32_t tg = 0, xb = 0, nb = 0;
    Map pm = identity();
    if (lane == f) {
        uint32_t acc = a0;
        bool found = false;
#pragma unroll
        for (uint32_t u = 0; u < PIECE_L; u++) {
            if (!found) {
                Map st;
                step(x[u], K, st);
                const uint32_t bu = apply(st, acc);
                if (bu >= TOP) {
                    found = true;
                    tg = first + u;
                    xb = x[u];
                    nb = __float_as_uint(__fadd_rn(__uint_as_float(bits_of(K, acc)), __uint_as_float(x[u])));
                } else {
                    acc = bu;
                    pm = compose(pm, st);
                }
            }
        }
    }
    tg = __shfl_sync(FULL_MASK, tg, f);
    xb = __shfl_sync(FULL_MASK, xb, f);
    nb = __shfl_sync(FULL_MASK, nb, f);
    const Map m1 = compose(Map{__shfl_sync(FULL_MASK, excl.e, f), __shfl_sync(FULL_MASK, excl.o, f)},
                           Map{__shfl_sync(FULL_MASK, pm.e, f), __shfl_sync(FULL_MASK, pm.o, f)});
    if (!in_domain(nb)) return;
    const uint32_t K2 = exponent_of(nb);
    const Map m2 = warp_compose(lane_maps(x, K2, first, tg, good), lane);   // the terms after tg
    r0 = make_uint4(REC_CROSS | (tg << 8), K | (K2 << 8), m1.e, m1.o);
    r1 = make_uint4(xb, m2.e, m2.o, 0u);
}

// The record of piece q >= SERIAL_PIECES of a giant row (valid in lane 0).
__device__ __forceinline__ void piece_record(const PrArgs &a, const float *rv, uint32_t n, uint32_t p0, uint32_t q,
                                             float *stage, unsigned lane, uint4 &r0, uint4 &r1)
{
    using namespace bwseq;
    r0 = make_uint4(REC_NONE, 0u, 0u, 0u);
    r1 = make_uint4(0u, 0u, 0u, 0u);
    const uint32_t b = q * SEG_EDGES, len = min(SEG_EDGES, n - b);
    float v[PIECE_L];                                // the terms, coalesced (issued first)
#pragma unroll
    for (uint32_t u = 0; u < PIECE_L; u++) {
        const uint32_t k = u * 32 + lane;
        v[u] = k < len ? __ldcg(rv + b + k) : 0.0f;
    }
    // The guess: the earlier pieces' sums added in float.  Its error (a few
    // ulps) is far below the sequential sum's own drift from the exact sum,
    // and a guess off the true running sum's binade only sends the piece
    // to exact evaluation.  (Adding in double cost more: GB300's FP64 pipe
    // is narrow, and every piece adds all the sums before it.)
    constexpr uint32_t PRE_U = 4;
    float pre = 0.0f;
    for (uint32_t i0 = 0; i0 < q; i0 += 32 * PRE_U) {
        float f[PRE_U];
#pragma unroll
        for (uint32_t k = 0; k < PRE_U; k++) {
            const uint32_t i = i0 + k * 32 + lane;
            f[k] = i < q ? __ldcg(a.piece_sum + p0 + i) : 0.0f;
        }
#pragma unroll
        for (uint32_t k = 0; k < PRE_U; k++) pre += f[k];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) pre += __shfl_xor_sync(FULL_MASK, pre, o);   // same bits in every lane
    // restage so that lane l holds terms l*PIECE_L .. (element k at k + k / 32)
#pragma unroll
    for (uint32_t u = 0; u < PIECE_L; u++) stage[u * 33 + lane] = v[u];
    __syncwarp();
    uint32_t x[PIECE_L];
#pragma unroll
    for (uint32_t u = 0; u < PIECE_L; u++) {
        const uint32_t k = lane * PIECE_L + u;
        x[u] = __float_as_uint(stage[k + (k >> 5)]);   // past the end: +0, the identity
    }
    __syncwarp();
    const uint32_t guess = __float_as_uint(pre);
    record_of_terms(x, guess, lane, r0, r1);
}

// The exact evaluation of piece q from the running sum `sb` (rare: kept
// out of line, so that the kernel's frequent paths stay small in the
// instruction cache).  Returns {ok, new sb}.
__device__ __noinline__ uint2 piece_exact(const float *rv, uint32_t n, uint32_t q, uint32_t sb, float *stage,
                                          unsigned lane)
{
    const uint32_t b = q * SEG_EDGES;
    const bool ok = warp_sequential_continue<PIECE_L>(rv, b, min(n, b + SEG_EDGES), sb, stage, lane);
    return make_uint2(ok ? 1u : 0u, sb);
}

// Piece q from the running sum `sb`: its record when it holds for that sum,
// else the exact evaluation of its terms.  False when a term or the sum
// leaves the maps' domain.
// exact(q, sb) evaluates piece q from sb and returns {ok, new sb}.
template<class Exact>
__device__ __forceinline__ bool piece_advance(uint32_t q, const uint4 &r0, const uint4 &r1, uint32_t &sb, Exact exact)
{
    using namespace bwseq;
    const uint32_t kind = r0.x & 0xffu, K = r0.y & 0xffu;
    if ((kind == REC_BINADE || kind == REC_CROSS) && in_domain(sb) && exponent_of(sb) == K) {
        const uint32_t a1 = apply(Map{r0.z, r0.w}, significand_of(sb));
        if (kind == REC_BINADE && a1 < TOP) {
            sb = bits_of(K, a1);
            return true;
        }
        Map st;
        if (kind == REC_CROSS && a1 < TOP && step(r1.x, K, st) && apply(st, a1) >= TOP) {
            const uint32_t nb = __float_as_uint(__fadd_rn(__uint_as_float(bits_of(K, a1)), __uint_as_float(r1.x)));
            const uint32_t K2 = (r0.y >> 8) & 0xffu;
            if (in_domain(nb) && exponent_of(nb) == K2) {
                const uint32_t a3 = apply(Map{r1.y, r1.z}, significand_of(nb));
                if (a3 < TOP) {
                    sb = bits_of(K2, a3);
                    return true;
                }
            }
        }
    }
    const uint2 r = exact(q, sb);
    sb = r.y;
    return r.x != 0;
}

// The row's sum from the records rec[0 .. pieces) of its pieces (the warp
// of the last piece to finish): rec[0] holds the running sum after the
// serial start (REC_STATE), map records begin at piece `first`.  Groups of
// 32 records: the run of map records in the current sum's binade is
// applied with one scan, up to the first piece it cannot take, which
// piece_advance takes (exact(q, sb) evaluates piece q from sb; plain() is
// the whole row's plain loop, for terms outside the maps' domain).
template<class Exact, class Plain>
__device__ __forceinline__ float combine_records(const uint4 *rec, uint32_t first, uint32_t pieces, unsigned lane,
                                                 Exact exact, Plain plain)
{
    using namespace bwseq;
    uint32_t sb = __ldcg(rec).y;                     // REC_STATE of piece 0
    bool ok = true;
    for (uint32_t g = first; g < pieces && ok; g += 32) {
        const uint32_t cnt = min(32u, pieces - g);
        const uint4 zero = make_uint4(0u, 0u, 0u, 0u);
        const uint4 r0 = lane < cnt ? __ldcg(rec + 2 * (g + lane)) : zero;
        const uint4 r1 = lane < cnt ? __ldcg(rec + 2 * (g + lane) + 1) : zero;
        uint32_t pos = 0;
        while (pos < cnt && ok) {
            const uint32_t K = exponent_of(sb);
            const bool live = lane >= pos && lane < cnt;
            const bool simple = live && in_domain(sb) && (r0.x & 0xffu) == REC_BINADE && (r0.y & 0xffu) == K;
            Map incl = simple ? Map{r0.z, r0.w} : identity();
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const Map y{__shfl_up_sync(FULL_MASK, incl.e, o), __shfl_up_sync(FULL_MASK, incl.o, o)};
                if (lane >= static_cast<unsigned>(o)) incl = compose(y, incl);
            }
            const uint32_t av = apply(incl, significand_of(sb));
            const unsigned stops = __ballot_sync(FULL_MASK, live && (!simple || av >= TOP));
            const uint32_t s = stops ? __ffs(stops) - 1 : cnt;
            if (s > pos) sb = bits_of(K, __shfl_sync(FULL_MASK, av, s - 1));   // pieces pos .. s-1
            if (s >= cnt) break;
            const uint4 q0{__shfl_sync(FULL_MASK, r0.x, s), __shfl_sync(FULL_MASK, r0.y, s),
                           __shfl_sync(FULL_MASK, r0.z, s), __shfl_sync(FULL_MASK, r0.w, s)};
            const uint4 q1{__shfl_sync(FULL_MASK, r1.x, s), __shfl_sync(FULL_MASK, r1.y, s),
                           __shfl_sync(FULL_MASK, r1.z, s), __shfl_sync(FULL_MASK, r1.w, s)};
            ok = piece_advance(g + s, q0, q1, sb, exact);
            pos = s + 1;
        }
    }
    return ok ? __uint_as_float(sb) : plain();
}

// k_pr_long_sums: the records of a giant row whose terms are in vals[].
__device__ __forceinline__ float combine_pieces(const PrArgs &a, const float *rv, uint32_t n, uint32_t p0,
                                                uint32_t pieces, float *stage, unsigned lane)
{
    return combine_records(a.piece_map + 2 * static_cast<uint64_t>(p0), SERIAL_PIECES, pieces, lane,
                           [&](uint32_t q, uint32_t sb) { return piece_exact(rv, n, q, sb, stage, lane); },
                           [&]() { return warp_plain_sum(rv, n, lane); });
}


// FIRST: the div variants' first iteration, which also translates the
// sources when the hub-first order was taken (first_pk; no hub cache then).
template<bool NODIV, int BLOCK, bool FIRST = false>
__global__ void __launch_bounds__(BLOCK, pull_min_blocks(BLOCK)) k_pr_pull_items(PrArgs a)
{
    constexpr int PULL_WARPS = BLOCK / 32;
    resolve_args(a);
    extern __shared__ __align__(16) float smem_f[];
    const unsigned lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint64_t warp = gtid() >> 5, warps = gthreads() >> 5;
    const float *src = NODIV ? (a.gat_in ? a.gat_in : a.pr_in) : a.contrib_in;
    const uint2 *pk = (FIRST && a.slot) ? a.first_pk : nullptr;
    uint32_t *const gat_out = a.gat_e_out;
    const uint32_t *ge = pk ? a.rev_e : a.gat_e;
    const float base_nd = nodiv_base(a.n);
    float *buf = smem_f + wib * PULL_BUF;
    uint32_t *s_end = reinterpret_cast<uint32_t *>(smem_f + PULL_WARPS * PULL_BUF) + wib * 33;
    float *hub = smem_f + PULL_WARPS * (PULL_BUF + 33);
    const uint32_t hubs = pk ? 0u : a.hub_count;       // multiple of 4
    for (uint32_t i = threadIdx.x; i < hubs / 4; i += blockDim.x)
        reinterpret_cast<float4 *>(hub)[i] = __ldg(reinterpret_cast<const float4 *>(src) + i);
    __syncthreads();
    float dsum = 0.0f;
    // the next item's descriptor is loaded one item ahead
    uint4 w_next = warp < a.work_count ? a.work[warp] : make_uint4(0, 0, 0, 0);
    for (uint64_t it = warp; it < a.work_count; it += warps) {
        const uint4 w = w_next;
        if (it + warps < a.work_count) w_next = a.work[it + warps];
        const uint32_t r0 = w.x, r1 = w.y & ROW_MASK, e0 = w.z, e1 = w.w;
        if (w.y & LONG_FLAG) {
            // exact piece: store the gathered terms in edge order (the
            // long-row sums run in k_pr_long_sums after this kernel) and
            // their float sum in any order, from which the pieces of giant
            // rows guess the running sum of the row
            const uint32_t len = e1 - e0;
            float part = 0.0f;
            for (uint32_t base = 0; base < len; base += 32 * GATHER_UNROLL) {
                uint32_t idx[GATHER_UNROLL];
#pragma unroll
                for (int u = 0; u < GATHER_UNROLL; u++) {
                    const uint32_t k = base + u * 32 + lane;
                    idx[u] = k < len ? __ldcs(ge + e0 + k) : 0u;
                }
#pragma unroll
                for (int u = 0; u < GATHER_UNROLL; u++) {
                    const uint32_t k = base + u * 32 + lane;
                    if (k < len) {
                        const float v = (FIRST && pk) ? gather_first(pk, gat_out, idx[u], e0 + k)
                                                      : gather1(src, hub, hubs, idx[u]);
                        __stcg(a.vals + e0 + k, v);
                        part += v;
                    }
                }
            }
            for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(FULL_MASK, part, o);
            if (lane == 0) a.piece_sum[it] = part;   // pieces lead the list: item = piece
            continue;
        }
        // up to 32 rows rows[r0 + l]: lane l owns one; its row end and
        // consolidation inputs are loaded alongside the gathers
        const uint32_t rows = r1 - r0, len = e1 - e0;
        uint32_t row = 0;
        FinishIn fin{0.0f, 0u, 0u};
        if (lane < rows) {
            row = a.rows[r0 + lane];
            fin = finish_load<NODIV>(a, row);
        }
        if (w.y & CONST_FLAG) {                            // no in-edges: the sum is +0
            if (lane < rows) dsum += finish_store<NODIV>(a, row, 0.0f, base_nd, fin);
            continue;
        }
        if (lane < rows) s_end[lane] = a.rev_v[row + 1] - e0;
        gather_into<FIRST>(ge, src, hub, hubs, e0, len, buf, lane, pk, gat_out);
        __syncwarp();
        if (lane < rows) {
            const uint32_t b = lane ? s_end[lane - 1] : 0u, e = s_end[lane];
            float sum = 0.0f;
            for (uint32_t i = b; i < e; i++) sum = __fadd_rn(sum, buf[i]);
            dsum += finish_store<NODIV>(a, row, sum, base_nd, fin);
        }
        __syncwarp();
    }
    add_diff(a.diff, dsum);
}

// Long-row sums of the exact variants (vertex-pull, vertex-pull-nodiv),
// after the iteration's work-list kernel has stored every long row's terms
// in vals[] (edge order) and every piece's float sum in piece_sum[].  Jobs
// are taken in order from a counter (no static share, so a warp that drew a
// long job takes fewer):
//  * first batches of 32 long rows of at most GIANT_ROW terms and similar
//    length, one row per lane (batch_sequential_sum): the longest chains of
//    dependent additions start first.
//  * then the pieces of the rows above GIANT_ROW terms, longest rows
//    first.  Piece 0 adds the row's first SERIAL_TERMS terms in order (one
//    lane, from shared memory).  Every later piece guesses the running sum at its start (the
//    float sums of the pieces before it, added in float) and records, in
//    the guessed binade, the map of its terms -- or, when the guess crosses
//    into the next binade inside the piece, the map of the terms before the
//    crossing term, that term, and the map of the terms after it in the new
//    binade.  The row's last piece to finish combines the records in order,
//    scanning runs of map records with the warp: a record that holds for
//    the true running sum (same binade, crossing where recorded) is applied,
//    any other piece is evaluated exactly from the true running sum
//    (warp_sequential_continue).  The guesses only decide how much work the
//    combination does, never its result.
// Every sum is the reference's sequential loop, bit-identical.  The last
// warp to finish resets the job counters for the next iteration; each
// giant row's combining piece resets the row's arrival counter.
constexpr int LONG_SUM_THREADS = 256;
constexpr int LONG_SUM_BLOCKS_PER_SM = 2;            // registers <= 128
constexpr uint32_t LONG_SUM_WARP_SMEM = BATCH_RING > 33 * PIECE_L ? BATCH_RING : 33 * PIECE_L;   // floats
constexpr size_t LONG_SUM_SMEM = (LONG_SUM_THREADS / 32) * LONG_SUM_WARP_SMEM * sizeof(float);
template<bool NODIV>
__global__ void __launch_bounds__(LONG_SUM_THREADS, LONG_SUM_BLOCKS_PER_SM) k_pr_long_sums(PrArgs a, uint32_t *ctr)
{
    extern __shared__ __align__(16) float long_smem[];   // per warp: the batch ring or a piece's stage
    resolve_args(a);
    const unsigned lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    float *const ring = long_smem + wib * LONG_SUM_WARP_SMEM;
    float *const stage_w = ring;
    const uint32_t L = *a.long_total, G = *a.giant_total, PG = *a.giant_pieces;
    const uint32_t MB = (L - G + 31) / 32;
    const uint32_t jobs = MB + PG;
    const float base_nd = nodiv_base(a.n);
    float dsum = 0.0f;
    for (;;) {
        uint32_t job = 0;
        if (lane == 0) job = atomicAdd(&ctr[0], 1u);
        job = __shfl_sync(FULL_MASK, job, 0);
        if (job >= jobs) break;
        if (job < MB) {
            const uint32_t k = G + job * 32 + lane;
            uint32_t row = 0, beg = 0, len = 0;
            FinishIn fin{0.0f, 0u, 0u};
            if (k < L) {
                row = a.long_rows[k];
                fin = finish_load<NODIV>(a, row);
                beg = a.rev_v[row];
                len = a.rev_v[row + 1] - beg;
            }
            const float sum = batch_sequential_sum(a.vals, beg, len, ring, lane);
            if (k < L) dsum += finish_store<NODIV>(a, row, sum, base_nd, fin);
        } else {
            job -= MB;
            const uint4 w = a.work[job];
            const uint32_t row = w.x, beg = a.rev_v[row], n = a.rev_v[row + 1] - beg;
            const uint32_t q = (w.z - beg) / SEG_EDGES, pieces = (n + SEG_EDGES - 1) / SEG_EDGES, p0 = job - q;
            const float *rv = a.vals + beg;
            uint4 r0 = make_uint4(REC_NONE, 0u, 0u, 0u), r1 = make_uint4(0u, 0u, 0u, 0u);
            if (q == 0) {
                r0 = make_uint4(REC_STATE, warp_serial_start(rv, stage_w, lane), 0u, 0u);
            } else if (q >= SERIAL_PIECES) {
                piece_record(a, rv, n, p0, q, stage_w, lane, r0, r1);
            }
            uint32_t last = 0;
            if (lane == 0) {
                a.piece_map[2 * static_cast<uint64_t>(job)] = r0;
                a.piece_map[2 * static_cast<uint64_t>(job) + 1] = r1;
                last = atomic_add_acq_rel(&a.long_count[row], 1u) + 1 == pieces ? 1u : 0u;
            }
            if (__shfl_sync(FULL_MASK, last, 0)) {
                __syncwarp();                         // orders every lane's reads after lane 0's acquire
                const float total = combine_pieces(a, rv, n, p0, pieces, stage_w, lane);
                if (lane == 0) {
                    dsum += finish_vertex<NODIV>(a, row, total, base_nd);
                    a.long_count[row] = 0;
                }
            }
        }
    }
    add_diff(a.diff, dsum);
    // the last warp out resets the job counter
    if (lane == 0) {
        const uint32_t warps = gridDim.x * (blockDim.x / 32);
        if (atomicAdd(&ctr[1], 1u) + 1 == warps) {
            ctr[0] = 0;
            ctr[1] = 0;
        }
    }
}

// Every rank set to one value (graphs without edges).
__global__ void k_pr_fill(float *__restrict__ ranks, uint64_t n, float value)
{
    for (uint64_t v = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; v < n; v += uint64_t(gridDim.x) * blockDim.x)
        ranks[v] = value;
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
    uint4 *work = nullptr;
    uint32_t *long_count = nullptr;    // arrival counters per long row
    uint32_t *scratch = nullptr;       // every other per-run array (one allocation)
    float *vals = nullptr;             // exact long rows: gathered terms (edge-indexed)
    uint32_t *rows = nullptr;          // rows with in-edges, then rows without
    uint32_t *long_rows = nullptr;     // long rows by decreasing length
    uint32_t *long_total = nullptr;    // device: number of long rows
    uint32_t *giant_total = nullptr;   // device: how many of them exceed GIANT_ROW
    uint32_t *giant_pieces = nullptr;  // device: the pieces of those
    float *piece_sum = nullptr;        // exact pieces: their float sums
    uint4 *piece_map = nullptr;        // giant-row pieces: records (two uint4 each)
    uint32_t *sum_ctr = nullptr;       // k_pr_long_sums' job and finish counters
    const uint32_t *count_all = nullptr;       // device: items in the list
    const uint32_t *count_nonconst = nullptr;  // device: items before the CONST ones
};

struct Geometry { unsigned block, grid; size_t smem; };

Geometry geometry(const bw_context *ctx, int variant, const bw_launch_config *cfg)
{
    Geometry g{256, static_cast<unsigned>(ctx->sm_count) * 8, 0};
    if (variant == PR_PULL_SEGMENTED || variant == PR_VERTEX_PULL || variant == PR_VERTEX_PULL_NODIV) {
        // block_size picks the shape (default WIDE); one resident wave
        g.block = (cfg && cfg->block_size == PULL_NARROW) ? PULL_NARROW : PULL_WIDE;
        g.grid = static_cast<unsigned>(ctx->sm_count) * pull_min_blocks(static_cast<int>(g.block));
        if (cfg && cfg->grid_size) g.grid = cfg->grid_size;
        g.smem = pull_fixed_smem(static_cast<int>(g.block));  // + the hub cache (run_pagerank)
        return g;
    }
    const uint32_t W = (cfg && cfg->warp_size) ? cfg->warp_size : 32;
    const uint32_t C = (cfg && cfg->chunk_size) ? cfg->chunk_size : 32;
    if (cfg && cfg->block_size) g.block = cfg->block_size;
    if (cfg && cfg->grid_size) g.grid = cfg->grid_size;
    // C staged values (push: contributions; pull: accumulators) and C + 1 offsets per virtual warp
    if (variant == PR_VERTEX_PUSH_WARP || variant == PR_VERTEX_PULL_WARP || variant == PR_VERTEX_PULL_WARP_NODIV)
        g.smem = (g.block / W) * (C * 4 + (C + 1) * 4);
    return g;
}

int validate_cfg(const bw_context *ctx, int variant, const bw_launch_config *cfg)
{
    if (!cfg) return BW_OK;
    const bool items = variant == PR_PULL_SEGMENTED || variant == PR_VERTEX_PULL || variant == PR_VERTEX_PULL_NODIV;
    if (items) {
        // work-list kernels: block_size picks the shape, chunk_size the
        // hub-cache entries per block (a multiple of 4)
        if (cfg->block_size && cfg->block_size != PULL_WIDE && cfg->block_size != PULL_NARROW)
            return BW_ERR_INVALID_ARGUMENT;
        if (cfg->chunk_size % 4) return BW_ERR_INVALID_ARGUMENT;
        // warp_size: the long-row threshold, a row of at most it fits an item
        if (cfg->warp_size > SEG_EDGES) return BW_ERR_INVALID_ARGUMENT;
        return BW_OK;
    }
    if (cfg->block_size && (cfg->block_size % 32 || cfg->block_size > 256)) {
        // every other PageRank kernel is built for at most 256 threads, the
        // warp variants for 512
        const bool warp = variant == PR_VERTEX_PUSH_WARP || variant == PR_VERTEX_PULL_WARP ||
                          variant == PR_VERTEX_PULL_WARP_NODIV;
        if (cfg->block_size % 32 || cfg->block_size > (warp ? 512u : 256u)) return BW_ERR_INVALID_ARGUMENT;
    }
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
    if (g->fwd_vertices) {
        // the forward CSR's row lengths are the counts the reference's
        // degree kernels produce, at the cost of one pass over N
        k_row_lengths<<<ctx->sm_count * 4, 256, 0, s>>>(g->fwd_vertices, g->vertex_count, deg);
        ctx->launches++;
        BW_CUDA(cudaGetLastError());
        return BW_OK;
    }
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
        k_count_ids_private<<<ctx->sm_count * 2, 1024, 0, s>>>(g->rev_edges, g->edge_count, 1,
                                                               g->vertex_count, deg);
        break;
    }
    ctx->launches++;
    BW_CUDA(cudaGetLastError());
    return BW_OK;
}

int build_segments(bw_context *ctx, const bw_graph_view *g, uint32_t seg_long, PrRun &run, cudaStream_t s)
{
    const uint64_t n = g->vertex_count, m = g->edge_count;
    if (n > ROW_MASK) return BW_ERR_TOO_LARGE;
    const uint64_t windows = (n + 31) / 32;
    const uint64_t lcap = m / (seg_long + 1) + 1;          // long rows at most
    // Pieces <= M / SEG_EDGES + lcap; short items <= N + W; CONST <= W.
    const uint64_t cap = 2 * windows + n + m / SEG_EDGES + lcap + 16;
    const uint64_t tiles = (n + ROW_TILE - 1) / ROW_TILE;
    // one allocation, 256-byte aligned regions (sizes in words)
    auto al = [](uint64_t w) { return (w + 63) & ~uint64_t(63); };
    uint64_t at = 0;
    const uint64_t o_pe = at; at += al(tiles + 1);
    const uint64_t o_pl = at; at += al(tiles + 1);
    const uint64_t o_lkey0 = at; at += al(lcap);
    const uint64_t o_lkey1 = at; at += al(lcap);
    const uint64_t o_lid0 = at; at += al(lcap);
    const uint64_t o_lid1 = at; at += al(lcap);
    const uint64_t o_pcnt = at; at += al(lcap + 1);
    const uint64_t o_ppos = at; at += al(lcap + 1);
    const uint64_t o_wcnt = at; at += al(2 * windows + 1);
    const uint64_t o_first = at; at += al(2 * windows + 1);
    const uint64_t o_tot = at; at += al(12);   // lengths, giant rows, long-sum counters (tot + 8)
    const uint64_t o_sort = at; at += al(sortk::digit_sort_words<LONG_SORT_BINS>(LONG_SORT_GRID));
    const uint64_t o_part = at; at += al(std::max(sortk::scan_parts(lcap + 1), sortk::scan_parts(2 * windows + 1)));
    BW_CUDA(ctx_malloc_async(ctx, reinterpret_cast<void **>(&run.scratch), at * sizeof(uint32_t), s));
    BW_CUDA(ctx_malloc_async(ctx, reinterpret_cast<void **>(&run.work), cap * sizeof(uint4), s));
    BW_CUDA(ctx_malloc_async(ctx, reinterpret_cast<void **>(&run.long_count), n * sizeof(uint32_t), s));
    BW_CUDA(ctx_malloc_async(ctx, reinterpret_cast<void **>(&run.rows), n * sizeof(uint32_t), s));
    uint32_t *S = run.scratch;
    uint32_t *part_e = S + o_pe, *part_l = S + o_pl, *part = S + o_part;
    uint32_t *pcnt = S + o_pcnt, *ppos = S + o_ppos, *wcnt = S + o_wcnt, *first = S + o_first, *tot = S + o_tot;
    const uint32_t *ne = part_e + tiles;
    run.long_total = part_l + tiles;
    run.giant_total = tot + 2;
    run.sum_ctr = tot + 8;
    run.giant_pieces = tot + 5;
    const unsigned grid = ctx->sm_count * 4;
    // 1. the stable partition of the rows (with / without in-edges) and the
    //    long rows in row order
    k_rows_count<<<static_cast<unsigned>(tiles), sortk::SCAN_THREADS, 0, s>>>(g->rev_vertices, n, seg_long,
                                                                             part_e, part_l);
    sortk::k_scan_parts<<<1, 1024, 0, s>>>(part_e, tiles);
    sortk::k_scan_parts<<<1, 1024, 0, s>>>(part_l, tiles);
    k_rows_partition<<<static_cast<unsigned>(tiles), sortk::SCAN_THREADS, 0, s>>>(
        g->rev_vertices, n, seg_long, part_e, part_l, tiles, run.rows, S + o_lkey0, S + o_lid0);
    // 2. long rows by decreasing length (long_row_key), their pieces in that order
    BW_CUDA((sortk::digit_sort<LONG_SORT_BINS, LONG_SORT_WARPS>(
        LongRowDigit{S + o_lkey0}, LongRowPut{S + o_lkey0, S + o_lid0, S + o_lkey1, S + o_lid1}, lcap,
        run.long_total, LONG_SORT_GRID, S + o_sort, s)));
    const uint32_t *long_len = S + o_lkey1;
    run.long_rows = S + o_lid1;
    k_piece_count<<<grid, 256, 0, s>>>(long_len, run.long_total, lcap, pcnt);
    BW_CUDA(cudaMemsetAsync(pcnt + lcap, 0, sizeof(uint32_t), s));
    BW_CUDA(sortk::scan_exclusive(pcnt, ppos, lcap + 1, part, s));
    k_piece_emit<<<grid, 256, 0, s>>>(g->rev_vertices, run.long_rows, long_len, run.long_total, ppos,
                                      run.work, run.long_count, run.giant_total, run.giant_pieces);
    BW_CUDA(cudaMemsetAsync(run.sum_ctr, 0, 2 * sizeof(uint32_t), s));
    // 3. short and CONST items after the pieces: a warp per 32 windows of
    //    32 rows
    const uint64_t seg_warps = (windows + 31) / 32;
    const unsigned seg_grid = static_cast<unsigned>(
        std::min<uint64_t>((seg_warps + SEG_WARPS - 1) / SEG_WARPS, uint64_t(ctx->sm_count) * 32));
    k_seg_count<<<seg_grid, SEG_WARPS * 32, 0, s>>>(g->rev_vertices, run.rows, ne, n, seg_long, wcnt);
    BW_CUDA(cudaMemsetAsync(wcnt + 2 * windows, 0, sizeof(uint32_t), s));
    BW_CUDA(sortk::scan_exclusive(wcnt, first, 2 * windows + 1, part, s));
    k_seg_emit<<<seg_grid, SEG_WARPS * 32, 0, s>>>(g->rev_vertices, run.rows, ne, n, seg_long, first, ppos + lcap,
                                                  run.work, tot);
    // rows count/partition, two tile scans, sort 4, piece count/scan 3/emit, seg count/scan 3/emit
    ctx->launches += 20;
    BW_CUDA(cudaGetLastError());
    run.count_nonconst = tot;
    run.count_all = tot + 1;
    if (m) {
        // 4 floats past the edges: the batch sums' 16-byte copies (k_pr_long_sums)
        BW_CUDA(ctx_malloc_async(ctx, reinterpret_cast<void **>(&run.vals), (m + 4) * sizeof(float), s));
        const uint64_t pcap = m / SEG_EDGES + lcap + 1;     // pieces at most
        BW_CUDA(ctx_malloc_async(ctx, reinterpret_cast<void **>(&run.piece_map), 2 * pcap * sizeof(uint4), s));
        BW_CUDA(ctx_malloc_async(ctx, reinterpret_cast<void **>(&run.piece_sum), pcap * sizeof(float), s));
    }
    return BW_OK;
}

void free_run(PrRun &run, cudaStream_t s)
{
    if (run.work) cudaFreeAsync(run.work, s);
    if (run.long_count) cudaFreeAsync(run.long_count, s);
    if (run.scratch) cudaFreeAsync(run.scratch, s);
    if (run.vals) cudaFreeAsync(run.vals, s);
    if (run.piece_map) cudaFreeAsync(run.piece_map, s);
    if (run.piece_sum) cudaFreeAsync(run.piece_sum, s);
    if (run.rows) cudaFreeAsync(run.rows, s);
    run = PrRun{};
}

// The long-row sums of one iteration of the work-list variants.
template<bool NODIV>
void launch_long_sums(const bw_context *ctx, const PrArgs &a, cudaStream_t s)
{
    k_pr_long_sums<NODIV><<<ctx->sm_count * LONG_SUM_BLOCKS_PER_SM, LONG_SUM_THREADS, LONG_SUM_SMEM, s>>>(a, a.sum_ctr);
}

// The work-list kernel of the div variants; the first iteration's instance
// translates the sources when first_pk is set.
void launch_pull_items_div(const PrArgs &a, const Geometry &geo, cudaStream_t s)
{
    const size_t smem = geo.smem + a.hub_count * 4;
    if (geo.block == PULL_WIDE) {
        if (a.first_pk) k_pr_pull_items<false, PULL_WIDE, true><<<geo.grid, geo.block, smem, s>>>(a);
        else k_pr_pull_items<false, PULL_WIDE><<<geo.grid, geo.block, smem, s>>>(a);
    } else {
        if (a.first_pk) k_pr_pull_items<false, PULL_NARROW, true><<<geo.grid, geo.block, smem, s>>>(a);
        else k_pr_pull_items<false, PULL_NARROW><<<geo.grid, geo.block, smem, s>>>(a);
    }
}

int launch_iteration(bw_context *ctx, int variant, PrArgs &a, const Geometry &geo, cudaStream_t s)
{
    switch (variant) {
      case PR_EDGE_LIST:
        if (a.hot_dst) k_pr_edge_hot<0><<<ctx->sm_count * 2, HOT_THREADS, HOT_SLOTS * sizeof(float), s>>>(a);
        else k_pr_edge<0><<<geo.grid, geo.block, 0, s>>>(a);
        break;
      case PR_REV_EDGE_LIST: k_pr_edge<1><<<geo.grid, geo.block, 0, s>>>(a); break;
      case PR_STRUCT_EDGE_LIST:
        if (a.hot_pairs) k_pr_edge_hot<2><<<ctx->sm_count * 2, HOT_THREADS, HOT_SLOTS * sizeof(float), s>>>(a);
        else k_pr_edge<2><<<geo.grid, geo.block, 0, s>>>(a);
        break;
      case PR_REV_STRUCT_EDGE_LIST: k_pr_edge<3><<<geo.grid, geo.block, 0, s>>>(a); break;
      case PR_VERTEX_PUSH:
        k_pr_vertex_push<<<geo.grid, geo.block, 0, s>>>(a);
        k_pr_heavy_tiles<0><<<ctx->sm_count * 4, 256, 0, s>>>(a);
        ctx->launches++;
        break;
      case PR_VERTEX_PUSH_WARP:
        k_pr_vertex_push_warp<<<geo.grid, geo.block, geo.smem, s>>>(a);
        k_pr_heavy_tiles<1><<<ctx->sm_count * 4, 256, 0, s>>>(a);
        ctx->launches++;
        break;
      case PR_VERTEX_PULL:
        launch_pull_items_div(a, geo, s);
        launch_long_sums<false>(ctx, a, s);
        ctx->launches++;
        break;
      case PR_VERTEX_PULL_NODIV:
        if (geo.block == PULL_WIDE) k_pr_pull_items<true, PULL_WIDE><<<geo.grid, geo.block, geo.smem + a.hub_count * 4, s>>>(a);
        else k_pr_pull_items<true, PULL_NARROW><<<geo.grid, geo.block, geo.smem + a.hub_count * 4, s>>>(a);
        launch_long_sums<true>(ctx, a, s);
        ctx->launches++;
        break;
      case PR_VERTEX_PULL_WARP:
        k_pr_vertex_pull_warp<false><<<geo.grid, geo.block, geo.smem, s>>>(a);
        k_pr_heavy_tiles<2><<<ctx->sm_count * 4, 256, 0, s>>>(a);
        k_pr_heavy_finish<false><<<ctx->sm_count * 2, 256, 0, s>>>(a);
        ctx->launches += 2;
        break;
      case PR_VERTEX_PULL_WARP_NODIV:
        k_pr_vertex_pull_warp<true><<<geo.grid, geo.block, geo.smem, s>>>(a);
        k_pr_heavy_tiles<3><<<ctx->sm_count * 4, 256, 0, s>>>(a);
        k_pr_heavy_finish<true><<<ctx->sm_count * 2, 256, 0, s>>>(a);
        ctx->launches += 2;
        break;
      case PR_PULL_SEGMENTED:
        // the vertex-pull kernel pair under the variant's own tuned shape
        launch_pull_items_div(a, geo, s);
        launch_long_sums<false>(ctx, a, s);
        ctx->launches++;
        break;
      default: return BW_ERR_UNKNOWN_VARIANT;
    }
    ctx->launches++;
    if (!is_fused(variant)) {
        k_consolidate_div<<<ctx->sm_count * 8, 256, 0, s>>>(a, uses_rowlen(variant) ? 1 : 0);
        ctx->launches++;
    }
    BW_CUDA(cudaGetLastError());
    return BW_OK;
}

// Scratch of the hub-first source order of one run.
struct Relabel {
    uint32_t *slot = nullptr;     // vertex -> position in the gathered array
    uint32_t *gat_e = nullptr;    // reverse-CSR sources as positions
    uint32_t *on = nullptr;       // device: the order was taken
    uint2 *pk = nullptr;          // div: {slot, first contribution} per vertex (the
                                  // first iteration translates the sources)
    void *scratch = nullptr;
};

// Orders vertices by decreasing out-degree class (floor(log2(deg))), stable
// in vertex order, and translates the reverse CSR's sources (one pass over
// M).  Runs after the degrees, inside the timed region.  Unless `force`, a
// one-block kernel decides on the device whether the first `hubs` entries
// would cover at least 5% more of the edges than in vertex order; the slot
// and translation kernels, and every iteration, read that decision.
int build_relabel(bw_context *ctx, const bw_graph_view *g, const uint32_t *deg, uint32_t hubs, bool force,
                  bool first_translates, Relabel &r, cudaStream_t s)
{
    const uint64_t n = g->vertex_count, m = g->edge_count;
    const uint32_t grid = ctx->sm_count * RELABEL_BLOCKS_PER_SM;
    const uint64_t order_words = (n + 63) & ~uint64_t(63);
    const uint64_t sort_words = (sortk::digit_sort_words<RELABEL_BINS>(grid) + 63) & ~uint64_t(63);
    // order, the sort's scratch, three 64-bit coverage counters, the decision
    BW_CUDA(ctx_malloc_async(ctx, &r.scratch, (order_words + sort_words + 8) * sizeof(uint32_t), s));
    BW_CUDA(ctx_malloc_async(ctx, reinterpret_cast<void **>(&r.slot), n * sizeof(uint32_t), s));
    BW_CUDA(ctx_malloc_async(ctx, reinterpret_cast<void **>(&r.gat_e), (m ? m : 1) * sizeof(uint32_t), s));
    if (first_translates) BW_CUDA(ctx_malloc_async(ctx, reinterpret_cast<void **>(&r.pk), n * sizeof(uint2), s));
    uint32_t *order = static_cast<uint32_t *>(r.scratch);
    auto *cov = reinterpret_cast<unsigned long long *>(order + order_words + sort_words);
    r.on = order + order_words + sort_words + 6;
    // vertices by degree class, stable (one counting-sort pass), with their
    // slots (and first-iteration entries) written by the sort itself
    const float init = 1.0f / static_cast<float>(n);        // k_pr_init's 1/N, IEEE single
    BW_CUDA((sortk::digit_sort<RELABEL_BINS, RELABEL_WARPS>(RelabelDigit{deg}, RelabelPut{order, r.slot, r.pk, deg, init},
                                                           n, nullptr, grid, order + order_words, s)));
    ctx->launches += 5;                  // count, three scan launches, scatter
    if (force) {
        BW_CUDA(cudaMemsetAsync(r.on, 1, sizeof(uint32_t), s));
    } else {
        const uint64_t k = std::min<uint64_t>(hubs, n);
        BW_CUDA(cudaMemsetAsync(cov, 0, 3 * sizeof(unsigned long long), s));
        if (k) {
            k_relabel_coverage<<<static_cast<unsigned>((k + 1023) / 1024), 1024, 0, s>>>(deg, order, k, m, cov, r.on);
            ctx->launches++;
        } else {
            BW_CUDA(cudaMemsetAsync(r.on, 0, sizeof(uint32_t), s));
        }
    }
    if (m && !first_translates) {
        k_relabel_edges<<<ctx->sm_count * 8, 256, 0, s>>>(g->rev_edges, m, r.on, r.slot, r.gat_e);
        ctx->launches++;
    }
    BW_CUDA(cudaGetLastError());
    return BW_OK;
}

void free_relabel(Relabel &r, cudaStream_t s)
{
    if (r.scratch) cudaFreeAsync(r.scratch, s);
    if (r.slot) cudaFreeAsync(r.slot, s);
    if (r.gat_e) cudaFreeAsync(r.gat_e, s);
    if (r.pk) cudaFreeAsync(r.pk, s);
    r = Relabel{};
}

// Runs a (possibly switching) schedule of variants of one semantics class.
// A graph without edges (its edge arrays may be null): every in-sum is +0
// and every out-degree 0, so every iteration gives each vertex the same
// rank, consolidateRank's (float)((1 - d) / N + (double)(d * 0))
// (pagerank/pagerank.cu:125-140) or consolidateRankNoDiv's
// (1 - d) / (float)N + d * 0 (pagerank/pagerank.cu:142-165), and the
// first iteration's diff is N |rank - 1/N|.  Computed on the host in IEEE
// single and double arithmetic, bit-identical to the device's
// consolidation; one fill kernel writes the ranks.
int run_edgeless(bw_context *ctx, uint64_t n, bool nodiv, uint32_t iterations, float *ranks, int time_iterations,
                 float *iteration_ms, bw_pagerank_result *result, float *diffs_host, cudaStream_t s)
{
    const float init = 1.0f / static_cast<float>(n);
    const float value = iterations == 0 ? init
                        : nodiv ? (1.0f - DAMPING) / static_cast<float>(n)
                                : static_cast<float>((1.0 - static_cast<double>(DAMPING)) / static_cast<double>(n));
    BW_CUDA(cudaEventRecord(ctx->ev_start, s));
    k_pr_fill<<<ctx->sm_count * 4, 256, 0, s>>>(ranks, n, value);
    BW_CUDA(cudaGetLastError());
    BW_CUDA(cudaEventRecord(ctx->ev_stop, s));
    BW_CUDA(cudaEventSynchronize(ctx->ev_stop));
    const float first = static_cast<float>(static_cast<double>(n) * std::fabs(static_cast<double>(value) - init));
    if (diffs_host)
        for (uint32_t j = 0; j < iterations; j++) diffs_host[j] = j == 0 ? first : 0.0f;
    if (time_iterations && iteration_ms)
        for (uint32_t j = 0; j < iterations; j++) iteration_ms[j] = 0.0f;
    if (result) {
        float ms = 0.0f;
        BW_CUDA(cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop));
        result->iterations = iterations;
        result->kernel_launches = 1;
        result->last_diff = iterations == 0 ? 0.0f : iterations == 1 ? first : 0.0f;
        result->device_ms = ms;
    }
    return BW_OK;
}

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
    bool need_exact = false, need_heavy = false, any_rowlen = false, any_deg = false,
         all_items = true, hot_el = false, hot_st = false;
    for (uint32_t i = 0; i < schedule_len; i++) {
        const int v = schedule[i];
        all_items = all_items && (v == PR_VERTEX_PULL || v == PR_VERTEX_PULL_NODIV || v == PR_PULL_SEGMENTED);
        if (v < 0 || v >= PR_VARIANT_COUNT) return BW_ERR_UNKNOWN_VARIANT;
        if (is_nodiv(v) != nodiv) return BW_ERR_INVALID_ARGUMENT;
        BW_TRY(validate_cfg(ctx, v, cfg));
        reps |= kPrReps[v];
        if (v == PR_PULL_SEGMENTED || v == PR_VERTEX_PULL || v == PR_VERTEX_PULL_NODIV) need_exact = true;
        if (v == PR_VERTEX_PUSH || v == PR_VERTEX_PUSH_WARP || v == PR_VERTEX_PULL_WARP ||
            v == PR_VERTEX_PULL_WARP_NODIV)
            need_heavy = true;
        if (uses_rowlen(v)) any_rowlen = true; else any_deg = true;
        if (v == PR_EDGE_LIST) hot_el = true;
        if (v == PR_STRUCT_EDGE_LIST) hot_st = true;
    }
    if (g->edge_count == 0) {
        if (!g->fwd_vertices && !g->rev_vertices) return BW_ERR_MISSING_REPRESENTATION;
        return run_edgeless(ctx, g->vertex_count, nodiv, iterations, ranks, time_iterations, iteration_ms, result,
                            diffs_host, as_stream(stream));
    }
    BW_TRY(check_reps(g, reps));
    if (any_rowlen && any_deg && !g->fwd_vertices) return BW_ERR_MISSING_REPRESENTATION;
    cudaStream_t s = as_stream(stream);
    const uint64_t n = g->vertex_count;
    BW_TRY(ensure_pr_scratch(ctx, n, iterations));
    ctx->launches = 0;
    if (time_iterations) BW_TRY(ensure_level_events(ctx, iterations + 1));

    PrRun exact_run;
    // the long-row threshold: warp_size of the work-list variants' launch
    // configuration (0: SEG_LONG), rows up to it summed in the work-list kernel
    const uint32_t seg_long = (cfg && cfg->warp_size) ? cfg->warp_size : SEG_LONG;
    if (need_exact) BW_TRY(build_segments(ctx, g, seg_long, exact_run, s));
    // heavy-unit tiles of the push and warp-pull variants
    uint4 *heavy_q = nullptr;
    uint32_t *heavy_small = nullptr;                 // 8 counters, then the chunk list
    const uint32_t chunk_c = (cfg && cfg->chunk_size) ? cfg->chunk_size : 32;
    const uint64_t heavy_cap = g->edge_count / HEAVY_TILE + g->edge_count / PUSH_GIANT + 2;
    if (need_heavy) {
        BW_CUDA(ctx_malloc_async(ctx, reinterpret_cast<void **>(&heavy_q), heavy_cap * sizeof(uint4), s));
        BW_CUDA(ctx_malloc_async(ctx, reinterpret_cast<void **>(&heavy_small),
                                 (8 + n / chunk_c + 1) * sizeof(uint32_t), s));
        BW_CUDA(cudaMemsetAsync(heavy_small, 0, 8 * sizeof(uint32_t), s));
    }

    PrArgs a{};
    a.fwd_v = g->fwd_vertices; a.fwd_e = g->fwd_edges; a.rev_v = g->rev_vertices; a.rev_e = g->rev_edges;
    a.fwd_in = g->fwd_in_edges; a.rev_in = g->rev_in_edges;
    a.fwd_s = reinterpret_cast<const uint2 *>(g->fwd_struct_edges);
    a.rev_s = reinterpret_cast<const uint2 *>(g->rev_struct_edges);
    a.n = n; a.m = g->edge_count;
    a.base_div = (1.0 - static_cast<double>(0.85f)) / static_cast<double>(n);
    a.deg = ctx->pr_deg;
    a.acc = ctx->pr_acc;
    a.gat_e = g->rev_edges;
    if (need_exact) {
        BW_CUDA(cudaFuncSetAttribute(k_pr_long_sums<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     static_cast<int>(LONG_SUM_SMEM)));
        BW_CUDA(cudaFuncSetAttribute(k_pr_long_sums<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     static_cast<int>(LONG_SUM_SMEM)));
        // hub cache entries per block: chunk_size when given, else the
        // default for the shape; never more than the block's share of
        // shared memory allows
        const int block = (cfg && cfg->block_size == PULL_NARROW) ? PULL_NARROW : PULL_WIDE;
        const uint64_t per_sm = static_cast<uint64_t>(pull_min_blocks(block));
        const size_t fixed = pull_fixed_smem(block);
        const size_t share = std::min<size_t>(ctx->max_smem_optin, ctx->max_smem_per_sm / per_sm);
        const uint64_t room = share > fixed + 1024 ? (share - fixed - 1024) / sizeof(float) : 0;
        const uint64_t want = (cfg && cfg->chunk_size) ? cfg->chunk_size
                                                       : (block == PULL_WIDE ? PULL_WIDE_HUBS : PULL_NARROW_HUBS);
        a.hub_count = static_cast<uint32_t>(std::min<uint64_t>(std::min<uint64_t>(n, room), want)) & ~3u;
        const int bytes = static_cast<int>(fixed + a.hub_count * sizeof(float));
        if (block == PULL_WIDE) {
            BW_CUDA(cudaFuncSetAttribute(k_pr_pull_items<false, PULL_WIDE>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
            BW_CUDA(cudaFuncSetAttribute(k_pr_pull_items<false, PULL_WIDE, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
            BW_CUDA(cudaFuncSetAttribute(k_pr_pull_items<true, PULL_WIDE>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        } else {
            BW_CUDA(cudaFuncSetAttribute(k_pr_pull_items<false, PULL_NARROW>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
            BW_CUDA(cudaFuncSetAttribute(k_pr_pull_items<false, PULL_NARROW, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
            BW_CUDA(cudaFuncSetAttribute(k_pr_pull_items<true, PULL_NARROW>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        }
    }
    a.warp_size = (cfg && cfg->warp_size) ? cfg->warp_size : 32;
    a.chunk_size = (cfg && cfg->chunk_size) ? cfg->chunk_size : 32;
    a.heavy_q = heavy_q;
    a.heavy_ctr = heavy_small;
    a.heavy_chunks = heavy_small ? heavy_small + 8 : nullptr;
    a.heavy_cap = static_cast<uint32_t>(heavy_cap);

    BW_CUDA(cudaEventRecord(ctx->ev_start, s));
    // Degrees inside the timed region, as pagerank/pagerank.cpp:102-112.
    BW_TRY(launch_degrees(ctx, g, schedule[0], ctx->pr_deg, s));
    if (any_rowlen && any_deg) {
        // mixed schedule: make the degree buffer valid for every variant
        k_row_lengths<<<ctx->sm_count * 4, 256, 0, s>>>(g->fwd_vertices, n, ctx->pr_deg);
        ctx->launches++;
    }
    BW_CUDA(cudaMemsetAsync(ctx->pr_diffs, 0, (iterations + 1) * sizeof(float), s));
    Relabel rl;
    const uint32_t flags = cfg ? cfg->flags : 0u;
    const bool force = (flags & BW_LAUNCH_RELABEL) != 0;
    bool relabel = false;                 // may be taken (the device decides)
    if (all_items && g->edge_count > 0 && !(flags & BW_LAUNCH_NO_RELABEL) &&
        (force || (iterations >= 4 && a.hub_count > 0))) {
        // div: the first iteration translates the sources itself
        const int rc = build_relabel(ctx, g, ctx->pr_deg, a.hub_count, force, !nodiv, rl, s);
        if (rc != BW_OK) {
            free_relabel(rl, s);
            free_run(exact_run, s);
            return rc;
        }
        relabel = true;
        a.slot = rl.slot;
        a.gat_e = rl.gat_e;
        a.gat_e_out = rl.gat_e;
        a.relabel_on = rl.on;
    }
    // forward edge lists: the hot destinations' slots and the rewritten
    // destination stream, once per run (inside the timed region)
    uint32_t *hot_buf = nullptr, *hot_dst_buf = nullptr;
    uint2 *hot_pairs_buf = nullptr;
    if ((hot_el || hot_st) && n < HOT_BIT) {
        BW_CUDA(cudaFuncSetAttribute(k_pr_edge_hot<0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     static_cast<int>(HOT_SLOTS * sizeof(float))));
        BW_CUDA(cudaFuncSetAttribute(k_pr_edge_hot<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     static_cast<int>(HOT_SLOTS * sizeof(float))));
        uint32_t *indeg = nullptr;
        BW_CUDA(ctx_malloc_async(ctx, reinterpret_cast<void **>(&hot_buf),
                                 (2 * n + HOT_SLOTS + 64) * sizeof(uint32_t), s));
        indeg = hot_buf;
        uint32_t *slot_of = hot_buf + n, *hot_vertex = hot_buf + 2 * n, *bins = hot_buf + 2 * n + HOT_SLOTS;
        const unsigned grid = ctx->sm_count * 4;
        if (g->rev_vertices) {
            k_row_lengths<<<grid, 256, 0, s>>>(g->rev_vertices, n, indeg);      // in-degrees
        } else {
            BW_CUDA(cudaMemsetAsync(indeg, 0, n * sizeof(uint32_t), s));
            if (hot_el) k_count_ids<<<grid * 2, 256, 0, s>>>(g->fwd_edges, g->edge_count, 1, indeg);
            else k_count_ids<<<grid * 2, 256, 0, s>>>(g->fwd_struct_edges + 1, g->edge_count, 2, indeg);
        }
        BW_CUDA(cudaMemsetAsync(bins, 0, 64 * sizeof(uint32_t), s));
        k_hot_classes<<<grid, 256, 0, s>>>(indeg, n, bins);
        k_hot_pick<<<1, 32, 0, s>>>(bins);
        k_hot_assign<<<grid, 256, 0, s>>>(indeg, n, bins, slot_of, hot_vertex);
        ctx->launches += 4;
        if (hot_el) {
            BW_CUDA(ctx_malloc_async(ctx, reinterpret_cast<void **>(&hot_dst_buf), g->edge_count * sizeof(uint32_t), s));
            k_hot_translate<false><<<grid * 2, 256, 0, s>>>(g->fwd_edges, nullptr, g->edge_count, slot_of,
                                                             hot_dst_buf, nullptr);
            ctx->launches++;
            a.hot_dst = hot_dst_buf;
        }
        if (hot_st) {
            BW_CUDA(ctx_malloc_async(ctx, reinterpret_cast<void **>(&hot_pairs_buf), g->edge_count * sizeof(uint2), s));
            k_hot_translate<true><<<grid * 2, 256, 0, s>>>(nullptr, a.fwd_s, g->edge_count, slot_of, nullptr,
                                                            hot_pairs_buf);
            ctx->launches++;
            a.hot_pairs = hot_pairs_buf;
        }
        a.hot_vertex = hot_vertex;
        a.hot_count = bins + 34;
        BW_CUDA(cudaGetLastError());
    }
    // nodiv + relabelled sources: the gathered copy of the ranks, in slot order
    float *gat[2] = {ctx->pr_buf[1], ctx->pr_acc};
    const bool nodiv_gat = nodiv && relabel;

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
                                                 nodiv_gat ? gat[0] : nullptr, first_rowlen);
    ctx->launches++;
    BW_CUDA(cudaGetLastError());

    // loop_mode 1: the iterations are captured (on a private stream: the
    // caller's may be the legacy default stream, which cannot capture) into
    // one CUDA graph that is then launched once on the caller's stream; the
    // launches and their order are the same
    cudaGraph_t loop_graph = nullptr;
    cudaStream_t ls = s;
    // BW_LAUNCH_L2_WINDOW: the gathered vector persisting in L2 (div: both
    // contribution buffers; nodiv: the rank buffers it gathers from)
    L2Window win, win_ls;
    const bool l2w = cfg && (cfg->flags & BW_LAUNCH_L2_WINDOW);
    const void *l2_base = nodiv ? static_cast<const void *>(nb[0] < nb[1] ? nb[0] : nb[1])
                                : static_cast<const void *>(ctx->pr_buf[0]);
    const size_t l2_bytes = nodiv ? n * sizeof(float)
                                  : static_cast<size_t>(ctx->pr_buf[1] - ctx->pr_buf[0] + n) * sizeof(float);
    if (l2w) BW_TRY(l2_window_begin(ctx, s, l2_base, l2_bytes, win));
    if (loop_mode == 1) {
        BW_CUDA(cudaStreamCreateWithFlags(&ls, cudaStreamNonBlocking));
        if (l2w) {
            const int rc = l2_window_begin(ctx, ls, l2_base, l2_bytes, win_ls, false);
            if (rc != BW_OK) { cudaStreamDestroy(ls); return rc; }
        }
        const cudaError_t e = cudaStreamBeginCapture(ls, cudaStreamCaptureModeRelaxed);
        if (e != cudaSuccess) {
            cudaStreamDestroy(ls);
            BW_CUDA(e);
        }
    }
    int loop_status = BW_OK;
    for (uint32_t j = 1; j <= iterations && loop_status == BW_OK; j++) {
        const int v = schedule[std::min<uint32_t>(j - 1, schedule_len - 1)];
        if (time_iterations) BW_CUDA(cudaEventRecord(ctx->level_events[j - 1], ls));
        a.not_last = iterations > j ? 1 : 0;
        a.diff = ctx->pr_diffs + (j - 1);
        a.first_pk = j == 1 ? rl.pk : nullptr;
        if (nodiv) {
            a.pr_in = nb[(j - 1) & 1];
            a.pr_out = nb[j & 1];
            if (nodiv_gat) {
                a.gat_in = gat[(j - 1) & 1];
                a.gat_out = gat[j & 1];
            }
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
        const PrRun &items = exact_run;
        a.work = items.work;
        a.long_count = items.long_count;
        a.vals = items.vals;
        a.rows = items.rows;
        a.long_rows = items.long_rows;
        a.long_total = items.long_total;
        a.giant_total = items.giant_total;
        a.giant_pieces = items.giant_pieces;
        a.piece_sum = items.piece_sum;
        a.piece_map = items.piece_map;
        a.sum_ctr = items.sum_ctr;
        // div: rows without in-edges hold the same rank and contribution in
        // both buffers once iterations 1 and 2 have written them
        a.count_dev = items.work ? ((!nodiv && j > 2) ? items.count_nonconst : items.count_all) : nullptr;
        Geometry geo = geometry(ctx, v, cfg);
        loop_status = launch_iteration(ctx, v, a, geo, ls);
    }
    if (loop_mode == 1) {
        const cudaError_t e = cudaStreamEndCapture(ls, &loop_graph);
        l2_window_end(win_ls);
        cudaStreamDestroy(ls);
        if (loop_status == BW_OK && e != cudaSuccess) {
            set_last_error(e, "cudaStreamEndCapture");
            loop_status = BW_ERR_CUDA;
        }
        if (loop_status == BW_OK) {
            cudaGraphExec_t exec = nullptr;
            cudaError_t le = cudaGraphInstantiate(&exec, loop_graph, 0);
            if (le == cudaSuccess) le = cudaGraphLaunch(exec, s);
            if (exec) cudaGraphExecDestroy(exec);
            if (le != cudaSuccess) {
                set_last_error(le, "PageRank iteration graph");
                loop_status = BW_ERR_CUDA;
            }
        }
        if (loop_graph) cudaGraphDestroy(loop_graph);
    }
    BW_TRY(loop_status);
    if (time_iterations) BW_CUDA(cudaEventRecord(ctx->level_events[iterations], s));
    BW_CUDA(cudaEventRecord(ctx->ev_stop, s));
    float diffs_dev_last = 0.0f;
    if (diffs_host && iterations)
        BW_CUDA(cudaMemcpyAsync(diffs_host, ctx->pr_diffs, iterations * sizeof(float), cudaMemcpyDeviceToHost, s));
    if (iterations)
        BW_CUDA(cudaMemcpyAsync(&diffs_dev_last, ctx->pr_diffs + iterations - 1, sizeof(float),
                                cudaMemcpyDeviceToHost, s));
    BW_CUDA(cudaStreamSynchronize(s));
    free_run(exact_run, s);
    free_relabel(rl, s);
    if (heavy_q) cudaFreeAsync(heavy_q, s);
    if (heavy_small) cudaFreeAsync(heavy_small, s);
    if (hot_buf) cudaFreeAsync(hot_buf, s);
    if (hot_dst_buf) cudaFreeAsync(hot_dst_buf, s);
    if (hot_pairs_buf) cudaFreeAsync(hot_pairs_buf, s);
    if (time_iterations && iteration_ms) {
        for (uint32_t j = 0; j < iterations; j++)
            BW_CUDA(cudaEventElapsedTime(&iteration_ms[j], ctx->level_events[j], ctx->level_events[j + 1]));
    }
    if (result) {
        float ms = 0.0f;
        BW_CUDA(cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop));
        result->iterations = iterations;
        result->kernel_launches = ctx->launches;
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

}  // extern "C"

// A schedule run in either loop mode, with the per-iteration diffs (the
// learned PageRank run's entry).
int bw::pagerank_run_schedule_loop(bw_context *ctx, const bw_graph_view *g, const int32_t *schedule,
                                   uint32_t schedule_len, uint32_t iterations, float *ranks, int loop_mode,
                                   bw_pagerank_result *result, float *diffs, cudaStream_t stream)
{
    return run_pagerank(ctx, g, schedule, schedule_len, iterations, ranks, nullptr, loop_mode, 0, nullptr, result,
                        diffs, stream);
}

extern "C" {

int bw_pagerank_run_schedule(bw_context *ctx, const bw_graph_view *g, const int32_t *schedule,
                             uint32_t schedule_len, uint32_t iterations, float *ranks,
                             const bw_launch_config *cfg, int time_iterations,
                             float *iteration_ms, bw_pagerank_result *result, void *stream)
{
    return run_pagerank(ctx, g, schedule, schedule_len, iterations, ranks, cfg, BW_LOOP_HOST,
                        time_iterations, iteration_ms, result, nullptr, stream);
}

}  // extern "C"
