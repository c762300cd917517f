// BFS level kernels.  One template per reference kernel family
// (bfs/edgelist.cu, rev_edgelist.cu, struct_edgelist.cu,
// rev_struct_edgelist.cu, vertex_push.cu, vertex_pull.cu,
// vertex_push_warp.cu, vertex_pull_warp.cu), parameterised on the
// frontier-count reduction of bfs/bfs.hpp:32-116 and on SIDE (emit the next
// frontier queue and the frontier statistics, needed when levels of
// different variants follow each other), plus the GB300 variants
// frontier-push and frontier-pull.
//
// Every variant computes the same level relation (exact BFS depths): a
// vertex at `depth` gives each unvisited out-neighbour depth + 1, and the
// frontier counter counts each newly visited vertex exactly once.
#pragma once

#include <cooperative_groups.h>
#include "bw_internal.cuh"

namespace bw {
namespace cg = cooperative_groups;

enum Reduction { RED_NORMAL = 0, RED_BULK = 1, RED_WARP = 2, RED_BLOCK = 3 };
enum EdgeLayout { FWD_SOA = 0, REV_SOA = 1, FWD_AOS = 2, REV_AOS = 3 };

// Hub handling of frontier-push: vertices above HEAVY_DEGREE edges are cut
// into HUB_CHUNK-edge chunks that any warp of a second kernel can take.
constexpr uint32_t HEAVY_DEGREE = 256;
constexpr uint32_t HUB_CHUNK = 256;

__device__ __forceinline__ int level_depth(const BfsArgs &a)
{ return a.depth >= 0 ? a.depth : *((volatile int32_t *) &a.ctl->depth); }

__device__ __forceinline__ void reset_slot(LevelSlot *s)
{
    s->frontier = 0; s->qlen = 0; s->fedges = 0; s->lsum = 0.f; s->lsq = 0.f;
    s->lmax_bits = 0; s->heavy = 0;
}

// Frontier counter with the four reference strategies
// (bfs/bfs.hpp:32-116).  finish() must be reached by every thread.
template<int RED>
struct Counter {
    uint32_t c = 0;
    __device__ __forceinline__ void hit(uint32_t *g)
    {
        if constexpr (RED == RED_NORMAL) atomicAdd(g, 1u);
        else c++;
    }
    __device__ __forceinline__ void finish(uint32_t *g)
    {
        if constexpr (RED == RED_BULK) {
            if (c) atomicAdd(g, c);
        } else if constexpr (RED == RED_WARP) {
            uint32_t s = __reduce_add_sync(FULL_MASK, c);
            if ((threadIdx.x & 31) == 0 && s) atomicAdd(g, s);
        } else if constexpr (RED == RED_BLOCK) {
            __shared__ uint32_t part[32];
            const unsigned lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
            uint32_t s = __reduce_add_sync(FULL_MASK, c);
            if (lane == 0) part[wid] = s;
            __syncthreads();
            if (wid == 0) {
                s = lane < (blockDim.x >> 5) ? part[lane] : 0u;
                s = __reduce_add_sync(FULL_MASK, s);
                if (lane == 0 && s) atomicAdd(g, s);
            }
        }
    }
};

// Warp-aggregated append of `v` to a queue; safe in divergent code.
__device__ __forceinline__ void queue_append(uint32_t *q, uint32_t *len, uint32_t v)
{
    cg::coalesced_group g = cg::coalesced_threads();
    uint32_t base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(len, g.size());
    base = g.shfl(base, 0);
    q[base + g.thread_rank()] = v;
}

// Side outputs: next frontier queue + frontier degree statistics.
template<bool SIDE>
struct Side {
    unsigned long long fe = 0;
    float ls = 0.f, lq = 0.f, lm = 0.f;
    __device__ __forceinline__ void visit(const BfsArgs &a, uint32_t *qnext, LevelSlot *s, uint32_t v)
    {
        if constexpr (SIDE) {
            if (qnext) queue_append(qnext, &s->qlen, v);   // null: statistics only
            const uint32_t d = a.outdeg[v];
            const float l = __log2f(1.0f + static_cast<float>(d));
            fe += d; ls += l; lq += l * l; lm = fmaxf(lm, l);
        }
    }
    __device__ __forceinline__ void finish(LevelSlot *s)
    {
        if constexpr (SIDE) {
            for (int o = 16; o > 0; o >>= 1) {
                fe += __shfl_xor_sync(FULL_MASK, fe, o);
                ls += __shfl_xor_sync(FULL_MASK, ls, o);
                lq += __shfl_xor_sync(FULL_MASK, lq, o);
                lm = fmaxf(lm, __shfl_xor_sync(FULL_MASK, lm, o));
            }
            if ((threadIdx.x & 31) == 0 && fe) {
                atomicAdd(&s->fedges, fe);
                atomicAdd(&s->lsum, ls);
                atomicAdd(&s->lsq, lq);
                atomicMax(&s->lmax_bits, __float_as_uint(lm));
            }
        }
    }
};

// Relax v to nd; true for exactly one caller per newly visited vertex.
// The plain pre-check only filters: a stale read can only be INF or nd.
__device__ __forceinline__ bool relax(int32_t *levels, uint32_t v, int32_t nd)
{
    return levels[v] > nd && atomicMin(&levels[v], nd) > nd;
}

// Warp-reduce an out-edge count into slot->fedges (every lane must call).
__device__ __forceinline__ void flush_edges(LevelSlot *s, unsigned long long fe)
{
    for (int o = 16; o > 0; o >>= 1) fe += __shfl_xor_sync(FULL_MASK, fe, o);
    if ((threadIdx.x & 31) == 0 && fe) atomicAdd(&s->fedges, fe);
}

__device__ __forceinline__ uint64_t gtid()
{ return blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; }
__device__ __forceinline__ uint64_t gthreads()
{ return uint64_t(gridDim.x) * blockDim.x; }

// ---------------------------------------------------------------------------
// Edge-list families (bfs/edgelist.cu:3-22, rev_edgelist.cu:3-21,
// struct_edgelist.cu:3-22, rev_struct_edgelist.cu:3-22).  Every level
// streams all M edges; edges are read 4 per thread with 16-byte streaming
// loads (evict-first, so the depth array keeps L2).  The reverse families
// test the sequential destination first, which skips the random source
// gather for already-visited destinations.
// ---------------------------------------------------------------------------
template<int RED, bool SIDE, int LAYOUT>
__global__ void __launch_bounds__(512) k_bfs_edge(BfsArgs a)
{
    const int32_t depth = level_depth(a), nd = depth + 1;
    LevelSlot *slot = &a.ctl->slot[depth % 3];
    if (blockIdx.x == 0 && threadIdx.x == 0) reset_slot(&a.ctl->slot[(depth + 1) % 3]);
    uint32_t *qnext = (depth & 1) ? a.q0 : a.q1;
    int32_t *lv = a.levels;
    Counter<RED> cnt;
    Side<SIDE> side;

    auto edge = [&](uint32_t row, uint32_t col) {
        // FWD: row = source, col = destination.  REV: row = destination,
        // col = source.
        if constexpr (LAYOUT == FWD_SOA || LAYOUT == FWD_AOS) {
            if (lv[row] == depth && relax(lv, col, nd)) { cnt.hit(&slot->frontier); side.visit(a, qnext, slot, col); }
        } else {
            if (lv[row] > nd && lv[col] == depth && atomicMin(&lv[row], nd) > nd) {
                cnt.hit(&slot->frontier);
                side.visit(a, qnext, slot, row);
            }
        }
    };

    const uint64_t m = a.m;
    bool aligned;
    if constexpr (LAYOUT == FWD_SOA) aligned = !((reinterpret_cast<uintptr_t>(a.fwd_in) | reinterpret_cast<uintptr_t>(a.fwd_e)) & 15);
    else if constexpr (LAYOUT == REV_SOA) aligned = !((reinterpret_cast<uintptr_t>(a.rev_in) | reinterpret_cast<uintptr_t>(a.rev_e)) & 15);
    else if constexpr (LAYOUT == FWD_AOS) aligned = !(reinterpret_cast<uintptr_t>(a.fwd_s) & 15);
    else aligned = !(reinterpret_cast<uintptr_t>(a.rev_s) & 15);
    const uint64_t groups = aligned ? m >> 2 : 0;
    const uint64_t stride = gthreads();
    for (uint64_t g = gtid(); g < groups; g += stride) {
        if constexpr (LAYOUT == FWD_SOA || LAYOUT == REV_SOA) {
            const uint32_t *rows = LAYOUT == FWD_SOA ? a.fwd_in : a.rev_in;
            const uint32_t *cols = LAYOUT == FWD_SOA ? a.fwd_e : a.rev_e;
            const uint4 r = __ldcs(reinterpret_cast<const uint4 *>(rows) + g);
            const uint4 c = __ldcs(reinterpret_cast<const uint4 *>(cols) + g);
            edge(r.x, c.x); edge(r.y, c.y); edge(r.z, c.z); edge(r.w, c.w);
        } else {
            const uint2 *pairs = LAYOUT == FWD_AOS ? a.fwd_s : a.rev_s;
            const uint4 p0 = __ldcs(reinterpret_cast<const uint4 *>(pairs) + 2 * g);
            const uint4 p1 = __ldcs(reinterpret_cast<const uint4 *>(pairs) + 2 * g + 1);
            edge(p0.x, p0.y); edge(p0.z, p0.w); edge(p1.x, p1.y); edge(p1.z, p1.w);
        }
    }
    for (uint64_t e = (groups << 2) + gtid(); e < m; e += stride) {
        if constexpr (LAYOUT == FWD_SOA) edge(a.fwd_in[e], a.fwd_e[e]);
        else if constexpr (LAYOUT == REV_SOA) edge(a.rev_in[e], a.rev_e[e]);
        else if constexpr (LAYOUT == FWD_AOS) edge(a.fwd_s[e].x, a.fwd_s[e].y);
        else edge(a.rev_s[e].x, a.rev_s[e].y);
    }
    cnt.finish(&slot->frontier);
    side.finish(slot);
}

// ---------------------------------------------------------------------------
// vertex-push (bfs/vertex_push.cu:3-26): thread per vertex; a frontier
// vertex's owner walks its CSR row.  Depths are scanned 4 per thread.  A
// row longer than BFS_PUSH_HEAVY is expanded by the owner's whole warp
// (lane-strided, coalesced) instead of by its one thread, whose serial
// chain of relaxations would otherwise hold the level: a hub's row is the
// level's critical path.
// ---------------------------------------------------------------------------
constexpr uint32_t BFS_PUSH_HEAVY = 32;
constexpr int BFS_PUSH_UNROLL = 8;
// Rows above BFS_PUSH_GIANT edges are cut into HUB_CHUNK chunks for
// k_bfs_hub_chunks (the level's second kernel), as frontier-push does: one
// warp expanding a hub of R-MAT's lowest ids would hold the level.
constexpr uint32_t BFS_PUSH_GIANT = 1024;

__device__ __forceinline__ void queue_hub_chunks(const BfsArgs &a, LevelSlot *slot, uint32_t v, uint32_t s,
                                                 uint32_t e)
{
    const uint32_t chunks = (e - s + HUB_CHUNK - 1) / HUB_CHUNK;
    const uint32_t base = atomicAdd(&slot->heavy, chunks);
    for (uint32_t c = 0; c < chunks; c++) a.heavy[base + c] = make_uint2(v, s + c * HUB_CHUNK);
}

// Relaxes the neighbours E[first + k * step] (k < BFS_PUSH_UNROLL, below
// `end`): their indices, then their depths, are all in flight before the
// relaxations, and only a neighbour not yet visited costs an atomic.
template<int RED, bool SIDE>
__device__ __forceinline__ void relax_neighbours(const BfsArgs &a, const uint32_t *E, int32_t *lv, int32_t nd,
                                                 uint32_t first, uint32_t step, uint32_t end, Counter<RED> &cnt,
                                                 Side<SIDE> &side, uint32_t *qnext, LevelSlot *slot)
{
    uint32_t u[BFS_PUSH_UNROLL];
    int32_t d[BFS_PUSH_UNROLL];
#pragma unroll
    for (int k = 0; k < BFS_PUSH_UNROLL; k++) {
        const uint32_t i = first + k * step;
        u[k] = i < end ? __ldg(E + i) : 0u;
    }
#pragma unroll
    for (int k = 0; k < BFS_PUSH_UNROLL; k++) d[k] = first + k * step < end ? lv[u[k]] : nd;
#pragma unroll
    for (int k = 0; k < BFS_PUSH_UNROLL; k++)
        if (d[k] > nd && atomicMin(&lv[u[k]], nd) > nd) { cnt.hit(&slot->frontier); side.visit(a, qnext, slot, u[k]); }
}

template<int RED, bool SIDE>
__global__ void __launch_bounds__(512) k_bfs_vertex_push(BfsArgs a)
{
    const int32_t depth = level_depth(a), nd = depth + 1;
    LevelSlot *slot = &a.ctl->slot[depth % 3];
    if (blockIdx.x == 0 && threadIdx.x == 0) reset_slot(&a.ctl->slot[(depth + 1) % 3]);
    uint32_t *qnext = (depth & 1) ? a.q0 : a.q1;
    int32_t *lv = a.levels;
    Counter<RED> cnt;
    Side<SIDE> side;
    const unsigned lane = threadIdx.x & 31;
    const uint64_t n = a.n, stride = gthreads();
    // every lane calls it (warp-uniform loops); rows [s, e) of frontier
    // vertices, empty for the others
    auto relax_batch = [&](uint32_t first, uint32_t step, uint32_t end) {
        relax_neighbours(a, a.fwd_e, lv, nd, first, step, end, cnt, side, qnext, slot);
    };
    auto expand = [&](uint32_t v, uint32_t s, uint32_t e) {
        const bool giant = e - s > BFS_PUSH_GIANT;
        if (giant) queue_hub_chunks(a, slot, v, s, e);
        const bool heavy = !giant && e - s > BFS_PUSH_HEAVY;
        if (!heavy && !giant)
            for (uint32_t i = s; i < e; i += BFS_PUSH_UNROLL) relax_batch(i, 1, e);
        for (unsigned hv = __ballot_sync(FULL_MASK, heavy); hv; hv &= hv - 1) {
            const unsigned l = __ffs(hv) - 1;
            const uint32_t hs = __shfl_sync(FULL_MASK, s, l), he = __shfl_sync(FULL_MASK, e, l);
            for (uint32_t base = hs; base < he; base += 32 * BFS_PUSH_UNROLL) relax_batch(base + lane, 32, he);
        }
    };
    const uint64_t groups = (reinterpret_cast<uintptr_t>(lv) & 15) ? 0 : n >> 2;
    for (uint64_t g0 = gtid() - lane; g0 < groups; g0 += stride) {
        const uint64_t g = g0 + lane;
        int4 l = make_int4(-1, -1, -1, -1);
        if (g < groups) l = reinterpret_cast<const int4 *>(lv)[g];
        const int32_t d4[4] = {l.x, l.y, l.z, l.w};
#pragma unroll
        for (int k = 0; k < 4; k++) {
            uint32_t s = 0, e = 0;
            if (d4[k] == depth) {
                s = a.fwd_v[4 * g + k];
                e = a.fwd_v[4 * g + k + 1];
            }
            expand(static_cast<uint32_t>(4 * g + k), s, e);
        }
    }
    for (uint64_t v0 = (groups << 2) + gtid() - lane; v0 < n; v0 += stride) {
        const uint64_t v = v0 + lane;
        uint32_t s = 0, e = 0;
        if (v < n && lv[v] == depth) {
            s = a.fwd_v[v];
            e = a.fwd_v[v + 1];
        }
        expand(static_cast<uint32_t>(v), s, e);
    }
    cnt.finish(&slot->frontier);
    side.finish(slot);
}

// ---------------------------------------------------------------------------
// vertex-pull (bfs/vertex_pull.cu:3-31): thread per vertex; an unvisited
// vertex scans its reverse row and stops at the first parent at `depth`.
// The row is scanned BFS_PULL_UNROLL edges at a time: their indices, then
// their depths, are in flight together (a chain of dependent loads per
// edge would otherwise bound the thread); the few loads past the first
// parent are the price of the early exit.
// ---------------------------------------------------------------------------
constexpr int BFS_PULL_UNROLL = 4;

template<int RED, bool SIDE>
__global__ void __launch_bounds__(512) k_bfs_vertex_pull(BfsArgs a)
{
    const int32_t depth = level_depth(a), nd = depth + 1;
    LevelSlot *slot = &a.ctl->slot[depth % 3];
    if (blockIdx.x == 0 && threadIdx.x == 0) reset_slot(&a.ctl->slot[(depth + 1) % 3]);
    uint32_t *qnext = (depth & 1) ? a.q0 : a.q1;
    int32_t *lv = a.levels;
    Counter<RED> cnt;
    Side<SIDE> side;
    const uint64_t n = a.n, stride = gthreads();
    for (uint64_t v = gtid(); v < n; v += stride) {
        if (lv[v] <= nd) continue;
        const uint32_t s = a.rev_v[v], e = a.rev_v[v + 1];
        bool found = false;
        for (uint32_t i = s; i < e && !found; i += BFS_PULL_UNROLL) {
            uint32_t p[BFS_PULL_UNROLL];
#pragma unroll
            for (int k = 0; k < BFS_PULL_UNROLL; k++) p[k] = i + k < e ? __ldg(a.rev_e + i + k) : 0u;
#pragma unroll
            for (int k = 0; k < BFS_PULL_UNROLL; k++) found |= i + k < e && lv[p[k]] == depth;
        }
        if (found) {
            lv[v] = nd;
            cnt.hit(&slot->frontier);
            side.visit(a, qnext, slot, static_cast<uint32_t>(v));
        }
    }
    cnt.finish(&slot->frontier);
    side.finish(slot);
}

// ---------------------------------------------------------------------------
// Virtual-warp families (bfs/vertex_push_warp.cu:19-60,
// vertex_pull_warp.cu:17-71): a virtual warp of W lanes (W | 32) takes a
// chunk of C vertices, stages their depths and row offsets in shared memory
// ((W-lane group) x (C + C + 1) words, ImplementationTemplate.hpp:166-167)
// and expands / scans each row with its W lanes.  The pull form stops a
// row as soon as any lane has found a parent (the reference scans the
// whole row) and writes back only the depths it changed.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned subwarp_mask(uint32_t W)
{
    if (W >= 32) return FULL_MASK;
    const unsigned lane = threadIdx.x & 31;
    return ((1u << W) - 1u) << (lane & ~(W - 1u));
}

template<int RED, bool SIDE, bool PULL>
__global__ void __launch_bounds__(512) k_bfs_vwarp(BfsArgs a)
{
    extern __shared__ uint32_t smem[];
    const int32_t depth = level_depth(a), nd = depth + 1;
    LevelSlot *slot = &a.ctl->slot[depth % 3];
    if (blockIdx.x == 0 && threadIdx.x == 0) reset_slot(&a.ctl->slot[(depth + 1) % 3]);
    uint32_t *qnext = (depth & 1) ? a.q0 : a.q1;
    int32_t *lv = a.levels;
    Counter<RED> cnt;
    Side<SIDE> side;

    const uint32_t W = a.warp_size, C = a.chunk_size;
    const uint32_t per_block = blockDim.x / W;
    const uint32_t vw = threadIdx.x / W, lane = threadIdx.x % W;
    const unsigned mask = subwarp_mask(W);
    int32_t *my_lv = reinterpret_cast<int32_t *>(smem) + vw * C;
    uint32_t *my_off = smem + per_block * C + vw * (C + 1);
    const uint32_t *V = PULL ? a.rev_v : a.fwd_v;
    const uint32_t *E = PULL ? a.rev_e : a.fwd_e;
    const uint64_t n = a.n;
    const uint64_t total_vw = uint64_t(gridDim.x) * per_block;

    for (uint64_t chunk = blockIdx.x * uint64_t(per_block) + vw; chunk * C < n; chunk += total_vw) {
        const uint64_t v0 = chunk * C;
        const uint32_t cntv = static_cast<uint32_t>(min(uint64_t(C), n - v0));
        for (uint32_t i = lane; i < cntv; i += W) my_lv[i] = lv[v0 + i];
        for (uint32_t i = lane; i < cntv + 1; i += W) my_off[i] = V[v0 + i];
        __syncwarp(mask);
        for (uint32_t v = 0; v < cntv; v++) {
            const uint32_t s = my_off[v], e = my_off[v + 1];
            if constexpr (!PULL) {
                if (my_lv[v] == depth) {
                    if (e - s > BFS_PUSH_GIANT) {             // to k_bfs_hub_chunks
                        if (lane == 0) queue_hub_chunks(a, slot, static_cast<uint32_t>(v0 + v), s, e);
                    } else {
                        for (uint32_t base = s; base < e; base += W * BFS_PUSH_UNROLL)
                            relax_neighbours(a, E, lv, nd, base + lane, W, e, cnt, side, qnext, slot);
                    }
                }
            } else {
                if (my_lv[v] > depth) {
                    bool found = false;
                    for (uint32_t base = s; base < e; base += W) {
                        const uint32_t i = base + lane;
                        const bool hit = i < e && lv[__ldg(E + i)] == depth;
                        if (__any_sync(mask, hit)) { found = true; break; }
                    }
                    if (found && lane == 0) my_lv[v] = nd;
                }
            }
        }
        __syncwarp(mask);
        if constexpr (PULL) {
            for (uint32_t i = lane; i < cntv; i += W) {
                if (my_lv[i] == nd && lv[v0 + i] != nd) {
                    lv[v0 + i] = nd;
                    cnt.hit(&slot->frontier);
                    side.visit(a, qnext, slot, static_cast<uint32_t>(v0 + i));
                }
            }
            __syncwarp(mask);
        }
    }
    cnt.finish(&slot->frontier);
    side.finish(slot);
}

// ---------------------------------------------------------------------------
// frontier-push (GB300 variant): top-down over the frontier queue only.
// A warp takes 32 queue entries; their rows are concatenated (warp prefix
// sum of degrees) and the warp's lanes sweep the concatenation, so every
// lane does the same amount of edge work and reads within a row coalesce.
// Rows above HEAVY_DEGREE are cut into HUB_CHUNK chunks queued for
// k_bfs_hub_chunks, which spreads a hub over the whole GPU.
// Always emits the next queue.
// ---------------------------------------------------------------------------
template<bool SIDE>
__global__ void __launch_bounds__(256) k_bfs_frontier_push(BfsArgs a)
{
    __shared__ uint32_t s_excl[8][32];
    __shared__ uint32_t s_start[8][32];
    if (a.skip_check && *((volatile uint32_t *) &a.ctl->skip)) return;
    const int32_t depth = level_depth(a), nd = depth + 1;
    LevelSlot *slot = &a.ctl->slot[depth % 3];
    if (blockIdx.x == 0 && threadIdx.x == 0) reset_slot(&a.ctl->slot[(depth + 1) % 3]);
    const uint32_t *qin = (depth & 1) ? a.q1 : a.q0;
    uint32_t *qnext = (depth & 1) ? a.q0 : a.q1;
    const uint32_t qlen = *((volatile uint32_t *) &a.ctl->slot[(depth + 2) % 3].qlen);
    int32_t *lv = a.levels;
    Counter<RED_WARP> cnt;
    Side<SIDE> side;
    const unsigned lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint64_t warp = gtid() >> 5, warps = gthreads() >> 5;
    unsigned long long fe = 0;   // next-frontier out-edges (cluster-path gating)

    for (uint64_t t = warp * 32; t < qlen; t += warps * 32) {
        const uint64_t i = t + lane;
        uint32_t v = 0, s = 0, d = 0;
        if (i < qlen) {
            v = qin[i];
            s = a.fwd_v[v];
            d = a.fwd_v[v + 1] - s;
        }
        if (d > HEAVY_DEGREE) {
            const uint32_t chunks = (d + HUB_CHUNK - 1) / HUB_CHUNK;
            const uint32_t base = atomicAdd(&slot->heavy, chunks);
            for (uint32_t c = 0; c < chunks; c++) a.heavy[base + c] = make_uint2(v, s + c * HUB_CHUNK);
            d = 0;
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
        for (uint32_t k = lane; k < total; k += 32) {
            // owner = last lane with excl <= k
            int lo = 0, hi = 31;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (s_excl[wib][mid] <= k) lo = mid; else hi = mid - 1;
            }
            const uint32_t u = __ldg(a.fwd_e + s_start[wib][lo] + (k - s_excl[wib][lo]));
            if (relax(lv, u, nd)) {
                cnt.hit(&slot->frontier);
                queue_append(qnext, &slot->qlen, u);
                if constexpr (SIDE) side.visit(a, nullptr, nullptr, u);
                else if (a.skip_check) fe += a.outdeg[u];
            }
        }
        __syncwarp();
    }
    cnt.finish(&slot->frontier);
    side.finish(slot);
    if constexpr (!SIDE) flush_edges(slot, fe);
}

template<bool SIDE>
__global__ void __launch_bounds__(256) k_bfs_hub_chunks(BfsArgs a)
{
    if (a.skip_check && *((volatile uint32_t *) &a.ctl->skip)) return;
    const int32_t depth = level_depth(a), nd = depth + 1;
    LevelSlot *slot = &a.ctl->slot[depth % 3];
    uint32_t *qnext = (depth & 1) ? a.q0 : a.q1;
    const uint32_t chunks = *((volatile uint32_t *) &slot->heavy);
    int32_t *lv = a.levels;
    Counter<RED_WARP> cnt;
    Side<SIDE> side;
    const unsigned lane = threadIdx.x & 31;
    const uint64_t warp = gtid() >> 5, warps = gthreads() >> 5;
    unsigned long long fe = 0;
    for (uint64_t c = warp; c < chunks; c += warps) {
        const uint2 h = a.heavy[c];
        const uint32_t end = min(h.y + HUB_CHUNK, a.fwd_v[h.x + 1]);
        for (uint32_t i = h.y + lane; i < end; i += 32) {
            const uint32_t u = __ldcs(a.fwd_e + i);
            if (relax(lv, u, nd)) {
                cnt.hit(&slot->frontier);
                queue_append(qnext, &slot->qlen, u);
                if constexpr (SIDE) side.visit(a, nullptr, nullptr, u);
                else if (a.skip_check) fe += a.outdeg[u];
            }
        }
    }
    cnt.finish(&slot->frontier);
    side.finish(slot);
    if constexpr (!SIDE) flush_edges(slot, fe);
}

// ---------------------------------------------------------------------------
// frontier-pull (GB300 variant): bottom-up.  Each lane owns one unvisited
// vertex and checks up to 8 in-neighbours on its own; vertices still
// unresolved with longer rows are then swept by the whole warp 32
// in-neighbours at a time with a ballot early exit, so skewed in-degrees
// do not serialise a lane.  Emits the next queue when SIDE.
// ---------------------------------------------------------------------------
template<bool SIDE>
__global__ void __launch_bounds__(256) k_bfs_frontier_pull(BfsArgs a)
{
    const int32_t depth = level_depth(a), nd = depth + 1;
    LevelSlot *slot = &a.ctl->slot[depth % 3];
    if (blockIdx.x == 0 && threadIdx.x == 0) reset_slot(&a.ctl->slot[(depth + 1) % 3]);
    uint32_t *qnext = (depth & 1) ? a.q0 : a.q1;
    int32_t *lv = a.levels;
    Counter<RED_WARP> cnt;
    Side<SIDE> side;
    const unsigned lane = threadIdx.x & 31;
    const uint64_t warp = gtid() >> 5, warps = gthreads() >> 5;
    const uint64_t n = a.n;
    constexpr uint32_t SOLO = 8;

    for (uint64_t t = warp * 32; t < n; t += warps * 32) {
        const uint64_t v = t + lane;
        bool open = v < n && lv[v] > nd;
        bool found = false;
        uint32_t s = 0, e = 0;
        if (open) {
            s = a.rev_v[v];
            e = a.rev_v[v + 1];
            const uint32_t lim = min(e, s + SOLO);
            for (uint32_t i = s; i < lim; i++) {
                if (lv[__ldg(a.rev_e + i)] == depth) { found = true; break; }
            }
            open = !found && e > lim;
            s = lim;
        }
        unsigned pending = __ballot_sync(FULL_MASK, open);
        while (pending) {
            const int owner = __ffs(pending) - 1;
            pending &= pending - 1;
            const uint32_t rs = __shfl_sync(FULL_MASK, s, owner);
            const uint32_t re = __shfl_sync(FULL_MASK, e, owner);
            bool got = false;
            for (uint32_t b = rs; b < re; b += 32) {
                const uint32_t i = b + lane;
                const bool hit = i < re && lv[__ldg(a.rev_e + i)] == depth;
                if (__any_sync(FULL_MASK, hit)) { got = true; break; }
            }
            if (lane == static_cast<unsigned>(owner)) found = got;
        }
        if (found) {
            lv[v] = nd;
            cnt.hit(&slot->frontier);
            side.visit(a, qnext, slot, static_cast<uint32_t>(v));
        }
    }
    cnt.finish(&slot->frontier);
    side.finish(slot);
}

// ---------------------------------------------------------------------------
// frontier-push, small-frontier path (device loop only): one cluster of
// CLUSTER_CTAS blocks keeps expanding levels, separated by cluster barriers,
// while the frontier stays at or below CLUSTER_CAP vertices -- the
// high-diameter case (2-D grids, BFS tails) where one launch per level would
// dominate.  It does the per-level bookkeeping of the device-loop step for
// every level but the last, sets ctl->skip so the regular frontier-push
// kernels of the same loop iteration return at once, and leaves the last
// level to the step kernel.  A frontier above the cap at entry is left to
// the regular kernels.  Data written by other CTAs of the cluster (queues,
// hub chunks, counters) is read through L2 (L1 is not coherent).
// ---------------------------------------------------------------------------
constexpr uint32_t CLUSTER_CAP = 65536;            // frontier vertices
constexpr unsigned long long CLUSTER_EDGE_CAP = 65536;   // frontier out-edges
constexpr uint32_t CLUSTER_STAGE = 8192;           // next-frontier entries staged per block

// Per-level accumulators of one block of the cluster kernel: every thread
// counts locally, the block reduces once per level and issues one global
// atomic per counter (per-warp atomics on the shared level slot serialise
// at L2 and dominated short levels).  Newly visited vertices are staged in
// shared memory and copied to the global next-frontier queue in one block
// once the level is done; entries beyond the stage go to the queue directly.
template<bool SIDE>
struct ClusterLevel {
    uint32_t hits = 0;
    unsigned long long fe = 0;
    float ls = 0.f, lq = 0.f, lm = 0.f;

    __device__ __forceinline__ void visit(const BfsArgs &a, uint32_t *stage, uint32_t *stage_n, uint32_t *qnext,
                                          LevelSlot *slot, uint32_t v)
    {
        hits++;
        cg::coalesced_group g = cg::coalesced_threads();
        uint32_t base = 0;
        if (g.thread_rank() == 0) base = atomicAdd(stage_n, g.size());
        base = g.shfl(base, 0) + g.thread_rank();
        if (base < CLUSTER_STAGE) stage[base] = v;
        else queue_append(qnext, &slot->qlen, v);
        const uint32_t d = a.outdeg[v];
        fe += d;
        if constexpr (SIDE) {
            const float l = __log2f(1.0f + static_cast<float>(d));
            ls += l; lq += l * l; lm = fmaxf(lm, l);
        }
    }

    // Every thread of the block calls; ends with the staged entries in the
    // global queue and the level's counters in `slot`.
    __device__ __forceinline__ void finish(uint32_t *stage, uint32_t *stage_n, uint32_t *qnext, LevelSlot *slot)
    {
        __shared__ unsigned long long r_fe[CLUSTER_THREADS / 32];
        __shared__ uint32_t r_hits[CLUSTER_THREADS / 32];
        __shared__ float r_ls[CLUSTER_THREADS / 32], r_lq[CLUSTER_THREADS / 32], r_lm[CLUSTER_THREADS / 32];
        __shared__ uint32_t q_base;
        const unsigned lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        for (int o = 16; o > 0; o >>= 1) {
            hits += __shfl_xor_sync(FULL_MASK, hits, o);
            fe += __shfl_xor_sync(FULL_MASK, fe, o);
            if constexpr (SIDE) {
                ls += __shfl_xor_sync(FULL_MASK, ls, o);
                lq += __shfl_xor_sync(FULL_MASK, lq, o);
                lm = fmaxf(lm, __shfl_xor_sync(FULL_MASK, lm, o));
            }
        }
        if (lane == 0) { r_hits[wid] = hits; r_fe[wid] = fe; r_ls[wid] = ls; r_lq[wid] = lq; r_lm[wid] = lm; }
        __syncthreads();
        const uint32_t staged = min(*stage_n, CLUSTER_STAGE);
        if (threadIdx.x == 0) {
            uint32_t h = 0;
            unsigned long long e = 0;
            float s1 = 0.f, s2 = 0.f, mx = 0.f;
            for (unsigned w = 0; w < CLUSTER_THREADS / 32; w++) {
                h += r_hits[w]; e += r_fe[w]; s1 += r_ls[w]; s2 += r_lq[w]; mx = fmaxf(mx, r_lm[w]);
            }
            if (h) atomicAdd(&slot->frontier, h);
            if (e) atomicAdd(&slot->fedges, e);
            if constexpr (SIDE) {
                if (h) {
                    atomicAdd(&slot->lsum, s1);
                    atomicAdd(&slot->lsq, s2);
                    atomicMax(&slot->lmax_bits, __float_as_uint(mx));
                }
            }
            q_base = staged ? atomicAdd(&slot->qlen, staged) : 0u;
        }
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < staged; i += blockDim.x) qnext[q_base + i] = stage[i];
        hits = 0; fe = 0; ls = lq = lm = 0.f;
    }
};

template<bool SIDE>
__global__ void __cluster_dims__(CLUSTER_CTAS, 1, 1) __launch_bounds__(CLUSTER_THREADS)
k_bfs_cluster(BfsArgs a)
{
    __shared__ uint32_t s_excl[CLUSTER_THREADS / 32][32];
    __shared__ uint32_t s_start[CLUSTER_THREADS / 32][32];
    __shared__ uint32_t s_stage[CLUSTER_STAGE];
    __shared__ uint32_t s_stage_n;
    cg::cluster_group cl = cg::this_cluster();
    BfsCtl *ctl = a.ctl;
    const unsigned rank = cl.block_rank();
    const bool leader = rank == 0 && threadIdx.x == 0;
    int32_t L = *((volatile int32_t *) &ctl->depth);
    const uint32_t max_levels = *((volatile uint32_t *) &ctl->max_levels);
    uint32_t qlen = *((volatile uint32_t *) &ctl->slot[(L + 2) % 3].qlen);
    const unsigned long long fedges = *((volatile unsigned long long *) &ctl->slot[(L + 2) % 3].fedges);
    // same values in every block: a large or edge-heavy frontier is left to
    // the full-GPU kernels
    if (qlen == 0 || qlen > CLUSTER_CAP || fedges > CLUSTER_EDGE_CAP) return;
    int32_t *lv = a.levels;
    const unsigned lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint64_t warp = uint64_t(rank) * (CLUSTER_THREADS / 32) + wib;
    const uint64_t warps = uint64_t(CLUSTER_CTAS) * (CLUSTER_THREADS / 32);
    ClusterLevel<SIDE> acc;
    for (;;) {
        const int32_t nd = L + 1;
        LevelSlot *slot = &ctl->slot[L % 3];
        if (leader) reset_slot(&ctl->slot[(L + 1) % 3]);
        if (threadIdx.x == 0) s_stage_n = 0;
        __syncthreads();
        const uint32_t *qin = (L & 1) ? a.q1 : a.q0;
        uint32_t *qnext = (L & 1) ? a.q0 : a.q1;
        for (uint64_t t = warp * 32; t < qlen; t += warps * 32) {
            const uint64_t i = t + lane;
            uint32_t v = 0, s = 0, d = 0;
            if (i < qlen) {
                v = __ldcg(qin + i);
                s = a.fwd_v[v];
                d = a.fwd_v[v + 1] - s;
            }
            if (d > HEAVY_DEGREE) {
                const uint32_t chunks = (d + HUB_CHUNK - 1) / HUB_CHUNK;
                const uint32_t base = atomicAdd(&slot->heavy, chunks);
                for (uint32_t c = 0; c < chunks; c++) a.heavy[base + c] = make_uint2(v, s + c * HUB_CHUNK);
                d = 0;
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
            for (uint32_t k = lane; k < total; k += 32) {
                int lo = 0, hi = 31;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (s_excl[wib][mid] <= k) lo = mid; else hi = mid - 1;
                }
                const uint32_t u = __ldg(a.fwd_e + s_start[wib][lo] + (k - s_excl[wib][lo]));
                if (relax(lv, u, nd)) acc.visit(a, s_stage, &s_stage_n, qnext, slot, u);
            }
            __syncwarp();
        }
        acc.finish(s_stage, &s_stage_n, qnext, slot);
        cl.sync();
        const uint32_t chunks = __ldcg(&slot->heavy);
        if (chunks) {                                      // hub chunks: a second phase
            if (threadIdx.x == 0) s_stage_n = 0;
            __syncthreads();
            for (uint64_t c = warp; c < chunks; c += warps) {
                const uint2 h = __ldcg(a.heavy + c);
                const uint32_t end = min(h.y + HUB_CHUNK, a.fwd_v[h.x + 1]);
                for (uint32_t i = h.y + lane; i < end; i += 32) {
                    const uint32_t u = __ldg(a.fwd_e + i);
                    if (relax(lv, u, nd)) acc.visit(a, s_stage, &s_stage_n, qnext, slot, u);
                }
            }
            acc.finish(s_stage, &s_stage_n, qnext, slot);
            cl.sync();
        }
        const uint32_t f = __ldcg(&slot->qlen);
        const unsigned long long fnext = __ldcg(&slot->fedges);
        if (f == 0 || f > CLUSTER_CAP || fnext > CLUSTER_EDGE_CAP || static_cast<uint32_t>(L) + 2 > max_levels) {
            if (leader) ctl->skip = 1;                     // level L is left to the step kernel
            return;
        }
        if (leader) {                                      // the step kernel's bookkeeping for level L
            LevelSlot sl;
            sl.frontier = __ldcg(&slot->frontier);
            sl.qlen = f;
            sl.fedges = __ldcg(&slot->fedges);
            sl.lsum = __ldcg(&slot->lsum);
            sl.lsq = __ldcg(&slot->lsq);
            sl.lmax_bits = __ldcg(&slot->lmax_bits);
            sl.heavy = static_cast<uint32_t>(ctl->variant);
            if (a.log && static_cast<uint32_t>(L) < a.log_cap) a.log[L] = sl;
            ctl->visited += sl.frontier;
            ctl->traversed += sl.fedges;
            ctl->levels_done = static_cast<uint32_t>(L) + 1;
            ctl->depth = L + 1;
        }
        qlen = f;
        L++;
    }
}

}  // namespace bw
