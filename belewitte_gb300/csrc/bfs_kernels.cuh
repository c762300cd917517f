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
    s->frontier = 0; s->qlen = 0; s->fedges = 0; s->lsum = 0; s->lsq = 0;
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
    unsigned long long ls = 0, lq = 0;     // fixed point (lsum_fx, lsq_fx)
    float lm = 0.f;
    __device__ __forceinline__ void visit(const BfsArgs &a, uint32_t *qnext, LevelSlot *s, uint32_t v)
    {
        if constexpr (SIDE) {
            if (qnext) queue_append(qnext, &s->qlen, v);   // null: statistics only
            const uint32_t d = a.outdeg[v];
            const float l = __log2f(1.0f + static_cast<float>(d));
            fe += d; ls += lsum_fx(l); lq += lsq_fx(l); lm = fmaxf(lm, l);
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
    // The same, one set of atomics per block (every thread of the block
    // calls): the level's slot is one address per counter, and per-warp
    // atomics from every warp of a large level serialise there.
    __device__ __forceinline__ void finish_block(LevelSlot *s)
    {
        if constexpr (SIDE) {
            __shared__ unsigned long long b_fe[32];
            __shared__ unsigned long long b_ls[32], b_lq[32];
            __shared__ float b_lm[32];
            const unsigned lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
            for (int o = 16; o > 0; o >>= 1) {
                fe += __shfl_xor_sync(FULL_MASK, fe, o);
                ls += __shfl_xor_sync(FULL_MASK, ls, o);
                lq += __shfl_xor_sync(FULL_MASK, lq, o);
                lm = fmaxf(lm, __shfl_xor_sync(FULL_MASK, lm, o));
            }
            if (lane == 0) { b_fe[wid] = fe; b_ls[wid] = ls; b_lq[wid] = lq; b_lm[wid] = lm; }
            __syncthreads();
            if (wid == 0) {
                const bool in = lane < (blockDim.x >> 5);
                fe = in ? b_fe[lane] : 0ull; ls = in ? b_ls[lane] : 0ull; lq = in ? b_lq[lane] : 0ull;
                lm = in ? b_lm[lane] : 0.f;
                for (int o = 16; o > 0; o >>= 1) {
                    fe += __shfl_xor_sync(FULL_MASK, fe, o);
                    ls += __shfl_xor_sync(FULL_MASK, ls, o);
                    lq += __shfl_xor_sync(FULL_MASK, lq, o);
                    lm = fmaxf(lm, __shfl_xor_sync(FULL_MASK, lm, o));
                }
                if (lane == 0 && fe) {
                    atomicAdd(&s->fedges, fe);
                    atomicAdd(&s->lsum, ls);
                    atomicAdd(&s->lsq, lq);
                    atomicMax(&s->lmax_bits, __float_as_uint(lm));
                }
            }
        }
    }
};

// Next-queue appends staged per warp in shared memory: the whole warp calls
// add() at a convergent point; a full stage goes to the queue with one
// global atomic and coalesced stores.  One counter address takes every
// append of a level, so a large level otherwise serialises on it.
constexpr uint32_t WARP_STAGE = 256;
struct WarpQueue {
    uint32_t *stage;      // this warp's WARP_STAGE entries of shared memory
    uint32_t n = 0;       // staged (warp-uniform)
    __device__ __forceinline__ void add(bool hit, uint32_t v, uint32_t *q, uint32_t *len)
    {
        const unsigned lane = threadIdx.x & 31;
        const unsigned m = __ballot_sync(FULL_MASK, hit);
        if (hit) stage[n + __popc(m & ((1u << lane) - 1u))] = v;
        n += __popc(m);
        if (n > WARP_STAGE - 32) flush(q, len);
    }
    __device__ __forceinline__ void flush(uint32_t *q, uint32_t *len)
    {
        __syncwarp();
        uint32_t base = 0;
        if ((threadIdx.x & 31) == 0 && n) base = atomicAdd(len, n);
        base = __shfl_sync(FULL_MASK, base, 0);
        for (uint32_t i = threadIdx.x & 31; i < n; i += 32) q[base + i] = stage[i];
        n = 0;
        __syncwarp();
    }
};

// Hint that the 128-byte line holding p will be read soon (L2 only).
// Callers pass addresses inside their arrays.
__device__ __forceinline__ void prefetch_l2(const void *p)
{
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

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
    side.finish_block(slot);
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
    side.finish_block(slot);
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
    __shared__ uint32_t s_stage[SIDE ? 16 : 1][SIDE ? WARP_STAGE : 1];
    WarpQueue wq;
    wq.stage = s_stage[SIDE ? (threadIdx.x >> 5) : 0];
    const unsigned lane = threadIdx.x & 31;
    const uint64_t n = a.n, stride = gthreads();
    // whole-warp steps (the next queue is staged with one ballot per step)
    for (uint64_t v0 = gtid() - lane; v0 < n; v0 += stride) {
        const uint64_t v = v0 + lane;
        bool found = false;
        if (v < n && lv[v] > nd) {
            const uint32_t s = a.rev_v[v], e = a.rev_v[v + 1];
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
                side.visit(a, nullptr, slot, static_cast<uint32_t>(v));   // statistics; the queue below
            }
        }
        if constexpr (SIDE) if (qnext) wq.add(found, static_cast<uint32_t>(v), qnext, &slot->qlen);
    }
    if constexpr (SIDE) if (qnext) wq.flush(qnext, &slot->qlen);
    cnt.finish(&slot->frontier);
    side.finish_block(slot);
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
    side.finish_block(slot);
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
    __shared__ uint32_t s_stage[8][WARP_STAGE];
    if (a.skip_check && *((volatile uint32_t *) &a.ctl->skip)) return;
    const int32_t depth = level_depth(a), nd = depth + 1;
    LevelSlot *slot = &a.ctl->slot[depth % 3];
    if (blockIdx.x == 0 && threadIdx.x == 0) reset_slot(&a.ctl->slot[(depth + 1) % 3]);
    const uint32_t *qin = (depth & 1) ? a.q1 : a.q0;
    uint32_t *qnext = (depth & 1) ? a.q0 : a.q1;
    const uint32_t qlen = *((volatile uint32_t *) &a.ctl->slot[(depth + 2) % 3].qlen);
    int32_t *lv = a.levels;
    Counter<RED_BLOCK> cnt;
    Side<SIDE> side;
    const unsigned lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint64_t warp = gtid() >> 5, warps = gthreads() >> 5;
    unsigned long long fe = 0;   // next-frontier out-edges (cluster-path gating)
    WarpQueue wq;
    wq.stage = s_stage[wib];

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
        // edge k of the concatenated rows: a per-lane cursor over the rows'
        // exclusive offsets; whole-warp steps, so that the new vertices are
        // staged with one ballot per step
        uint32_t seg = 0;
        for (uint32_t k0 = 0; k0 < total; k0 += 32) {
            const uint32_t k = k0 + lane;
            bool got = false;
            uint32_t u = 0;
            if (k < total) {
                while (seg < 31 && s_excl[wib][seg + 1] <= k) seg++;
                u = __ldg(a.fwd_e + s_start[wib][seg] + (k - s_excl[wib][seg]));
                got = relax(lv, u, nd);
            }
            if (got) {
                cnt.hit(&slot->frontier);
                if constexpr (SIDE) side.visit(a, nullptr, nullptr, u);
                else if (a.skip_check) fe += a.outdeg[u];
            }
            wq.add(got, u, qnext, &slot->qlen);
        }
        __syncwarp();
    }
    wq.flush(qnext, &slot->qlen);
    cnt.finish(&slot->frontier);
    side.finish_block(slot);
    if constexpr (!SIDE) flush_edges(slot, fe);
}

template<bool SIDE>
__global__ void __launch_bounds__(256) k_bfs_hub_chunks(BfsArgs a)
{
    __shared__ uint32_t s_stage[8][WARP_STAGE];
    if (a.skip_check && *((volatile uint32_t *) &a.ctl->skip)) return;
    const int32_t depth = level_depth(a), nd = depth + 1;
    LevelSlot *slot = &a.ctl->slot[depth % 3];
    uint32_t *qnext = (depth & 1) ? a.q0 : a.q1;
    const uint32_t chunks = *((volatile uint32_t *) &slot->heavy);
    int32_t *lv = a.levels;
    Counter<RED_BLOCK> cnt;
    Side<SIDE> side;
    const unsigned lane = threadIdx.x & 31;
    const uint64_t warp = gtid() >> 5, warps = gthreads() >> 5;
    unsigned long long fe = 0;
    WarpQueue wq;
    wq.stage = s_stage[threadIdx.x >> 5];
    for (uint64_t c = warp; c < chunks; c += warps) {
        const uint2 h = a.heavy[c];
        const uint32_t end = min(h.y + HUB_CHUNK, a.fwd_v[h.x + 1]);
        for (uint32_t i0 = h.y; i0 < end; i0 += 32) {
            const uint32_t i = i0 + lane;
            bool got = false;
            uint32_t u = 0;
            if (i < end) {
                u = __ldcs(a.fwd_e + i);
                got = relax(lv, u, nd);
            }
            if (got) {
                cnt.hit(&slot->frontier);
                if constexpr (SIDE) side.visit(a, nullptr, nullptr, u);
                else if (a.skip_check) fe += a.outdeg[u];
            }
            wq.add(got, u, qnext, &slot->qlen);
        }
    }
    wq.flush(qnext, &slot->qlen);
    cnt.finish(&slot->frontier);
    side.finish_block(slot);
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
    __shared__ uint32_t s_stage[8][WARP_STAGE];
    const int32_t depth = level_depth(a), nd = depth + 1;
    LevelSlot *slot = &a.ctl->slot[depth % 3];
    if (blockIdx.x == 0 && threadIdx.x == 0) reset_slot(&a.ctl->slot[(depth + 1) % 3]);
    uint32_t *qnext = (depth & 1) ? a.q0 : a.q1;
    int32_t *lv = a.levels;
    Counter<RED_BLOCK> cnt;
    Side<SIDE> side;
    const unsigned lane = threadIdx.x & 31;
    const uint64_t warp = gtid() >> 5, warps = gthreads() >> 5;
    const uint64_t n = a.n;
    constexpr uint32_t SOLO = 8;
    WarpQueue wq;
    wq.stage = s_stage[threadIdx.x >> 5];

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
            side.visit(a, nullptr, slot, static_cast<uint32_t>(v));   // statistics; the queue below
        }
        if constexpr (SIDE) wq.add(found, static_cast<uint32_t>(v), qnext, &slot->qlen);
    }
    if constexpr (SIDE) wq.flush(qnext, &slot->qlen);
    cnt.finish(&slot->frontier);
    side.finish_block(slot);
}

// ---------------------------------------------------------------------------
// frontier-push, small-frontier path (device loop only): one cluster of
// CLUSTER_CTAS blocks keeps expanding levels while the frontier stays small
// -- the high-diameter case (2-D grids, BFS tails) where one launch per
// level would dominate.  A level is then a short chain of dependent
// accesses, so the kernel keeps all else on chip:
//  * each block holds a share of the frontier in shared memory as
//    {vertex, row start, row end}: a level reads no queue and no offsets
//    from global memory;
//  * a neighbour is claimed with one atomicMin on its depth, issued with
//    its row bounds' loads and the lane's other claims; the winner puts the
//    bounds in its block's next list;
//  * after the level's one cluster barrier, every block reads the blocks'
//    counts and then its equal share of the next frontier from the other
//    blocks' shared memory (a wavefront found by one block would otherwise
//    stay with it).  The next lists alternate between two buffers, so the
//    copy needs no second barrier.
// Rows above CLUSTER_HEAVY edges are left to the full-GPU kernels (their
// hub chunks spread such a row over every SM): a frontier with one is not
// taken on, and a level that finds one hands over.  So do a frontier above
// the caps and a block list overflow (the overflow went to the global queue
// already): the blocks write their lists to the global queue after the
// overflow, the leader fills the level's slot as the regular kernels would
// have, sets ctl->skip so that the regular frontier-push kernels of the loop
// iteration return at once, and leaves that level's bookkeeping to the step
// kernel.  The leader does the bookkeeping of the levels it completes.
// ---------------------------------------------------------------------------
constexpr uint32_t CLUSTER_HEAVY = 1024;           // rows above: the full-GPU kernels
constexpr int CLUSTER_UNROLL = 4;
static_assert(CLUSTER_THREADS == 32 * 32, "the block's counts are reduced by one warp, one lane per warp");
// dynamic shared memory: the level's share and two next lists, each of
// {vertex, row start, row end}
constexpr size_t CLUSTER_SMEM = 3 * 3 * CLUSTER_LIST * sizeof(uint32_t);

struct ClusterCounts {
    uint32_t frontier;            // new vertices of the level found by this block
    uint32_t listed;              // of those, in the block's next list
    unsigned long long fedges;    // their out-edges
    unsigned long long ls, lq;    // log-degree statistics (STATS == 1), fixed point
    float lm;
    uint32_t heavy;               // of those, rows above CLUSTER_HEAVY
};

// STATS: 0 none; 1 the log-degree statistics of every level (accumulated
// per claim, for a level log); 2 only those of a level handed over (what
// the next level's choice reads), computed from its frontier at handover.
template<int STATS>
__global__ void __cluster_dims__(CLUSTER_CTAS, 1, 1) __launch_bounds__(CLUSTER_THREADS)
k_bfs_cluster(BfsArgs a)
{
    extern __shared__ uint32_t cl_lists[];
    __shared__ ClusterCounts s_cnt[2];             // by level parity; read by the other blocks
    __shared__ ClusterCounts s_tot;                // the cluster's totals
    __shared__ uint32_t s_pre[CLUSTER_CTAS + 1];    // exclusive prefix of the blocks' next lists
    __shared__ unsigned long long r_fe[CLUSTER_THREADS / 32];
    __shared__ uint32_t r_hits[CLUSTER_THREADS / 32], r_heavy[CLUSTER_THREADS / 32];
    __shared__ unsigned long long r_ls[CLUSTER_THREADS / 32], r_lq[CLUSTER_THREADS / 32];
    __shared__ float r_lm[CLUSTER_THREADS / 32];
    __shared__ uint32_t s_n, s_cur_n;
    __shared__ unsigned long long s_hand[3];       // this block's part of a handed-over frontier's statistics
    cg::cluster_group cl = cg::this_cluster();
    BfsCtl *ctl = a.ctl;
    const unsigned rank = cl.block_rank(), tid = threadIdx.x, lane = tid & 31, wib = tid >> 5;
    const bool leader = rank == 0 && tid == 0;
    int32_t L = *((volatile int32_t *) &ctl->depth);
    const uint32_t max_levels = *((volatile uint32_t *) &ctl->max_levels);
    const uint32_t qlen = *((volatile uint32_t *) &ctl->slot[(L + 2) % 3].qlen);
    const unsigned long long fedges = *((volatile unsigned long long *) &ctl->slot[(L + 2) % 3].fedges);
    // same values in every block: a large or edge-heavy frontier is left to
    // the full-GPU kernels
    if (qlen == 0 || qlen > CLUSTER_CAP || fedges > CLUSTER_EDGE_CAP) return;
    int32_t *lv = a.levels;
    // buffer 0: the level's share; buffers 1 and 2: next lists, alternating
    uint32_t *lst_v[3], *lst_s[3], *lst_e[3];
    for (int b = 0; b < 3; b++) {
        lst_v[b] = cl_lists + (3 * b) * CLUSTER_LIST;
        lst_s[b] = cl_lists + (3 * b + 1) * CLUSTER_LIST;
        lst_e[b] = cl_lists + (3 * b + 2) * CLUSTER_LIST;
    }
    {   // this block's share of the level's queue, with the rows' bounds
        const uint32_t *qin = (L & 1) ? a.q1 : a.q0;
        const uint32_t per = (qlen + CLUSTER_CTAS - 1) / CLUSTER_CTAS;
        const uint32_t b = min(qlen, rank * per), cnt = min(per, qlen - b);   // cnt <= CLUSTER_LIST
        uint32_t heavy = 0;
        for (uint32_t i = tid; i < cnt; i += CLUSTER_THREADS) {
            const uint32_t v = __ldcg(qin + b + i);
            const uint32_t rs = a.fwd_v[v], re = a.fwd_v[v + 1];
            lst_v[0][i] = v;
            lst_s[0][i] = rs;
            lst_e[0][i] = re;
            heavy |= re - rs > CLUSTER_HEAVY ? 1u : 0u;
        }
        heavy = __syncthreads_or(heavy);
        if (tid == 0) {
            s_cur_n = cnt;
            s_cnt[1].heavy = heavy;
        }
        cl.sync();
        uint32_t any = 0;
        if (tid < CLUSTER_CTAS) any = cl.map_shared_rank(&s_cnt[1], tid)->heavy;
        any = __syncthreads_or(any);
        cl.sync();                                   // nobody leaves while its flag may be read
        if (any) return;                             // a hub row: the full-GPU kernels take this level
    }
    int p = 0;                                       // next lists: buffer 1 + p
    for (;;) {
        const int32_t nd = L + 1;
        LevelSlot *slot = &ctl->slot[L % 3];
        uint32_t *qnext = (L & 1) ? a.q0 : a.q1;
        if (leader) reset_slot(&ctl->slot[(L + 1) % 3]);
        if (tid == 0) s_n = 0;
        __syncthreads();
        const uint32_t ncur = s_cur_n;
        const uint32_t *cs = lst_s[0], *ce = lst_e[0];
        uint32_t *nv = lst_v[1 + p], *ns = lst_s[1 + p], *ne = lst_e[1 + p];
        uint32_t hits = 0, heavy = 0;
        unsigned long long fe = 0;
        unsigned long long ls = 0, lq = 0;
        float lm = 0.f;
        // a claimed neighbour u with row [us, ue): its counts and its entry k
        auto claim = [&](uint32_t u, uint32_t us, uint32_t ue, uint32_t k) {
            // Next-line prefetch: where vertex ids follow the graph's
            // geometry (grids, meshes, road networks) the wavefront reaches
            // u's id neighbours within a few levels, and the first touch of
            // their lines would put an HBM miss on the level's critical path.
            if (ue + 32 < a.m) prefetch_l2(a.fwd_e + ue + 32);
            if (u + 33 <= a.n) prefetch_l2(a.fwd_v + u + 33);
            if (u + 32 < a.n) prefetch_l2(lv + u + 32);
            hits++;
            fe += ue - us;
            heavy += ue - us > CLUSTER_HEAVY ? 1u : 0u;
            if constexpr (STATS == 1) {
                const float l = __log2f(1.0f + static_cast<float>(ue - us));
                ls += lsum_fx(l); lq += lsq_fx(l); lm = fmaxf(lm, l);
            }
            if (k < CLUSTER_LIST) {
                nv[k] = u;
                ns[k] = us;
                ne[k] = ue;
            } else {                                     // overflow: straight to the global queue
                qnext[atomicAdd(&slot->qlen, 1u)] = u;
            }
        };
        // 32 entries per warp step, their rows concatenated
        for (uint32_t t = wib * 32; t < ncur; t += CLUSTER_THREADS) {
            const uint32_t i = t + lane;
            uint32_t s = 0, d = 0;
            if (i < ncur) {
                s = cs[i];
                d = ce[i] - s;
            }
            uint32_t incl = d;
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(FULL_MASK, incl, o);
                if (lane >= static_cast<unsigned>(o)) incl += y;
            }
            const uint32_t total = __shfl_sync(FULL_MASK, incl, 31), excl = incl - d;
            for (uint32_t k0 = 0; k0 < total; k0 += 32 * CLUSTER_UNROLL) {
                uint32_t u[CLUSTER_UNROLL];
#pragma unroll
                for (int jj = 0; jj < CLUSTER_UNROLL; jj++) {
                    // edge k of the concatenated rows belongs to the last
                    // lane whose exclusive prefix is <= k (that lane's row
                    // is not empty): a binary search over the lanes
                    const uint32_t k = k0 + jj * 32 + lane;
                    uint32_t seg = 0;
#pragma unroll
                    for (uint32_t b = 16; b > 0; b >>= 1)
                        if (__shfl_sync(FULL_MASK, excl, seg + b) <= k) seg += b;
                    const uint32_t rs = __shfl_sync(FULL_MASK, s, seg), ex = __shfl_sync(FULL_MASK, excl, seg);
                    u[jj] = k < total ? __ldg(a.fwd_e + rs + (k - ex)) : 0xffffffffu;
                }
                // A level is a chain of dependent accesses, so every lane's
                // neighbours go out together: their row bounds (loaded
                // whether or not the claim wins) and their atomics are all
                // in flight before any result is used.
                uint32_t us[CLUSTER_UNROLL], ue[CLUSTER_UNROLL];
                int32_t old[CLUSTER_UNROLL];
#pragma unroll
                for (int jj = 0; jj < CLUSTER_UNROLL; jj++) {
                    us[jj] = ue[jj] = 0;
                    if (u[jj] != 0xffffffffu) {
                        us[jj] = __ldg(a.fwd_v + u[jj]);
                        ue[jj] = __ldg(a.fwd_v + u[jj] + 1);
                    }
                }
#pragma unroll
                for (int jj = 0; jj < CLUSTER_UNROLL; jj++)
                    old[jj] = u[jj] != 0xffffffffu ? atomicMin(&lv[u[jj]], nd) : nd;
                // the winners' entries: one shared atomic per warp and step
#pragma unroll
                for (int jj = 0; jj < CLUSTER_UNROLL; jj++) {
                    const bool win = old[jj] > nd;
                    const unsigned wm = __ballot_sync(FULL_MASK, win);
                    if (wm == 0) continue;
                    uint32_t base = 0;
                    if (lane == 0) base = atomicAdd(&s_n, static_cast<uint32_t>(__popc(wm)));
                    base = __shfl_sync(FULL_MASK, base, 0);
                    if (win) claim(u[jj], us[jj], ue[jj], base + __popc(wm & ((1u << lane) - 1u)));
                }
            }
        }
        // the block's counts
        for (int o = 16; o > 0; o >>= 1) {
            hits += __shfl_xor_sync(FULL_MASK, hits, o);
            heavy += __shfl_xor_sync(FULL_MASK, heavy, o);
            fe += __shfl_xor_sync(FULL_MASK, fe, o);
            if constexpr (STATS == 1) {
                ls += __shfl_xor_sync(FULL_MASK, ls, o);
                lq += __shfl_xor_sync(FULL_MASK, lq, o);
                lm = fmaxf(lm, __shfl_xor_sync(FULL_MASK, lm, o));
            }
        }
        if (lane == 0) {
            r_hits[wib] = hits; r_heavy[wib] = heavy; r_fe[wib] = fe;
            r_ls[wib] = ls; r_lq[wib] = lq; r_lm[wib] = lm;
        }
        __syncthreads();
        if (wib == 0) {                                  // the block's totals: one warp, in parallel
            ClusterCounts c{};
            c.frontier = r_hits[lane]; c.heavy = r_heavy[lane]; c.fedges = r_fe[lane];
            c.ls = r_ls[lane]; c.lq = r_lq[lane]; c.lm = r_lm[lane];
            for (int o = 16; o > 0; o >>= 1) {
                c.frontier += __shfl_xor_sync(FULL_MASK, c.frontier, o);
                c.heavy += __shfl_xor_sync(FULL_MASK, c.heavy, o);
                c.fedges += __shfl_xor_sync(FULL_MASK, c.fedges, o);
                c.ls += __shfl_xor_sync(FULL_MASK, c.ls, o);
                c.lq += __shfl_xor_sync(FULL_MASK, c.lq, o);
                c.lm = fmaxf(c.lm, __shfl_xor_sync(FULL_MASK, c.lm, o));
            }
            c.listed = min(s_n, CLUSTER_LIST);
            if (lane == 0) s_cnt[p] = c;
        }
        cl.sync();                                       // every block's counts, list and overflow are out
        if (wib == 0) {                                  // the cluster's totals, read by one warp
            ClusterCounts c{};
            if (lane < CLUSTER_CTAS) c = *cl.map_shared_rank(&s_cnt[p], lane);
            uint32_t incl = c.listed;                    // prefix of the lists over ranks
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(FULL_MASK, incl, o);
                if (lane >= static_cast<unsigned>(o)) incl += y;
            }
            if (lane < CLUSTER_CTAS) s_pre[lane + 1] = incl;
            if (lane == 0) s_pre[0] = 0;
            for (int o = 16; o > 0; o >>= 1) {
                c.frontier += __shfl_xor_sync(FULL_MASK, c.frontier, o);
                c.listed += __shfl_xor_sync(FULL_MASK, c.listed, o);
                c.heavy += __shfl_xor_sync(FULL_MASK, c.heavy, o);
                c.fedges += __shfl_xor_sync(FULL_MASK, c.fedges, o);
                c.ls += __shfl_xor_sync(FULL_MASK, c.ls, o);
                c.lq += __shfl_xor_sync(FULL_MASK, c.lq, o);
                c.lm = fmaxf(c.lm, __shfl_xor_sync(FULL_MASK, c.lm, o));
            }
            if (lane == 0) s_tot = c;
        }
        __syncthreads();
        const uint32_t f = s_tot.frontier, listed_all = s_tot.listed;
        const unsigned long long fe_all = s_tot.fedges;
        const unsigned long long ls_all = s_tot.ls, lq_all = s_tot.lq;
        const float lm_all = s_tot.lm;
        if (f == 0 || f > CLUSTER_CAP || fe_all > CLUSTER_EDGE_CAP || listed_all < f || s_tot.heavy ||
            static_cast<uint32_t>(L) + 2 > max_levels) {
            // hand level L to the step kernel: the next queue (overflow first,
            // then the blocks' lists) and the level's slot
            const uint32_t at = (f - listed_all) + s_pre[rank], mine = s_cnt[p].listed;
            for (uint32_t i = tid; i < mine; i += CLUSTER_THREADS) qnext[at + i] = nv[i];
            unsigned long long hls = ls_all, hlq = lq_all;
            float hlm = lm_all;
            if constexpr (STATS == 2) {
                // The handed-over frontier's log-degree statistics: this
                // block's list entries and its slice of the overflow, which
                // the other blocks wrote to the global queue before the
                // counts' cluster barrier (read past L1).
                unsigned long long ls = 0, lq = 0;
                float lm = 0.f;
                auto add = [&](uint32_t deg) {
                    const float l = __log2f(1.0f + static_cast<float>(deg));
                    ls += lsum_fx(l); lq += lsq_fx(l); lm = fmaxf(lm, l);
                };
                for (uint32_t i = tid; i < mine; i += CLUSTER_THREADS) add(ne[i] - ns[i]);
                const uint32_t ov = f - listed_all, per = (ov + CLUSTER_CTAS - 1) / CLUSTER_CTAS;
                const uint32_t ob = min(ov, rank * per), oe = min(ov, ob + per);
                for (uint32_t i = ob + tid; i < oe; i += CLUSTER_THREADS) {
                    const uint32_t v = __ldcg(qnext + i);
                    add(a.fwd_v[v + 1] - a.fwd_v[v]);
                }
                for (int o = 16; o > 0; o >>= 1) {
                    ls += __shfl_xor_sync(FULL_MASK, ls, o);
                    lq += __shfl_xor_sync(FULL_MASK, lq, o);
                    lm = fmaxf(lm, __shfl_xor_sync(FULL_MASK, lm, o));
                }
                if (lane == 0) { r_ls[wib] = ls; r_lq[wib] = lq; r_lm[wib] = lm; }
                __syncthreads();
                if (wib == 0) {
                    ls = r_ls[lane]; lq = r_lq[lane]; lm = r_lm[lane];
                    for (int o = 16; o > 0; o >>= 1) {
                        ls += __shfl_xor_sync(FULL_MASK, ls, o);
                        lq += __shfl_xor_sync(FULL_MASK, lq, o);
                        lm = fmaxf(lm, __shfl_xor_sync(FULL_MASK, lm, o));
                    }
                    if (lane == 0) { s_hand[0] = ls; s_hand[1] = lq; s_hand[2] = __float_as_uint(lm); }
                }
                cl.sync();                               // every block's part is out
                if (leader) {
                    hls = hlq = 0;
                    hlm = 0.f;
                    for (unsigned q = 0; q < CLUSTER_CTAS; q++) {
                        const unsigned long long *h = cl.map_shared_rank(s_hand, q);
                        hls += h[0]; hlq += h[1];
                        hlm = fmaxf(hlm, __uint_as_float(static_cast<uint32_t>(h[2])));
                    }
                }
            }
            if (leader) {
                slot->frontier = f;
                slot->qlen = f;
                slot->fedges = fe_all;
                slot->lsum = hls;
                slot->lsq = hlq;
                slot->lmax_bits = __float_as_uint(hlm);
                slot->heavy = 0;
                ctl->skip = 1;
            }
            cl.sync();                                   // no block leaves while others may read its shared memory
            return;
        }
        if (leader) {                                      // the step kernel's bookkeeping for level L
            LevelSlot sl;
            sl.frontier = f;
            sl.qlen = f;
            sl.fedges = fe_all;
            sl.lsum = ls_all;
            sl.lsq = lq_all;
            sl.lmax_bits = __float_as_uint(lm_all);
            sl.heavy = static_cast<uint32_t>(ctl->variant);
            if (a.log && static_cast<uint32_t>(L) < a.log_cap) a.log[L] = sl;
            ctl->visited += f;
            ctl->traversed += fe_all;
            ctl->levels_done = static_cast<uint32_t>(L) + 1;
            ctl->depth = L + 1;
        }
        // this block's equal share of the next frontier, gathered from the
        // blocks' next lists (rank order) into the level buffer
        {
            const uint32_t per = (f + CLUSTER_CTAS - 1) / CLUSTER_CTAS;
            const uint32_t b = min(f, rank * per), cnt = min(per, f - b);
            for (uint32_t i = tid; i < cnt; i += CLUSTER_THREADS) {
                const uint32_t j = b + i;
                unsigned q = 0;
                while (q + 1 < CLUSTER_CTAS && s_pre[q + 1] <= j) q++;
                const uint32_t k = j - s_pre[q];
                lst_s[0][i] = *cl.map_shared_rank(ns + k, q);
                lst_e[0][i] = *cl.map_shared_rank(ne + k, q);
            }
            if (tid == 0) s_cur_n = cnt;
        }
        p ^= 1;
        L++;
    }
}

}  // namespace bw
