// Device-wide exclusive scan and stable counting sort by a digit, used by
// the per-run set-up of the PageRank work-list variants (inside the timed
// region), so that every kernel a timed run launches is the library's own.
//
// Scan: three launches over tiles of SCAN_TILE words (tile sums; one block
// scanning the tile sums; each tile scanned and offset).  The scanned array
// may alias the input.
//
// Counting sort: a stable sort of `count` items by a digit below BINS,
// where `count` may live on the device (the host never waits for it).  The
// grid is fixed; each block takes one contiguous range of items and each of
// its warps one contiguous sub-range, walked 32 items at a time.
//   1. k_digit_count: each block's digit histogram -> hist[d * grid + b];
//   2. an exclusive scan of hist (digit-major): the first output position
//      of block b's items of digit d;
//   3. k_digit_scatter: each warp counts its sub-range per digit, the
//      block turns the counts into per-warp bases, and each warp walks its
//      sub-range again, ranking equal digits by lane (__match_any_sync).
// Items of equal digit keep their input order: lanes in lane order, steps
// in order, warps and blocks in order.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace bw {
namespace sortk {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 16;                          // consecutive words per thread
constexpr uint64_t SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

// Words of tile sums a scan of `count` words needs.
inline uint64_t scan_parts(uint64_t count) { return (count + SCAN_TILE - 1) / SCAN_TILE + 1; }

// Block-wide exclusive scan of one value per thread; `total` is the block's
// sum.  `ws` is shared scratch of THREADS / 32 words.
template<int THREADS>
__device__ __forceinline__ uint32_t block_exclusive(uint32_t v, uint32_t &total, uint32_t *ws)
{
    constexpr int NW = THREADS / 32;
    const unsigned lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= static_cast<unsigned>(o)) x += y;
    }
    if (lane == 31) ws[wid] = x;
    __syncthreads();
    if (wid == 0) {
        uint32_t w = lane < NW ? ws[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= static_cast<unsigned>(o)) w += y;
        }
        if (lane < NW) ws[lane] = w;                    // inclusive warp totals
    }
    __syncthreads();
    total = ws[NW - 1];
    const uint32_t before = wid ? ws[wid - 1] : 0u;
    __syncthreads();                                    // ws may be reused by the caller
    return before + x - v;
}

// part[b] = sum of tile b of in[0, count).
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_reduce(const uint32_t *__restrict__ in, uint64_t count,
                                                              uint32_t *__restrict__ part)
{
    __shared__ uint32_t ws[SCAN_THREADS / 32];
    const uint64_t t0 = blockIdx.x * SCAN_TILE;
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        const uint64_t i = t0 + k * SCAN_THREADS + threadIdx.x;
        if (i < count) s += in[i];
    }
    uint32_t total;
    block_exclusive<SCAN_THREADS>(s, total, ws);
    if (threadIdx.x == 0) part[blockIdx.x] = total;
}

// Exclusive scan of part[0, tiles) in place, one block; part[tiles] = total.
__global__ void __launch_bounds__(1024) k_scan_parts(uint32_t *part, uint64_t tiles)
{
    __shared__ uint32_t ws[32];
    uint32_t carry = 0;
    for (uint64_t base = 0; base < tiles; base += 1024) {
        const uint64_t i = base + threadIdx.x;
        const uint32_t v = i < tiles ? part[i] : 0u;
        uint32_t total;
        const uint32_t ex = block_exclusive<1024>(v, total, ws);
        if (i < tiles) part[i] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0) part[tiles] = carry;
}

// out[i] = part[tile] + the exclusive prefix of in[] within the tile.  The
// tile is staged in shared memory with one pad word per 32 (word j at
// j + j / 32), so that both the coalesced copies and each thread's run of
// SCAN_ITEMS consecutive words are free of bank conflicts.
__device__ __forceinline__ uint32_t scan_pad(uint32_t j) { return j + (j >> 5); }

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_apply(const uint32_t *in, uint64_t count,
                                                             const uint32_t *__restrict__ part, uint32_t *out)
{
    __shared__ uint32_t tile[SCAN_TILE + SCAN_TILE / 32];
    __shared__ uint32_t ws[SCAN_THREADS / 32];
    const uint64_t t0 = blockIdx.x * SCAN_TILE;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        const uint64_t i = t0 + k * SCAN_THREADS + threadIdx.x;
        tile[scan_pad(k * SCAN_THREADS + threadIdx.x)] = i < count ? in[i] : 0u;
    }
    __syncthreads();
    const uint32_t j0 = threadIdx.x * SCAN_ITEMS;
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) s += tile[scan_pad(j0 + k)];
    uint32_t total;
    uint32_t run = part[blockIdx.x] + block_exclusive<SCAN_THREADS>(s, total, ws);
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        const uint32_t v = tile[scan_pad(j0 + k)];
        tile[scan_pad(j0 + k)] = run;
        run += v;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        const uint64_t i = t0 + k * SCAN_THREADS + threadIdx.x;
        if (i < count) out[i] = tile[scan_pad(k * SCAN_THREADS + threadIdx.x)];
    }
}

// Exclusive scan of in[0, count) into out[0, count); `part` holds
// scan_parts(count) words and ends with the total (part[tiles]).
inline cudaError_t scan_exclusive(const uint32_t *in, uint32_t *out, uint64_t count, uint32_t *part,
                                  cudaStream_t s)
{
    const uint64_t tiles = (count + SCAN_TILE - 1) / SCAN_TILE;
    if (tiles == 0) {
        return cudaMemsetAsync(part, 0, sizeof(uint32_t), s);
    }
    k_scan_reduce<<<static_cast<unsigned>(tiles), SCAN_THREADS, 0, s>>>(in, count, part);
    k_scan_parts<<<1, 1024, 0, s>>>(part, tiles);
    k_scan_apply<<<static_cast<unsigned>(tiles), SCAN_THREADS, 0, s>>>(in, count, part, out);
    return cudaGetLastError();
}

// The range of items [lo, hi) of block b among `grid` blocks, and of warp w
// among WARPS warps within it (whole 32-item steps except at the end).
__device__ __forceinline__ void digit_range(uint64_t count, uint32_t b, uint32_t grid, uint32_t w, uint32_t warps,
                                            uint64_t &lo, uint64_t &hi)
{
    const uint64_t per_warp = ((count + uint64_t(grid) * warps - 1) / (uint64_t(grid) * warps) + 31) & ~uint64_t(31);
    lo = (uint64_t(b) * warps + w) * per_warp;
    hi = lo + per_warp;
    if (lo > count) lo = count;
    if (hi > count) hi = count;
}

// Pass 1: hist[d * grid + b] = items of block b with digit d; hist[BINS * grid] = 0.
// Src: uint32_t digit(uint64_t i) const.
template<int BINS, int WARPS, class Src>
__global__ void __launch_bounds__(WARPS * 32) k_digit_count(Src src, uint64_t count_host, const uint32_t *count_dev,
                                                            uint32_t *__restrict__ hist)
{
    __shared__ uint32_t h[BINS];
    for (int d = threadIdx.x; d < BINS; d += WARPS * 32) h[d] = 0;
    __syncthreads();
    const uint64_t count = count_dev ? *count_dev : count_host;
    const unsigned lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint64_t lo, hi;
    digit_range(count, blockIdx.x, gridDim.x, w, WARPS, lo, hi);
    for (uint64_t i = lo + lane; i < hi; i += 32) atomicAdd(&h[src.digit(i)], 1u);
    __syncthreads();
    for (int d = threadIdx.x; d < BINS; d += WARPS * 32) hist[uint64_t(d) * gridDim.x + blockIdx.x] = h[d];
    if (blockIdx.x == 0 && threadIdx.x == 0) hist[uint64_t(BINS) * gridDim.x] = 0u;
}

// Pass 3: out.put(position, i) for every item, `off` the scanned histogram.
// Shared memory: WARPS * BINS words (dynamic).
template<int BINS, int WARPS, class Src, class Dst>
__global__ void __launch_bounds__(WARPS * 32) k_digit_scatter(Src src, Dst dst, uint64_t count_host,
                                                              const uint32_t *count_dev,
                                                              const uint32_t *__restrict__ off)
{
    extern __shared__ uint32_t cnt[];                   // [WARPS][BINS]
    for (int k = threadIdx.x; k < WARPS * BINS; k += WARPS * 32) cnt[k] = 0;
    __syncthreads();
    const uint64_t count = count_dev ? *count_dev : count_host;
    const unsigned lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t *mine = cnt + w * BINS;
    uint64_t lo, hi;
    digit_range(count, blockIdx.x, gridDim.x, w, WARPS, lo, hi);
    // per-warp counts
    for (uint64_t i0 = lo; i0 < hi; i0 += 32) {
        const uint64_t i = i0 + lane;
        const bool valid = i < hi;
        const uint32_t d = valid ? src.digit(i) : static_cast<uint32_t>(BINS);
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        if (valid && lane == static_cast<unsigned>(__ffs(peers) - 1)) mine[d] += __popc(peers);
    }
    __syncthreads();
    // per-warp bases: the block's first position of digit d, then the warps in order
    for (int d = threadIdx.x; d < BINS; d += WARPS * 32) {
        uint32_t run = off[uint64_t(d) * gridDim.x + blockIdx.x];
#pragma unroll
        for (int k = 0; k < WARPS; k++) {
            const uint32_t c = cnt[k * BINS + d];
            cnt[k * BINS + d] = run;
            run += c;
        }
    }
    __syncthreads();
    const uint32_t below = (1u << lane) - 1u;
    for (uint64_t i0 = lo; i0 < hi; i0 += 32) {
        const uint64_t i = i0 + lane;
        const bool valid = i < hi;
        const uint32_t d = valid ? src.digit(i) : static_cast<uint32_t>(BINS);
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        uint32_t base = 0;
        if (valid) base = mine[d];
        __syncwarp();
        if (valid) {
            dst.put(base + __popc(peers & below), i);
            if (lane == static_cast<unsigned>(__ffs(peers) - 1)) mine[d] = base + __popc(peers);
        }
        __syncwarp();
    }
}

// Words of scratch a digit sort over `grid` blocks needs: the histogram
// (BINS * grid + 1) and its scan's tile sums.
template<int BINS>
inline uint64_t digit_sort_words(uint32_t grid)
{
    const uint64_t h = uint64_t(BINS) * grid + 1;
    return h + scan_parts(h);
}

// Stable sort of `count` items (count_dev, when given, is read on the
// device) by src.digit(i) < BINS; dst.put(position, i) writes each item.
template<int BINS, int WARPS, class Src, class Dst>
inline cudaError_t digit_sort(Src src, Dst dst, uint64_t count_host, const uint32_t *count_dev, uint32_t grid,
                              uint32_t *scratch, cudaStream_t s)
{
    const uint64_t h = uint64_t(BINS) * grid + 1;
    uint32_t *hist = scratch, *part = scratch + h;
    k_digit_count<BINS, WARPS, Src><<<grid, WARPS * 32, 0, s>>>(src, count_host, count_dev, hist);
    cudaError_t e = scan_exclusive(hist, hist, h, part, s);
    if (e != cudaSuccess) return e;
    const size_t smem = sizeof(uint32_t) * WARPS * BINS;
    if (smem > 48 * 1024) {
        e = cudaFuncSetAttribute(k_digit_scatter<BINS, WARPS, Src, Dst>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        if (e != cudaSuccess) return e;
    }
    k_digit_scatter<BINS, WARPS, Src, Dst><<<grid, WARPS * 32, smem, s>>>(src, dst, count_host, count_dev, hist);
    return cudaGetLastError();
}

}  // namespace sortk
}  // namespace bw
