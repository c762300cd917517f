// Degree statistics of a device-resident graph: the graph-details figures
// (graph-details.cpp:36-61) that SwitchImplementation::loadGraph gives a
// predictor as graph properties (ImplementationTemplate.hpp:622-649), with
// the conventions of utils/StatisticalSummary.hpp:30-76 -- min, lower
// quantile, mean, median, upper quantile, max and standard deviation of the
// per-vertex degree.
//
// The degrees (row lengths of the offsets, summed for "abs") are sorted on
// the device; the order statistics are read at the summary's indices.  The
// sums of d and d^2 are exact integers (one 128-bit partial per block), so
// the mean is the host's exactly and the standard deviation is the exact
// sample deviation rounded once, where the host's Welford loop in double
// accumulates rounding on the way (the two agree to about 1e-12 relative).
#include <cmath>
#include <utility>
#include <vector>

#include <cub/cub.cuh>

#include "bw_internal.cuh"

namespace bw {
namespace {

constexpr int STAT_THREADS = 256;

// deg[v]: out (fwd), in (rev) or abs (both, or out only when undirected).
__global__ void k_degrees(const uint32_t *__restrict__ fwd, const uint32_t *__restrict__ rev, uint64_t n,
                          unsigned long long *__restrict__ deg)
{
    for (uint64_t v = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; v < n; v += uint64_t(gridDim.x) * blockDim.x) {
        unsigned long long d = 0;
        if (fwd) d += fwd[v + 1] - fwd[v];
        if (rev) d += rev[v + 1] - rev[v];
        deg[v] = d;
    }
}

// Per-block exact sums of d and d^2 (partial[2b] = sum d, [2b+1] = sum d^2;
// as 128-bit integers).
__global__ void __launch_bounds__(STAT_THREADS) k_degree_sums(const unsigned long long *__restrict__ deg, uint64_t n,
                                                              unsigned __int128 *__restrict__ partial)
{
    unsigned __int128 s1 = 0, s2 = 0;
    for (uint64_t v = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; v < n; v += uint64_t(gridDim.x) * blockDim.x) {
        const unsigned __int128 d = deg[v];
        s1 += d;
        s2 += d * d;
    }
    __shared__ unsigned __int128 r1[STAT_THREADS], r2[STAT_THREADS];
    r1[threadIdx.x] = s1;
    r2[threadIdx.x] = s2;
    __syncthreads();
    for (unsigned o = STAT_THREADS / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            r1[threadIdx.x] += r1[threadIdx.x + o];
            r2[threadIdx.x] += r2[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partial[2 * blockIdx.x] = r1[0];
        partial[2 * blockIdx.x + 1] = r2[0];
    }
}

}  // namespace
}  // namespace bw

using namespace bw;

extern "C" int bw_degree_statistics_device(bw_context *ctx, const bw_graph_view *g, int undirected, int kind,
                                           double out[7], void *stream)
{
    if (!ctx || !g || !out || kind < 0 || kind > 2 || g->vertex_count == 0) return BW_ERR_INVALID_ARGUMENT;
    const uint64_t n = g->vertex_count;
    // Degrees::abs counts out + in edges, but only out edges for an
    // undirected graph (utils/Graph.hpp:1153-1172)
    const uint32_t *fwd = (kind == 0 || kind == 2) ? g->fwd_vertices : nullptr;
    const uint32_t *rev = (kind == 1 || (kind == 0 && !undirected)) ? g->rev_vertices : nullptr;
    if ((kind != 1 && !fwd) || ((kind == 1 || (kind == 0 && !undirected)) && !rev))
        return BW_ERR_MISSING_REPRESENTATION;
    cudaStream_t s = as_stream(stream);
    const unsigned blocks = static_cast<unsigned>(ctx->sm_count) * 2;
    size_t sort_bytes = 0;
    cub::DoubleBuffer<unsigned long long> keys(nullptr, nullptr);
    BW_CUDA(cub::DeviceRadixSort::SortKeys(nullptr, sort_bytes, keys, static_cast<int64_t>(n), 0, 64, s));
    unsigned long long *buf = nullptr;
    unsigned __int128 *partial = nullptr;
    void *temp = nullptr;
    int rc = BW_OK;
    do {
        cudaError_t e;
        if ((e = ctx_malloc_async(ctx, reinterpret_cast<void **>(&buf), 2 * n * sizeof(unsigned long long), s)) ||
            (e = ctx_malloc_async(ctx, reinterpret_cast<void **>(&partial), 2 * blocks * sizeof(unsigned __int128), s)) ||
            (e = ctx_malloc_async(ctx, &temp, sort_bytes, s))) {
            set_last_error(e, "degree statistics scratch");
            rc = e == cudaErrorMemoryAllocation ? BW_ERR_OUT_OF_MEMORY : BW_ERR_CUDA;
            break;
        }
        k_degrees<<<blocks * 4, 256, 0, s>>>(fwd, rev, n, buf);
        k_degree_sums<<<blocks, STAT_THREADS, 0, s>>>(buf, n, partial);
        keys = cub::DoubleBuffer<unsigned long long>(buf, buf + n);
        if ((e = cub::DeviceRadixSort::SortKeys(temp, sort_bytes, keys, static_cast<int64_t>(n), 0, 64, s))) {
            set_last_error(e, "degree sort");
            rc = BW_ERR_CUDA;
            break;
        }
        // the summary's indices (StatisticalSummary.hpp:30-76): the median
        // of the whole, of the lower half and of the upper half
        auto median_idx = [](uint64_t cnt) {
            return cnt % 2 == 0 ? std::pair<uint64_t, uint64_t>{cnt / 2 - 1, cnt / 2}
                                : std::pair<uint64_t, uint64_t>{cnt / 2, cnt / 2};
        };
        std::pair<uint64_t, uint64_t> med{0, 0}, lo{0, 0}, hi{0, 0};
        const uint64_t half = n / 2;
        if (n > 1) {
            med = median_idx(n);
            lo = median_idx(half);
            hi = {lo.first + half + (n % 2), lo.second + half + (n % 2)};
        }
        const uint64_t at[8] = {0, lo.first, lo.second, med.first, med.second, hi.first, hi.second, n - 1};
        unsigned long long v[8];
        const unsigned long long *sorted = keys.Current();
        for (int i = 0; i < 8; i++)
            if ((e = cudaMemcpyAsync(&v[i], sorted + at[i], sizeof v[i], cudaMemcpyDeviceToHost, s))) break;
        std::vector<unsigned __int128> hp(2 * blocks);
        if (!e) e = cudaMemcpyAsync(hp.data(), partial, hp.size() * sizeof(unsigned __int128), cudaMemcpyDeviceToHost, s);
        if (!e) e = cudaStreamSynchronize(s);
        if (e) {
            set_last_error(e, "degree statistics read-back");
            rc = BW_ERR_CUDA;
            break;
        }
        unsigned __int128 s1 = 0, s2 = 0;
        for (unsigned b = 0; b < blocks; b++) {
            s1 += hp[2 * b];
            s2 += hp[2 * b + 1];
        }
        out[0] = static_cast<double>(v[0]);
        out[1] = (static_cast<double>(v[1]) + static_cast<double>(v[2])) / 2.0;
        out[2] = static_cast<double>(s1) / static_cast<double>(n);
        out[3] = (static_cast<double>(v[3]) + static_cast<double>(v[4])) / 2.0;
        out[4] = (static_cast<double>(v[5]) + static_cast<double>(v[6])) / 2.0;
        out[5] = static_cast<double>(v[7]);
        // sample deviation (the summary divides by count - 1): n * sum d^2 -
        // (sum d)^2 is n^2 times the population variance, exact in 128 bits
        if (n < 2) {
            out[6] = 0.0;
        } else {
            const unsigned __int128 num = static_cast<unsigned __int128>(n) * s2 - s1 * s1;
            out[6] = std::sqrt(static_cast<double>(num) / static_cast<double>(n) / static_cast<double>(n - 1));
        }
    } while (0);
    if (buf) cudaFreeAsync(buf, s);
    if (partial) cudaFreeAsync(partial, s);
    if (temp) cudaFreeAsync(temp, s);
    ctx->launches += 2;
    return rc;
}
