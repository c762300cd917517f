// Random-gather ceiling of the GPU: independent 4-byte loads at positions
// of an array given by a streamed index array, with nothing else to do.
// PageRank's pull kernels gather one value of a vertex-sized vector per
// edge; when that vector lives in L2 (16 MB for 4M vertices) they are bound
// by how fast the memory system serves such scattered loads, not by HBM
// bandwidth.  This kernel measures that rate on the same device, with the
// same unrolling and the same L2-only loads as the pull kernels' gathers, so
// that their time can be set against it.  It has no counterpart in the
// reference: it is a measurement, like the copy and GEMM peaks.
#include "bw_internal.cuh"

namespace bw {
namespace {

constexpr int PROBE_THREADS = 1024;
constexpr int PROBE_UNROLL = 16;

__global__ void __launch_bounds__(PROBE_THREADS) k_gather_probe(const float *__restrict__ src, uint64_t n,
                                                                const uint32_t *__restrict__ idx, uint64_t m,
                                                                float *__restrict__ partial)
{
    __shared__ float warp_sums[PROBE_THREADS / 32];
    float acc = 0.0f;
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t base = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; base < m; base += stride * PROBE_UNROLL) {
        uint32_t id[PROBE_UNROLL];
#pragma unroll
        for (int u = 0; u < PROBE_UNROLL; u++) {
            const uint64_t i = base + u * stride;
            id[u] = i < m ? __ldcs(idx + i) : 0xffffffffu;
        }
#pragma unroll
        for (int u = 0; u < PROBE_UNROLL; u++)
            if (id[u] < n) acc += __ldcg(src + id[u]);
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) warp_sums[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        float s = threadIdx.x < blockDim.x / 32 ? warp_sums[threadIdx.x] : 0.0f;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) partial[blockIdx.x] = s;
    }
}

}  // namespace
}  // namespace bw

using namespace bw;

extern "C" int bw_gather_probe(bw_context *ctx, const float *src, uint64_t n, const uint32_t *idx, uint64_t m,
                               float *partial, void *stream)
{
    if (!ctx || !src || !partial || (m && !idx)) return BW_ERR_INVALID_ARGUMENT;
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    k_gather_probe<<<ctx->sm_count, PROBE_THREADS, 0, s>>>(src, n, idx, m, partial);
    BW_CUDA(cudaGetLastError());
    return BW_OK;
}
