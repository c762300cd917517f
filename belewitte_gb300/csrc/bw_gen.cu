// Device-side graph generation: the host generators' counter-based edges
// evaluated on the GPU, then radix-sorted, de-duplicated and turned into
// forward and reverse CSR in HBM.  Input preparation for large graphs (the
// host path takes minutes at R-MAT scale 24); not a hot path.
#include <algorithm>

#include <cub/cub.cuh>

#include "bw_hash.h"
#include "bw_internal.cuh"

namespace bw {
namespace {

constexpr uint64_t INVALID_KEY = ~0ULL;

struct GenParams {
    int kind;
    uint64_t p0, p1, seed;
    bwgen::RmatParams rmat;
    int vb;
    int symmetrise;
    int drop_self;
};

__global__ void k_gen_keys(GenParams p, uint64_t count, uint64_t *keys)
{
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < count; i += stride) {
        uint64_t s = 0, d = 0;
        switch (p.kind) {
          case 0: bwgen::rmat_edge(p.rmat, p.seed, i, s, d); break;
          case 1: bwgen::er_edge(p.p0, p.seed, i, s, d); break;
          case 2: bwgen::grid_edge(p.p0, p.p1, i, s, d); break;
          case 3: bwgen::ba_edge(p.p1, p.seed, i, s, d); break;
          default: bwgen::rmat_edge_n(p.rmat, p.p0, p.seed, i, s, d); break;
        }
        const bool drop = p.drop_self && s == d;
        if (p.symmetrise) {
            keys[2 * i] = drop ? INVALID_KEY : (s << p.vb) | d;
            keys[2 * i + 1] = (drop || s == d) ? INVALID_KEY : (d << p.vb) | s;
        } else {
            keys[i] = drop ? INVALID_KEY : (s << p.vb) | d;
        }
    }
}

__global__ void k_keys_to_csr(const uint64_t *keys, uint64_t m, int vb, uint64_t n, uint32_t *off, uint32_t *edges)
{
    const uint64_t mask = (uint64_t(1) << vb) - 1;
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < m; i += stride) {
        const uint64_t row = keys[i] >> vb;
        edges[i] = static_cast<uint32_t>(keys[i] & mask);
        const uint64_t prev = i == 0 ? 0 : (keys[i - 1] >> vb) + 1;
        for (uint64_t r = prev; r <= row; r++) off[r] = static_cast<uint32_t>(i);
        if (i == m - 1)
            for (uint64_t r = row + 1; r <= n; r++) off[r] = static_cast<uint32_t>(m);
    }
}

__global__ void k_fill_offsets(uint32_t *off, uint64_t n, uint32_t value)
{
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i <= n; i += stride) off[i] = value;
}

__global__ void k_transpose_keys(uint64_t *keys, uint64_t m, int vb)
{
    const uint64_t mask = (uint64_t(1) << vb) - 1;
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < m; i += stride) {
        const uint64_t k = keys[i];
        keys[i] = ((k & mask) << vb) | (k >> vb);
    }
}

int bits_for(uint64_t n)
{
    int b = 0;
    while (b < 64 && (uint64_t(1) << b) < n) b++;
    return b < 1 ? 1 : b;
}

}  // namespace
}  // namespace bw

using namespace bw;

extern "C" {

void bw_device_graph_free(bw_device_graph *g)
{
    if (!g) return;
    if (g->rev_vertices && g->rev_vertices != g->fwd_vertices) cudaFree(g->rev_vertices);
    if (g->rev_edges && g->rev_edges != g->fwd_edges) cudaFree(g->rev_edges);
    if (g->fwd_vertices) cudaFree(g->fwd_vertices);
    if (g->fwd_edges) cudaFree(g->fwd_edges);
    *g = bw_device_graph{};
}

int bw_generate_device(int kind, uint64_t p0, uint64_t p1, double a, double b, double c, uint64_t seed,
                       int symmetrise, bw_device_graph *out, void *stream)
{
    if (!out || kind < 0 || kind > 4) return BW_ERR_INVALID_ARGUMENT;
    *out = bw_device_graph{};
    cudaStream_t s = as_stream(stream);
    GenParams gp{};
    gp.kind = kind;
    gp.seed = seed;
    gp.p0 = p0;
    gp.p1 = p1;
    gp.drop_self = 1;
    uint64_t n = 0, count = 0;
    bool dedupe = true;
    switch (kind) {
      case 0:
        if (p0 < 1 || p0 > 31 || p1 == 0 || a < 0 || b < 0 || c < 0 || a + b + c > 1.0)
            return BW_ERR_INVALID_ARGUMENT;
        n = uint64_t(1) << p0;
        count = n * p1;
        gp.rmat = bwgen::rmat_params(static_cast<uint32_t>(p0), a, b, c);
        gp.symmetrise = symmetrise != 0;
        break;
      case 1:
        if (p0 < 2 || p0 > 0xffffffffULL) return BW_ERR_INVALID_ARGUMENT;
        n = p0; count = p1;
        gp.symmetrise = symmetrise != 0;
        break;
      case 2:
        if (p0 == 0 || p1 == 0 || p0 * p1 > 0xffffffffULL) return BW_ERR_INVALID_ARGUMENT;
        n = p0 * p1; count = 2 * n;
        gp.symmetrise = 1;
        dedupe = false;
        break;
      case 3:
        if (p0 < 2 || p0 > 0xffffffffULL || p1 == 0) return BW_ERR_INVALID_ARGUMENT;
        n = p0; count = p0 * p1;
        gp.symmetrise = 1;
        break;
      default:
        if (p0 < 2 || p0 > 0x80000000ULL || p1 == 0 || a < 0 || b < 0 || c < 0 || a + b + c > 1.0)
            return BW_ERR_INVALID_ARGUMENT;
        n = p0;
        count = n * p1;
        gp.rmat = bwgen::rmat_params(static_cast<uint32_t>(bits_for(n)), a, b, c);
        gp.symmetrise = symmetrise != 0;
        break;
    }
    gp.vb = bits_for(n);
    const int key_bits = 2 * gp.vb;
    const uint64_t total = count * (gp.symmetrise ? 2 : 1);
    int dev = 0, sm = 0;
    BW_CUDA(cudaGetDevice(&dev));
    BW_CUDA(cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev));

    uint64_t *keys = nullptr, *alt = nullptr, *num_sel = nullptr;
    void *temp = nullptr;
    size_t temp_bytes = 0;
    int rc = BW_OK;
    auto fail = [&](cudaError_t e, const char *what) {
        set_last_error(e, what);
        rc = e == cudaErrorMemoryAllocation ? BW_ERR_OUT_OF_MEMORY : BW_ERR_CUDA;
    };
    do {
        cudaError_t e;
        if ((e = cudaMallocAsync(reinterpret_cast<void **>(&keys), total * 8, s)) != cudaSuccess) { fail(e, "alloc keys"); break; }
        if ((e = cudaMallocAsync(reinterpret_cast<void **>(&alt), total * 8, s)) != cudaSuccess) { fail(e, "alloc alt"); break; }
        if ((e = cudaMallocAsync(reinterpret_cast<void **>(&num_sel), 8, s)) != cudaSuccess) { fail(e, "alloc count"); break; }
        k_gen_keys<<<sm * 8, 256, 0, s>>>(gp, count, keys);
        // Sort on all 64 bits so INVALID keys (all ones) go last.
        cub::DoubleBuffer<uint64_t> db(keys, alt);
        cub::DeviceRadixSort::SortKeys(nullptr, temp_bytes, db, static_cast<int64_t>(total), 0, 64, s);
        size_t uniq_bytes = 0;
        cub::DeviceSelect::Unique(nullptr, uniq_bytes, keys, alt, num_sel, static_cast<int64_t>(total), s);
        temp_bytes = std::max(temp_bytes, uniq_bytes);
        if ((e = cudaMallocAsync(&temp, temp_bytes, s)) != cudaSuccess) { fail(e, "alloc temp"); break; }
        if ((e = cub::DeviceRadixSort::SortKeys(temp, temp_bytes, db, static_cast<int64_t>(total), 0, 64, s)) != cudaSuccess) {
            fail(e, "SortKeys"); break;
        }
        uint64_t *sorted = db.Current();
        uint64_t *other = db.Alternate();
        uint64_t m = 0;
        if (dedupe) {
            if ((e = cub::DeviceSelect::Unique(temp, temp_bytes, sorted, other, num_sel, static_cast<int64_t>(total), s)) != cudaSuccess) {
                fail(e, "Unique"); break;
            }
            uint64_t h = 0;
            cudaMemcpyAsync(&h, num_sel, 8, cudaMemcpyDeviceToHost, s);
            uint64_t last = 0;
            if ((e = cudaStreamSynchronize(s)) != cudaSuccess) { fail(e, "sync"); break; }
            if (h) {
                cudaMemcpyAsync(&last, other + h - 1, 8, cudaMemcpyDeviceToHost, s);
                cudaStreamSynchronize(s);
            }
            m = (h && last == INVALID_KEY) ? h - 1 : h;
            std::swap(sorted, other);
        } else {
            // no duplicates possible: count the valid prefix
            uint64_t lo = 0, hi = total;
            while (lo < hi) {   // first INVALID key (sorted ascending)
                uint64_t mid = (lo + hi) / 2, v = 0;
                cudaMemcpyAsync(&v, sorted + mid, 8, cudaMemcpyDeviceToHost, s);
                cudaStreamSynchronize(s);
                if (v == INVALID_KEY) hi = mid; else lo = mid + 1;
            }
            m = lo;
        }
        if (m > 0xffffffffULL) { rc = BW_ERR_TOO_LARGE; break; }
        out->vertex_count = n;
        out->edge_count = m;
        out->undirected = gp.symmetrise ? 1 : 0;
        if ((e = cudaMalloc(reinterpret_cast<void **>(&out->fwd_vertices), (n + 1) * 4)) != cudaSuccess) { fail(e, "alloc"); break; }
        if ((e = cudaMalloc(reinterpret_cast<void **>(&out->fwd_edges), (m ? m : 1) * 4)) != cudaSuccess) { fail(e, "alloc"); break; }
        if (m) k_keys_to_csr<<<sm * 8, 256, 0, s>>>(sorted, m, gp.vb, n, out->fwd_vertices, out->fwd_edges);
        else k_fill_offsets<<<sm, 256, 0, s>>>(out->fwd_vertices, n, 0);
        if (gp.symmetrise) {
            out->rev_vertices = out->fwd_vertices;
            out->rev_edges = out->fwd_edges;
        } else {
            if ((e = cudaMalloc(reinterpret_cast<void **>(&out->rev_vertices), (n + 1) * 4)) != cudaSuccess) { fail(e, "alloc"); break; }
            if ((e = cudaMalloc(reinterpret_cast<void **>(&out->rev_edges), (m ? m : 1) * 4)) != cudaSuccess) { fail(e, "alloc"); break; }
            if (m) {
                k_transpose_keys<<<sm * 8, 256, 0, s>>>(sorted, m, gp.vb);
                cub::DoubleBuffer<uint64_t> db2(sorted, other);
                if ((e = cub::DeviceRadixSort::SortKeys(temp, temp_bytes, db2, static_cast<int64_t>(m), 0, key_bits, s)) != cudaSuccess) {
                    fail(e, "SortKeys rev"); break;
                }
                k_keys_to_csr<<<sm * 8, 256, 0, s>>>(db2.Current(), m, gp.vb, n, out->rev_vertices, out->rev_edges);
            } else {
                k_fill_offsets<<<sm, 256, 0, s>>>(out->rev_vertices, n, 0);
            }
        }
        if ((e = cudaGetLastError()) != cudaSuccess) { fail(e, "generator kernels"); break; }
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) { fail(e, "sync"); break; }
    } while (0);
    if (keys) cudaFreeAsync(keys, s);
    if (alt) cudaFreeAsync(alt, s);
    if (num_sel) cudaFreeAsync(num_sel, s);
    if (temp) cudaFreeAsync(temp, s);
    cudaStreamSynchronize(s);
    if (rc) bw_device_graph_free(out);
    return rc;
}

}  // extern "C"
