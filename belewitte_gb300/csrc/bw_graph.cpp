// Host-side graph substrate: seeded generators, CSR construction, the
// reference's .graph file format and degree statistics.
//
// Everything here is deterministic for a given seed regardless of thread
// count or CPU architecture: random numbers come from a counter-based hash
// (splitmix64 finaliser) indexed by (seed, edge, draw), thresholds are
// compared as integers, and sorting is a stable LSD radix sort.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include <omp.h>

#include "belewitte_gb300.h"
#include "bw_hash.h"

namespace {

using bwgen::bounded;
using bwgen::hash3;

inline int bits_for(uint64_t n)
{
    int b = 0;
    while (b < 64 && (uint64_t(1) << b) < n) b++;
    return b < 1 ? 1 : b;
}

// Stable parallel LSD radix sort of 64-bit keys on their low `key_bits`.
void radix_sort(std::vector<uint64_t>& keys, int key_bits)
{
    const size_t n = keys.size();
    if (n < 2) return;
    constexpr int BITS = 11;
    constexpr size_t B = size_t(1) << BITS;
    const int passes = (key_bits + BITS - 1) / BITS;
    std::vector<uint64_t> tmp(n);
    uint64_t *src = keys.data(), *dst = tmp.data();
    const int T = omp_get_max_threads();
    std::vector<size_t> hist(static_cast<size_t>(T) * B);

    for (int p = 0; p < passes; p++) {
        const int shift = p * BITS;
        int nt_shared = 1;
#pragma omp parallel num_threads(T)
        {
            const int t = omp_get_thread_num();
            const int nt = omp_get_num_threads();
#pragma omp single
            nt_shared = nt;
            const size_t lo = n * t / nt, hi = n * (t + 1) / nt;
            size_t *h = &hist[static_cast<size_t>(t) * B];
            std::fill(h, h + B, 0);
            for (size_t i = lo; i < hi; i++) h[(src[i] >> shift) & (B - 1)]++;
#pragma omp barrier
#pragma omp single
            {
                size_t sum = 0;
                for (size_t d = 0; d < B; d++) {
                    for (int tt = 0; tt < nt_shared; tt++) {
                        size_t c = hist[static_cast<size_t>(tt) * B + d];
                        hist[static_cast<size_t>(tt) * B + d] = sum;
                        sum += c;
                    }
                }
            }
            for (size_t i = lo; i < hi; i++) {
                uint64_t k = src[i];
                dst[h[(k >> shift) & (B - 1)]++] = k;
            }
        }
        std::swap(src, dst);
    }
    if (src != keys.data()) std::memcpy(keys.data(), src, n * sizeof(uint64_t));
}

// Remove adjacent duplicates of a sorted vector in parallel.
void parallel_unique(std::vector<uint64_t>& keys)
{
    const size_t n = keys.size();
    if (n < 2) return;
    const int T = omp_get_max_threads();
    std::vector<size_t> counts(static_cast<size_t>(T) + 1, 0);
    std::vector<uint64_t> out(n);
    size_t total = 0;
#pragma omp parallel num_threads(T)
    {
        const int t = omp_get_thread_num(), nt = omp_get_num_threads();
        const size_t lo = n * t / nt, hi = n * (t + 1) / nt;
        size_t c = 0;
        for (size_t i = lo; i < hi; i++)
            if (i == 0 || keys[i] != keys[i - 1]) c++;
        counts[static_cast<size_t>(t) + 1] = c;
#pragma omp barrier
#pragma omp single
        {
            for (int k = 1; k <= nt; k++) counts[k] += counts[k - 1];
            total = counts[static_cast<size_t>(nt)];
        }
        size_t w = counts[static_cast<size_t>(t)];
        for (size_t i = lo; i < hi; i++)
            if (i == 0 || keys[i] != keys[i - 1]) out[w++] = keys[i];
    }
    out.resize(total);
    keys.swap(out);
}

// Sorted keys (row << vb | col) -> CSR arrays (malloc'd).
int keys_to_csr(const std::vector<uint64_t>& keys, int vb, uint64_t n,
                uint32_t **offsets_out, uint32_t **edges_out)
{
    const size_t m = keys.size();
    uint32_t *off = static_cast<uint32_t *>(std::malloc((n + 1) * sizeof(uint32_t)));
    uint32_t *edg = static_cast<uint32_t *>(std::malloc((m ? m : 1) * sizeof(uint32_t)));
    if (!off || !edg) { std::free(off); std::free(edg); return BW_ERR_OUT_OF_MEMORY; }
    const uint64_t mask = (uint64_t(1) << vb) - 1;
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < m; i++) {
        const uint64_t row = keys[i] >> vb;
        edg[i] = static_cast<uint32_t>(keys[i] & mask);
        const uint64_t prev = i == 0 ? 0 : (keys[i - 1] >> vb) + 1;
        for (uint64_t r = prev; r <= row; r++) off[r] = static_cast<uint32_t>(i);
    }
    const uint64_t last = m == 0 ? 0 : (keys[m - 1] >> vb) + 1;
    for (uint64_t r = last; r <= n; r++) off[r] = static_cast<uint32_t>(m);
    *offsets_out = off;
    *edges_out = edg;
    return BW_OK;
}

// Build a bw_host_graph from packed keys (row << vb | col), already filtered.
int finish_graph(std::vector<uint64_t>& keys, uint64_t n, int vb, bool dedupe,
                 bool undirected, bw_host_graph *out)
{
    radix_sort(keys, 2 * vb);
    if (dedupe) parallel_unique(keys);
    if (keys.size() > 0xffffffffULL) return BW_ERR_TOO_LARGE;
    std::memset(out, 0, sizeof *out);
    out->vertex_count = n;
    out->edge_count = keys.size();
    out->undirected = undirected ? 1 : 0;
    int rc = keys_to_csr(keys, vb, n, &out->fwd_vertices, &out->fwd_edges);
    if (rc) return rc;
    if (undirected) {
        out->rev_vertices = out->fwd_vertices;
        out->rev_edges = out->fwd_edges;
        return BW_OK;
    }
    const uint64_t mask = (uint64_t(1) << vb) - 1;
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < keys.size(); i++) {
        const uint64_t k = keys[i];
        keys[i] = ((k & mask) << vb) | (k >> vb);
    }
    radix_sort(keys, 2 * vb);
    return keys_to_csr(keys, vb, n, &out->rev_vertices, &out->rev_edges);
}

// Generate keys in parallel: gen(i, &s, &d) for i in [0, count); each thread
// writes into its own buffer, buffers are concatenated in thread order so
// the pre-sort sequence does not matter for the (sorted) result anyway.
template<typename Gen>
int generate_keys(uint64_t count, uint64_t n, int flags, Gen gen,
                  std::vector<uint64_t>& keys)
{
    const int vb = bits_for(n);
    const int T = omp_get_max_threads();
    const uint64_t per = (flags & BW_BUILD_SYMMETRISE) ? 2 : 1;
    std::vector<size_t> counts(static_cast<size_t>(T) + 1, 0);
    std::vector<size_t> starts(static_cast<size_t>(T) + 1, 0);
    try {
        keys.resize(count * per);
    } catch (const std::bad_alloc&) {
        return BW_ERR_OUT_OF_MEMORY;
    }
#pragma omp parallel num_threads(T)
    {
        const int t = omp_get_thread_num(), nt = omp_get_num_threads();
        const uint64_t lo = count * t / nt, hi = count * (t + 1) / nt;
        size_t w = lo * per;
        starts[static_cast<size_t>(t)] = w;
        for (uint64_t i = lo; i < hi; i++) {
            uint64_t s, d;
            gen(i, s, d);
            if ((flags & BW_BUILD_DROP_SELF_LOOPS) && s == d) continue;
            keys[w++] = (s << vb) | d;
            if ((flags & BW_BUILD_SYMMETRISE) && s != d) keys[w++] = (d << vb) | s;
        }
        counts[static_cast<size_t>(t) + 1] = w - lo * per;
        (void) nt;
    }
    // Compact the per-thread runs.
    size_t write = 0;
    for (int t = 0; t < T; t++) {
        const size_t from = starts[static_cast<size_t>(t)];
        const size_t c = counts[static_cast<size_t>(t) + 1];
        if (c && write != from) std::memmove(&keys[write], &keys[from], c * sizeof(uint64_t));
        write += c;
    }
    keys.resize(write);
    return BW_OK;
}

} // namespace

extern "C" {

void bw_host_graph_free(bw_host_graph *g)
{
    if (!g) return;
    if (g->rev_vertices != g->fwd_vertices) std::free(g->rev_vertices);
    if (g->rev_edges != g->fwd_edges) std::free(g->rev_edges);
    std::free(g->fwd_vertices);
    std::free(g->fwd_edges);
    std::memset(g, 0, sizeof *g);
}

int bw_graph_from_edges(uint64_t vertex_count, uint64_t count,
                        const uint32_t *src, const uint32_t *dst, int flags,
                        bw_host_graph *out)
{
    if (!out || (count && (!src || !dst))) return BW_ERR_INVALID_ARGUMENT;
    if (vertex_count == 0 || vertex_count > 0xffffffffULL) return BW_ERR_INVALID_ARGUMENT;
    for (uint64_t i = 0; i < count; i++)
        if (src[i] >= vertex_count || dst[i] >= vertex_count) return BW_ERR_INVALID_ARGUMENT;
    const int vb = bits_for(vertex_count);
    std::vector<uint64_t> keys;
    int rc = generate_keys(count, vertex_count, flags,
        [&](uint64_t i, uint64_t& s, uint64_t& d) { s = src[i]; d = dst[i]; }, keys);
    if (rc) return rc;
    return finish_graph(keys, vertex_count, vb, (flags & BW_BUILD_DEDUPE) != 0,
                        (flags & BW_BUILD_SYMMETRISE) != 0, out);
}

int bw_generate_rmat(uint32_t scale, uint32_t edge_factor, double a, double b,
                     double c, uint64_t seed, int symmetrise, bw_host_graph *out)
{
    if (!out || scale < 1 || scale > 31 || edge_factor == 0) return BW_ERR_INVALID_ARGUMENT;
    if (a < 0 || b < 0 || c < 0 || a + b + c > 1.0) return BW_ERR_INVALID_ARGUMENT;
    const uint64_t n = uint64_t(1) << scale;
    const uint64_t count = n * edge_factor;
    const bwgen::RmatParams p = bwgen::rmat_params(scale, a, b, c);
    const int flags = BW_BUILD_DROP_SELF_LOOPS | BW_BUILD_DEDUPE |
                      (symmetrise ? BW_BUILD_SYMMETRISE : 0);
    std::vector<uint64_t> keys;
    int rc = generate_keys(count, n, flags,
        [&](uint64_t e, uint64_t& s, uint64_t& d) { bwgen::rmat_edge(p, seed, e, s, d); }, keys);
    if (rc) return rc;
    return finish_graph(keys, n, bits_for(n), true, symmetrise != 0, out);
}

int bw_generate_rmat_n(uint64_t n, uint32_t edge_factor, double a, double b,
                       double c, uint64_t seed, int symmetrise, bw_host_graph *out)
{
    if (!out || n < 2 || n > 0x80000000ULL || edge_factor == 0) return BW_ERR_INVALID_ARGUMENT;
    if (a < 0 || b < 0 || c < 0 || a + b + c > 1.0) return BW_ERR_INVALID_ARGUMENT;
    const int vb = bits_for(n);
    const bwgen::RmatParams p = bwgen::rmat_params(static_cast<uint32_t>(vb), a, b, c);
    const int flags = BW_BUILD_DROP_SELF_LOOPS | BW_BUILD_DEDUPE |
                      (symmetrise ? BW_BUILD_SYMMETRISE : 0);
    std::vector<uint64_t> keys;
    int rc = generate_keys(n * edge_factor, n, flags,
        [&](uint64_t e, uint64_t& s, uint64_t& d) { bwgen::rmat_edge_n(p, n, seed, e, s, d); }, keys);
    if (rc) return rc;
    return finish_graph(keys, n, vb, true, symmetrise != 0, out);
}

int bw_generate_er(uint64_t n, uint64_t m, uint64_t seed, int symmetrise,
                   bw_host_graph *out)
{
    if (!out || n < 2 || n > 0xffffffffULL) return BW_ERR_INVALID_ARGUMENT;
    const int flags = BW_BUILD_DROP_SELF_LOOPS | BW_BUILD_DEDUPE |
                      (symmetrise ? BW_BUILD_SYMMETRISE : 0);
    std::vector<uint64_t> keys;
    int rc = generate_keys(m, n, flags,
        [&](uint64_t e, uint64_t& s, uint64_t& d) { bwgen::er_edge(n, seed, e, s, d); }, keys);
    if (rc) return rc;
    return finish_graph(keys, n, bits_for(n), true, symmetrise != 0, out);
}

int bw_generate_grid(uint32_t h, uint32_t w, bw_host_graph *out)
{
    if (!out || h == 0 || w == 0) return BW_ERR_INVALID_ARGUMENT;
    const uint64_t n = uint64_t(h) * w;
    if (n > 0xffffffffULL) return BW_ERR_TOO_LARGE;
    // Candidate edge i: vertex v = i / 2, direction i % 2 (0 right, 1 down);
    // invalid candidates become self-loops and are dropped.
    const int flags = BW_BUILD_DROP_SELF_LOOPS | BW_BUILD_SYMMETRISE;
    std::vector<uint64_t> keys;
    int rc = generate_keys(2 * n, n, flags,
        [&](uint64_t i, uint64_t& s, uint64_t& d) { bwgen::grid_edge(h, w, i, s, d); }, keys);
    if (rc) return rc;
    return finish_graph(keys, n, bits_for(n), false, true, out);
}

int bw_generate_ba(uint64_t n, uint32_t m, uint64_t seed, bw_host_graph *out)
{
    if (!out || n < 2 || n > 0xffffffffULL || m == 0) return BW_ERR_INVALID_ARGUMENT;
    // Batagelj-Brandes linear preferential attachment: slot 2k holds vertex
    // k / m, slot 2k+1 copies a uniformly chosen earlier slot.  Resolving a
    // slot follows the copy chain backwards, which makes every edge
    // independent and the generator parallel.
    const uint64_t count = n * m;
    const int flags = BW_BUILD_DROP_SELF_LOOPS | BW_BUILD_DEDUPE | BW_BUILD_SYMMETRISE;
    std::vector<uint64_t> keys;
    int rc = generate_keys(count, n, flags,
        [&](uint64_t k, uint64_t& s, uint64_t& d) { bwgen::ba_edge(m, seed, k, s, d); }, keys);
    if (rc) return rc;
    return finish_graph(keys, n, bits_for(n), true, true, out);
}

// ---------------------------------------------------------------------------
// .graph file format (utils/Graph.hpp:784-807, 977-1063, 1112-1151).
// v1 header: 10 x uint32 = {version=1, 0, 0, undirected, vertex_size,
// edge_size, vertex_count(u64), edge_count(u64)}; then vertices
// [(N+1) x vertex_size], edges [M x edge_size] and, for directed graphs,
// reverse vertices and edges.  v0 header: 3 x uint32 = {undirected, N, M},
// 4-byte fields throughout.
// ---------------------------------------------------------------------------
int bw_graph_file_read(const char *path, bw_host_graph *out)
{
    if (!path || !out) return BW_ERR_INVALID_ARGUMENT;
    std::FILE *f = std::fopen(path, "rb");
    if (!f) return BW_ERR_IO;
    std::fseek(f, 0, SEEK_END);
    long sz = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (sz < 12) { std::fclose(f); return BW_ERR_FORMAT; }
    std::vector<uint32_t> head(10, 0);
    size_t got = std::fread(head.data(), 1, std::min<size_t>(40, static_cast<size_t>(sz)), f);
    (void) got;
    uint32_t version = (head[1] == 0 && head[2] == 0) ? head[0] : 0;
    uint64_t n, m;
    uint32_t undirected, vsize = 4, esize = 4;
    size_t header_bytes;
    if (version == 0) {
        undirected = head[0]; n = head[1]; m = head[2];
        header_bytes = 12;
    } else if (version == 1) {
        undirected = head[3]; vsize = head[4]; esize = head[5];
        std::memcpy(&n, &head[6], 8);
        std::memcpy(&m, &head[8], 8);
        header_bytes = 40;
    } else {
        std::fclose(f);
        return BW_ERR_FORMAT;
    }
    if (vsize != 4 || esize != 4) { std::fclose(f); return BW_ERR_TOO_LARGE; }
    const uint64_t per_dir = (n + 1) * 4 + m * 4;
    const uint64_t expect = header_bytes + per_dir * (undirected ? 1 : 2);
    if (static_cast<uint64_t>(sz) != expect || n > 0xffffffffULL || m > 0xffffffffULL) {
        std::fclose(f);
        return BW_ERR_FORMAT;
    }
    std::memset(out, 0, sizeof *out);
    out->vertex_count = n;
    out->edge_count = m;
    out->undirected = undirected ? 1 : 0;
    auto alloc = [](uint64_t cnt) { return static_cast<uint32_t *>(std::malloc((cnt ? cnt : 1) * 4)); };
    out->fwd_vertices = alloc(n + 1);
    out->fwd_edges = alloc(m);
    std::fseek(f, static_cast<long>(header_bytes), SEEK_SET);
    bool ok = out->fwd_vertices && out->fwd_edges &&
              std::fread(out->fwd_vertices, 4, n + 1, f) == n + 1 &&
              std::fread(out->fwd_edges, 4, m, f) == m;
    if (ok && !undirected) {
        out->rev_vertices = alloc(n + 1);
        out->rev_edges = alloc(m);
        ok = out->rev_vertices && out->rev_edges &&
             std::fread(out->rev_vertices, 4, n + 1, f) == n + 1 &&
             std::fread(out->rev_edges, 4, m, f) == m;
    } else if (ok) {
        out->rev_vertices = out->fwd_vertices;
        out->rev_edges = out->fwd_edges;
    }
    std::fclose(f);
    if (!ok) { bw_host_graph_free(out); return BW_ERR_FORMAT; }
    // Structural checks: monotone offsets ending at M, targets < N.
    for (int dir = 0; dir < (undirected ? 1 : 2); dir++) {
        const uint32_t *v = dir ? out->rev_vertices : out->fwd_vertices;
        const uint32_t *e = dir ? out->rev_edges : out->fwd_edges;
        bool bad = v[0] != 0 || v[n] != m;
        for (uint64_t i = 0; i < n && !bad; i++) bad = v[i] > v[i + 1];
        for (uint64_t i = 0; i < m && !bad; i++) bad = e[i] >= n;
        if (bad) { bw_host_graph_free(out); return BW_ERR_FORMAT; }
    }
    return BW_OK;
}

int bw_graph_file_write(const char *path, const bw_host_graph *g)
{
    if (!path || !g || !g->fwd_vertices) return BW_ERR_INVALID_ARGUMENT;
    if (g->vertex_count > 0xffffffffULL || g->edge_count > 0xffffffffULL) return BW_ERR_TOO_LARGE;
    std::FILE *f = std::fopen(path, "wb");
    if (!f) return BW_ERR_IO;
    uint32_t head[10] = {1, 0, 0, static_cast<uint32_t>(g->undirected ? 1 : 0), 4, 4, 0, 0, 0, 0};
    std::memcpy(&head[6], &g->vertex_count, 8);
    std::memcpy(&head[8], &g->edge_count, 8);
    const uint64_t n = g->vertex_count, m = g->edge_count;
    bool ok = std::fwrite(head, 4, 10, f) == 10 &&
              std::fwrite(g->fwd_vertices, 4, n + 1, f) == n + 1 &&
              (m == 0 || std::fwrite(g->fwd_edges, 4, m, f) == m);
    if (ok && !g->undirected) {
        ok = std::fwrite(g->rev_vertices, 4, n + 1, f) == n + 1 &&
             (m == 0 || std::fwrite(g->rev_edges, 4, m, f) == m);
    }
    if (std::fclose(f) != 0) ok = false;
    return ok ? BW_OK : BW_ERR_IO;
}

int bw_degree_statistics(const bw_host_graph *g, int kind, double out[7])
{
    if (!g || !out || kind < 0 || kind > 2 || g->vertex_count == 0) return BW_ERR_INVALID_ARGUMENT;
    const uint64_t n = g->vertex_count;
    std::vector<double> deg(n);
    for (uint64_t v = 0; v < n; v++) {
        double d = 0;
        // Degrees::abs counts out + in edges, but only out edges for an
        // undirected graph (utils/Graph.hpp:1153-1172).
        if (kind == 0 || kind == 2) d += g->fwd_vertices[v + 1] - g->fwd_vertices[v];
        if (kind == 1 || (kind == 0 && !g->undirected))
            d += g->rev_vertices[v + 1] - g->rev_vertices[v];
        deg[v] = d;
    }
    // Quantile / Welford conventions of utils/StatisticalSummary.hpp:30-76.
    auto median_idx = [](size_t cnt) {
        return cnt % 2 == 0 ? std::pair<size_t, size_t>{cnt / 2 - 1, cnt / 2}
                            : std::pair<size_t, size_t>{cnt / 2, cnt / 2};
    };
    std::pair<size_t, size_t> med{0, 0}, lo{0, 0}, hi{0, 0};
    const size_t half = n / 2;
    if (n > 1) {
        med = median_idx(n);
        lo = median_idx(half);
        hi = lo;
        hi.first += half + (n % 2);
        hi.second += half + (n % 2);
    }
    std::sort(deg.begin(), deg.end());
    double total = 0, M = 0, S = 0;
    long k = 1;
    for (double v : deg) {
        total += v;
        double tmpM = M;
        M += (v - tmpM) / static_cast<double>(k);
        S += (v - tmpM) * (v - M);
        k++;
    }
    out[0] = deg.front();
    out[1] = (deg[lo.first] + deg[lo.second]) / 2.0;
    out[2] = total / static_cast<double>(n);
    out[3] = (deg[med.first] + deg[med.second]) / 2.0;
    out[4] = (deg[hi.first] + deg[hi.second]) / 2.0;
    out[5] = deg.back();
    out[6] = (k - 2 == 0) ? 0.0 : std::sqrt(S / static_cast<double>(k - 2));
    return BW_OK;
}

} // extern "C"
