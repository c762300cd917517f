// Counter-based edge generators shared by the host (bw_graph.cpp) and the
// device (bw_gen.cu) so both produce bit-identical graphs for a seed.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define BW_HD __host__ __device__ __forceinline__
#else
#define BW_HD inline
#endif

namespace bwgen {

BW_HD uint64_t mix64(uint64_t z)
{
    z += 0x9e3779b97f4a7c15ULL;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

BW_HD uint64_t hash3(uint64_t seed, uint64_t a, uint64_t b)
{ return mix64(mix64(seed ^ mix64(a)) ^ (b * 0xd1b54a32d192ed03ULL)); }

// Uniform integer in [0, n) (multiply-shift of a 64-bit hash).
BW_HD uint64_t bounded(uint64_t h, uint64_t n)
{
#if defined(__CUDA_ARCH__)
    return __umul64hi(h, n);
#else
    return static_cast<uint64_t>((static_cast<unsigned __int128>(h) * n) >> 64);
#endif
}

struct RmatParams {
    uint32_t scale;
    uint64_t ta, tab, tabc;   // cumulative a, a+b, a+b+c scaled to 2^32
};

inline RmatParams rmat_params(uint32_t scale, double a, double b, double c)
{
    const double two32 = 4294967296.0;
    return RmatParams{scale, static_cast<uint64_t>(a * two32), static_cast<uint64_t>((a + b) * two32),
                      static_cast<uint64_t>((a + b + c) * two32)};
}

// R-MAT edge e: one 32-bit uniform per level picks the quadrant, most
// significant bit first; a hash gives two levels.
BW_HD void rmat_edge(const RmatParams &p, uint64_t seed, uint64_t e, uint64_t &s, uint64_t &d)
{
    uint64_t sv = 0, dv = 0, h = 0;
    for (uint32_t l = 0; l < p.scale; l++) {
        uint64_t r;
        if ((l & 1) == 0) { h = hash3(seed, e, l >> 1); r = h & 0xffffffffULL; }
        else r = h >> 32;
        const uint64_t sb = r >= p.tab, db = (r >= p.ta && r < p.tab) || r >= p.tabc;
        sv = (sv << 1) | sb;
        dv = (dv << 1) | db;
    }
    s = sv;
    d = dv;
}

// R-MAT over n vertices, n not necessarily a power of two (p.scale =
// ceil(log2 n)): the power-of-two generator's edge e with both endpoints
// scaled by n / 2^scale (multiply-shift), so the low ids keep the hubs.
BW_HD void rmat_edge_n(const RmatParams &p, uint64_t n, uint64_t seed, uint64_t e, uint64_t &s, uint64_t &d)
{
    rmat_edge(p, seed, e, s, d);
    s = (s * n) >> p.scale;
    d = (d * n) >> p.scale;
}

BW_HD void er_edge(uint64_t n, uint64_t seed, uint64_t e, uint64_t &s, uint64_t &d)
{
    s = bounded(hash3(seed, e, 0), n);
    d = bounded(hash3(seed, e, 1), n);
}

// Grid candidate i: vertex i / 2, direction i % 2 (0 right, 1 down);
// a missing neighbour yields a self-loop, which is dropped.
BW_HD void grid_edge(uint64_t h, uint64_t w, uint64_t i, uint64_t &s, uint64_t &d)
{
    const uint64_t v = i >> 1, row = v / w, col = v % w;
    s = v;
    if ((i & 1) == 0) d = (col + 1 < w) ? v + 1 : v;
    else d = (row + 1 < h) ? v + w : v;
}

// Barabasi-Albert (Batagelj-Brandes): slot 2k holds vertex k / m, slot
// 2k+1 copies a uniformly chosen earlier slot; resolving follows the copy
// chain backwards, so every edge k is independent.
BW_HD void ba_edge(uint64_t m, uint64_t seed, uint64_t k, uint64_t &s, uint64_t &d)
{
    s = k / m;
    uint64_t slot = 2 * k + 1;
    while (slot & 1) {
        const uint64_t kk = slot >> 1;
        slot = bounded(hash3(seed, kk, 7), 2 * kk + 1);
    }
    d = (slot >> 1) / m;
}

}  // namespace bwgen
