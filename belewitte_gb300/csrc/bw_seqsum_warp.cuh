// Warp-parallel, bit-exact sequential float sums over a row of terms, on
// top of the binade maps of bw_seqsum.h.  Shared by the PageRank exact
// long-row sums (terms staged in memory) and the batched kernel (terms
// gathered on the fly).
#pragma once
#include <stdint.h>

#include "bw_internal.cuh"
#include "bw_seqsum.h"

namespace bw {

// The sequential sum s = fl(s + vals[i]) over i = b..e-1, continued from
// the running sum with bits `sb` -- bit-identical to one thread's loop --
// evaluated window by window (32 x L terms, staged in shared memory, the
// next window's loads in flight).  Terms at row positions below
// SERIAL_TERMS are added by lane 0 in order: there the sum doubles every
// few terms, and a binade crossing costs the map scan a restart.  The rest
// uses the binade maps of bw_seqsum.h: each lane composes the maps of its L
// consecutive terms as a tree (depth log2 L, branch-free steps), the warp
// scans the lanes' maps, and the lane that holds the next binade crossing
// adds that term with one float addition.  `stage` holds 33 x L floats of
// shared memory per warp; load(i) returns the row's term at position i
// (called for i < e only).  False when a
// term or the sum leaves the maps' domain (the caller then runs the plain
// loop); `sb` is warp-uniform.
constexpr uint32_t SERIAL_TERMS = 1024;   // measured: 64 was 23% slower on R-MAT-22

template<uint32_t L, class Load>
__device__ __forceinline__ bool warp_sequential_continue_load(Load load, uint32_t b, uint32_t e, uint32_t &sb,
                                                              float *stage, unsigned lane)
{
    using namespace bwseq;
    static_assert((L & (L - 1)) == 0 && L <= 32, "L: a power of two up to 32");
    constexpr uint32_t WIN = 32 * L;
    bool ok = true;
    float pre[L];
#pragma unroll
    for (uint32_t u = 0; u < L; u++) pre[u] = b + u * 32 + lane < e ? load(b + u * 32 + lane) : 0.0f;
    for (uint32_t w = b; w < e && ok; w += WIN) {
        // window [w, w + WIN): coalesced loads, staged so that lane l reads
        // terms l*L .. l*L + L-1 (element k at k + k / 32: no bank conflicts)
#pragma unroll
        for (uint32_t u = 0; u < L; u++) stage[u * 33 + lane] = pre[u];
        __syncwarp();
        uint32_t x[L];
#pragma unroll
        for (uint32_t u = 0; u < L; u++) {
            const uint32_t k = lane * L + u;
            x[u] = __float_as_uint(stage[k + (k >> 5)]);
        }
        const uint32_t nw = w + WIN;
#pragma unroll
        for (uint32_t u = 0; u < L; u++)
            pre[u] = nw + u * 32 + lane < e ? load(nw + u * 32 + lane) : 0.0f;
        const uint32_t lim = min(WIN, e - w), first = lane * L;
        uint32_t pos = 0;                  // first term of the window not yet added
        if (w < SERIAL_TERMS) {            // early terms: lane 0 adds them in order
            const uint32_t upto = min(lim, SERIAL_TERMS - w);
            uint32_t bits = 0;
            if (lane == 0) {
                float acc = __uint_as_float(sb);
                for (uint32_t i = 0; i < upto; i++) acc = __fadd_rn(acc, stage[i + (i >> 5)]);
                bits = __float_as_uint(acc);
            }
            sb = __shfl_sync(FULL_MASK, bits, 0);
            pos = upto;
        }
        __syncwarp();                      // stage is rewritten by the next window
        for (uint32_t guard = 0; pos < lim; guard++) {
            if (guard > WIN + 1) { ok = false; break; }
            if (sb == 0) {
                // the sum is still +0: it becomes the first nonzero term
                uint32_t hit = L, hv = 0;
#pragma unroll
                for (uint32_t u = 0; u < L; u++)
                    if (hit == L && first + u >= pos && first + u < lim && (x[u] & 0x7fffffffu)) { hit = u; hv = x[u]; }
                const unsigned any = __ballot_sync(FULL_MASK, hit < L);
                if (!any) break;
                const unsigned f = __ffs(any) - 1;
                sb = __shfl_sync(FULL_MASK, hv, f);
                pos = f * L + __shfl_sync(FULL_MASK, hit, f) + 1;
                if (!in_domain(sb)) { ok = false; break; }
                continue;
            }
            if (!in_domain(sb)) { ok = false; break; }
            const uint32_t K = exponent_of(sb), A = significand_of(sb);
            // this lane's terms as maps (inactive terms: +0, the identity),
            // composed as a tree
            Map t[L];
            bool good = true;
#pragma unroll
            for (uint32_t u = 0; u < L; u++) {
                const bool live = first + u >= pos && first + u < lim;
                t[u] = step_select(live ? x[u] : 0u, K, good);
            }
#pragma unroll
            for (uint32_t st = 1; st < L; st <<= 1) {
#pragma unroll
                for (uint32_t u = 0; u + st < L; u += 2 * st) t[u] = compose_short(t[u], t[u + st]);
            }
            const Map m = saturated(t[0]);
            if (__any_sync(FULL_MASK, !good)) { ok = false; break; }
            Map incl = m;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const Map y{__shfl_up_sync(FULL_MASK, incl.e, o), __shfl_up_sync(FULL_MASK, incl.o, o)};
                if (lane >= static_cast<unsigned>(o)) incl = compose(y, incl);
            }
            Map excl{__shfl_up_sync(FULL_MASK, incl.e, 1), __shfl_up_sync(FULL_MASK, incl.o, 1)};
            if (lane == 0) excl = identity();
            const uint32_t a0 = apply(excl, A), a1 = apply(m, a0);
            const unsigned cross = __ballot_sync(FULL_MASK, a1 >= TOP);
            if (!cross) {
                sb = bits_of(K, __shfl_sync(FULL_MASK, a1, 31));
                break;
            }
            // the first lane whose run leaves the binade finds the term
            const unsigned f = __ffs(cross) - 1;
            uint32_t nb = 0, np = 0;
            if (lane == f) {
                uint32_t acc = a0;
#pragma unroll
                for (uint32_t u = 0; u < L; u++) {
                    if (np == 0 && first + u >= pos && first + u < lim) {
                        Map tu;
                        step(x[u], K, tu);
                        const uint32_t bu = apply(tu, acc);
                        if (bu >= TOP) {
                            nb = __float_as_uint(__fadd_rn(__uint_as_float(bits_of(K, acc)), __uint_as_float(x[u])));
                            np = first + u + 1;
                        } else {
                            acc = bu;
                        }
                    }
                }
            }
            np = __shfl_sync(FULL_MASK, np, f);
            sb = __shfl_sync(FULL_MASK, nb, f);
            if (np <= pos || exponent_of(sb) == 0xffu) { ok = false; break; }
            pos = np;
        }
    }
    return ok;
}

}  // namespace bw
