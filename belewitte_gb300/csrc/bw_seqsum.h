// Parallel, bit-exact evaluation of a sequential float sum
//
//     s = +0;  for i in 0..n-1:  s = fl(s + x[i])      (round to nearest even)
//
// which is how the reference's vertex-pull kernels add a vertex's in-row
// (pagerank/vertex_pull.cu:23-27).  A plain loop is a chain of n dependent
// additions; for the in-row of an R-MAT hub (10^5 terms) that chain alone is
// hundreds of microseconds.  For terms that are non-negative and normal the
// same rounding sequence can be computed in parallel:
//
// While the running sum s stays in one binade [2^k, 2^(k+1)) every value it
// takes is an integer multiple A of the binade's ulp u (A in [2^23, 2^24)).
// Adding a term x rounds s + x to the u grid, so A grows by q = floor(x/u)
// plus 0 or 1 depending on the remainder r = x - q u:
//     r < u/2 -> +0,   r > u/2 -> +1,   r = u/2 (tie) -> the +0/+1 that makes
//     the new A even, which depends only on the parity of A + q.
// So each term is a map of A that depends on A's parity only: a pair
// (increment if A is even, increment if A is odd).  Such maps compose
// associatively, so a warp can compose each lane's run of terms, scan the
// lanes' maps, and obtain every lane's starting A at once.  The only thing
// the maps cannot express is the sum leaving the binade (A + increment >=
// 2^24); the first term where that happens is found by the lane that holds
// it, added with one real float addition, and the scan restarts after it in
// the new binade.  Partial sums of non-negative terms never decrease, so a
// row crosses at most a few dozen binades.
//
// Terms outside the domain (negative, subnormal, infinite, NaN) and a sum
// that overflows are reported to the caller, which then runs the plain loop.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define BWS_HD __host__ __device__ __forceinline__
#else
#define BWS_HD inline
#endif

namespace bwseq {

constexpr uint32_t ONE = 1u << 23;     // implicit significand bit
constexpr uint32_t TOP = 1u << 24;     // smallest significand outside the binade
constexpr uint32_t SAT = 1u << 25;     // saturation: "certainly leaves the binade"

// Increment of the running significand A (in ulps of the current binade)
// when A is even (e) and when A is odd (o).
struct Map {
    uint32_t e, o;
};

BWS_HD Map identity() { return Map{0u, 0u}; }

BWS_HD uint32_t saturate(uint32_t v) { return v < SAT ? v : SAT; }

// f first, then g.
BWS_HD Map compose(Map f, Map g)
{
    return Map{saturate(f.e + ((f.e & 1u) ? g.o : g.e)),
               saturate(f.o + ((f.o & 1u) ? g.e : g.o))};
}

BWS_HD uint32_t apply(Map f, uint32_t a) { return a + ((a & 1u) ? f.o : f.e); }

// Map of adding the term with bits `xb` to a sum in the binade with biased
// exponent k (1..254).  False when the term is outside the domain.
BWS_HD bool step(uint32_t xb, uint32_t k, Map &m)
{
    if ((xb & 0x7fffffffu) == 0) {                 // +0 or -0: s + 0 = s for s > 0
        m = identity();
        return true;
    }
    const uint32_t kx = (xb >> 23) & 0xffu;
    if ((xb >> 31) || kx == 0 || kx == 0xffu) return false;
    if (kx >= k) {                                 // x >= 2^23 ulps: leaves the binade
        m = Map{SAT, SAT};
        return true;
    }
    const uint32_t d = k - kx;                     // x / u = mx / 2^d
    if (d >= 25) {                                 // x < u / 2: no change
        m = identity();
        return true;
    }
    const uint32_t mx = (xb & 0x7fffffu) | ONE;
    const uint32_t q = mx >> d, rem = mx & ((1u << d) - 1u), half = 1u << (d - 1u);
    if (rem != half) {
        const uint32_t v = q + (rem > half ? 1u : 0u);
        m = Map{v, v};
    } else {                                       // tie: round to the even significand
        m = Map{q + (q & 1u), q + 1u - (q & 1u)};
    }
    return true;
}

// The same map without branches (selects only), for warps whose lanes take
// different cases at once; `ok` is cleared for terms outside the domain.
// Both increments are one rounding of mx / 2^d (mx the term's significand,
// d = k - kx): to nearest with ties to an even quotient (A even: the sum's
// new significand is even) or to an odd one (A odd), each an addition and
// a shift: (mx + half - 1 + lsb(q)) >> d and (mx + half - lsb(q)) >> d.
BWS_HD Map step_select(uint32_t xb, uint32_t k, bool &ok)
{
    const uint32_t kx = (xb >> 23) & 0xffu;
    const bool zero = (xb << 1) == 0u;
    ok = ok && (zero || xb - 0x00800000u < 0x7f000000u);   // +-0, or positive and normal
    const int32_t d = static_cast<int32_t>(k) - static_cast<int32_t>(kx);
    const uint32_t dd = static_cast<uint32_t>(d < 1 ? 1 : (d > 24 ? 24 : d));
    const uint32_t mx = (xb & 0x7fffffu) | ONE;
    const uint32_t half = 1u << (dd - 1u), qb = (mx >> dd) & 1u;
    uint32_t e = (mx + half - 1u + qb) >> dd, o = (mx + half - qb) >> dd;
    const bool big = d <= 0, tiny = d >= 25 || zero;
    e = big ? SAT : (tiny ? 0u : e);
    o = big ? SAT : (tiny ? 0u : o);
    return Map{e, o};
}

// compose() without saturation, for short runs whose increments cannot
// overflow (at most 64 maps of at most SAT each); saturate() the result.
// Any run whose true total reaches SAT still totals at least SAT, so the
// saturated result equals compose()'s.
BWS_HD Map compose_short(Map f, Map g)
{
    return Map{f.e + ((f.e & 1u) ? g.o : g.e), f.o + ((f.o & 1u) ? g.e : g.o)};
}

BWS_HD Map saturated(Map m) { return Map{saturate(m.e), saturate(m.o)}; }

BWS_HD uint32_t exponent_of(uint32_t sb) { return (sb >> 23) & 0xffu; }
BWS_HD uint32_t significand_of(uint32_t sb) { return (sb & 0x7fffffu) | ONE; }
BWS_HD uint32_t bits_of(uint32_t k, uint32_t a) { return (k << 23) | (a & 0x7fffffu); }

// A positive normal running sum: the state the maps work on.
BWS_HD bool in_domain(uint32_t sb)
{
    const uint32_t k = exponent_of(sb);
    return !(sb >> 31) && k != 0 && k != 0xffu;
}

}  // namespace bwseq
