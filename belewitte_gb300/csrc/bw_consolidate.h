// The reference's PageRank consolidation adds a double base term to a float
// product and rounds to float:
//     new_rank = (float)(((1.0 - d) / N) + (double)(d * acc))
// (pagerank/pagerank.cu:132).  GB300 runs FP64 instructions at a small
// fraction of the FP32 rate, so this header performs the same two IEEE
// round-to-nearest-even steps -- double addition, then conversion to float --
// with 64-bit integer arithmetic.  Valid for a positive normal double B and a
// float x >= 0 (zero or normal); the result is bit-identical to the FP64 path
// (checked exhaustively on edge cases and randomly in tests).
#pragma once
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define BWC_HD __host__ __device__ __forceinline__
#else
#define BWC_HD inline
#endif

namespace bwcons {

// Unpacked positive double: value = m * 2^(e - 1075), m in [2^52, 2^53).
struct Unpacked {
    uint64_t m;
    int32_t e;
};

BWC_HD Unpacked unpack_double(uint64_t bits)
{
    return Unpacked{(bits & ((uint64_t(1) << 52) - 1)) | (uint64_t(1) << 52), static_cast<int32_t>((bits >> 52) & 0x7ff)};
}

// fl32(fl64(B + x)) for B = double with bits `b_bits` (positive, normal) and
// x >= 0 normal float or zero.  `ok` is false for inputs outside that domain
// (subnormal x or a result outside the normal float range).
BWC_HD uint32_t add_round_bits(uint64_t b_bits, uint32_t x_bits, bool &ok)
{
    ok = true;
    const Unpacked B = unpack_double(b_bits);
    uint64_t M;
    int32_t E;
    const uint32_t ex = (x_bits >> 23) & 0xff, fx = x_bits & 0x7fffff;
    if ((x_bits & 0x7fffffff) == 0) {
        M = B.m;
        E = B.e;
    } else {
        if (ex == 0 || ex == 0xff || (x_bits >> 31)) { ok = false; return 0; }
        const Unpacked X{(static_cast<uint64_t>(fx) | (uint64_t(1) << 23)) << 29, static_cast<int32_t>(ex) - 127 + 1023};
        const Unpacked &hi = B.e >= X.e ? B : X;
        const Unpacked &lo = B.e >= X.e ? X : B;
        const uint32_t d = static_cast<uint32_t>(hi.e - lo.e);
        const uint64_t a = hi.m << 10;                    // 63 bits: 53 significant + 10 guard
        const uint64_t full = lo.m << 10;
        uint64_t b;
        bool sticky;
        if (d >= 63) {
            b = 0;
            sticky = full != 0;
        } else {
            b = full >> d;
            sticky = d ? (full & ((uint64_t(1) << d) - 1)) != 0 : false;
        }
        uint64_t s = a + b;
        int32_t e = hi.e;
        if (s >> 63) {                                    // carry: renormalise
            sticky = sticky || (s & 1);
            s >>= 1;
            e += 1;
        }
        // round the 53-bit significand (bits 62..10) to nearest even
        const uint64_t low = s & 0x3ff, half = 0x200;
        const uint64_t lsb = (s >> 10) & 1;
        const bool up = low > half || (low == half && (sticky || lsb));
        M = (s >> 10) + (up ? 1 : 0);
        if (M >> 53) {
            M >>= 1;
            e += 1;
        }
        E = e;
        if (E >= 0x7ff) { ok = false; return 0; }
    }
    // double (M, E) -> float, round to nearest even on the 29 dropped bits
    const uint64_t low29 = M & ((uint64_t(1) << 29) - 1), half29 = uint64_t(1) << 28;
    const uint64_t lsb = (M >> 29) & 1;
    uint64_t F = (M >> 29) + ((low29 > half29 || (low29 == half29 && lsb)) ? 1 : 0);
    int32_t e32 = E - 1023 + 127;
    if (F >> 24) {
        F >>= 1;
        e32 += 1;
    }
    if (e32 <= 0 || e32 >= 0xff) { ok = false; return 0; }
    return (static_cast<uint32_t>(e32) << 23) | static_cast<uint32_t>(F & 0x7fffff);
}

}  // namespace bwcons
