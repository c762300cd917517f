"""The integer emulation of the reference's double-precision consolidation
(csrc/bw_consolidate.h) against real double arithmetic on the CPU:
fl32(fl64(B + x)) for every base term B = (1.0 - 0.85f) / N the library
uses and x = 0.85f * acc over many magnitudes, plus rounding edge cases."""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "belewitte_gb300" / "csrc" / "bw_consolidate.h"

CHECKER = r"""
#include <cstdio>
#include <cstring>
#include <cmath>
#include <cstdint>
#include "bw_consolidate.h"

static uint64_t rng = 0x9e3779b97f4a7c15ULL;
static uint64_t next() { rng ^= rng << 13; rng ^= rng >> 7; rng ^= rng << 17; return rng; }

static int check(double B, float x) {
    uint64_t bb; std::memcpy(&bb, &B, 8);
    uint32_t xb; std::memcpy(&xb, &x, 4);
    volatile double sum = B + static_cast<double>(x);
    volatile float want = static_cast<float>(sum);
    uint32_t wb; float w = want; std::memcpy(&wb, &w, 4);
    bool ok;
    uint32_t got = bwcons::add_round_bits(bb, xb, ok);
    if (!ok) return 0;                       // outside the domain: not used by the kernels
    if (got != wb) {
        std::printf("MISMATCH B=%a x=%a got=%08x want=%08x\n", B, (double)x, got, wb);
        return 1;
    }
    return 0;
}

int main() {
    int bad = 0;
    long tested = 0;
    const float d = 0.85f;
    // every base term for N up to 2^25 in geometric steps, random products
    for (double n = 1; n < 40e6; n = n * 1.37 + 1) {
        const double B = (1.0 - static_cast<double>(d)) / std::floor(n);
        for (int i = 0; i < 4000; i++) {
            uint64_t r = next();
            int shift = static_cast<int>(r % 60) - 40;            // x relative to B: 2^-40 .. 2^20
            float mant = 1.0f + static_cast<float>((r >> 8) & 0xffffff) / 16777216.0f;
            float x = static_cast<float>(B * std::ldexp(1.0, shift)) * mant;
            bad += check(B, x); tested++;
        }
        bad += check(B, 0.0f); tested++;
    }
    // ties: x such that B + x sits on float and double rounding boundaries
    for (int i = 0; i < 2000000; i++) {
        uint64_t r = next();
        double B = std::ldexp(1.0 + static_cast<double>(r & ((1ULL << 52) - 1)) / 4503599627370496.0,
                              -static_cast<int>(r >> 58) - 20);
        float base = static_cast<float>(B);
        uint32_t fb; std::memcpy(&fb, &base, 4);
        uint32_t k = static_cast<uint32_t>(next() % 5);
        fb = fb - 2 + k;
        float nearby; std::memcpy(&nearby, &fb, 4);
        float x = static_cast<float>(static_cast<double>(nearby) - B);
        if (!(x > 0)) x = static_cast<float>(std::fabs(static_cast<double>(x)));
        bad += check(B, x); tested++;
        float x2 = std::nextafter(x, 1.0f);
        bad += check(B, x2); tested++;
    }
    std::printf("tested %ld bad %d\n", tested, bad);
    return bad ? 1 : 0;
}
"""


def test_integer_consolidation_matches_double(tmp_path):
    src = tmp_path / "check.cpp"
    src.write_text(CHECKER)
    exe = tmp_path / "check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", f"-I{HEADER.parent}", str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout[-2000:]
    assert "bad 0" in out.stdout
