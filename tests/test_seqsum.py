"""The warp-parallel evaluation of a sequential float sum (csrc/bw_seqsum.h)
against the plain loop s = fl(s + x[i]) on the CPU.

The checker emulates the warp algorithm the PageRank kernels run on the
longest rows (32 lanes x 8 or 32 terms per window, per-lane map
composition, lane scan, binade crossings found by one lane) with the
header's helpers, and compares the bits of the result with a
sequential float loop compiled with -ffp-contract=off.  Inputs cover wide
dynamic ranges, long runs of equal terms (which hit round-half-even ties
at every step once the sum is large), constructed ties, zeros, leading
zeros and out-of-domain terms (which must be reported)."""
import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "belewitte_gb300" / "csrc" / "bw_seqsum.h"

CHECKER = r"""
#include <cstdio>
#include <cstring>
#include <cmath>
#include <cstdint>
#include <vector>
#include "bw_seqsum.h"
using namespace bwseq;

static uint32_t fb(float f) { uint32_t b; std::memcpy(&b, &f, 4); return b; }
static float bf(uint32_t b) { float f; std::memcpy(&f, &b, 4); return f; }

static uint32_t sequential(const std::vector<float> &x) {
    volatile float s = 0.0f;
    for (float v : x) s = s + v;
    return fb(s);
}

// Terms added in order by one lane before the map scan takes over (the
// kernel's SERIAL_TERMS), and terms per lane (the window is 32 x L; with
// L > 8 a lane composes its maps as a tree of branch-free steps, as the
// wide kernel does); the checker runs several settings, including serial
// starts that end inside a window.
static uint32_t serial_terms = 0;
static uint32_t L = 8;

// Warp emulation; returns false when the kernel would fall back.
static bool warp_sum(const std::vector<float> &vals, uint32_t &out) {
    const uint32_t WIN = 32 * L, n = vals.size();
    uint32_t sb = 0;
    for (uint32_t w = 0; w < n; w += WIN) {
        uint32_t pos = 0;
        if (w < serial_terms) {            // terms [w, serial_terms) in order by one lane
            volatile float acc = bf(sb);
            uint32_t i = w;
            for (; i < n && i < w + WIN && i < serial_terms; i++) acc = acc + vals[i];
            sb = fb(acc);
            pos = i - w;
        }
        uint32_t x[32][32];
        for (uint32_t lane = 0; lane < 32; lane++)
            for (uint32_t u = 0; u < L; u++) {
                const uint32_t k = lane * L + u;
                x[lane][u] = w + k < n ? fb(vals[w + k]) : 0u;
            }
        const uint32_t lim = n - w < WIN ? n - w : WIN;
        int guard = 0;
        while (pos < lim) {
            if (++guard > 1000) return false;
            if (sb != 0 && !in_domain(sb)) return false;
            if (sb == 0) {
                int f = -1; uint32_t hu = 0;
                for (uint32_t lane = 0; lane < 32 && f < 0; lane++)
                    for (uint32_t u = 0; u < L; u++) {
                        const uint32_t i = lane * L + u;
                        if (i >= pos && i < lim && (x[lane][u] & 0x7fffffffu)) { f = lane; hu = u; break; }
                    }
                if (f < 0) break;
                sb = x[f][hu];
                pos = f * L + hu + 1;
                if (!in_domain(sb)) return false;
                continue;
            }
            const uint32_t K = exponent_of(sb), A = significand_of(sb);
            Map m[32];
            for (uint32_t lane = 0; lane < 32; lane++) {
                if (L > 8) {                       // branch-free steps composed as a tree
                    Map t[32];
                    bool good = true;
                    for (uint32_t u = 0; u < L; u++) {
                        const uint32_t i = lane * L + u;
                        t[u] = step_select(i >= pos && i < lim ? x[lane][u] : 0u, K, good);
                    }
                    if (!good) return false;
                    for (uint32_t st = 1; st < L; st <<= 1)
                        for (uint32_t u = 0; u + st < L; u += 2 * st) t[u] = compose(t[u], t[u + st]);
                    m[lane] = t[0];
                    continue;
                }
                m[lane] = identity();
                for (uint32_t u = 0; u < L; u++) {
                    const uint32_t i = lane * L + u;
                    if (i >= pos && i < lim) {
                        Map t;
                        if (!step(x[lane][u], K, t)) return false;
                        m[lane] = compose(m[lane], t);
                    }
                }
            }
            // Kogge-Stone inclusive scan, then shift for the exclusive one
            Map incl[32];
            for (int l = 0; l < 32; l++) incl[l] = m[l];
            for (int o = 1; o < 32; o <<= 1) {
                Map prev[32];
                for (int l = 0; l < 32; l++) prev[l] = incl[l];
                for (int l = o; l < 32; l++) incl[l] = compose(prev[l - o], prev[l]);
            }
            int f = -1;
            uint32_t a0f = 0, a1last = 0;
            for (int l = 0; l < 32; l++) {
                const Map ex = l ? incl[l - 1] : identity();
                const uint32_t a0 = apply(ex, A), a1 = apply(m[l], a0);
                if (a1 >= TOP && f < 0) { f = l; a0f = a0; }
                if (l == 31) a1last = a1;
            }
            if (f < 0) { sb = bits_of(K, a1last); break; }
            uint32_t a = a0f, nb = 0, np = 0;
            for (uint32_t u = 0; u < L && np == 0; u++) {
                const uint32_t i = f * L + u;
                if (i >= pos && i < lim) {
                    Map t; step(x[f][u], K, t);
                    const uint32_t b = apply(t, a);
                    if (b >= TOP) {
                        volatile float s0 = bf(bits_of(K, a));
                        volatile float s1 = s0 + bf(x[f][u]);
                        nb = fb(s1); np = i + 1;
                    } else a = b;
                }
            }
            if (np <= pos) return false;
            sb = nb; pos = np;
            if (exponent_of(sb) == 0xffu) return false;
        }
    }
    out = sb;
    return true;
}

static uint64_t rng = 0x243f6a8885a308d3ULL;
static uint64_t nxt() { rng ^= rng << 13; rng ^= rng >> 7; rng ^= rng << 17; return rng; }
static double unit() { return (nxt() >> 11) * (1.0 / 9007199254740992.0); }

static int bad = 0, tested = 0, fallback = 0;
static void check(const std::vector<float> &x, bool expect_domain) {
    uint32_t got;
    const bool ok = warp_sum(x, got);
    tested++;
    if (!ok) {
        fallback++;
        if (expect_domain) { std::printf("unexpected fallback n=%zu\n", x.size()); bad++; }
        return;
    }
    const uint32_t want = sequential(x);
    if (got != want) {
        if (bad < 10) std::printf("MISMATCH n=%zu got %08x (%a) want %08x (%a)\n", x.size(), got, bf(got), want, bf(want));
        bad++;
    }
}

static void run_all();

int main() {
    for (uint32_t l : {8u, 32u})
        for (uint32_t st : {0u, 64u, 300u, 1024u}) { L = l; serial_terms = st; run_all(); }
    std::printf("tested %d fallback %d bad %d\n", tested, fallback, bad);
    return bad ? 1 : 0;
}

static void run_all() {
    // 1. log-uniform magnitudes over wide ranges, many lengths
    for (int t = 0; t < 3000; t++) {
        const uint32_t n = 1 + nxt() % (t < 2500 ? 3000 : 40000);
        const int span = 1 + nxt() % 40;
        std::vector<float> x(n);
        for (auto &v : x) v = static_cast<float>(std::ldexp(1.0 + unit(), -static_cast<int>(nxt() % span) - 10));
        check(x, true);
    }
    // 2. equal terms: ties at every step once the sum is large
    for (int t = 0; t < 300; t++) {
        const uint32_t n = 1 + nxt() % 200000;
        const float v = static_cast<float>(std::ldexp(1.0 + (nxt() % 8) / 8.0, -static_cast<int>(nxt() % 30)));
        std::vector<float> x(n, v);
        check(x, true);
    }
    // 3. PageRank-like: 1/N-scale contributions divided by small degrees
    for (int t = 0; t < 300; t++) {
        const uint32_t n = 256 + nxt() % 100000;
        const float base = 1.0f / static_cast<float>(1u << (10 + nxt() % 14));
        std::vector<float> x(n);
        for (auto &v : x) v = base / static_cast<float>(1 + nxt() % 64);
        check(x, true);
    }
    // 4. zeros: leading, interleaved, all
    for (int t = 0; t < 300; t++) {
        const uint32_t n = 1 + nxt() % 2000;
        std::vector<float> x(n);
        const uint32_t lead = nxt() % (n + 1);
        for (uint32_t i = 0; i < n; i++)
            x[i] = (i < lead || nxt() % 3 == 0) ? ((nxt() & 1) ? 0.0f : -0.0f) : static_cast<float>(unit());
        check(x, true);
    }
    // 5. constructed ties and near-ties against the running sum
    for (int t = 0; t < 2000; t++) {
        const uint32_t n = 2 + nxt() % 3000;
        std::vector<float> x(n);
        float s = 0.0f;
        for (uint32_t i = 0; i < n; i++) {
            if (s > 0.0f && nxt() % 2) {
                const int e = static_cast<int>((fb(s) >> 23) & 0xff) - 150;       // ulp exponent of s
                const int sh = static_cast<int>(nxt() % 20);
                const double ulp = std::ldexp(1.0, e);
                double v = ulp * (static_cast<double>(nxt() % (1u << sh)) + 0.5);  // exact half-ulp multiples
                if (nxt() % 3 == 0) v = std::nextafter(v, 0.0);
                x[i] = static_cast<float>(v);
                if (!(x[i] >= 0.0f)) x[i] = 0.0f;
            } else {
                x[i] = static_cast<float>(std::ldexp(1.0 + unit(), -static_cast<int>(nxt() % 30)));
            }
            s = s + x[i];
        }
        check(x, true);
    }
    // 6. increasing and decreasing magnitudes: a crossing in most windows
    for (int t = 0; t < 200; t++) {
        const uint32_t n = 1000 + nxt() % 20000;
        std::vector<float> x(n);
        for (uint32_t i = 0; i < n; i++) x[i] = static_cast<float>(std::ldexp(1.0 + unit(), static_cast<int>(i / 200) - 60));
        check(x, true);
        std::vector<float> y(x.rbegin(), x.rend());
        check(y, true);
    }
    // 7. out-of-domain terms are reported, never summed wrongly
    {
        std::vector<float> x(600, 1.0f); x[300] = -1.0f; check(x, false);
        std::vector<float> y(600, 1.0f); y[7] = 1e-40f; check(y, false);
        std::vector<float> z(600, 1.0f); z[599] = INFINITY; check(z, false);
        std::vector<float> w(600, 3e38f); check(w, false);
    }
}
"""


def test_warp_sequential_sum_matches_loop(tmp_path):
    src = tmp_path / "check.cpp"
    src.write_text(CHECKER)
    exe = tmp_path / "check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", f"-I{HEADER.parent}", str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stdout[-3000:]
    assert "bad 0" in out.stdout


STEP_CHECK = r"""
#include <cstdio>
#include <cstdint>
#include "bw_seqsum.h"
using namespace bwseq;
static uint64_t rng = 0x9e3779b97f4a7c15ULL;
static uint64_t nxt() { rng ^= rng << 13; rng ^= rng >> 7; rng ^= rng << 17; return rng; }
int main() {
    long bad = 0, n = 0;
    for (long i = 0; i < 20000000; i++) {
        uint32_t xb = static_cast<uint32_t>(nxt());
        if (i % 7 == 0) xb &= 0x807fffffu;            // zero exponent: zeros and subnormals
        if (i % 11 == 0) xb = 0;
        const uint32_t k = 1 + static_cast<uint32_t>(nxt() % 254);
        Map a; const bool oka = step(xb, k, a);
        bool okb = true; const Map b = step_select(xb, k, okb);
        n++;
        if (oka != okb || (oka && (a.e != b.e || a.o != b.o))) {
            if (bad < 5) std::printf("x=%08x k=%u step=(%u,%u,%d) select=(%u,%u,%d)\n", xb, k, a.e, a.o, oka, b.e, b.o, okb);
            bad++;
        }
    }
    std::printf("tested %ld bad %ld\n", n, bad);
    return bad ? 1 : 0;
}
"""


def test_branch_free_step_matches(tmp_path):
    """step_select (the wide kernel's branch-free form) equals step on 20M
    random terms and binades, including zeros, subnormals, negatives and
    inf/NaN."""
    src = tmp_path / "step.cpp"
    src.write_text(STEP_CHECK)
    exe = tmp_path / "step"
    subprocess.run(["g++", "-O2", "-std=c++17", f"-I{HEADER.parent}", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stdout[-2000:]
