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

// Warp emulation of the continuation over terms [b, e) from the running sum
// sb (warp_sequential_continue); returns false when the kernel would fall
// back.
static bool warp_continue(const std::vector<float> &vals, uint32_t b, uint32_t e, uint32_t &sb) {
    const uint32_t WIN = 32 * L, n = e;
    for (uint32_t w = b; w < n; w += WIN) {
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
                        for (uint32_t u = 0; u + st < L; u += 2 * st) t[u] = compose_short(t[u], t[u + st]);
                    m[lane] = saturated(t[0]);
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
    return true;
}

static bool warp_sum(const std::vector<float> &vals, uint32_t &out) {
    uint32_t sb = 0;
    if (!warp_continue(vals, 0, vals.size(), sb)) return false;
    out = sb;
    return true;
}

static uint64_t rng = 0x243f6a8885a308d3ULL;
static uint64_t nxt() { rng ^= rng << 13; rng ^= rng >> 7; rng ^= rng << 17; return rng; }
static double unit() { return (nxt() >> 11) * (1.0 / 9007199254740992.0); }

// Piece-parallel emulation (the giant rows of k_pr_long_sums): pieces of
// 512 terms; piece 0 adds the first 1024 terms in order; every later piece
// guesses the running sum at its start (the float sums of the pieces before
// it, added in double) and records, in the guessed binade, the map of its
// terms, or -- when the guessed sum crosses into the next binade inside the
// piece -- the map before the crossing term, that term, and the map of the
// rest in the new binade.  The combination applies a record where it holds
// for the true running sum and evaluates the piece exactly otherwise.
// guess_mode 1 replaces the guesses by wrong ones (a neighbouring binade,
// a shifted significand, or none) at random: the result must not change.
static int guess_mode = 0;
static long pieces_mapped = 0, pieces_crossed = 0, pieces_exact = 0;
struct Rec { uint32_t kind = 0, K = 0, K2 = 0, tg = 0, xb = 0; Map m1{0, 0}, m2{0, 0}; };

static Rec make_record(const std::vector<float> &vals, uint32_t b, uint32_t e, uint32_t guess) {
    Rec r;
    if (!in_domain(guess)) return r;
    const uint32_t K = exponent_of(guess);
    bool good = true;
    Map total = identity();
    for (uint32_t i = b; i < e; i++) total = compose(total, step_select(fb(vals[i]), K, good));
    if (!good) return r;
    uint32_t acc = significand_of(guess), nb = 0;
    int tg = -1;
    Map m1 = identity();
    for (uint32_t i = b; i < e && tg < 0; i++) {
        Map st; step(fb(vals[i]), K, st);
        const uint32_t bu = apply(st, acc);
        if (bu >= TOP) {
            tg = static_cast<int>(i - b);
            volatile float s0 = bf(bits_of(K, acc));
            volatile float s1 = s0 + vals[i];
            nb = fb(s1);
        } else { acc = bu; m1 = compose(m1, st); }
    }
    if (tg < 0) { r.kind = 1; r.K = K; r.m1 = total; return r; }
    if (!in_domain(nb)) return r;
    const uint32_t K2 = exponent_of(nb);
    Map m2 = identity();
    for (uint32_t i = b + tg + 1; i < e; i++) m2 = compose(m2, step_select(fb(vals[i]), K2, good));
    r.kind = 3; r.K = K; r.K2 = K2; r.tg = tg; r.xb = fb(vals[b + tg]); r.m1 = m1; r.m2 = m2;
    return r;
}

static bool piece_advance(const std::vector<float> &vals, uint32_t b, uint32_t e, const Rec &r, uint32_t &sb) {
    if ((r.kind == 1 || r.kind == 3) && in_domain(sb) && exponent_of(sb) == r.K) {
        const uint32_t a1 = apply(r.m1, significand_of(sb));
        if (r.kind == 1 && a1 < TOP) { sb = bits_of(r.K, a1); pieces_mapped++; return true; }
        Map st;
        if (r.kind == 3 && a1 < TOP && step(r.xb, r.K, st) && apply(st, a1) >= TOP) {
            volatile float s0 = bf(bits_of(r.K, a1));
            volatile float s1 = s0 + bf(r.xb);
            const uint32_t nb = fb(s1);
            if (in_domain(nb) && exponent_of(nb) == r.K2) {
                const uint32_t a3 = apply(r.m2, significand_of(nb));
                if (a3 < TOP) { sb = bits_of(r.K2, a3); pieces_crossed++; return true; }
            }
        }
    }
    pieces_exact++;
    return warp_continue(vals, b, e, sb);
}

static bool piece_sum(const std::vector<float> &vals, uint32_t &out) {
    const uint32_t PIECE = 512, n = vals.size(), P = (n + PIECE - 1) / PIECE;
    const uint32_t save_l = L, save_st = serial_terms;
    L = PIECE / 32; serial_terms = 1024;
    std::vector<float> ps(P);
    for (uint32_t p = 0; p < P; p++) {              // in any order: here backwards
        volatile float s = 0.0f;
        for (uint32_t i = std::min(n, (p + 1) * PIECE); i-- > p * PIECE;) s = s + vals[i];
        ps[p] = s;
    }
    std::vector<Rec> rec(P);
    for (uint32_t q = 2; q < P; q++) {
        double pre = 0.0;
        for (uint32_t i = 0; i < q; i++) pre += ps[i];
        uint32_t g = fb(static_cast<float>(pre));
        if (guess_mode == 1) {
            const uint32_t r = nxt() % 5;
            if (r == 1 && exponent_of(g) > 1) g -= 1u << 23;
            if (r == 2 && exponent_of(g) < 0xfdu) g += 1u << 23;
            if (r == 3) g = 0;
            if (r == 4) g ^= static_cast<uint32_t>(nxt()) & 0x7fffffu;
        }
        rec[q] = make_record(vals, q * PIECE, std::min(n, q * PIECE + PIECE), g);
    }
    volatile float s0 = 0.0f;                        // the serial start
    for (uint32_t i = 0; i < std::min(n, 1024u); i++) s0 = s0 + vals[i];
    uint32_t sb = fb(s0);
    bool ok = true;
    for (uint32_t q = 2; q < P && ok; q++) ok = piece_advance(vals, q * PIECE, std::min(n, q * PIECE + PIECE), rec[q], sb);
    L = save_l; serial_terms = save_st;
    if (!ok) return false;
    out = sb;
    return true;
}


static int bad = 0, tested = 0, fallback = 0;
static bool use_pieces = false;
static void check(const std::vector<float> &x, bool expect_domain) {
    uint32_t got;
    const bool ok = use_pieces ? piece_sum(x, got) : warp_sum(x, got);
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

static void run_giant();

int main(int argc, char **argv) {
    if (argc > 1) {                                  // the piece-parallel scheme
        use_pieces = true;
        for (int mode : {0, 1}) { guess_mode = mode; run_giant(); }
        std::printf("mapped %ld crossed %ld exact %ld\n", pieces_mapped, pieces_crossed, pieces_exact);
    } else {
        for (uint32_t l : {8u, 32u})
            for (uint32_t st : {0u, 64u, 300u, 1024u}) { L = l; serial_terms = st; run_all(); }
    }
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

// Rows above the giant threshold, as the piece-parallel scheme sees them.
static void run_giant() {
    // log-uniform magnitudes
    for (int t = 0; t < 150; t++) {
        const uint32_t n = 4097 + nxt() % 60000;
        const int span = 1 + nxt() % 40;
        std::vector<float> x(n);
        for (auto &v : x) v = static_cast<float>(std::ldexp(1.0 + unit(), -static_cast<int>(nxt() % span) - 10));
        check(x, true);
    }
    // equal terms: running sums at exact powers of two, ties at every step
    for (int t = 0; t < 60; t++) {
        const uint32_t n = 4097 + nxt() % 200000;
        const float v = static_cast<float>(std::ldexp(1.0 + (nxt() % 8) / 8.0, -static_cast<int>(nxt() % 30)));
        std::vector<float> x(n, v);
        check(x, true);
    }
    // PageRank-like terms, hub-sized rows
    for (int t = 0; t < 60; t++) {
        const uint32_t n = 4097 + nxt() % 120000;
        const float base = 1.0f / static_cast<float>(1u << (10 + nxt() % 14));
        std::vector<float> x(n);
        for (auto &v : x) v = base / static_cast<float>(1 + nxt() % 64);
        check(x, true);
    }
    // growing magnitudes: a binade crossing in most pieces; and shrinking
    for (int t = 0; t < 60; t++) {
        const uint32_t n = 4097 + nxt() % 30000;
        std::vector<float> x(n);
        const uint32_t step = n / 100 + 1 + nxt() % 600;   // up to 2^40: no overflow
        for (uint32_t i = 0; i < n; i++) x[i] = static_cast<float>(std::ldexp(1.0 + unit(), static_cast<int>(i / step) - 60));
        check(x, true);
        std::vector<float> y(x.rbegin(), x.rend());
        check(y, true);
    }
    // zeros through the serial start and beyond, then terms
    for (int t = 0; t < 40; t++) {
        const uint32_t n = 4097 + nxt() % 20000, lead = nxt() % n;
        std::vector<float> x(n);
        for (uint32_t i = 0; i < n; i++) x[i] = i < lead ? 0.0f : static_cast<float>(std::ldexp(1.0 + unit(), -20));
        check(x, true);
    }
    // one huge term late in the row: every later guess is far off
    for (int t = 0; t < 40; t++) {
        const uint32_t n = 4097 + nxt() % 20000;
        std::vector<float> x(n, 1e-6f);
        x[2048 + nxt() % (n - 2048)] = 1e3f;
        check(x, true);
    }
    // out of domain in a mapped piece: reported
    {
        std::vector<float> x(9000, 1.0f); x[7000] = -1.0f; check(x, false);
        std::vector<float> y(9000, 1.0f); y[5000] = 1e-40f; check(y, false);
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


def test_piece_parallel_sum_matches_loop(tmp_path):
    """The giant-row scheme of k_pr_long_sums (per 512-term piece, maps in a
    guessed binade with the guessed crossing term, combined in order with
    exact re-evaluation where a record does not hold) equals the plain loop
    bit for bit, with the real guesses and with guesses made wrong at
    random."""
    src = tmp_path / "check.cpp"
    src.write_text(CHECKER)
    exe = tmp_path / "check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", f"-I{HEADER.parent}", str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe), "pieces"], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stdout[-3000:]
    assert "bad 0" in out.stdout
    assert "fallback 4 " in out.stdout          # the two out-of-domain rows, in both modes
    words = out.stdout.split("mapped ")[1].split()
    mapped, crossed, exact = int(words[0]), int(words[2]), int(words[4])
    assert mapped > exact and crossed > 0       # the records do the bulk of the work


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
