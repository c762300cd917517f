/*
 * oracle.c -- CPU restatement of the reference's BFS and PageRank semantics.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py load this library, and only as the checker or
 * the timed CPU baseline.  The product (libbelewitte_gb300.so and the plugin
 * libraries) never links or calls it.
 *
 * Parity pinning: the reference ships no tests or golden vectors.  This
 * restatement is pinned against the reference's own CUDA kernels, compiled
 * unmodified from the reference sources into cubins under oracle/_ref/ and run on
 * the GPU by oracle/ref_launch.c (see tests/test_reference_pin.py), and the
 * fixtures in tests/golden/ were produced by that run.
 *
 * Compile with -ffp-contract=off: every float operation below is a separate
 * IEEE single-precision operation unless it calls fmaf() explicitly, which is
 * how the reference kernels' arithmetic is restated.
 */
#include <limits.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "oracle.h"

/* Reference damping factor: pagerank/pagerank.hpp:9 (const float 0.85f). */
static const float DAMPING = 0.85f;

/*
 * Level-synchronous BFS over the forward CSR.
 *
 * Every reference BFS variant computes the same per-level relation:
 * a vertex u with levels[u] == depth relaxes each out-neighbour v with
 * atomicMin(levels[v], depth+1) and counts the visit when the old value was
 * larger (bfs/edgelist.cu:13-19, bfs/vertex_push.cu:11-23,
 * bfs/vertex_push_warp.cu:51-56), or, pulling, an unvisited v takes depth+1
 * when any in-neighbour has levels == depth (bfs/vertex_pull.cu:12-28,
 * bfs/vertex_pull_warp.cu:53-67).  Both give exact BFS depths and the same
 * per-level count of newly visited vertices.  The host loop runs levels
 * until a level visits nothing (bfs/bfs.cpp:80-107) and unreached vertices
 * keep INT_MAX (bfs/bfs.cpp:71-74).
 *
 * levels[n] out; level_counts[] (optional) receives the per-level visit
 * count (the reference's `frontier`), including the final 0.  Returns the
 * number of levels run, or -1 when max_levels is hit.
 */
int64_t or_bfs(uint64_t n, const uint32_t *off, const uint32_t *edges,
               uint32_t root, int32_t *levels, uint32_t *level_counts,
               uint64_t max_levels)
{
    uint32_t *cur = (uint32_t *) malloc((n ? n : 1) * sizeof(uint32_t));
    uint32_t *next = (uint32_t *) malloc((n ? n : 1) * sizeof(uint32_t));
    uint64_t cur_len = 0, next_len, level = 0;
    for (uint64_t i = 0; i < n; i++) levels[i] = INT_MAX;
    if (root >= n) { free(cur); free(next); return 0; }
    levels[root] = 0;
    cur[cur_len++] = root;
    for (;;) {
        if (level >= max_levels) { free(cur); free(next); return -1; }
        next_len = 0;
        int32_t nd = (int32_t) level + 1;
        for (uint64_t i = 0; i < cur_len; i++) {
            uint32_t u = cur[i];
            for (uint32_t e = off[u]; e < off[u + 1]; e++) {
                uint32_t v = edges[e];
                if (levels[v] > nd) { levels[v] = nd; next[next_len++] = v; }
            }
        }
        if (level_counts) level_counts[level] = (uint32_t) next_len;
        level++;
        if (next_len == 0) break;
        uint32_t *t = cur; cur = next; next = t;
        cur_len = next_len;
    }
    free(cur);
    free(next);
    return (int64_t) level;
}

/*
 * CPU BFS baseline: the reference's only CPU BFS, evolve/Connectivity.cpp:29-77
 * (level-synchronous, parallel over vertices, atomic-min on depths, repeat
 * while any depth changed), with OpenMP in place of TBB and a root
 * parameter in place of vertex 0.  Returns the number of levels run.
 */
int64_t or_bfs_parallel(uint64_t n, const uint32_t *off, const uint32_t *edges,
                        uint32_t root, int32_t *levels, int threads)
{
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void) threads;
#endif
    for (uint64_t i = 0; i < n; i++) levels[i] = INT_MAX;
    if (root >= n) return 0;
    levels[root] = 0;
    int64_t level = 0;
    int changed = 1;
    while (changed) {
        changed = 0;
        const int32_t cur = (int32_t) level, nd = (int32_t) level + 1;
#pragma omp parallel for schedule(dynamic, 1024) reduction(| : changed)
        for (int64_t u = 0; u < (int64_t) n; u++) {
            if (levels[u] != cur) continue;
            for (uint32_t e = off[u]; e < off[u + 1]; e++) {
                uint32_t v = edges[e];
                int32_t old = __atomic_load_n(&levels[v], __ATOMIC_RELAXED);
                while (old > nd) {
                    if (__atomic_compare_exchange_n(&levels[v], &old, nd, 0,
                                                    __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
                        changed = 1;
                        break;
                    }
                }
            }
        }
        level++;
    }
    return level;
}

/* Out-degree of every vertex; all reference degree kernels compute this
 * (pagerank/pagerank.cu:40-123: forward edge lists count inEdges (sources),
 * reverse ones count outEdges (sources), reverseCSRComputeDegrees counts
 * each reverse-row entry; the push variants use the CSR row length,
 * pagerank/vertex_push.cu:20-25). */
void or_out_degrees(uint64_t n, const uint32_t *rev_off, const uint32_t *rev_edges,
                    uint32_t *deg)
{
    memset(deg, 0, n * sizeof(uint32_t));
    for (uint64_t v = 0; v < n; v++)
        for (uint32_t e = rev_off[v]; e < rev_off[v + 1]; e++) deg[rev_edges[e]]++;
}

/*
 * FP32 PageRank with the reference's exact arithmetic, summing each
 * destination's contributions in increasing source order: that is the
 * sequential order of vertex-pull (pagerank/vertex_pull.cu:23-27) and of the
 * edge-list variants processed one edge at a time (their float atomics make
 * the GPU order arbitrary; this is the canonical one).
 *
 *  semantics OR_PR_DIV:   acc[v] = sum pr[u] / (float) deg[u]
 *                         (pagerank/vertex_pull.cu:26, edgelist.cu:18-21)
 *                         pr[v]  = (float)((1.0 - 0.85f)/N + (double)(0.85f*acc))
 *                         (consolidateRank, pagerank/pagerank.cu:131-136)
 *  semantics OR_PR_NODIV: acc[v] = sum pr[u]   (vertex_pull_nodiv.cu:23-25)
 *                         pr[v]  = fmaf(0.85f, acc, (1 - 0.85f)/(float)N),
 *                         then / (float) deg[v] when deg != 0 and this is
 *                         not the last iteration
 *                         (consolidateRankNoDiv, pagerank.cu:153-161)
 * Initial ranks 1.0f / N, accumulator 0 (pagerank/pagerank.cpp:88-92);
 * exactly `iterations` iterations (pagerank.cpp:115-125, notLast =
 * iterations > j).  The nodiv initial ranks are NOT pre-divided, so the
 * first nodiv iteration sums raw 1/N values (pagerank.cpp:88).
 *
 * diffs[] (optional) gets sum |pr_new - pr_old| per iteration in double.
 */
void or_pagerank(int semantics, uint64_t n, const uint32_t *rev_off,
                 const uint32_t *rev_edges, const uint32_t *deg,
                 uint32_t iterations, float *pr, double *diffs)
{
    float *acc = (float *) malloc((n ? n : 1) * sizeof(float));
    const float init = 1.0f / (float) n;
    for (uint64_t v = 0; v < n; v++) pr[v] = init;
    const double base_div = (1.0 - (double) DAMPING) / (double) n;
    const float base_nodiv = (1 - DAMPING) / (float) n;
    for (uint32_t j = 1; j <= iterations; j++) {
        for (uint64_t v = 0; v < n; v++) {
            float s = 0.0f;
            if (semantics == OR_PR_DIV) {
                for (uint32_t e = rev_off[v]; e < rev_off[v + 1]; e++) {
                    uint32_t u = rev_edges[e];
                    s += pr[u] / (float) deg[u];
                }
            } else {
                for (uint32_t e = rev_off[v]; e < rev_off[v + 1]; e++) s += pr[rev_edges[e]];
            }
            acc[v] = s;
        }
        const int not_last = iterations > j;
        double diff = 0.0;
        for (uint64_t v = 0; v < n; v++) {
            float nr;
            if (semantics == OR_PR_DIV) {
                float scaled = DAMPING * acc[v];
                nr = (float) (base_div + (double) scaled);
                diff += fabs((double) nr - (double) pr[v]);
            } else {
                nr = fmaf(DAMPING, acc[v], base_nodiv);
                diff += fabs((double) nr - (double) pr[v]);
                if (deg[v] != 0 && not_last) nr = nr / (float) deg[v];
            }
            pr[v] = nr;
        }
        if (diffs) diffs[j - 1] = diff;
    }
    free(acc);
}

/*
 * FP64 PageRank with the same two semantics (no float rounding anywhere):
 * the accuracy yardstick for every FP32 variant.
 */
void or_pagerank_f64(int semantics, uint64_t n, const uint32_t *rev_off,
                     const uint32_t *rev_edges, const uint32_t *deg,
                     uint32_t iterations, double *pr)
{
    double *acc = (double *) malloc((n ? n : 1) * sizeof(double));
    for (uint64_t v = 0; v < n; v++) pr[v] = 1.0 / (double) n;
    for (uint32_t j = 1; j <= iterations; j++) {
        for (uint64_t v = 0; v < n; v++) {
            double s = 0.0;
            for (uint32_t e = rev_off[v]; e < rev_off[v + 1]; e++) {
                uint32_t u = rev_edges[e];
                s += semantics == OR_PR_DIV ? pr[u] / (double) deg[u] : pr[u];
            }
            acc[v] = s;
        }
        const int not_last = iterations > j;
        for (uint64_t v = 0; v < n; v++) {
            double nr = 0.15 / (double) n + 0.85 * acc[v];
            if (semantics == OR_PR_NODIV && deg[v] != 0 && not_last) nr /= (double) deg[v];
            pr[v] = nr;
        }
    }
    free(acc);
}

/*
 * Multi-threaded FP32 PageRank (div semantics, vertex-pull order) for the
 * CPU baseline: the reference has no CPU PageRank, so this times the
 * restatement of vertex-pull + consolidateRank with OpenMP over vertices.
 * Bit-identical to or_pagerank(OR_PR_DIV, ...).
 */
void or_pagerank_parallel(uint64_t n, const uint32_t *rev_off,
                          const uint32_t *rev_edges, const uint32_t *deg,
                          uint32_t iterations, float *pr, int threads)
{
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void) threads;
#endif
    float *contrib = (float *) malloc((n ? n : 1) * sizeof(float));
    float *next = (float *) malloc((n ? n : 1) * sizeof(float));
    const float init = 1.0f / (float) n;
    const double base = (1.0 - (double) DAMPING) / (double) n;
#pragma omp parallel for schedule(static)
    for (int64_t v = 0; v < (int64_t) n; v++) pr[v] = init;
    for (uint32_t j = 1; j <= iterations; j++) {
#pragma omp parallel for schedule(static)
        for (int64_t u = 0; u < (int64_t) n; u++)
            contrib[u] = deg[u] ? pr[u] / (float) deg[u] : 0.0f;
#pragma omp parallel for schedule(dynamic, 4096)
        for (int64_t v = 0; v < (int64_t) n; v++) {
            float s = 0.0f;
            for (uint32_t e = rev_off[v]; e < rev_off[v + 1]; e++) s += contrib[rev_edges[e]];
            float scaled = DAMPING * s;
            next[v] = (float) (base + (double) scaled);
        }
        memcpy(pr, next, n * sizeof(float));
    }
    free(contrib);
    free(next);
}

/* The reference's --validate PageRank output line format
 * (pagerank/pagerank.cpp:135-141): setprecision(digits10 + 1) = 7
 * significant digits in default float notation. */
int or_format_rank(float value, char *buf, int len)
{
    return snprintf(buf, (size_t) len, "%.7g", (double) value);
}

/*
 * Seeded R-MAT graph, built without the product library, so that the
 * reference arm of the benchmark and the CPU baselines can make the very
 * graph the GPU runs on.  It restates the library's own counter-based
 * generator (not a reference algorithm; the reference's generator is
 * evolve/gen-graph.cpp, which has no R-MAT): edge e draws scale quadrant
 * choices, two per 64-bit hash of (seed, e, level / 2), most significant
 * bit first, with the cumulative probabilities a, a+b, a+b+c scaled to 2^32.
 * Self-loops and duplicates are dropped; rows of the forward and reverse
 * CSR are sorted.  The CSR arrays are malloc'd (or_graph_free).
 */
static uint64_t or_mix64(uint64_t z)
{
    z += 0x9e3779b97f4a7c15ULL;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

static uint64_t or_hash3(uint64_t seed, uint64_t a, uint64_t b)
{
    return or_mix64(or_mix64(seed ^ or_mix64(a)) ^ (b * 0xd1b54a32d192ed03ULL));
}

static int or_cmp_u32(const void *x, const void *y)
{
    const uint32_t a = *(const uint32_t *) x, b = *(const uint32_t *) y;
    return (a > b) - (a < b);
}

/* Counting sort of (src[i], dst[i]) pairs, i < count, into rows of n
 * (pairs with src == UINT32_MAX skipped); every row sorted and de-duplicated
 * when `unique`.  Deterministic for any thread count: threads own contiguous
 * input ranges and write each row's entries in input order. */
static int or_pairs_to_csr(uint64_t n, uint64_t count, const uint32_t *src, const uint32_t *dst,
                           int unique, uint32_t **off_out, uint32_t **edges_out, uint64_t *m_out)
{
    int T = 1;
#ifdef _OPENMP
    T = omp_get_max_threads();
#endif
    uint64_t *cnt = (uint64_t *) calloc((size_t) T * (n + 1), sizeof(uint64_t));
    uint32_t *buf = (uint32_t *) malloc((count ? count : 1) * sizeof(uint32_t));
    uint64_t *start = (uint64_t *) malloc((n + 1) * sizeof(uint64_t));
    uint32_t *len = (uint32_t *) malloc((n ? n : 1) * sizeof(uint32_t));
    if (!cnt || !buf || !start || !len) { free(cnt); free(buf); free(start); free(len); return -1; }
#pragma omp parallel num_threads(T)
    {
        int t = 0;
#ifdef _OPENMP
        t = omp_get_thread_num();
#endif
        const uint64_t lo = count * (uint64_t) t / (uint64_t) T, hi = count * (uint64_t) (t + 1) / (uint64_t) T;
        uint64_t *c = cnt + (size_t) t * (n + 1);
        for (uint64_t i = lo; i < hi; i++)
            if (src[i] != UINT32_MAX) c[src[i]]++;
#pragma omp barrier
#pragma omp single
        {
            uint64_t sum = 0;
            for (uint64_t r = 0; r < n; r++) {
                start[r] = sum;
                for (int tt = 0; tt < T; tt++) {
                    const uint64_t k = cnt[(size_t) tt * (n + 1) + r];
                    cnt[(size_t) tt * (n + 1) + r] = sum;
                    sum += k;
                }
            }
            start[n] = sum;
        }
        for (uint64_t i = lo; i < hi; i++)
            if (src[i] != UINT32_MAX) buf[c[src[i]]++] = dst[i];
    }
    free(cnt);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t r = 0; r < (int64_t) n; r++) {
        uint32_t *row = buf + start[r];
        const uint64_t k = start[r + 1] - start[r];
        if (k > 1) qsort(row, k, sizeof(uint32_t), or_cmp_u32);
        uint64_t w = k;
        if (unique && k > 1) {
            w = 1;
            for (uint64_t i = 1; i < k; i++)
                if (row[i] != row[w - 1]) row[w++] = row[i];
        }
        len[r] = (uint32_t) w;
    }
    uint32_t *off = (uint32_t *) malloc((n + 1) * sizeof(uint32_t));
    uint64_t m = 0;
    for (uint64_t r = 0; r < n; r++) m += len[r];
    uint32_t *edges = (uint32_t *) malloc((m ? m : 1) * sizeof(uint32_t));
    if (!off || !edges || m > 0xffffffffULL) { free(off); free(edges); free(buf); free(start); free(len); return -1; }
    uint64_t acc = 0;
    for (uint64_t r = 0; r < n; r++) { off[r] = (uint32_t) acc; acc += len[r]; }
    off[n] = (uint32_t) acc;
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t r = 0; r < (int64_t) n; r++)
        memcpy(edges + off[r], buf + start[r], (size_t) len[r] * sizeof(uint32_t));
    free(buf); free(start); free(len);
    *off_out = off; *edges_out = edges; *m_out = m;
    return 0;
}

int or_generate_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c, uint64_t seed,
                     int symmetrise, or_graph *out)
{
    memset(out, 0, sizeof *out);
    if (scale < 1 || scale > 31 || edge_factor == 0) return -1;
    const uint64_t n = (uint64_t) 1 << scale, count = n * edge_factor, total = count * (symmetrise ? 2 : 1);
    const double two32 = 4294967296.0;
    const uint64_t ta = (uint64_t) (a * two32), tab = (uint64_t) ((a + b) * two32),
                   tabc = (uint64_t) ((a + b + c) * two32);
    uint32_t *src = (uint32_t *) malloc(total * sizeof(uint32_t));
    uint32_t *dst = (uint32_t *) malloc(total * sizeof(uint32_t));
    if (!src || !dst) { free(src); free(dst); return -1; }
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < (int64_t) count; e++) {
        uint64_t sv = 0, dv = 0, h = 0;
        for (uint32_t l = 0; l < scale; l++) {
            uint64_t r;
            if ((l & 1) == 0) { h = or_hash3(seed, (uint64_t) e, l >> 1); r = h & 0xffffffffULL; }
            else r = h >> 32;
            const uint64_t sb = r >= tab, db = (r >= ta && r < tab) || r >= tabc;
            sv = (sv << 1) | sb;
            dv = (dv << 1) | db;
        }
        const int loop = sv == dv;
        if (symmetrise) {
            src[2 * e] = loop ? UINT32_MAX : (uint32_t) sv;  dst[2 * e] = (uint32_t) dv;
            src[2 * e + 1] = loop ? UINT32_MAX : (uint32_t) dv;  dst[2 * e + 1] = (uint32_t) sv;
        } else {
            src[e] = loop ? UINT32_MAX : (uint32_t) sv;  dst[e] = (uint32_t) dv;
        }
    }
    int rc = or_pairs_to_csr(n, total, src, dst, 1, &out->fwd_off, &out->fwd_edges, &out->m);
    free(src); free(dst);
    if (rc) return rc;
    out->n = n;
    if (symmetrise) {
        out->rev_off = out->fwd_off;
        out->rev_edges = out->fwd_edges;
        return 0;
    }
    /* reverse CSR: the forward edges counted by destination, in source
     * order (so each reverse row comes out sorted) */
    const uint64_t m = out->m;
    uint32_t *rs = (uint32_t *) malloc((m ? m : 1) * sizeof(uint32_t));
    if (!rs) { or_graph_free(out); return -1; }
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t u = 0; u < (int64_t) n; u++)
        for (uint32_t k = out->fwd_off[u]; k < out->fwd_off[u + 1]; k++) rs[k] = (uint32_t) u;
    uint64_t m2 = 0;
    rc = or_pairs_to_csr(n, m, out->fwd_edges, rs, 0, &out->rev_off, &out->rev_edges, &m2);
    free(rs);
    if (rc || m2 != m) { or_graph_free(out); return -1; }
    return 0;
}

void or_graph_free(or_graph *g)
{
    if (g->rev_off != g->fwd_off) free(g->rev_off);
    if (g->rev_edges != g->fwd_edges) free(g->rev_edges);
    free(g->fwd_off);
    free(g->fwd_edges);
    memset(g, 0, sizeof *g);
}
