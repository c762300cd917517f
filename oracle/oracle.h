/* oracle.h -- CPU restatement of the reference's BFS / PageRank semantics.
 * TEST INFRASTRUCTURE ONLY (tests/, smoke(), bench.py's CPU baseline). */
#ifndef BW_ORACLE_H
#define BW_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { OR_PR_DIV = 0, OR_PR_NODIV = 1 };

int64_t or_bfs(uint64_t n, const uint32_t *off, const uint32_t *edges,
               uint32_t root, int32_t *levels, uint32_t *level_counts,
               uint64_t max_levels);
int64_t or_bfs_parallel(uint64_t n, const uint32_t *off, const uint32_t *edges,
                        uint32_t root, int32_t *levels, int threads);
void or_out_degrees(uint64_t n, const uint32_t *rev_off,
                    const uint32_t *rev_edges, uint32_t *deg);
void or_pagerank(int semantics, uint64_t n, const uint32_t *rev_off,
                 const uint32_t *rev_edges, const uint32_t *deg,
                 uint32_t iterations, float *pr, double *diffs);
void or_pagerank_f64(int semantics, uint64_t n, const uint32_t *rev_off,
                     const uint32_t *rev_edges, const uint32_t *deg,
                     uint32_t iterations, double *pr);
void or_pagerank_parallel(uint64_t n, const uint32_t *rev_off,
                          const uint32_t *rev_edges, const uint32_t *deg,
                          uint32_t iterations, float *pr, int threads);
int or_format_rank(float value, char *buf, int len);

/* A seeded R-MAT graph (forward + reverse CSR, malloc'd), made without the
 * product library; identical to its bw_generate_rmat graph. */
typedef struct {
    uint64_t n, m;
    uint32_t *fwd_off, *fwd_edges, *rev_off, *rev_edges;
} or_graph;
int or_generate_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c, uint64_t seed,
                     int symmetrise, or_graph *out);
void or_graph_free(or_graph *g);

#ifdef __cplusplus
}
#endif
#endif
