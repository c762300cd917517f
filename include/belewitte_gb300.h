/*
 * belewitte_gb300.h -- C ABI of the GB300 (sm_103a) BFS and PageRank kernel
 * libraries.
 *
 * Everything here is plain C: pointers, sizes and status codes.  Device
 * pointers are CUDA global-memory addresses owned by the caller; the library
 * never frees caller memory.  The only memory the library owns is the scratch
 * of a bw_context (frontier queues, counters, degree and rank buffers, CUDA
 * graphs), released by bw_context_destroy().  Streams are passed as `void *`
 * holding a cudaStream_t (NULL = legacy default stream).
 *
 * The reference drives its kernels through a C++ plugin surface
 * (ImplementationTemplate.hpp GraphKernel::operator() -> CUDABackend::runKernel,
 * CUDA.hpp:256-263) with per-algorithm device globals for the frontier / diff
 * counters (bfs/bfs.cu:5-18, pagerank/pagerank.cu:4-17).  Each entry point
 * below names the reference interface it replaces.  Errors are returned as
 * status codes instead of the reference's print-and-exit (CUDA.cpp:7-26,
 * utils/Util.hpp:67-74).
 */
#ifndef BELEWITTE_GB300_H
#define BELEWITTE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------ */
/* Status codes                                                              */
/* ------------------------------------------------------------------------ */
enum bw_status {
    BW_OK = 0,
    BW_ERR_INVALID_ARGUMENT = 1,    /* NULL pointer, size out of range, ... */
    BW_ERR_MISSING_REPRESENTATION = 2, /* variant needs a rep the view lacks */
    BW_ERR_UNKNOWN_VARIANT = 3,
    BW_ERR_CUDA = 4,                /* a CUDA runtime call failed */
    BW_ERR_OUT_OF_MEMORY = 5,
    BW_ERR_LEVEL_LIMIT = 6,         /* traversal exceeded its level cap */
    BW_ERR_TOO_LARGE = 7,           /* counts beyond the uint32 format */
    BW_ERR_IO = 8,                  /* graph file could not be read/written */
    BW_ERR_FORMAT = 9,              /* graph file is malformed */
    BW_ERR_NO_DEVICE = 10
};

/* Human readable text of a status code (static storage). */
const char *bw_status_string(int status);
/* Text of the last CUDA error seen by this thread (static storage). */
const char *bw_last_error(void);
/* Library version / commit stamp; reference: Algorithm.hpp:8 KERNEL_COMMIT. */
const char *bw_version(void);

/* ------------------------------------------------------------------------ */
/* Graph representations                                                     */
/* ------------------------------------------------------------------------ */
/*
 * Device view of one graph in every representation the reference's
 * GraphLoader builds (GraphLoader.hpp:123-211, GraphRep.hpp:9-73).
 * All arrays are uint32, in device memory, and any pointer may be NULL when
 * no selected variant needs it.
 *
 *   CSR forward   : fwd_vertices[N+1], fwd_edges[M]   (rows = sources)
 *   CSR reverse   : rev_vertices[N+1], rev_edges[M]   (rows = destinations,
 *                   each row sorted by source id)
 *   EdgeList fwd  : inEdges = fwd_in_edges[M] (source), outEdges = fwd_edges
 *   EdgeList rev  : inEdges = rev_in_edges[M] (destination),
 *                   outEdges = rev_edges (source)
 *   StructEdgeList: {in,out} pairs, fwd_struct_edges[2M] / rev_struct_edges[2M]
 *
 * For a symmetric graph the forward and reverse arrays may alias.
 *
 * A graph without edges (edge_count 0) needs only fwd_vertices or
 * rev_vertices; its edge arrays may be NULL.  Every BFS entry point then
 * gives the root depth 0 and every other vertex INT_MAX after one level,
 * and PageRank gives every vertex the constant rank of a zero in-sum, with
 * no level or iteration kernel run.
 */
typedef struct bw_graph_view {
    uint64_t vertex_count;
    uint64_t edge_count;
    const uint32_t *fwd_vertices;
    const uint32_t *fwd_edges;
    const uint32_t *rev_vertices;
    const uint32_t *rev_edges;
    const uint32_t *fwd_in_edges;
    const uint32_t *rev_in_edges;
    const uint32_t *fwd_struct_edges;
    const uint32_t *rev_struct_edges;
} bw_graph_view;

/*
 * Host graph in CSR form (forward + reverse), allocated by the library with
 * malloc and released by bw_host_graph_free().  Replaces the mmapped
 * Graph<V,E> of utils/Graph.hpp:977-1063 as the in-memory form.
 */
typedef struct bw_host_graph {
    uint64_t vertex_count;
    uint64_t edge_count;
    int32_t undirected;        /* 1: reverse arrays alias the forward ones */
    int32_t reserved;
    uint32_t *fwd_vertices;
    uint32_t *fwd_edges;
    uint32_t *rev_vertices;
    uint32_t *rev_edges;
} bw_host_graph;

void bw_host_graph_free(bw_host_graph *g);

/*
 * Build a graph from a directed edge list (host arrays).  Self-loops are
 * dropped when BW_BUILD_DROP_SELF_LOOPS is set, duplicate edges are removed
 * when BW_BUILD_DEDUPE is set, and every edge (u,v) gains (v,u) when
 * BW_BUILD_SYMMETRISE is set.  Rows come out sorted by neighbour id, which
 * is the order utils/Graph.hpp:1146-1151 (output -> sort -> writeEdges)
 * produces.
 */
enum bw_build_flags {
    BW_BUILD_DROP_SELF_LOOPS = 1,
    BW_BUILD_DEDUPE = 2,
    BW_BUILD_SYMMETRISE = 4
};
int bw_graph_from_edges(uint64_t vertex_count, uint64_t count,
                        const uint32_t *src, const uint32_t *dst, int flags,
                        bw_host_graph *out);

/*
 * Seeded synthetic generators (counter-based hashing, so the same seed gives
 * the same graph on every machine and thread count).  All drop self-loops and
 * duplicate edges.
 *   R-MAT(a,b,c,d=1-a-b-c), 2^scale vertices, edge_factor*2^scale samples.
 *   R-MAT over n vertices (any n >= 2): edge_factor*n samples of the R-MAT
 *     of scale ceil(log2 n), both endpoints scaled by n / 2^scale.
 *   Erdos-Renyi G(n,m): m uniform (u,v) samples.
 *   2-D 4-neighbour grid h x w, both directions (evolve/gen-graph.cpp:96-123).
 *   Barabasi-Albert: n vertices, m attachments each, both directions.
 */
int bw_generate_rmat(uint32_t scale, uint32_t edge_factor, double a, double b,
                     double c, uint64_t seed, int symmetrise,
                     bw_host_graph *out);
int bw_generate_rmat_n(uint64_t n, uint32_t edge_factor, double a, double b,
                       double c, uint64_t seed, int symmetrise,
                       bw_host_graph *out);
int bw_generate_er(uint64_t n, uint64_t m, uint64_t seed, int symmetrise,
                   bw_host_graph *out);
int bw_generate_grid(uint32_t h, uint32_t w, bw_host_graph *out);
int bw_generate_ba(uint64_t n, uint32_t m, uint64_t seed, bw_host_graph *out);

/*
 * Device-resident graph in forward + reverse CSR, produced by the device
 * generators below and released with bw_device_graph_free().  The arrays
 * are device pointers; for an undirected graph the reverse arrays alias
 * the forward ones.
 */
typedef struct bw_device_graph {
    uint64_t vertex_count;
    uint64_t edge_count;
    int32_t undirected;
    int32_t reserved;
    uint32_t *fwd_vertices;
    uint32_t *fwd_edges;
    uint32_t *rev_vertices;
    uint32_t *rev_edges;
} bw_device_graph;

/*
 * The same seeded generators evaluated on the GPU (identical counter-based
 * hash, so they return exactly the graph the host generators return).
 * kind: 0 R-MAT(p0 = scale, p1 = edge factor, a, b, c),
 *       1 Erdos-Renyi(p0 = n, p1 = m),
 *       2 grid(p0 = h, p1 = w),
 *       3 Barabasi-Albert(p0 = n, p1 = m),
 *       4 R-MAT over any vertex count (p0 = n, p1 = edge factor, a, b, c;
 *         as bw_generate_rmat_n).
 * Sorting uses CUB radix sort (input preparation, not a hot path).
 */
int bw_generate_device(int kind, uint64_t p0, uint64_t p1, double a, double b,
                       double c, uint64_t seed, int symmetrise,
                       bw_device_graph *out, void *stream);
void bw_device_graph_free(bw_device_graph *g);

/*
 * The reference's .graph file format, versions 0 and 1
 * (utils/Graph.hpp:784-807 header/size rules, 977-1063 reader,
 * 1112-1120 writer).  Only 4-byte vertex/edge fields are supported (the
 * 8-byte form exists only for graphs beyond uint32 counts).
 */
int bw_graph_file_read(const char *path, bw_host_graph *out);
int bw_graph_file_write(const char *path, const bw_host_graph *g);

/*
 * Degree statistics of graph-details / SwitchImplementation::loadGraph
 * (graph-details.cpp:36-61, ImplementationTemplate.hpp:622-649,
 * utils/StatisticalSummary.hpp:8-80).  kind: 0 = abs, 1 = in, 2 = out.
 * out[7] = {min, lower quantile, mean, median, upper quantile, max, stddev}.
 */
int bw_degree_statistics(const bw_host_graph *g, int kind, double out[7]);


/* ------------------------------------------------------------------------ */
/* Context                                                                   */
/* ------------------------------------------------------------------------ */
typedef struct bw_context bw_context;

/* Select `device` and create a context.  Replaces CUDABackend::setDevice
 * (CUDA.cpp:158-193) plus the per-algorithm device globals. */
int bw_context_create(int device, bw_context **out);
int bw_context_destroy(bw_context *ctx);
/* Device properties the launch geometry uses. */
int bw_context_sm_count(const bw_context *ctx);

/*
 * Launch geometry.  Zero fields take defaults.  block/grid = 0 selects the
 * reference's Backend::computeDivision (Backend.cpp:52-70) for the reference
 * variants and an SM-multiple persistent grid for the others.  warp_size /
 * chunk_size are the -w / -c options of the warp variants
 * (ImplementationTemplate.hpp:431-436, defaults 32/32).
 */
typedef struct bw_launch_config {
    uint32_t block_size;
    uint32_t grid_size;
    uint32_t warp_size;
    uint32_t chunk_size;
    uint32_t flags;               /* BW_LAUNCH_* (no reference counterpart) */
} bw_launch_config;

/*
 * The forward edge-list PageRank variants (edge-list, struct-edge-list) run
 * with one geometry, two 1024-thread blocks per SM: each block keeps the
 * hottest destinations' accumulators in shared memory (block_size and
 * grid_size do not apply to them).
 *
 * Work-list PageRank variants (vertex-pull, vertex-pull-nodiv,
 * pull-segmented): block_size 1024 (default) or 256 picks the block shape,
 * chunk_size the number of gathered-array entries each block caches in
 * shared memory (0 = default: 24,288 for block_size 1024, none for 256;
 * a multiple of 4), warp_size the long-row
 * threshold (0 = 256, at most 512): rows with more in-edges are cut into
 * pieces whose sequential sums a second kernel evaluates, shorter ones are
 * summed where they are gathered.  Relabelling stores the
 * gathered array in decreasing out-degree order so that the cached entries
 * are the hubs; it costs one gather per edge per run (for the div variants
 * inside their first iteration) and leaves every result unchanged.  By default it runs when the cached entries would cover
 * at least 5% more of the edges than in vertex order (and the run has at
 * least 4 iterations); BW_LAUNCH_RELABEL forces it, BW_LAUNCH_NO_RELABEL
 * turns it off.
 */
#define BW_LAUNCH_RELABEL 1u
#define BW_LAUNCH_NO_RELABEL 2u
/*
 * BW_LAUNCH_L2_WINDOW (no reference counterpart): for the run's kernels, an
 * L2 access-policy window marks the randomly gathered vector persisting --
 * PageRank's contribution buffers, BFS's depth array -- with a persisting
 * carve-out of L2 of that size (at most the device's maximum); both are
 * removed when the run ends.  Results are unchanged.  The window is a stream
 * attribute, so the run's stream must be a created one (the legacy default
 * stream returns BW_ERR_INVALID_ARGUMENT).
 */
#define BW_LAUNCH_L2_WINDOW 4u

/* Reference Backend::computeDivision for `count` items. */
void bw_compute_division(uint64_t count, uint32_t sm_count,
                         uint32_t max_threads_per_block,
                         uint32_t *block_out, uint32_t *grid_out);

/* Expand a CSR (device) into the EdgeList inEdges array (row id per edge)
 * and build the StructEdgeList {in,out} array; GraphLoader.hpp:134-143. */
int bw_expand_edge_list(const uint32_t *vertices, uint64_t vertex_count,
                        uint64_t edge_count, uint32_t *in_edges, void *stream);
int bw_build_struct_edges(const uint32_t *in_edges, const uint32_t *out_edges,
                          uint64_t edge_count, uint32_t *struct_edges,
                          void *stream);


/*
 * The same statistics of a device-resident graph, computed on the device
 * (graph-details.cpp:36-61 over a graph already loaded for the kernels):
 * degrees from the view's offsets (fwd_vertices for out, rev_vertices for
 * in; abs adds both, or takes out only when `undirected`), sorted on the
 * device for the order statistics; mean and standard deviation from exact
 * integer sums of d and d^2 (the host's Welford loop agrees to ~1e-12).
 * Synchronises `stream` to return the figures.
 */
int bw_degree_statistics_device(bw_context *ctx, const bw_graph_view *g, int undirected, int kind,
                                double out[7], void *stream);

/* ------------------------------------------------------------------------ */
/* BFS                                                                       */
/* ------------------------------------------------------------------------ */
/*
 * Variants.  Ids 0..31 are the reference's 32 names
 * (bfs/bfs.cpp:121-207): family * 4 + reduction with
 *   family    0 edge-list, 1 rev-edge-list, 2 struct-edge-list,
 *             3 rev-struct-edge-list, 4 vertex-push, 5 vertex-pull,
 *             6 vertex-push-warp, 7 vertex-pull-warp
 *   reduction 0 "" (per-visit atomic), 1 -bulk, 2 -warpreduce,
 *             3 -blockreduce                       (bfs/bfs.hpp:32-116)
 * Ids >= 32 are GB300 variants with no reference counterpart:
 *   32 frontier-push   (queue-driven top-down, warp/grid cooperative hubs)
 *   33 frontier-pull   (bottom-up over unvisited vertices, early exit)
 */
enum { BW_BFS_REFERENCE_VARIANTS = 32 };
int bw_bfs_variant_count(void);
const char *bw_bfs_variant_name(int variant);
int bw_bfs_variant_lookup(const char *name);     /* -1 when unknown */
/* Which representation a variant reads: bit0 fwd CSR, bit1 rev CSR,
 * bit2 fwd EdgeList, bit3 rev EdgeList, bit4 fwd Struct, bit5 rev Struct. */
int bw_bfs_variant_reps(int variant);

/*
 * Initialise depths: every vertex INT32_MAX, root 0; resets the frontier
 * queue to {root}.  Reference: bfs/bfs.cpp:69-76 (host fill + H2D).
 */
int bw_bfs_init(bw_context *ctx, uint64_t vertex_count, uint32_t root,
                int32_t *levels, void *stream);

/*
 * Run one BFS level at `depth` with `variant`, then read back the number of
 * vertices it newly visited into *frontier (host).  Replaces
 * resetFrontier(); kernel(loader, results, curr); getFrontier()
 * (bfs/bfs.cpp:95-98, bfs/bfs.cu:7-18).
 */
int bw_bfs_level(bw_context *ctx, const bw_graph_view *g, int variant,
                 int32_t *levels, int32_t depth, const bw_launch_config *cfg,
                 uint32_t *frontier, void *stream);

/* Per-level side statistics the level kernels accumulate (features). */
typedef struct bw_bfs_level_stats {
    uint32_t frontier_vertices;   /* newly visited at this level */
    uint32_t variant;             /* variant that ran the level */
    uint64_t frontier_edges;      /* sum of out-degrees of those vertices */
    float log_degree_sum;         /* sum of log2(1+deg) */
    float log_degree_sq_sum;      /* sum of log2(1+deg)^2 */
    float log_degree_max;
    float device_ms;              /* level time, when timing was requested */
} bw_bfs_level_stats;

/*
 * The statistics of a frontier, for a host-side switch that picks the
 * variant of each level (SwitchImplementation::predict,
 * ImplementationTemplate.hpp:768-827, fed by setProps, bfs/bfs.cpp:43-49).
 * depth < 0: the frontier {root} that level 0 expands (root's out-degree).
 * depth >= 0: the vertices the bw_bfs_level call at `depth` newly visited,
 * i.e. the frontier of level depth + 1; valid until three more levels run.
 * Needs the forward CSR (the level kernels then accumulate the statistics).
 * out->variant is 0xffffffff (not recorded) and out->device_ms 0.
 */
int bw_bfs_frontier_stats(bw_context *ctx, const bw_graph_view *g,
                          uint32_t root, int32_t depth,
                          bw_bfs_level_stats *out, void *stream);

typedef struct bw_bfs_result {
    uint32_t level_count;         /* levels run (last one found nothing) */
    uint32_t reserved;
    uint64_t visited;             /* vertices with a finite depth */
    uint64_t traversed_edges;     /* sum of out-degrees of visited vertices */
    double device_ms;             /* traversal time on the device */
} bw_bfs_result;

enum bw_loop_mode {
    BW_LOOP_HOST = 0,    /* host loop, one frontier read-back per level */
    BW_LOOP_GRAPH = 1    /* CUDA graph with a device-side conditional loop */
};

/*
 * Full traversal from `root` with a fixed variant.  `stats` (optional) gets
 * one entry per level, up to stats_capacity.  max_levels = 0 means
 * vertex_count + 1.  Reference: BFS::runImplementation (bfs/bfs.cpp:51-118).
 */
int bw_bfs_run(bw_context *ctx, const bw_graph_view *g, int variant,
               uint32_t root, int32_t *levels, const bw_launch_config *cfg,
               int loop_mode, uint32_t max_levels, bw_bfs_result *result,
               bw_bfs_level_stats *stats, uint32_t stats_capacity,
               void *stream);

/*
 * Traversal where `schedule[level]` names the variant of each level
 * (the last entry repeats).  Used to replay predictor choices and the
 * per-level oracle-best sequence.  Reference analogue: the kernels tuple
 * swap of SwitchImplementation::predict (ImplementationTemplate.hpp:675-689).
 */
int bw_bfs_run_schedule(bw_context *ctx, const bw_graph_view *g,
                        const int32_t *schedule, uint32_t schedule_len,
                        uint32_t root, int32_t *levels,
                        const bw_launch_config *cfg, uint32_t max_levels,
                        int time_levels, bw_bfs_result *result,
                        bw_bfs_level_stats *stats, uint32_t stats_capacity,
                        void *stream);

/* ------------------------------------------------------------------------ */
/* PageRank                                                                  */
/* ------------------------------------------------------------------------ */
/*
 * Variants 0..9 are the reference's names (pagerank/pagerank.cpp:205-351):
 *   0 edge-list, 1 rev-edge-list, 2 struct-edge-list, 3 rev-struct-edge-list,
 *   4 vertex-push, 5 vertex-pull, 6 vertex-push-warp, 7 vertex-pull-warp,
 *   8 vertex-pull-nodiv, 9 vertex-pull-warp-nodiv
 * Ids >= 10 are GB300 variants with no reference counterpart:
 *  10 pull-segmented  (edge-balanced tiles, CTA segmented reduction,
 *                      consolidation fused; div semantics)
 */
enum { BW_PAGERANK_REFERENCE_VARIANTS = 10 };
int bw_pagerank_variant_count(void);
const char *bw_pagerank_variant_name(int variant);
int bw_pagerank_variant_lookup(const char *name);
int bw_pagerank_variant_reps(int variant);

typedef struct bw_pagerank_result {
    uint32_t iterations;
    uint32_t kernel_launches; /* this library's kernels launched by the run */
    float last_diff;        /* sum |pr_new - pr_old| of the last iteration */
    float reserved_f;
    double device_ms;       /* the whole run on the device: degrees, set-up, iterations */
} bw_pagerank_result;

/*
 * PageRank with damping 0.85 and 1/N initial ranks for exactly `iterations`
 * iterations (the reference hard-codes 100, pagerank/pagerank.cpp:55).
 * `ranks` (device, N floats) receives the result.  Degrees are computed
 * inside the call, as the reference does inside its timed region
 * (pagerank/pagerank.cpp:102-112).  `diffs` (optional, host) receives the
 * per-iteration diff the reference reads back (pagerank.cpp:124).
 * loop_mode 0 launches the iterations from the host; 1 captures them into
 * one CUDA graph and launches it once (the same kernels in the same order;
 * the call must not itself be made inside a stream capture).
 */
int bw_pagerank_run(bw_context *ctx, const bw_graph_view *g, int variant,
                    uint32_t iterations, float *ranks,
                    const bw_launch_config *cfg, int loop_mode,
                    bw_pagerank_result *result, float *diffs, void *stream);

/*
 * Same, with a per-iteration variant schedule (last entry repeats).  All
 * scheduled variants must share one semantics class (div or nodiv).
 */
int bw_pagerank_run_schedule(bw_context *ctx, const bw_graph_view *g,
                             const int32_t *schedule, uint32_t schedule_len,
                             uint32_t iterations, float *ranks,
                             const bw_launch_config *cfg, int time_iterations,
                             float *iteration_ms, bw_pagerank_result *result,
                             void *stream);

/* ------------------------------------------------------------------------ */
/* Learned variant switching                                                 */
/* ------------------------------------------------------------------------ */
/*
 * A small MLP (12 -> 64 -> 64 -> K, ReLU, softmax, FP32) picks the variant
 * of each BFS level from 12 per-level features.  It has no counterpart in
 * the reference's kernels; it plays the role of the reference's predictor
 * .so (ImplementationTemplate.hpp:768-827, lookup()), evaluated on the
 * device.  Parameters live in one device float array:
 *   mu[12], sd[12] (feature normalisation), W1[64][12], b1[64],
 *   W2[64][64], b2[64], W3[K][64], b3[K].
 */
enum { BW_FEATURE_COUNT = 12, BW_MLP_HIDDEN = 64, BW_MLP_MAX_CLASSES = 16 };

uint32_t bw_mlp_param_count(uint32_t classes);

/* Features of the level about to run (identical to the device formula):
 * frontier = vertices at the current depth, visited/edges_visited include
 * the frontier. */
void bw_bfs_features(uint64_t frontier_vertices, uint64_t frontier_edges,
                     float log_degree_sum, float log_degree_sq_sum,
                     float log_degree_max, uint64_t vertex_count,
                     uint64_t edge_count, uint64_t visited,
                     uint64_t edges_visited, uint32_t level, float out[12]);

/*
 * Per-level profile: at a sampled level each candidate variant runs from the
 * same state (a candidate is undone by resetting the vertices it visited,
 * which its emitted frontier queue lists) and is timed on the device; the
 * traversal then continues.  Levels < 32 and every `sample_every`-th level
 * (0 or 1 = all) are sampled; other levels run candidates[default_index]
 * once and get level_ms = -1.  level_ms[level * K + k] and
 * features[level * 12 + i] are filled for each level run (level_count).
 */
int bw_bfs_profile(bw_context *ctx, const bw_graph_view *g, uint32_t root,
                   int32_t *levels, const int32_t *candidates, uint32_t K,
                   uint32_t max_levels, uint32_t repeats,
                   uint32_t sample_every, uint32_t default_index,
                   float *level_ms, float *features, uint32_t *level_count,
                   void *stream);

typedef struct bw_mlp_train_config {
    uint32_t steps;          /* optimiser steps */
    uint32_t batch;          /* minibatch size (<= 64) */
    float lr;                /* Adam step size */
    float beta1, beta2, eps; /* Adam moments */
    float weight_decay;
    uint32_t reserved;
    uint64_t seed;           /* minibatch sampling / initialisation */
} bw_mlp_train_config;

/* Initialise weights (seeded) and store the feature normalisation. */
int bw_mlp_init(float *params, uint32_t classes, const float *mu,
                const float *sd, uint64_t seed, void *stream);

/*
 * Train on n samples (device arrays): X[n][12] raw features, T[n][K] target
 * distribution, W[n] sample weights (NULL = 1).  Loss: weighted soft-target
 * cross-entropy.  One CTA runs every Adam step on the device.  loss_curve
 * (host, optional) receives the mean minibatch loss of each block of
 * steps/loss_points steps.
 */
int bw_mlp_train(bw_context *ctx, float *params, uint32_t classes,
                 const float *X, const float *T, const float *W, uint32_t n,
                 const bw_mlp_train_config *cfg, float *loss_curve,
                 uint32_t loss_points, void *stream);

/* Full-batch gradient of the mean loss (device grad[param_count]) and the
 * loss value (host); used to check the backward pass. */
int bw_mlp_gradient(bw_context *ctx, const float *params, uint32_t classes,
                    const float *X, const float *T, const float *W,
                    uint32_t n, float *grad, float *loss, void *stream);

/* Softmax probabilities probs[n][K] (device). */
int bw_mlp_predict(bw_context *ctx, const float *params, uint32_t classes,
                   const float *X, uint32_t n, float *probs, void *stream);

/* The same forward pass on the host, with host params, X and probs, and the
 * host loop's operation order (BW_LOOP_HOST below picks from it); a
 * predictor library built from a trained model calls it. */
int bw_mlp_predict_host(const float *params, uint32_t classes,
                        const float *X, uint32_t n, float *probs);

typedef struct bw_switch_config {
    const float *params;        /* device MLP parameters */
    uint32_t classes;           /* K */
    int32_t fallback;           /* index into candidates */
    const int32_t *candidates;  /* host array of K BFS variant ids */
    float threshold;            /* below this top probability use fallback */
    uint32_t flags;             /* BW_SWITCH_* */
} bw_switch_config;

/* BW_LOOP_GRAPH normally runs a level whose frontier frontier-push's
 * cluster kernel can take (at most 32,768 vertices and 65,536 out-edges)
 * with frontier-push when it is a candidate: that kernel then carries on
 * through the following small levels on chip, one cluster barrier per
 * level, which no per-level choice can match on high-diameter graphs.
 * BW_SWITCH_MLP_ONLY leaves every level to the MLP, as BW_LOOP_HOST does. */
enum { BW_SWITCH_MLP_ONLY = 1 };

/*
 * BFS whose every level runs the variant the MLP picks from that level's
 * features (fallback below the confidence threshold).  BW_LOOP_GRAPH runs
 * the prediction on the device inside the CUDA graph (a SWITCH conditional
 * node selects the level kernel); BW_LOOP_HOST predicts on the host.  The
 * depths are bit-identical to every fixed variant's; stats[level].variant
 * records the choices.
 */
int bw_bfs_run_learned(bw_context *ctx, const bw_graph_view *g,
                       const bw_switch_config *sw, uint32_t root,
                       int32_t *levels, int loop_mode, uint32_t max_levels,
                       bw_bfs_result *result, bw_bfs_level_stats *stats,
                       uint32_t stats_capacity, void *stream);

/*
 * The 12 features of PageRank iteration `iteration` (bw_bfs_features with
 * every vertex active: the frontier is the whole vertex set, N vertices and
 * M edges, with the log-degree moments of the in-degrees -- the
 * out-degrees when the view has no reverse CSR -- nothing unvisited, and
 * level 0 for the first iteration, 1 for every later one, which all do the
 * same work).  out: host, 12 floats.
 */
int bw_pagerank_features(bw_context *ctx, const bw_graph_view *g,
                         uint32_t iteration, float out[12], void *stream);

/*
 * PageRank whose every iteration runs the variant the MLP picks from that
 * iteration's features (above), the fallback below the confidence
 * threshold.  The features separate only the first iteration from the
 * rest, so the whole schedule is chosen before the run, which then runs as
 * bw_pagerank_run_schedule does (loop_mode as in bw_pagerank_run).  The
 * candidates must share one semantics class (all div or all nodiv
 * variants).  diffs (optional, host, `iterations` floats) as in
 * bw_pagerank_run; schedule_out (optional, host, `iterations` entries)
 * receives the variant chosen for each iteration.  It plays the part of
 * the reference's PageRank `switch` implementation
 * (pagerank/pagerank.cpp:174-358), which picks its kernel through a
 * predictor library.
 */
int bw_pagerank_run_learned(bw_context *ctx, const bw_graph_view *g,
                            const bw_switch_config *sw, uint32_t iterations,
                            float *ranks, int loop_mode,
                            bw_pagerank_result *result, float *diffs,
                            int32_t *schedule_out, void *stream);


/* ------------------------------------------------------------------------ */
/* Batched persistent traversal                                              */
/* ------------------------------------------------------------------------ */
/*
 * Many independent units in one persistent launch fed by a device work
 * queue (an atomic cursor over a list ordered largest first); each CTA takes
 * a unit and runs it to completion with CTA-level barriers between levels
 * and iterations.  No counterpart in the reference, which runs one
 * traversal per process (kernel-runner.cpp:222-256).
 *
 * BW_BATCH_GRAPHS: `g` is one concatenated CSR (forward + reverse, global
 *   vertex ids) of graph_count graphs; graph i owns vertices
 *   [graph_offsets[i], graph_offsets[i+1]).  Unit i = graph i: BFS from
 *   roots[i] (a global id), depths into levels[global id], then
 *   pr_iterations PageRank iterations of graph i alone (its own N in the
 *   base term, vertex-pull order: bit-identical to bw_pagerank_run on that
 *   graph) into ranks[global id].
 * BW_BATCH_SOURCES: graph_count = 1; unit i = BFS from roots[i];
 *   depths into levels[i * vertex_count + v].
 * graph_offsets, roots and `order` (unit ids, largest first; NULL = 0..n-1)
 * are device arrays.
 * cfg (optional): grid_size (0: two CTAs per SM where they fit), block_size
 * (0 or 512), and chunk_size as the push/pull divisor -- a BFS level whose
 * frontier holds more than 1/chunk_size of the unit's vertices runs
 * bottom-up (0: 24; the autotuner's tune_batch picks it per graph class).
 */
enum bw_batch_mode { BW_BATCH_GRAPHS = 0, BW_BATCH_SOURCES = 1 };

typedef struct bw_batch_result {
    uint64_t units;             /* units run */
    uint64_t traversed_edges;   /* BFS: sum over units of out-edges of reached vertices */
    double device_ms;
} bw_batch_result;

int bw_batch_run(bw_context *ctx, const bw_graph_view *g, int mode,
                 const uint32_t *graph_offsets, uint32_t graph_count,
                 const uint32_t *roots, const uint32_t *order,
                 uint32_t unit_count, uint32_t max_unit_vertices,
                 uint32_t pr_iterations, int32_t *levels, float *ranks,
                 const bw_launch_config *cfg, bw_batch_result *result,
                 void *stream);

/* ------------------------------------------------------------------------ */
/* Allocation-free BFS                                                       */
/* ------------------------------------------------------------------------ */
/*
 * No counterpart in the reference.  BFS (frontier-push) that allocates no
 * memory: for callers that cannot allocate device memory while running,
 * such as a serving process that reserves its HBM budget at start-up and
 * forbids cudaMalloc on the request path (it can synchronise the device and
 * fail under fragmentation), or a host application that loads this library
 * under an allocator policy it does not own.  The caller passes the graph
 * (forward CSR), the depth array (N int32, device) and a stream; the BFS
 * scratch (frontier queues, hub-chunk queue, counters) is a fixed file-scope
 * device array of about 9.2 MB that every GPU loading the library holds
 * until exit.  Limits: at most 1,048,576 vertices and 16,777,216 edges;
 * larger graphs return BW_ERR_TOO_LARGE.  The first call on a device looks up
 * that array's device address (with the device current) and keeps it for
 * the life of the process.  With lazy module loading (the CUDA 13 default)
 * that first call is also when the array is reserved on the device, so make
 * one warm-up call per device at start-up (a one-vertex graph will do),
 * before reserving the rest of the HBM budget and before any stream capture.
 * Do not call it again on a device after cudaDeviceReset: the kept address
 * belongs to the old context.  Each call reads every level's frontier size
 * back to the host, synchronising `stream` once per level, so it returns with
 * the BFS complete.  Every call shares the one array and re-initialises it:
 * calls that overlap on the GPU (other streams, other threads) race and must
 * not be issued.  Depths are identical to
 * bw_bfs_run(..., "frontier-push", ...); *level_count gets the levels run.
 */
int bw_bfs_run_noalloc(const bw_graph_view *g, uint32_t root, int32_t *levels,
                       uint32_t max_levels, uint32_t *level_count,
                       void *stream);

/*
 * Random-gather ceiling (a measurement; no counterpart in the reference):
 * partial[b] = sum over the loads block b issued of src[idx[i]], i < m,
 * skipping idx[i] >= n.  One block per SM (partial holds
 * bw_context_sm_count(ctx) floats), 16 independent loads in flight per
 * thread, L2-only loads -- the gathers of the PageRank pull kernels with
 * nothing else to do.  Time it on `stream` to get the device's rate of
 * scattered 4-byte loads, the bound of those kernels when their gathered
 * vector fits in L2.
 */
int bw_gather_probe(bw_context *ctx, const float *src, uint64_t n,
                    const uint32_t *idx, uint64_t m, float *partial,
                    void *stream);

#ifdef __cplusplus
}
#endif
#endif /* BELEWITTE_GB300_H */
