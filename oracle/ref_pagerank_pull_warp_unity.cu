// Second PageRank unity unit (see ref_pagerank_unity.cu): the reference's
// vertex-pull-warp kernels, compiled unmodified.  Test infrastructure only.
#include "pagerank/vertex_pull_warp.cu"
#include "pagerank/vertex_pull_warp_nodiv.cu"
