// Unity translation unit that compiles the reference's PageRank kernels
// unmodified (pagerank/*.cu, included from the reference tree at build
// time) into one cubin for the GPU-side parity pin.  The two warp-pull
// kernels declare their dynamic shared array with another element type, so
// they live in ref_pagerank_pull_warp_unity.cu.  Test infrastructure only.
#include "pagerank/pagerank.cu"
#include "pagerank/edgelist.cu"
#include "pagerank/rev_edgelist.cu"
#include "pagerank/struct_edgelist.cu"
#include "pagerank/rev_struct_edgelist.cu"
#include "pagerank/vertex_push.cu"
#include "pagerank/vertex_pull.cu"
#include "pagerank/vertex_pull_nodiv.cu"
#include "pagerank/vertex_push_warp.cu"
