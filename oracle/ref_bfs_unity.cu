// Unity translation unit that compiles the reference's BFS kernels
// unmodified (bfs/*.cu, included from the reference tree at build time)
// into one cubin for the GPU-side parity pin.  Test infrastructure only.
#include "bfs/bfs.cu"
#include "bfs/edgelist.cu"
#include "bfs/rev_edgelist.cu"
#include "bfs/struct_edgelist.cu"
#include "bfs/rev_struct_edgelist.cu"
#include "bfs/vertex_push.cu"
#include "bfs/vertex_pull.cu"
#include "bfs/vertex_push_warp.cu"
#include "bfs/vertex_pull_warp.cu"
