// Instantiations of the vertex BFS families (vertex-push, vertex-pull,
// vertex-push-warp, vertex-pull-warp x 4 reductions x side outputs) and of
// the GB300 frontier variants.
#include "bfs_kernels.cuh"

namespace bw {

template<int RED>
static BfsKernelFn pick(int family, bool side)
{
    switch (family) {
      case 4: return side ? k_bfs_vertex_push<RED, true> : k_bfs_vertex_push<RED, false>;
      case 5: return side ? k_bfs_vertex_pull<RED, true> : k_bfs_vertex_pull<RED, false>;
      case 6: return side ? k_bfs_vwarp<RED, true, false> : k_bfs_vwarp<RED, false, false>;
      default: return side ? k_bfs_vwarp<RED, true, true> : k_bfs_vwarp<RED, false, true>;
    }
}

BfsKernelFn bfs_vertex_kernel(int family, int reduction, bool side)
{
    switch (reduction) {
      case RED_NORMAL: return pick<RED_NORMAL>(family, side);
      case RED_BULK: return pick<RED_BULK>(family, side);
      case RED_WARP: return pick<RED_WARP>(family, side);
      default: return pick<RED_BLOCK>(family, side);
    }
}

BfsKernelFn bfs_frontier_push_kernel(bool side)
{ return side ? k_bfs_frontier_push<true> : k_bfs_frontier_push<false>; }

BfsKernelFn bfs_hub_kernel(bool side)
{ return side ? k_bfs_hub_chunks<true> : k_bfs_hub_chunks<false>; }

BfsKernelFn bfs_cluster_kernel(int stats)
{ return stats == 1 ? k_bfs_cluster<1> : stats == 2 ? k_bfs_cluster<2> : k_bfs_cluster<0>; }

size_t bfs_cluster_smem() { return CLUSTER_SMEM; }

int bfs_cluster_prepare()
{
    for (BfsKernelFn k : {k_bfs_cluster<0>, k_bfs_cluster<1>, k_bfs_cluster<2>})
        BW_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(CLUSTER_SMEM)));
    return BW_OK;
}

BfsKernelFn bfs_frontier_pull_kernel(bool side)
{ return side ? k_bfs_frontier_pull<true> : k_bfs_frontier_pull<false>; }

}  // namespace bw
