// Instantiations of the edge-list BFS families (4 layouts x 4 reductions x
// side outputs on/off).
#include "bfs_kernels.cuh"

namespace bw {

template<int LAYOUT, int RED>
static BfsKernelFn pick(bool side)
{ return side ? k_bfs_edge<RED, true, LAYOUT> : k_bfs_edge<RED, false, LAYOUT>; }

template<int LAYOUT>
static BfsKernelFn pick_red(int red, bool side)
{
    switch (red) {
      case RED_NORMAL: return pick<LAYOUT, RED_NORMAL>(side);
      case RED_BULK: return pick<LAYOUT, RED_BULK>(side);
      case RED_WARP: return pick<LAYOUT, RED_WARP>(side);
      default: return pick<LAYOUT, RED_BLOCK>(side);
    }
}

BfsKernelFn bfs_edge_kernel(int layout, int reduction, bool side)
{
    switch (layout) {
      case FWD_SOA: return pick_red<FWD_SOA>(reduction, side);
      case REV_SOA: return pick_red<REV_SOA>(reduction, side);
      case FWD_AOS: return pick_red<FWD_AOS>(reduction, side);
      default: return pick_red<REV_AOS>(reduction, side);
    }
}

}  // namespace bw
