// The 12 per-level features of the variant predictor, computed identically
// on the host and on the device from the level side-statistics
// (frontier size, frontier out-edges, log-degree moments) and the running
// totals.  The reference's switch reads `frontier abs/rel`, `visited
// abs/rel` and graph degree statistics (bfs/bfs.cpp:43-49,
// ImplementationTemplate.hpp:622-649); these features carry the same
// information plus the frontier's degree distribution.
#pragma once
#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define BWF_HD __host__ __device__ __forceinline__
#else
#define BWF_HD inline
#endif

namespace bwfeat {

constexpr int COUNT = 12;

// fv, fe: vertices / out-edges of the frontier about to be expanded;
// lsum, lsq, lmax: sum, sum of squares and max of log2(1 + out-degree) over
// the frontier; visited: vertices reached so far (frontier included);
// edges_visited: out-edges of those vertices; level: index of the level.
BWF_HD void compute(double fv, double fe, double lsum, double lsq, double lmax, double n, double m,
                    double visited, double edges_visited, double level, float *x)
{
    const double mean = fv > 0 ? lsum / fv : 0.0;
    const double var = fv > 0 ? lsq / fv - mean * mean : 0.0;
    const double unvisited = n - visited > 0 ? n - visited : 0.0;
    const double unvisited_edges = m - edges_visited > 0 ? m - edges_visited : 0.0;
    x[0] = static_cast<float>(log2(1.0 + fv));
    x[1] = static_cast<float>(log2(1.0 + fe));
    x[2] = static_cast<float>(log2(1.0 + unvisited));
    x[3] = static_cast<float>(mean);
    x[4] = static_cast<float>(var > 0 ? sqrt(var) : 0.0);
    x[5] = static_cast<float>(lmax);
    x[6] = static_cast<float>(log2(n > 1 ? n : 1.0));
    x[7] = static_cast<float>(log2(1.0 + m));
    x[8] = static_cast<float>(log2(1.0 + level));
    x[9] = static_cast<float>(n > 0 ? fv / n : 0.0);
    x[10] = static_cast<float>(m > 0 ? fe / m : 0.0);
    x[11] = static_cast<float>(m > 0 ? unvisited_edges / m : 0.0);
}

}  // namespace bwfeat
