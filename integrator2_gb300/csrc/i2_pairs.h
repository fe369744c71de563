// i2_pairs.h -- the pair lists of the four classes, built on the host or on the device with
// identical results.
//
// Lists are unordered pairs (i < j) sorted by (i, j); the self list holds (i, i).  A pair's class
// is the number of vertex indices its cells share (the reference counts them over all i < j
// pairs, src/Mesh3d.cu:93-142): one = common vertex, two = common edge, none = disjoint.  The
// disjoint list keeps the pairs whose centroid distance is below near_factor x the mean edge
// length, or every disjoint pair when near_factor <= 0 (the reference's runAllPairs lists).
//
// Both builders compute the near-field radius and the centroid grid with the same arithmetic:
// the mean edge length is summed in 64-bit fixed point (integer sums do not depend on the order
// of summation), and distances are formed without fused multiply-adds.
#pragma once

#include "i2_host.h"

#include <cstdint>
#include <vector>

namespace i2 {

// binary exponent applied to every edge length before it is rounded to an integer, so that the
// sum of at most `half_edges` lengths no larger than max_len stays below 2^62
int edge_sum_shift(double max_len, long long half_edges);

// mean length over the unique edges of the cells C (nc x 3 vertex indices into V)
double mean_edge_length(const double *V, const int *C, int nc);

// uniform grid over the cell centroids with cells of edge r (the near-field radius)
struct NearGrid {
    double lo[3] = {0, 0, 0};
    long long dims[3] = {1, 1, 1};
    double r = 0.0, r2 = 0.0;
};
NearGrid near_grid(const double *centres, int nc, double r);

// lists on the device: rows[cls] holds n[cls] int2 (i, j) rows
struct DevicePairLists {
    DevBuf<int2> rows[4];
    int64_t n[4] = {0, 0, 0, 0};
};

// the device builder: V, C, centres are the host copies (the radius and grid are set up from
// them), dV and dC the device copies of V and C.  All work is enqueued on s; the call returns
// after the lists are complete.
void build_pair_lists_device(const double *V, const int *C, const double *centres, int nv, int nc, const double *dV,
                             const int *dC, double near_factor, DevicePairLists &out, cudaStream_t s);

} // namespace i2
