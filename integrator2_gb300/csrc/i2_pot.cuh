// i2_pot.cuh -- bookkeeping of the breadth-first adaptive potential of hard adjacent pairs,
// shared by its FP64 kernels (plain form) and its double-float kernels (mixed and batched forms).
#pragma once

#include "i2_engine.h"

namespace i2 {

// seed: the root of every hard pair is split once (one warp per pair); its four children form
// depth 1.  Pairs beyond a quarter of the list capacity keep their tier value and are counted
// as overflows.
__device__ __forceinline__ int pot_seeded(const ClassArgs &A) { return min(*A.hard_cnt, A.pot_qcap / 4); }

// the seed's bookkeeping, once per segment before any depth kernel runs: depth 1 holds the
// roots' children, the deeper lists start empty
__device__ __forceinline__ void pot_seed_init(const ClassArgs &A)
{
    const int count = pot_seeded(A);
    A.pot_qcnt[1] = 4 * count;
    for (int d = 2; d <= kHardMaxDepth + 1; ++d) A.pot_qcnt[d] = 0;
    if (*A.hard_cnt > count) atomicAdd(A.hard_overflow, *A.hard_cnt - count);
}

__device__ __forceinline__ int pot_depth_count(const ClassArgs &A, int depth) { return min(A.pot_qcnt[depth], A.pot_qcap); }

// cell triangles of the parents of depth d's cells (written while depth d - 1 split them)
__device__ __forceinline__ double *pot_tri_list(const ClassArgs &A, int depth) { return depth % 2 ? A.pot_tri_a : A.pot_tri_b; }

} // namespace i2
