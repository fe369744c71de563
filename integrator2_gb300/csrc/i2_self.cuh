// i2_self.cuh -- self pairs (K_i, K_i): the per-lane pieces of the potential rule and the
// outputs, shared by the per-class kernel (i2_kernels_fp64.cu) and the batched tier-1 / self
// launch (i2_kernels_mixed.cu).
#pragma once

#include "i2_engine.h"

namespace i2 {

// J(K_i, K_i) by the chosen convention, potential by self_potential (i2_rules.cuh)
// eight lanes per pair: lanes 0..5 take one (edge, piece) of the self-pair rule each, the group
// sums them (an edge's pieces are integrated independently, so the pair's 6 x nself point
// evaluations run in parallel)
// Self pairs, five to a warp: lanes 6k .. 6k+5 (k < 5) take the six (edge, piece) integrals of
// one pair, the first of the six writes the pair's outputs, lanes 30 and 31 idle (groups of eight
// lanes left two of every eight idle).
constexpr int kSelfPairsPerWarp = 5;

// lane g (0..5) of a pair's group: one (edge, piece) of the edge rule, or, for the closed form
// (Q.nself == 0), the whole value on lane 0
__device__ __forceinline__ double self_piece_of(const ClassArgs &A, const QuadTables &Q, long long t, int g)
{
    const PanelJ K = load_panel(A.panels, A.pairs[t].x);
    const d3 P[3] = {K.A, K.B, K.C};
    if (Q.nself == 0) return g == 0 ? self_potential_closed(P) : 0.0;
    return self_potential_piece(P, g >> 1, g & 1, Q);
}

// the parts of a lane's six-lane group, added in a fixed order (every lane of the warp calls it)
__device__ __forceinline__ double self_gather6(double part)
{
    const int lane = threadIdx.x & 31, base = lane - lane % 6;
    double sum = 0.0;
    for (int k = 0; k < 6; ++k) sum += __shfl_sync(0xffffffffu, part, (base + k) & 31);
    return sum;
}

__device__ __forceinline__ void self_store(const ClassArgs &A, int self_sign, long long t, double part)
{
    const PanelJ K = load_panel(A.panels, A.pairs[t].x);
    const double th = self_sign == 0 ? 0.0 : (self_sign > 0 ? kTwoPi : -kTwoPi) * K.S;
    const d3 J = kInv4Pi * (th * K.n);
    double *raw = A.raw4 + 4 * t;
    raw[0] = 0.0; raw[1] = 0.0; raw[2] = 0.0; raw[3] = th;
    double *Jo = A.J3 + 3 * t;
    Jo[0] = J.x; Jo[1] = J.y; Jo[2] = J.z;
    A.P[t] = kInv4Pi * part;
}

} // namespace i2
