// i2_tiers.cuh -- tier 2b of the adjacent-pair potential, shared by the FP64 and mixed forms.
//
// The tiered rule (tier 1: graded Duffy 10 x 8 against 8 x 6; tier 2: 16 x 16 against the main
// rule; tier 2b: 24 x 24 against 16 x 16; then the adaptive rule) runs tier 2b as its own pass
// over the pairs tier 2 rejected, listed in ClassArgs::tier2b_list (count in cnt[kCntTier2b]).
// It is FP64 in both forms and costs 832 point evaluations per pair at the 1/64 FP64 rate; run
// inline in the tier-2 warps, a few warps that drew several such pairs set the kernel's length,
// whereas a pass over the compact list keeps every warp on one pair.
#pragma once

#include "i2_engine.h"

namespace i2 {

__device__ __forceinline__ double warp_sum(double x)
{
    for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
    return x;
}

// listed pair h, by one warp.  hi_known: padj[t] holds the pair's FP64 16 x 16 value, unscaled
// (the FP64 form's tier 2 computed it); otherwise it is computed here.
template <int CLS>
__device__ __forceinline__ void tier2b_item(const ClassArgs &A, const QuadTables &Q, bool hi_known, int h, int lane)
{
    const int t = A.tier2b_list[h];
    const int2 pr = A.pairs[t];
    const int3 ci = A.cells[pr.x], cj = A.cells[pr.y];
    const PanelJ K = load_panel(A.panels, pr.y);
    const double Si = A.panels[pr.x].v[0].w;
    int si, sj;
    if (CLS == kEdge) shifts_edge(ci, cj, si, sj);
    else shifts_vertex(ci, cj, si, sj);
    const Tri Ti = rotate(load_tri(A.panels, pr.x), si), Tj = rotate(Tri{K.A, K.B, K.C}, sj);
    const FarCtx F = make_far_ctx(K);
    PotEdge pe;
    const double sig = CLS == kEdge ? make_pot_edge(Ti, Tj, K, Si, pe) : 0.0;
    const double ph = hi_known ? A.padj[t]
                               : warp_sum(duffy_partial<CLS>(Ti, K, F, pe, Q.hi_u, Q.hi_uw, Q.hi_nu, Q.hi_v, Q.hi_vw, Q.hi_nv, lane, 32)) + sig;
    const double pt = warp_sum(duffy_partial<CLS>(Ti, K, F, pe, Q.top_u, Q.top_uw, Q.top_nu, Q.top_v, Q.top_vw, Q.top_nv, lane, 32)) + sig;
    if (lane != 0) return;
    if (fabs(pt - ph) <= A.top_tol * fabs(pt)) {
        A.padj[t] = kInv4Pi * pt;
    } else {
        A.padj[t] = kInv4Pi * ph;  // the adaptive rule's tolerance base
        A.hard_list[atomicAdd(A.hard_cnt, 1)] = t;
    }
}

// three 128-thread blocks per SM (at most 170 registers, a few spilled) rather than two at the
// unconstrained 178: the pass is latency-bound at the 1/64 FP64 rate
template <int CLS>
__global__ void __launch_bounds__(128, 3) k_pot_tier2b(ClassArgs A, QuadTables Q, int hi_known)
{
    const int count = A.cnt[kCntTier2b];
    const int lane = threadIdx.x & 31;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (long long h = warp_item_index(); h < count; h += nwarps) tier2b_item<CLS>(A, Q, hi_known != 0, (int)h, lane);
}

} // namespace i2
