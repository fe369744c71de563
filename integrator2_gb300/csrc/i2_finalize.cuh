// i2_finalize.cuh -- finalisation shared by the FP64, mixed and batched kernel chains.
#pragma once

#include "i2_engine.h"

namespace i2 {

__device__ __forceinline__ void store5(double *p, const acc5 &a)
{
    p[0] = a.px; p[1] = a.py; p[2] = a.pz; p[3] = a.th; p[4] = a.pot;
}
__device__ __forceinline__ acc5 load5(const double *p) { return acc5{p[0], p[1], p[2], p[3], p[4]}; }

// the reference's Runge criterion (evaluator3d.cu:76-99, cuda_math.cuh:270-300): the 1-norm of
// divide(I_L - I_{L-1}, 2^p I_{L-1} - I_L) with its small-value guards against EPS_INTEGRATION
__device__ __forceinline__ bool runge_unconverged(const acc5 &cur, const acc5 &prev, double pow2p)
{
    const double c[4] = {cur.px, cur.py, cur.pz, cur.th}, p[4] = {prev.px, prev.py, prev.pz, prev.th};
    double crit = 0.0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const double num = c[k] - p[k], den = pow2p * p[k] - c[k];
        const double lim = k < 3 ? kDoubleMin : kEps2;
        crit += fabs((fabs(num) < lim && fabs(den) < lim) ? 0.0 : num / den);
    }
    return crit > kEpsRunge;
}

template <int CLS>
__device__ inline void finalize_item(const ClassArgs &A, int mode, int t)
{
    const int2 pr = A.pairs[t];
    acc5 v;
    if (mode == kFixed) {
        v = load5(A.cur + 5 * (long long)t);
    } else {
        // compat: the reference swaps two buffers per iteration and rewrites only unconverged
        // entries (evaluatorJ3DK.cu:966-1011), so a pair that stopped at level L keeps I_L when
        // the class-wide loop ran an even number of further iterations, else I_{L-1}
        const int K = *A.maxlev, L = A.stop[t];
        const bool older = (mode == kAdaptiveCompat) && ((K - L) & 1);
        v = load5((older ? A.fin_b : A.fin_a) + 5 * (long long)t);
    }
    d3 psi = mk(v.px, v.py, v.pz);
    double th = v.th;
    if (CLS != kFar) {
        const double *sg = A.sing + 4 * (long long)t;
        psi = psi + mk(sg[0], sg[1], sg[2]);
        th += sg[3];
    }
    const double4_32a nj4 = A.panels[pr.y].v[3];
    const d3 J = finalize_j(CLS, psi, th, mk(nj4.x, nj4.y, nj4.z), A.panels[pr.x].v[0].w);
    double *raw = A.raw4 + 4 * (long long)t;
    raw[0] = psi.x; raw[1] = psi.y; raw[2] = psi.z; raw[3] = th;
    double *Jo = A.J3 + 3 * (long long)t;
    Jo[0] = J.x; Jo[1] = J.y; Jo[2] = J.z;
    A.P[t] = CLS == kFar ? kInv4Pi * v.pot : A.padj[t];
    if (A.level_out) A.level_out[t] = mode == kFixed ? -1 : A.stop[t];
}

// finalisation of every pair of one class from inside another kernel (grid-stride)
__device__ inline void finalize_all(int cls, const ClassArgs &A, int mode, long long first, long long stride)
{
    for (long long t = first; t < A.n; t += stride) {
        if (cls == kEdge) finalize_item<kEdge>(A, mode, (int)t);
        else if (cls == kVertex) finalize_item<kVertex>(A, mode, (int)t);
        else finalize_item<kFar>(A, mode, (int)t);
    }
}

} // namespace i2
