// i2_kernels_mixed.cu -- mixed-precision form of the pair-integral path (sm_103a).
//
// FP32: the regular-part quadrature of every class (the bulk of the work), with per-pair
//       offsets formed from double-float vertices, cancellation-free edge logs and
//       Kahan-compensated accumulation; the graded-Duffy potential of adjacent pairs (tiers 1-2).
// FP64: the closed-form singular parts of common-edge / common-vertex pairs (once per pair),
//       the refinement error estimator (convergence test on the compensated sums), hard
//       (folded / sliver) adjacent pairs' adaptive potential, self pairs.
// The kernel chain per class mirrors the FP64 form (i2_kernels_fp64.cu) and shares its
// finalisation, self and adaptive-potential kernels.
#include "i2_device_f32.cuh"
#include "i2_dfvec.cuh"
#include "i2_batch.cuh"
#include "i2_engine.h"
#include "i2_finalize.cuh"
#include "i2_self.cuh"
#include "i2_tiers.cuh"

#include <cooperative_groups.h>

namespace i2 {

__global__ void k_prepare_panels_f32(int nc, const double *__restrict__ V, const int *__restrict__ C, PanelF *__restrict__ out)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    d3 P[3];
    for (int k = 0; k < 3; ++k) {
        const int v = C[3 * c + k];
        P[k] = mk(V[3 * v], V[3 * v + 1], V[3 * v + 2]);
    }
    const d3 cr = cross(P[1] - P[0], P[2] - P[0]);
    const d3 n = unit(cr);
    const double S = norm(cr) * 0.5;
    const d3 ea = P[2] - P[1], eb = P[0] - P[2], ec = P[1] - P[0];
    PanelF p;
    const double lens[3] = {norm(ea), norm(eb), norm(ec)};
    for (int k = 0; k < 3; ++k) {
        const float hx = (float)P[k].x, hy = (float)P[k].y, hz = (float)P[k].z;
        const float lx = (float)(P[k].x - hx), ly = (float)(P[k].y - hy), lz = (float)(P[k].z - hz);
        p.v[2 * k] = make_float4(hx, hy, hz, k == 0 ? (float)S : (float)lens[k - 1]);
        p.v[2 * k + 1] = make_float4(lx, ly, lz, k == 0 ? (float)(2.0 * S) : (k == 1 ? (float)lens[1] : 0.0f));
    }
    // [2].w = |C-B|, [3].w = |A-C|, [4].w = |B-A|
    p.v[2].w = (float)lens[0];
    p.v[3].w = (float)lens[1];
    p.v[4].w = (float)lens[2];
    // constants that scale logs against the FP64 closed forms, rounded once from FP64: [5].w =
    // 1/sqrt(S), [7..9].w = 1/|edge| (an FP32 rsqrtf or a quotient of FP32-rounded lengths would be
    // off by up to a few ulps, a bias the log terms carry into every point)
    p.v[5].w = (float)(1.0 / sqrt(S));
    p.v[6] = make_float4((float)n.x, (float)n.y, (float)n.z, 0.0f);
    const d3 ta = unit(ea), tb = unit(eb), tc = unit(ec);
    p.v[7] = make_float4((float)ta.x, (float)ta.y, (float)ta.z, (float)(1.0 / lens[0]));
    p.v[8] = make_float4((float)tb.x, (float)tb.y, (float)tb.z, (float)(1.0 / lens[1]));
    p.v[9] = make_float4((float)tc.x, (float)tc.y, (float)tc.z, (float)(1.0 / lens[2]));
    out[c] = p;
}

// ------------------------------------------------------------------ FP32 fused regular parts
// The plain logs of the adjacent classes' integrands, ln((l + o.tau) s), have arguments that
// vanish only on a ray from one of K_j's vertices along an edge line, which the cells of a valid
// mesh keep away from.  Folded or overlapping cells can reach it, and there FP32 cancellation can
// make the argument negative; the floor keeps the log finite (the FP64 form's argument stays a
// small positive number there, and gives a large finite log too).
constexpr float kLogArgFloor = 1.17549435e-38f;  // the smallest normal float

// A common-edge pair in the frame of its shared edge JB -> JC (K_j = (JA, JB, JC), D = K_i's vertex
// off the edge, tc = unit(JC - JB), L = |JC - JB|, D_p = the part of D - JB normal to tc, h = |D_p|).
// A point x of K_i with barycentric weights (l_B, l_C, l_D) lies at the distance a = l_C L + l_D dB
// along the edge from JB, a' = l_B L + l_D dC back from JC, and p = l_D D_p off the edge line.  The
// terms of theta that vanish on the shared edge are formed from a, a' and p: they are small
// differences of offsets of size l, and FP32 offsets rounded at ulp(l) would leave them errors of
// ulp(l) / |p| (4e-6 of J on a jittered 320-cell sphere).  The constants are rounded once from FP64
// (store_edge_frame).
struct EdgeCtxF {
    f3 ta, tb;          // unit(JA - JC), unit(JB - JA) (the two log terms of Psi, from o_A)
    float ilvc;         // 1 / L
    float L, h, dB, dC; // dB = (D - JB).tc, dC = (JC - D).tc
    float dn;           // n_j . D_p: the distance to K_j's plane is l_D dn
    float g1, g2;       // D_p . (tb x tc), D_p . (ta x tc)
    float h1, h2;       // (tb - tc) . D_p, (ta - tc) . D_p
    float cb, ca;       // 1 - tb.tc, 1 - ta.tc (= |tb - tc|^2 / 2, |ta - tc|^2 / 2)
    float BAtc, BAp;    // (JB - JA).tc, (JB - JA).D_p
};
struct VertexCtxF {
    f3 AB, AC;       // JB - JA, JC - JA (JA = shared vertex)
    f3 ta, tb, tbc;
    // the asymptote's direction e and, formed in FP64 once per pair, w = tau x e and p = e -+ tau
    // for its two angle terms, c = |p|^2 / 2 = 1 -+ e.tau (when e is nearly parallel to +-tau, w
    // and p are small vectors that FP32 arithmetic on e and tau would keep only a few digits of)
    f3 e, w1, w2, p1, p2;
    float c1, c2;
    float inv_sqrt_si, lenBC;
};

// The common-edge regular integrand (the FP64 form's edge_integrand) at the point with offset o_A
// from JA and barycentric weights wb = (l_B, l_C, l_D) in K_i.  With o_B = a tc + p, o_C = -a' tc + p
// and l_B = |o_B|, l_C = |o_C|, the solid angle's denominator
//   l_A l_B l_C + (o_A.o_B) l_C + (o_B.o_C) l_A + (o_C.o_A) l_B = l_A Q + o_A.(l_C o_B + l_B o_C),
//   Q = l_B l_C - a a' + p^2,   l_C o_B + l_B o_C = (l_C a - l_B a') tc + (l_B + l_C) p,
// its height n_j.o_A = n_j.p, and the two edge angles' arguments
//   (o_B x tb).tc = p.(tb x tc),  (tb - tc).(l_B tb + o_B) = (l_B - a)(1 - tb.tc) + (tb - tc).p
// (and the same with o_C, ta, a') are rebuilt without cancellation where the point projects onto
// the edge (a, a' > 0):
//   l_B l_C - a a' = p^2 (a^2 + a'^2 + p^2) / (l_B l_C + a a'),
//   l_C a - l_B a' = p^2 (a - a')(a + a') / (l_C a + l_B a'),   l_B - a = p^2 / (l_B + a);
// outside that span the direct forms add terms of one sign.  Psi's two logs are returned as
// scalars (lg): the lanes sum them, and psi_from_logs applies the FP64 unit edges once per pair.
__device__ __forceinline__ void edge_integrand_f(f3 oA, f3 wb, const PanelJf &K, const EdgeCtxF &E, f3 &lg, float &th)
{
    const float lA = normf(oA);
    const float l1 = logf(fmaxf((lA + dotf(oA, E.tb)) * E.ilvc, kLogArgFloor));
    const float l2 = logf(fmaxf((lA - dotf(oA, E.ta)) * E.ilvc, kLogArgFloor));
    lg = f3{l1, l2, 0.0f};  // Psi = l1 tb + l2 ta, formed once per pair (psi_from_logs)
    const float lD = wb.z;
    const float a = fmaf(wb.y, E.L, lD * E.dB), ap = fmaf(wb.x, E.L, lD * E.dC);
    const float ph = lD * E.h, p2 = ph * ph;
    const float lB = sqrtf(fmaf(a, a, p2)), lC = sqrtf(fmaf(ap, ap, p2));
    float Q, W;
    if (a > 0.0f && ap > 0.0f) {
        Q = fmaf(p2, div_q(fmaf(a, a, fmaf(ap, ap, p2)), fmaf(lB, lC, a * ap)), p2);
        W = div_q(p2 * (a - ap) * (a + ap), fmaf(lC, a, lB * ap));
    } else {
        Q = fmaf(lB, lC, fmaf(-a, ap, p2));
        W = fmaf(lC, a, -lB * ap);
    }
    const float den = fmaf(lA, Q, fmaf(a + E.BAtc, W, (lB + lC) * fmaf(lD, E.BAp, p2)));
    const float lBa = a > 0.0f ? div_q(p2, lB + a) : lB - a;
    const float lCa = ap > 0.0f ? div_q(p2, lC + ap) : lC - ap;
    const float s1 = atan2f(lD * E.g1, fmaf(lBa, E.cb, lD * E.h1));
    const float s2 = atan2f(lD * E.g2, fmaf(lCa, E.ca, -lD * E.h2));
    th = 2.0f * atan2f(2.0f * K.S * (lD * E.dn), den) - 2.0f * (s1 - s2);
}

// Psi = L_bc tbc + l1 ta + l2 tb; its three logs are returned as scalars (lg), summed by the
// lanes and combined with the FP64 unit edges once per pair (psi_from_logs).
__device__ __forceinline__ void vertex_integrand_f(f3 oA, f3 oB, f3 oC, const PanelJf &K, const VertexCtxF &Vx, f3 &lg, float &th)
{
    const float lA = normf(oA), lB = normf(oB), lC = normf(oC);
    const float Lbc = edge_log_f32(lB, dotf(oB, Vx.tbc), oB, lC, dotf(oC, Vx.tbc), oC, Vx.tbc, Vx.lenBC);
    const float l1 = logf(fmaxf((lC + dotf(oC, Vx.ta)) * Vx.inv_sqrt_si, kLogArgFloor));
    const float l2 = logf(fmaxf((lB - dotf(oB, Vx.tb)) * Vx.inv_sqrt_si, kLogArgFloor));
    lg = f3{Lbc, l1, l2};
    const float den = lA * lB * lC + dotf(oA, oB) * lC + dotf(oB, oC) * lA + dotf(oC, oA) * lB;
    // The angle terms s1 = atan2(o_A.w1, l_A c1 - o_A.p1) and s2 = atan2(o_A.w2, l_A c2 - o_A.p2)
    // are both singular on the ray A + t e (the planes' intersection line, which may cross K_i):
    // there both arguments vanish, each angle depends on the direction of approach, and only
    // their sum is smooth.  Near the ray FP32 rounding of o_A decides those directions
    // independently for s1 and s2 (errors up to 0.04 in the sum were seen).  Both are therefore
    // formed from one deviation r = o_A - (o_A.e) e (projected again onto the plane normal to e),
    // with the exact identities (e.w = 0, |e| = 1)
    //   l_A c - o_A.p = q c - r.p,   o_A.w = r.w,
    //   q = l_A - o_A.e = |r|^2 / (l_A + o_A.e)  (cancellation-free for o_A.e > 0);
    // a rounding error in r then moves the point the two angles are taken at, consistently, and
    // their sum does not depend on the direction of r near the ray.  r.p keeps the small FP64
    // vector p (r.p = r.(+-tau) would cancel when e is nearly parallel to -+tau).
    const float oe = dotf(oA, Vx.e);
    f3 r = oA - oe * Vx.e;
    r = r - dotf(r, Vx.e) * Vx.e;
    const float q = oe > 0.0f ? div_q(dotf(r, r), lA + oe) : lA - oe;
    const float s1 = atan2f(dotf(r, Vx.w1), q * Vx.c1 - dotf(r, Vx.p1));
    const float s2 = atan2f(dotf(r, Vx.w2), q * Vx.c2 - dotf(r, Vx.p2));
    th = 2.0f * atan2f(2.0f * K.S * dotf(K.n, oA), den) - 2.0f * (s1 + s2);
}

struct TriF {
    f3 a, b, c;
};
__device__ __forceinline__ TriF childf(const TriF &t, int k)
{
    const f3 mbc = 0.5f * (t.b + t.c), mca = 0.5f * (t.c + t.a), mab = 0.5f * (t.a + t.b);
    switch (k) {
    case 0: return TriF{mab, t.b, mbc};
    case 1: return TriF{mbc, t.c, mca};
    case 2: return TriF{mca, t.a, mab};
    default: return TriF{mbc, mca, mab};
    }
}
__device__ __forceinline__ TriF subcellf(TriF t, int level, int s)
{
    for (int l = level - 1; l >= 0; --l) t = childf(t, (s >> (2 * l)) & 3);
    return t;
}



// one refinement level of the regular part, FP32 evaluation, FP64 bookkeeping (same contract
// as k_level of the FP64 form).  Work items are (pair, lane of its lane group) over a grid-stride
// loop starting at `first` with stride `stride` (multiples of 32), so the same body serves the
// per-class kernels and the batched persistent kernel.
// a level's active lists: the pairs to integrate (act_in, count *cnt_in; all pairs when
// act_in is null) and the list the unconverged ones go to
struct LevelLists {
    const int *act_in, *cnt_in;
    int *act_out, *cnt_out;
};

__device__ __forceinline__ LevelLists level_lists(const ClassArgs &A, int level, int mode)
{
    if (mode == kFixed || level == 0) return LevelLists{A.act_in, A.cnt_in, A.act_out, A.cnt_out};
    return LevelLists{level == 1 ? nullptr : (level % 2 ? A.act_b : A.act_a), level == 1 ? nullptr : A.cnt + (level - 1),
                      level % 2 ? A.act_a : A.act_b, A.cnt + level};
}

// relative error control: level 0's pass also integrates level 1 (see level_items_mixed), and
// the level-1 pass is skipped
__device__ __forceinline__ bool fuse_levels01(int level, int mode, int kmax) { return level == 0 && mode == kAdaptiveRelative && kmax >= 1; }
__host__ __device__ __forceinline__ bool level_pass_needed(int level, int mode) { return !(level == 1 && mode == kAdaptiveRelative); }

// Psi of an adjacent pair from the lanes' sums of its logs (common vertex: L_bc, l1, l2; common
// edge: l1, l2), with K_j's unit edges in FP64 (K_j rotated by sj).  Summing the logs and applying
// the directions once keeps their FP32 rounding out of Psi; over the common-vertex pairs of the
// 20,480-triangle jittered sphere (FP32 emulation) that rounding was most of the error.  The
// lanes' logs are scaled by an FP32 constant s' (1/sqrt(S_i), or 1/|JC - JB|) rounded once from
// the exact s: every point's l1 and l2 carry ln(s'/s), which integrates to (s'/s - 1) S_i and is
// taken off here (to first order; the second is below 1e-14).
template <int CLS>
__device__ __forceinline__ void psi_from_logs(const ClassArgs &A, int2 pr, int sj, acc5 &a)
{
    const double4_32a *pj = A.panels[pr.y].v;
    const d3 ta = xyz(pj[4 + (sj + 1) % 3]), tb = xyz(pj[4 + (sj + 2) % 3]);
    const double Si = A.panels[pr.x].v[0].w;
    d3 p;
    if (CLS == kVertex) {
        const double dl = ((double)A.panels_f[pr.x].v[5].w * sqrt(Si) - 1.0) * Si;
        p = a.px * xyz(pj[4 + sj]) + (a.py - dl) * ta + (a.pz - dl) * tb;
    } else {
        const double dl = ((double)A.panels_f[pr.y].v[7 + sj].w * pj[4 + sj].w - 1.0) * Si;
        p = (a.px - dl) * tb + (a.py - dl) * ta;
    }
    a.px = p.x;
    a.py = p.y;
    a.pz = p.z;
}

template <int CLS>
__device__ void level_items_mixed(const ClassArgs &A, const LevelLists &Lst, const QuadTablesF &Qf, int level, int mode, double tol,
                                  int kmax, long long first, long long stride, int G_cap)
{
    const int nsub = 1 << (2 * level);
    const bool listed = Lst.act_in != nullptr;
    const int count = listed ? *Lst.cnt_in : A.n;
    // lanes per pair: the fewest (a power of two, at most a warp: G_cap) that still give the grid
    // about two work items per thread -- at levels 1-2 the active pairs alone outnumber the
    // threads, and each extra lane repeats the pair's set-up (some twenty panel loads) and a
    // butterfly step for its 13 points; or the whole block once a pair has at least a block's
    // worth of sub-cells (levels 4 and 5, where only a few pairs remain and one warp per pair left
    // each lane hundreds of points in series).  count is the same for every thread, so G is
    // uniform.  first and stride are thread-linear and the item count is then a multiple of the
    // block, so every block runs the loop uniformly and the __syncthreads of the block-wide
    // reduction below is reached by all its threads.
    const bool block_group = blockDim.x > 32 && nsub >= (int)blockDim.x;
    int G = 1;
    if (block_group) G = (int)blockDim.x;
    else
        while (G < G_cap && G < nsub && (long long)count * G < 2 * stride) G <<= 1;
    const int per_lane = nsub / G;
    const long long total = (long long)count * G;
    const long long total_r = block_group ? total : (total + 31) & ~31LL;
    const float sub_scale = ldexpf(1.0f, -2 * level);
    // Relative error control always computes levels 0 and 1 of every pair (the criterion compares
    // two levels), so level 0 does both: one lane per pair (G is 1 at level 0) integrates the
    // pair's 13 level-0 points and its 4 x 13 level-1 points with one set-up, and decides at level 1
    // with level 0's sums still in registers -- no level-0 round trip through `cur`, no second
    // set-up; the level-1 pass is then skipped (level_pass_needed).  The sums are the same
    // operations as in two passes.
    const bool fused01 = fuse_levels01(level, mode, kmax);
    for (long long idx = first; idx < total_r; idx += stride) {
        const bool valid = idx < total;
        const int slot = (int)(idx / G);
        const int lane_g = (int)(idx % G);
        const int t = valid ? (listed ? Lst.act_in[slot] : slot) : 0;
        acc5 acc = zero5();
        kahan5 ks;  // this lane's sums (value s - c); zero for lanes past the last item
        kahan_zero(ks);
        kahan5 ks0;  // level 0's sums when levels 0 and 1 are fused (ks then holds level 1's)
        kahan_zero(ks0);
        int2 pr = make_int2(0, 0);
        int sj_pair = 0;  // K_j's rotation (adjacent classes)
        if (valid) {
            pr = A.pairs[t];
            const PanelJf K = load_panel_f(A.panels_f, pr.y);
            const float Ssub = A.panels_f[pr.x].v[0].w * sub_scale;
            int origin = 0;  // vertex of K_j the offsets are measured from
            EdgeCtxF E;
            VertexCtxF Vx;
            FarCtxF F;
            TriF Tb;  // common edge: K_i's vertices as barycentric roles (x = JB, y = JC, z = off the edge)
            if (CLS == kFar) {
                F.ea = df_edge(A.panels_f, pr.y, 2, 1);  // C - B
                F.eb = -1.0f * K.AC;                      // A - C
            } else {
                const int3 ci = A.cells[pr.x], cj = A.cells[pr.y];
                int si, sj;
                if (CLS == kEdge) shifts_edge(ci, cj, si, sj);
                else shifts_vertex(ci, cj, si, sj);
                origin = sj;
                sj_pair = sj;
                // unit edges of K_j in the rotated order, rounded from FP64 (the panel's unit edge
                // k is opposite vertex k): the closed forms subtract the asymptote along the same
                // directions, so FP32-normalised edges would leave a bias of a few ulps at every point
                const float4 *uj = A.panels_f[pr.y].v + 7;
                const f3 t_a = xyzf(uj[(sj + 1) % 3]), t_b = xyzf(uj[(sj + 2) % 3]), t_bc = xyzf(uj[sj]);
                if (CLS == kEdge) {
                    E.ta = t_a;
                    E.tb = t_b;
                    E.ilvc = uj[sj].w;  // 1 / |JC - JB|, the edge opposite JA
                    const float4 *ce = reinterpret_cast<const float4 *>(A.ctx_e + kPairCtxFloats * (long long)t);
                    const float4 q1 = ce[1], q2 = ce[2], q3 = ce[3], q4 = ce[4];
                    E.h = q1.x;
                    E.dB = q1.w;
                    E.dC = q2.x;
                    E.dn = q2.y;
                    E.g1 = q2.z;
                    E.g2 = q2.w;
                    E.h1 = q3.x;
                    E.h2 = q3.y;
                    E.cb = q3.z;
                    E.ca = q3.w;
                    E.BAtc = q4.x;
                    E.BAp = q4.y;
                    E.L = q4.z;
                    const int jb = sj == 0 ? cj.y : (sj == 1 ? cj.z : cj.x);
                    const int iv[3] = {ci.x, ci.y, ci.z};
                    f3 role[3];
#pragma unroll
                    for (int k = 0; k < 3; ++k)
                        role[k] = k == si ? f3{0.0f, 0.0f, 1.0f} : (iv[k] == jb ? f3{1.0f, 0.0f, 0.0f} : f3{0.0f, 1.0f, 0.0f});
                    Tb = TriF{role[0], role[1], role[2]};
                } else {
                    const f3 AB = df_edge(A.panels_f, pr.y, (sj + 1) % 3, sj), AC = df_edge(A.panels_f, pr.y, (sj + 2) % 3, sj);
                    Vx.AB = AB;
                    Vx.AC = AC;
                    Vx.ta = t_a;
                    Vx.tb = t_b;
                    Vx.lenBC = A.panels_f[pr.y].v[2 + sj].w;  // |JC - JB|, the edge opposite JA
                    Vx.tbc = t_bc;
                    const float4 *ce = reinterpret_cast<const float4 *>(A.ctx_e + kPairCtxFloats * (long long)t);
                    const float4 q0 = ce[0], q1 = ce[1], q2 = ce[2], q3 = ce[3];
                    Vx.w1 = xyzf(q0);
                    Vx.p1 = f3{q0.w, q1.x, q1.y};
                    Vx.w2 = f3{q1.z, q1.w, q2.x};
                    Vx.p2 = f3{q2.y, q2.z, q2.w};
                    Vx.e = xyzf(q3);
                    Vx.c1 = 0.5f * dotf(Vx.p1, Vx.p1);
                    Vx.c2 = 0.5f * dotf(Vx.p2, Vx.p2);
                    Vx.inv_sqrt_si = A.panels_f[pr.x].v[5].w;
                }
            }
            // K_i's vertices as offsets from K_j's vertex A (the shared vertex for the
            // common-vertex class, the vertex off the shared edge for the common-edge class), exact
            // in double-float and rounded once.  The disjoint and common-vertex classes form a
            // point's offsets from the other two vertices as (o_A - e_hi) - e_lo with K_j's edges in
            // double-float: o_A's rounding is then a shift of the point shared by all three offsets
            // (harmless), the two subtractions add half an ulp each, and no rounded edge vector
            // enters the logs (that would be a per-pair bias, amplified by the cancellation in Psi).
            // The common-edge class needs no offsets from B and C: its points come close to the
            // shared edge, where every offset from its ends would be rounded at ulp(offset) while
            // the edge terms depend on the point's distance to the edge line.  It walks K_i's
            // sub-cells a second time in barycentric coordinates (exact dyadic values at these
            // levels), from which edge_integrand_f places the point in the shared edge's frame.
            TriF T0;
            f3 ABh, ABl, ACh, ACl;
            df_offsets(A.panels_f, pr.x, pr.y, origin, T0.a, T0.b, T0.c);
            if (CLS != kEdge) {
                df_edge_pair(A.panels_f, pr.y, (origin + 1) % 3, origin, ABh, ABl);
                df_edge_pair(A.panels_f, pr.y, (origin + 2) % 3, origin, ACh, ACl);
            }
            // sub-cell sc of level lev into the Kahan sums k (sub-cell area Ss)
            auto add_subcell = [&](kahan5 &k, int lev, int sc, float Ss) {
                const TriF U0 = subcellf(T0, lev, sc);
                TriF Ub;
                if (CLS == kEdge) Ub = subcellf(Tb, lev, sc);
                float c0 = 0, c1 = 0, c2 = 0, c3 = 0, c4 = 0;
#pragma unroll 1
                for (int g = 0; g < Qf.npts; ++g) {
                    const float l1 = Qf.L1[g], l2 = Qf.L2[g], l3 = Qf.L3[g];
                    const f3 oA = l1 * U0.a + l2 * U0.b + l3 * U0.c;
                    f3 psi;  // the disjoint class's Psi; the adjacent classes' log coefficients (psi_from_logs)
                    float th, pot = 0.0f;
                    if (CLS == kEdge) {
                        edge_integrand_f(oA, l1 * Ub.a + l2 * Ub.b + l3 * Ub.c, K, E, psi, th);
                    } else {
                        const f3 oB = (oA - ABh) - ABl, oC = (oA - ACh) - ACl;
                        if (CLS == kFar) far_field_integrand_f(oA, oB, oC, K, F, psi, th, pot);
                        else vertex_integrand_f(oA, oB, oC, K, Vx, psi, th);
                    }
                    const float w = Qf.w[g];
                    c0 = fmaf(w, psi.x, c0);
                    c1 = fmaf(w, psi.y, c1);
                    c2 = fmaf(w, psi.z, c2);
                    c3 = fmaf(w, th, c3);
                    c4 = fmaf(w, pot, c4);
                }
                kahan_add(k, 0, Ss * c0);
                kahan_add(k, 1, Ss * c1);
                kahan_add(k, 2, Ss * c2);
                kahan_add(k, 3, Ss * c3);
                kahan_add(k, 4, Ss * c4);
            };
            // one copy of the loop for both passes: fused, step 0 is level 0's cell (its sums move
            // to ks0) and steps 1-4 level 1's sub-cells
            const int steps = fused01 ? 5 : per_lane;
            for (int j = 0; j < steps; ++j) {
                if (fused01) add_subcell(ks, j == 0 ? 0 : 1, j == 0 ? 0 : j - 1, j == 0 ? Ssub : Ssub * 0.25f);
                else add_subcell(ks, level, lane_g * per_lane + j, Ssub);
                if (fused01 && j == 0) {
                    ks0 = ks;
                    kahan_zero(ks);
                }
            }
        }
        // the lanes' Kahan pairs added across the group in FP32 (kahan_pair_add); lane 0 converts
        for (int off = 1; off < (G < 32 ? G : 32); off <<= 1) {
#pragma unroll
            for (int i = 0; i < 5; ++i) {
                const float s2 = __shfl_xor_sync(0xffffffffu, ks.s[i], off), c2 = __shfl_xor_sync(0xffffffffu, ks.c[i], off);
                kahan_pair_add(ks.s[i], ks.c[i], s2, c2);
            }
        }
        if (block_group) {
            // the warps' pairs through shared memory, added in warp order by thread 0 (at most
            // 256 threads, 8 warps)
            __shared__ float grp[8][10];
            const int w = threadIdx.x >> 5;
            if ((threadIdx.x & 31) == 0) {
#pragma unroll
                for (int i = 0; i < 5; ++i) {
                    grp[w][i] = ks.s[i];
                    grp[w][5 + i] = ks.c[i];
                }
            }
            __syncthreads();
            if (threadIdx.x == 0)
                for (int k = 1; k < (int)(blockDim.x >> 5); ++k)
#pragma unroll
                    for (int i = 0; i < 5; ++i) kahan_pair_add(ks.s[i], ks.c[i], grp[k][i], grp[k][5 + i]);
            __syncthreads();
        }
        if (!valid || lane_g != 0) continue;
        acc.px = (double)ks.s[0] - (double)ks.c[0];
        acc.py = (double)ks.s[1] - (double)ks.c[1];
        acc.pz = (double)ks.s[2] - (double)ks.c[2];
        acc.th = (double)ks.s[3] - (double)ks.c[3];
        acc.pot = (double)ks.s[4] - (double)ks.c[4];
        if (CLS != kFar) psi_from_logs<CLS>(A, pr, sj_pair, acc);
        double *cur = A.cur + 5 * (long long)t;
        int lev = level;  // the level decided on below
        LevelLists out = Lst;
        acc5 prev;
        if (fused01) {
            prev = acc5{(double)ks0.s[0] - (double)ks0.c[0], (double)ks0.s[1] - (double)ks0.c[1], (double)ks0.s[2] - (double)ks0.c[2],
                        (double)ks0.s[3] - (double)ks0.c[3], (double)ks0.s[4] - (double)ks0.c[4]};
            if (CLS != kFar) psi_from_logs<CLS>(A, pr, sj_pair, prev);
            lev = 1;
            out = level_lists(A, 1, mode);
        } else {
            if (mode == kFixed || level == 0) {
                cur[0] = acc.px; cur[1] = acc.py; cur[2] = acc.pz; cur[3] = acc.th; cur[4] = acc.pot;
                continue;
            }
            prev = acc5{cur[0], cur[1], cur[2], cur[3], cur[4]};
        }
        cur[0] = acc.px; cur[1] = acc.py; cur[2] = acc.pz; cur[3] = acc.th; cur[4] = acc.pot;
        // error estimator: the differences of successive levels (where cancellation sits) and the
        // singular part are formed in FP64; the norms of the resulting J and dJ are compared in FP32
        // (squared, no square roots), which is ample for a 1e-6..1e-2 tolerance
        const double4_32a nj4 = A.panels[pr.y].v[3];
        const f3 nf = f3{(float)nj4.x, (float)nj4.y, (float)nj4.z};
        double spx = 0.0, spy = 0.0, spz = 0.0, sth = 0.0;
        if (CLS != kFar) {
            const double *sg = A.sing + 4 * (long long)t;
            spx = sg[0]; spy = sg[1]; spz = sg[2]; sth = sg[3];
        }
        double th_tot = acc.th + sth;
        if (CLS == kVertex) {
            // the p-fix of the common-vertex class (evaluatorJ3DK.cu:224-264)
            const double ref = kTwoPi * A.panels[pr.x].v[0].w;
            int pf = 0;
            if (th_tot > ref) pf = -((int)trunc((th_tot - ref) / (2.0 * ref)) + 1);
            else if (th_tot < -ref) pf = ((int)trunc((-ref - th_tot) / (2.0 * ref)) + 1);
            th_tot += 2.0 * pf * ref;
        }
        const f3 psif = f3{(float)(acc.px + spx), (float)(acc.py + spy), (float)(acc.pz + spz)};
        const f3 Jf = (float)th_tot * nf + crossf(psif, nf);
        const f3 dpsif = f3{(float)(acc.px - prev.px), (float)(acc.py - prev.py), (float)(acc.pz - prev.pz)};
        const f3 dJf = (float)(acc.th - prev.th) * nf + crossf(dpsif, nf);
        const float tolf = (float)tol;
        bool unconv;
        if (mode == kAdaptiveCompat) {
            unconv = runge_unconverged(acc, prev, Qf.pow2p);
        } else {
            unconv = dotf(dJf, dJf) > tolf * tolf * dotf(Jf, Jf);
            if (CLS == kFar) unconv = unconv || fabsf((float)(acc.pot - prev.pot)) > tolf * fabsf((float)acc.pot);
        }
        atomicMax(A.maxlev, lev);
        if (!unconv || lev >= kmax) {
            A.stop[t] = lev;
            double *fa = A.fin_a + 5 * (long long)t;
            fa[0] = acc.px; fa[1] = acc.py; fa[2] = acc.pz; fa[3] = acc.th; fa[4] = acc.pot;
            if (mode == kAdaptiveCompat) {  // only the compat mode's buffer parity reads the previous level
                double *fb = A.fin_b + 5 * (long long)t;
                fb[0] = prev.px; fb[1] = prev.py; fb[2] = prev.pz; fb[3] = prev.th; fb[4] = prev.pot;
            }
        } else {
            out.act_out[atomicAdd(out.cnt_out, 1)] = t;
        }
    }
}

template <int CLS>
__global__ void __launch_bounds__(256, 2) k_level_mixed(ClassArgs A, QuadTablesF Qf, int level, int mode, double tol, int kmax)
{
    // the host sets this level's lists in A (level_chain_mixed)
    level_items_mixed<CLS>(A, LevelLists{A.act_in, A.cnt_in, A.act_out, A.cnt_out}, Qf, level, mode, tol, kmax,
                           (long long)blockIdx.x * blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x, 32);
}

// ------------------------------------------------------------------ adjacent pairs: singular parts + FP32 Duffy potential
// graded Duffy rule in FP32 over the pieces of K_i; point offsets to K_j's vertices are formed
// as (apex - vertex) + w with the apex offsets exact in double-float, so graded points that sit
// very close to a shared vertex keep their relative precision
template <int CLS>
__device__ float duffy_total_f(const PanelF *__restrict__ P, int pi, int pj, int si, const PanelJf &K, const FarCtxF &F,
                               int p1_vertex, const f3 &m_in, float c, float h, const float *uu, const float *uw, int nu,
                               const float *vv, const float *vw, int nv, int first = 0, int step = 1)
{
    // first / step select the points p = first, first + step, ... of the flattened (piece, radial,
    // angular) list, so that a warp can share one rule (step 32); the defaults sum all points
    f3 R0[3], R1[3], R2[3];  // K_i's vertices (rotated by si) as offsets from K_j's vertices 0, 1, 2
    {
        f3 a, b, cc;
        df_offsets(P, pi, pj, 0, a, b, cc);
        const f3 q0[3] = {a, b, cc};
        df_offsets(P, pi, pj, 1, a, b, cc);
        const f3 q1[3] = {a, b, cc};
        df_offsets(P, pi, pj, 2, a, b, cc);
        const f3 q2[3] = {a, b, cc};
        for (int k = 0; k < 3; ++k) {
            R0[k] = q0[(si + k) % 3];
            R1[k] = q1[(si + k) % 3];
            R2[k] = q2[(si + k) % 3];
        }
    }
    const int npieces = CLS == kEdge ? 2 : 1;
    const int per = nu * nv;
    float total = 0.0f, comp = 0.0f;  // compensated (Kahan) sum: the tier checks compare to 2e-7
#pragma unroll 1
    for (int p = first; p < npieces * per; p += step) {
        const int piece = p / per, q = p - piece * per, a = q / nv, b = q - a * nv;
        // apex slot and the two other corners of the piece, as offsets from K_j's vertex 0
        int ap;
        f3 B, Cc;
        if (CLS == kVertex) { ap = 0; B = R0[1]; Cc = R0[2]; }
        else {
            const f3 M = 0.5f * (R0[1] + R0[2]);
            if (piece == 0) { ap = 1; B = M; Cc = R0[0]; }
            else { ap = 2; B = R0[0]; Cc = M; }
        }
        const f3 dA = R0[ap], dB = R1[ap], dC = R2[ap];
        const f3 eB = B - dA, eC = Cc - dA;
        const float u = uu[a];
        const f3 w = u * ((1.0f - vv[b]) * eB + vv[b] * eC);
        f3 psi;
        float th, g;
        far_integrand_f(dA + w, dB + w, dC + w, K, F, psi, th, g);
        if (CLS == kEdge) {
            const f3 dP1 = p1_vertex == 0 ? dA : (p1_vertex == 1 ? dB : dC);
            const float sd = dotf(dP1 + w, m_in);
            if (sd > 0.0f) g += 2.0f * c * sd * logf(sd / h);
        }
        const float y = normf(crossf(eB, eC)) * uw[a] * u * vw[b] * g - comp;
        const float tt = total + y;
        comp = (tt - total) - y;
        total = tt;
    }
    return total;
}

// s ln s term along the shared edge of a common-edge pair, set up in FP64 (pairs holding a
// needle cell; the others form it in double-float in singular_mixed_item)
__device__ __forceinline__ void edge_sigma_setup(const ClassArgs &A, int2 pr, int si, int sj, double Si, f3 &m_in, float &c, float &h,
                                                 double &sig)
{
    const PanelJ K = load_panel(A.panels, pr.y);
    const Tri Ti0 = load_tri(A.panels, pr.x);
    const d3 Pi[3] = {Ti0.a, Ti0.b, Ti0.c}, Pj[3] = {K.A, K.B, K.C};
    const d3 JB = Pj[(sj + 1) % 3], JC = Pj[(sj + 2) % 3], IA = Pi[si];
    const d3 tau = unit(JC - JB), m = cross(tau, K.n), w = IA - JB;
    const d3 perp = w - dot(w, tau) * tau;
    const double hd = norm(perp);
    const d3 mi = (1.0 / hd) * perp;
    const double cd = -dot(m, mi);
    m_in = to_f3(mi);
    c = (float)cd;
    h = (float)hd;
    sig = (5.0 / 9.0) * cd * Si * hd;
}

// the shared-edge term's constants of a common-edge pair in ctx_e (written once per pair by the
// closed-form kernel, read by the potential's FP32 tiers): m_in, c, h, then the integral over K_i
// as a double's two halves
__device__ __forceinline__ void store_edge_sigma(const ClassArgs &A, long long t, f3 m_in, float c, float h, double sig)
{
    float4 *ce = reinterpret_cast<float4 *>(A.ctx_e + kPairCtxFloats * t);
    ce[0] = make_float4(m_in.x, m_in.y, m_in.z, c);
    ce[1] = make_float4(h, __int_as_float(__double2hiint(sig)), __int_as_float(__double2loint(sig)), 0.0f);
}

__device__ __forceinline__ void load_edge_sigma(const ClassArgs &A, long long t, f3 &m_in, float &c, float &h, double &sig)
{
    const float4 *ce = reinterpret_cast<const float4 *>(A.ctx_e + kPairCtxFloats * t);
    const float4 a = ce[0], b = ce[1];
    m_in = f3{a.x, a.y, a.z};
    c = a.w;
    h = b.x;
    sig = __hiloint2double(__float_as_int(b.y), __float_as_int(b.z));
}

// the shared-edge frame of a common-edge pair (EdgeCtxF) in ctx_e after the shared-edge term:
// [7] dB, [8..11] dC, n_j.D_p, D_p.(tb x tc), D_p.(ta x tc), [12..15] (tb - tc).D_p, (ta - tc).D_p,
// 1 - tb.tc, 1 - ta.tc, [16..18] (JB - JA).tc, (JB - JA).D_p, L; formed in FP64 and rounded once
// (h = |D_p| is the shared-edge term's h, [4])
__device__ __forceinline__ void store_edge_frame(const ClassArgs &A, int2 pr, int si, int sj, long long t)
{
    const PanelJ K = load_panel(A.panels, pr.y);
    const Tri Ti = load_tri(A.panels, pr.x);
    const d3 Pi[3] = {Ti.a, Ti.b, Ti.c}, Pj[3] = {K.A, K.B, K.C};
    const d3 JA = Pj[sj], JB = Pj[(sj + 1) % 3], JC = Pj[(sj + 2) % 3], D = Pi[si];
    const d3 tc = unit(JC - JB), ta = unit(JA - JC), tb = unit(JB - JA);
    const d3 w = D - JB, BA = JB - JA;
    const double dB = dot(w, tc);
    const d3 Dp = w - dB * tc, ub = tb - tc, ua = ta - tc;
    float *ce = A.ctx_e + kPairCtxFloats * t;
    ce[7] = (float)dB;
    reinterpret_cast<float4 *>(ce)[2] =
        make_float4((float)dot(JC - D, tc), (float)dot(K.n, Dp), (float)dot(Dp, cross(tb, tc)), (float)dot(Dp, cross(ta, tc)));
    reinterpret_cast<float4 *>(ce)[3] = make_float4((float)dot(ub, Dp), (float)dot(ua, Dp), (float)(0.5 * dot(ub, ub)), (float)(0.5 * dot(ua, ua)));
    reinterpret_cast<float4 *>(ce)[4] = make_float4((float)dot(BA, tc), (float)dot(BA, Dp), (float)norm(JC - JB), 0.0f);
}

// true when the common-edge closed form's factor 1 / (sin a (1 - c^2)) (closed_edge_unit's q_edge,
// c = c_mu or c_sigma) exceeds 1 / kEdgeClosedFormC2 outside the coplanar branch: the angles at the
// shared edge's ends from cosines and sines of FP64 unit edges (Ti, Tj rotated as the closed form
// takes them, the off-edge vertex first)
__device__ __forceinline__ bool edge_closed_form_cancels(const Tri &Ti, const Tri &Tj, d3 ni, d3 nj)
{
    const d3 ica = unit(Ti.a - Ti.c), icb = unit(Ti.b - Ti.c), iba = unit(Ti.a - Ti.b), ibc = unit(Ti.c - Ti.b);
    const d3 jba = unit(Tj.a - Tj.b), jbc = unit(Tj.c - Tj.b), jca = unit(Tj.a - Tj.c), jcb = unit(Tj.b - Tj.c);
    const double ca = dot(ica, icb), sa = norm(cross(ica, icb)), cb = dot(ibc, iba), sb = norm(cross(ibc, iba));
    const double cg = dot(jbc, jba), sg = norm(cross(jbc, jba)), cd = dot(jcb, jca), sd = norm(cross(jcb, jca));
    const double cx = dot(ni, nj);
    const double cmu = -(cb * cg + cx * sb * sg), csig = -(ca * cd + cx * sa * sd);
    return 1.0 - cmu * cmu < kEdgeClosedFormC2 || 1.0 - csig * csig < kEdgeClosedFormC2;
}

template <int CLS>
__device__ __forceinline__ void singular_mixed_item(const ClassArgs &A, const QuadTablesF &Qf, long long t)
{
    const int2 pr = A.pairs[t];
    const int3 ci = A.cells[pr.x], cj = A.cells[pr.y];
    const PanelJ Kd = load_panel(A.panels, pr.y);
    const double4_32a ni4 = A.panels[pr.x].v[3];
    const d3 ni = mk(ni4.x, ni4.y, ni4.z);
    const double Si = A.panels[pr.x].v[0].w;
    int si, sj;
    if (CLS == kEdge) shifts_edge(ci, cj, si, sj);
    else shifts_vertex(ci, cj, si, sj);
    // closed-form singular part (a4 / a5) and, for the vertex class, the asymptote's constants.
    // A pair that holds a needle cell is recomputed in FP64 after the level sweep, its J a small
    // difference of large parts: its closed form is FP64 too (the path below), so that the fix-up
    // reproduces the FP64 form.  So does a common-edge pair whose closed form cancels by more than
    // double-float can carry (edge_closed_form_cancels: none of the 61,440 pairs of the
    // 20,480-triangle jittered sphere, 4 to 7 in 800 on the reference's Fish and Krylo01 examples,
    // where double-float gave errors up to 4e-5).  Every other pair computes it in double-float, the pair
    // translated to K_j's vertex A in FP64 (the closed forms depend on vertex differences only)
    // and converted; the closed forms scale it by a power of two.
    const Tri Ti64 = rotate(load_tri(A.panels, pr.x), si), Tj64 = rotate(Tri{Kd.A, Kd.B, Kd.C}, sj);
    if (A.panels[pr.x].v[2].w > kNeedleCos || A.panels[pr.y].v[2].w > kNeedleCos ||  // as fixup_collect_item
        (CLS == kEdge && edge_closed_form_cancels(Ti64, Tj64, ni, Kd.n))) {
        const Tri &Ti = Ti64, &Tj = Tj64;
        d3 psi;
        double th;
        if (CLS == kEdge) {
            closed_edge(Ti, Tj, ni, Kd.n, Si, psi, th);
            f3 m_in;
            float c, h;
            double sig;
            edge_sigma_setup(A, pr, si, sj, Si, m_in, c, h, sig);
            store_edge_sigma(A, t, m_in, c, h, sig);
            store_edge_frame(A, pr, si, sj, t);
        } else {
            closed_vertex(Ti, Tj, ni, Kd.n, Si, psi, th);
            const d3 ta = unit(Tj.a - Tj.c), tb = unit(Tj.b - Tj.a);
            double dA, dB;
            const d3 e = vertex_direction(ni, Kd.n, ta, tb, dA, dB);
            const d3 w1 = cross(ta, e), p1 = e - ta, w2 = cross(tb, e), p2 = e + tb;
            float4 *ce = reinterpret_cast<float4 *>(A.ctx_e + kPairCtxFloats * (long long)t);
            // w1, p1, w2, p2 (12 floats), then e
            ce[0] = make_float4((float)w1.x, (float)w1.y, (float)w1.z, (float)p1.x);
            ce[1] = make_float4((float)p1.y, (float)p1.z, (float)w2.x, (float)w2.y);
            ce[2] = make_float4((float)w2.z, (float)p2.x, (float)p2.y, (float)p2.z);
            ce[3] = make_float4((float)e.x, (float)e.y, (float)e.z, 0.0f);
        }
        double *sg = A.sing + 4 * (long long)t;
        sg[0] = psi.x; sg[1] = psi.y; sg[2] = psi.z; sg[3] = th;
    } else {
        const Tri Ti0 = load_tri(A.panels, pr.x);
        const d3 o = Kd.A;
        const TriD Ti = to_df(rotate(Tri{Ti0.a - o, Ti0.b - o, Ti0.c - o}, si));
        const TriD Tj = to_df(rotate(Tri{mk(0.0, 0.0, 0.0), Kd.B - o, Kd.C - o}, sj));
        const df3 nid = to_df(ni), njd = to_df(Kd.n);
        df3 psi;
        dfl th;
        if (CLS == kEdge) {
            closed_edge(Ti, Tj, nid, njd, dfl(Si), psi, th);
            // the shared edge JB -> JC (Tj rotated: JA off the edge), as edge_sigma_setup
            const df3 tau = unit(Tj.c - Tj.b), m = cross(tau, njd), w = Ti.a - Tj.b;
            const df3 perp = w - dot(w, tau) * tau;
            const dfl hd = norm(perp);
            const df3 mi = (1.0f / hd) * perp;
            const dfl cd = -dot(m, mi);
            store_edge_sigma(A, t, f3{mi.x.hi, mi.y.hi, mi.z.hi}, cd.hi, hd.hi, (double)(((5.0 / 9.0) * cd) * (dfl(Si) * hd)));
            store_edge_frame(A, pr, si, sj, t);
        } else {
            closed_vertex(Ti, Tj, nid, njd, dfl(Si), psi, th);
            const df3 ta = unit(Tj.a - Tj.c), tb = unit(Tj.b - Tj.a);
            dfl dA, dB;
            const df3 e = vertex_direction(nid, njd, ta, tb, dA, dB);
            const df3 w1 = cross(ta, e), p1 = e - ta, w2 = cross(tb, e), p2 = e + tb;
            float4 *ce = reinterpret_cast<float4 *>(A.ctx_e + kPairCtxFloats * (long long)t);
            // w1, p1, w2, p2 (12 floats), then e
            ce[0] = make_float4(w1.x.hi, w1.y.hi, w1.z.hi, p1.x.hi);
            ce[1] = make_float4(p1.y.hi, p1.z.hi, w2.x.hi, w2.y.hi);
            ce[2] = make_float4(w2.z.hi, p2.x.hi, p2.y.hi, p2.z.hi);
            ce[3] = make_float4(e.x.hi, e.y.hi, e.z.hi, 0.0f);
        }
        double *sg = A.sing + 4 * (long long)t;
        sg[0] = (double)psi.x; sg[1] = (double)psi.y; sg[2] = (double)psi.z; sg[3] = (double)th;
    }
}

// tier 1 of the potential in FP32 (main graded Duffy rule, and the check rule unless the pair
// goes straight to the adaptive rule), by a group of 8 lanes per pair: the 128 points of the two
// rules, 16 per lane, would be a long serial chain for one thread.  The lanes' Kahan partial sums
// are added in FP64.
constexpr int kTier1Lanes = 8;

__device__ __forceinline__ double group_sum8(double x)
{
    const unsigned mask = 0xffu << (threadIdx.x & 24);
    for (int off = 1; off < kTier1Lanes; off <<= 1) x += __shfl_xor_sync(mask, x, off, kTier1Lanes);
    return x;
}

template <int CLS>
__device__ __forceinline__ void tier1_mixed_item(const ClassArgs &A, const QuadTablesF &Qf, long long t, int g)
{
    const int2 pr = A.pairs[t];
    const int3 ci = A.cells[pr.x], cj = A.cells[pr.y];
    int si, sj;
    if (CLS == kEdge) shifts_edge(ci, cj, si, sj);
    else shifts_vertex(ci, cj, si, sj);
    const PanelJf K = load_panel_f(A.panels_f, pr.y);
    const FarCtxF F{crossf(K.ta, K.n), crossf(K.tb, K.n), crossf(K.tc, K.n)};
    f3 m_in = f3{0, 0, 0};
    float c = 0.0f, h = 1.0f;
    double sig = 0.0;
    const int p1v = (sj + 1) % 3;  // JB, start of the shared edge in K_j's orientation
    if (CLS == kEdge) load_edge_sigma(A, t, m_in, c, h, sig);
    const double pmd = group_sum8((double)duffy_total_f<CLS>(A.panels_f, pr.x, pr.y, si, K, F, p1v, m_in, c, h, Qf.du_u, Qf.du_w, Qf.nu,
                                                             Qf.dv_v, Qf.dv_w, Qf.nv, g, kTier1Lanes)) + sig;
    if (g == 0) A.padj[t] = kInv4Pi * pmd;
    if (!A.hard_list) return;
    const double c10 = 0.98480775301220806;
    const double4_32a ni4 = A.panels[pr.x].v[3], nj4 = A.panels[pr.y].v[3];
    if (ni4.x * nj4.x + ni4.y * nj4.y + ni4.z * nj4.z < 0.5 || A.panels[pr.x].v[2].w > c10 || A.panels[pr.y].v[2].w > c10) {
        if (g == 0) A.hard_list[atomicAdd(A.hard_cnt, 1)] = (int)t;
        return;
    }
    const double pl = group_sum8((double)duffy_total_f<CLS>(A.panels_f, pr.x, pr.y, si, K, F, p1v, m_in, c, h, Qf.lo_u, Qf.lo_uw, Qf.lo_nu,
                                                            Qf.lo_v, Qf.lo_vw, Qf.lo_nv, g, kTier1Lanes)) + sig;
    if (g == 0 && fabs(pmd - pl) > A.tier_tol * fabs(pmd)) A.tier2_list[atomicAdd(A.tier2_cnt, 1)] = (int)t;
}

template <int CLS>
__global__ void __launch_bounds__(128) k_tier1_mixed(ClassArgs A, QuadTablesF Qf)
{
    // every pair's group of 8 lanes is one aligned group of a warp, and the whole group is valid
    // or invalid together
    const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid / kTier1Lanes < A.n) tier1_mixed_item<CLS>(A, Qf, gid / kTier1Lanes, (int)(gid % kTier1Lanes));
}

template <int CLS>
__global__ void __launch_bounds__(128) k_singular_mixed(ClassArgs A, QuadTablesF Qf)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < A.n) singular_mixed_item<CLS>(A, Qf, t);
}


// tier 2 in FP32, one warp per listed pair (the lanes share each rule's points); the pairs it
// rejects are listed for tier 2b, which runs in FP64 because the FP32 rules can share a bias of
// a few 1e-6 (a small, flat K_j beside a large K_i), and two biased rules agree with each other.
template <int CLS>
__device__ __forceinline__ void tier2_mixed_item(const ClassArgs &A, const QuadTablesF &Qf, const QuadTables &Q, int h, int lane)
{
    const int t = A.tier2_list[h];
    const int2 pr = A.pairs[t];
    const int3 ci = A.cells[pr.x], cj = A.cells[pr.y];
    int si, sj;
    if (CLS == kEdge) shifts_edge(ci, cj, si, sj);
    else shifts_vertex(ci, cj, si, sj);
    const PanelJf Kf = load_panel_f(A.panels_f, pr.y);
    const FarCtxF Ff{crossf(Kf.ta, Kf.n), crossf(Kf.tb, Kf.n), crossf(Kf.tc, Kf.n)};
    f3 m_in = f3{0, 0, 0};
    float c = 0.0f, hh = 1.0f;
    double sig = 0.0;
    const int p1v = (sj + 1) % 3;
    if (CLS == kEdge) load_edge_sigma(A, t, m_in, c, hh, sig);
    // the lanes' Kahan partial sums added in FP64 (an FP32 butterfly adds noise the tier bar sees)
    const double ph = warp_sum((double)duffy_total_f<CLS>(A.panels_f, pr.x, pr.y, si, Kf, Ff, p1v, m_in, c, hh, Qf.hi_u, Qf.hi_uw,
                                                          Qf.hi_nu, Qf.hi_v, Qf.hi_vw, Qf.hi_nv, lane, 32)) + sig;
    const double pm = A.padj[t] * (4.0 * kPi);
    if (lane != 0) return;
    if (fabs(ph - pm) <= A.tier_tol * fabs(ph)) A.padj[t] = kInv4Pi * ph;
    else A.tier2b_list[atomicAdd(A.cnt + kCntTier2b, 1)] = t;  // tier 2b next, in FP64 (i2_tiers.cuh)
}

template <int CLS>
__global__ void __launch_bounds__(128) k_pot_tier2_mixed(ClassArgs A, QuadTablesF Qf, QuadTables Q)
{
    const int count = *A.tier2_cnt;
    const int lane = threadIdx.x & 31;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int h = (int)warp_item_index(); h < count; h += nwarps) tier2_mixed_item<CLS>(A, Qf, Q, h, lane);
}

// ------------------------------------------------------------------ FP64 fix-up of ill-conditioned pairs
// A pair that holds a needle cell (a corner angle below 5 degrees) is ill-conditioned: its J is
// a small difference of large parts, and FP32 rounding of the bulk is amplified by a few thousand
// there (measured: errors up to 1e-3 on the 20,480-triangle jittered sphere, whose two needles
// have corners of 0.6 and 1.5 degrees).  After the mixed chain has finished, each such pair's
// regular part is recomputed in FP64 by one whole block, the threads striding over the 4^L
// sub-cells x 13 points (a few pairs at level 5 would otherwise set the time), and J (and the
// disjoint class's potential) is finalised again.  Other pairs cost two loads.
template <int CLS>
struct FixupPair {
    PanelJ K;
    Tri Ti;
    double Si;
    FarCtx F;
    EdgeCtx E;
    VertexCtx Vx;
};

// (Psi, Theta, potential) of the regular part at `level`, summed by the whole block (every thread
// receives the sums); red holds 5 doubles per warp
template <int CLS>
__device__ acc5 fixup_level_sum(const FixupPair<CLS> &p, const QuadTables &Q, int level, double *red)
{
    const int nsub = 1 << (2 * level);
    const double Ssub = p.Si * ldexp(1.0, -2 * level);
    acc5 acc = zero5();
    // the flattened (sub-cell, point) list over the block: level 0's 13 points already keep 13
    // threads busy (one thread per sub-cell left levels 0-2 nearly idle), at the price of one
    // sub-cell walk (at most kFixDirect midpoint splits) per point
    const int total = nsub * Q.npts;
    for (int j = threadIdx.x; j < total; j += blockDim.x) {
        const int sc = j / Q.npts, g = j - sc * Q.npts;
        const Tri T = subcell(p.Ti, level, sc);
        const d3 x = Q.L1[g] * T.a + Q.L2[g] * T.b + Q.L3[g] * T.c;
        d3 psi;
        double th, pot = 0.0;
        if (CLS == kFar) far_integrand(x, p.K, p.F, psi, th, pot);
        else if (CLS == kEdge) edge_integrand(x, p.K, p.E, psi, th);
        else vertex_integrand(x, p.K, p.Vx, psi, th);
        axpy5(acc, Ssub * Q.w[g], psi, th, pot);
    }
    for (int off = 16; off > 0; off >>= 1) {
        acc.px += __shfl_xor_sync(0xffffffffu, acc.px, off);
        acc.py += __shfl_xor_sync(0xffffffffu, acc.py, off);
        acc.pz += __shfl_xor_sync(0xffffffffu, acc.pz, off);
        acc.th += __shfl_xor_sync(0xffffffffu, acc.th, off);
        acc.pot += __shfl_xor_sync(0xffffffffu, acc.pot, off);
    }
    const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) store5(red + 5 * w, acc);
    __syncthreads();
    acc5 tot = zero5();
    for (int k = 0; k < nw; ++k) {
        const acc5 v = load5(red + 5 * k);
        tot.px += v.px; tot.py += v.py; tot.pz += v.pz; tot.th += v.th; tot.pot += v.pot;
    }
    return tot;
}

// the pairs that hold a needle cell, gathered into list[0 .. *count) (the class's active-list
// buffer, free once the level chain has finished)
// A disjoint pair needs it only when K_j, the cell integrated in closed form, is the needle: its
// two long, nearly antiparallel edges make Psi a small difference of nearly equal edge terms.  A
// needle K_i is only a small area the quadrature runs over.  Adjacent pairs share vertices with
// both cells, so either cell's needle counts there.  An adjacent pair is also gathered when its
// closed-form part, (Theta_s n_j + Psi_s x n_j) / (4 pi), exceeds the finalised J by kFixRatio:
// J is then a small difference of that part and an FP32 quadrature part of the same size (up to
// 355x |J| among the 20,480-triangle jittered sphere's common-vertex pairs).
template <int CLS>
__device__ __forceinline__ void fixup_collect_item(const ClassArgs &A, int *list, int *count, long long t)
{
    const int2 pr = A.pairs[t];
    bool take = (CLS != kFar && A.panels[pr.x].v[2].w > kNeedleCos) || A.panels[pr.y].v[2].w > kNeedleCos;
    if (CLS != kFar && !take) {
        const double *sg = A.sing + 4 * t, *J = A.J3 + 3 * t;
        const double4_32a nj4 = A.panels[pr.y].v[3];
        const d3 ps = cross(mk(sg[0], sg[1], sg[2]), mk(nj4.x, nj4.y, nj4.z));
        const double s2 = (sg[3] * sg[3] + dot(ps, ps)) * (kInv4Pi * kInv4Pi);  // |J_s|^2 (Psi_s x n_j is normal to n_j)
        take = s2 > kFixRatio * kFixRatio * (J[0] * J[0] + J[1] * J[1] + J[2] * J[2]);
    }
    if (take) list[atomicAdd(count, 1)] = (int)t;
}

template <int CLS>
__global__ void __launch_bounds__(256) k_fixup_collect(ClassArgs A, int *list, int *count)
{
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < A.n; t += (long long)gridDim.x * blockDim.x)
        fixup_collect_item<CLS>(A, list, count, t);
}

// pair t, by the whole block (red: 5 doubles per warp of shared memory)
template <int CLS>
__device__ __forceinline__ FixupPair<CLS> fixup_pair(const ClassArgs &A, int t, d3 &nj, d3 &spsi, double &sth)
{
    const int2 pr = A.pairs[t];
    const double4_32a ni4 = A.panels[pr.x].v[3], nj4 = A.panels[pr.y].v[3];
    const d3 ni = mk(ni4.x, ni4.y, ni4.z);
    nj = mk(nj4.x, nj4.y, nj4.z);
    FixupPair<CLS> p;
    p.K = load_panel(A.panels, pr.y);
    p.Ti = load_tri(A.panels, pr.x);
    p.Si = A.panels[pr.x].v[0].w;
    if (CLS == kFar) p.F = make_far_ctx(p.K);
    else {
        const int3 ci = A.cells[pr.x], cj = A.cells[pr.y];
        int si, sj;
        if (CLS == kEdge) {
            shifts_edge(ci, cj, si, sj);
            p.E = make_edge_ctx(p.K, sj);
        } else {
            shifts_vertex(ci, cj, si, sj);
            p.Vx = make_vertex_ctx(p.K, sj, ni, p.Si);
        }
    }
    spsi = mk(0, 0, 0);
    sth = 0.0;
    if (CLS != kFar) {
        const double *sg = A.sing + 4 * (long long)t;
        spsi = mk(sg[0], sg[1], sg[2]);
        sth = sg[3];
    }
    return p;
}

// the relative criterion between successive levels' sums (J, and P for the disjoint class)
template <int CLS>
__device__ __forceinline__ bool fixup_unconverged(const acc5 &nxt, const acc5 &prev, const FixupPair<CLS> &p, d3 nj, d3 spsi, double sth,
                                                  double tol)
{
    const d3 Jc = finalize_j(CLS, mk(nxt.px, nxt.py, nxt.pz) + spsi, nxt.th + sth, nj, p.Si);
    const d3 dJ = kInv4Pi * ((nxt.th - prev.th) * nj + cross(mk(nxt.px - prev.px, nxt.py - prev.py, nxt.pz - prev.pz), nj));
    bool unconv = norm(dJ) > tol * norm(Jc);
    if (CLS == kFar) unconv = unconv || fabs(nxt.pot - prev.pot) > tol * fabs(nxt.pot);
    return unconv;
}

// the kept level's sums plus the singular part, finalised into the pair's outputs
template <int CLS>
__device__ __forceinline__ void fixup_store(const ClassArgs &A, int t, const acc5 &acc, const FixupPair<CLS> &p, d3 nj, d3 spsi, double sth,
                                            int kept, int mode)
{
    const d3 psi = mk(acc.px, acc.py, acc.pz) + spsi;
    const double th = acc.th + sth;
    const d3 J = finalize_j(CLS, psi, th, nj, p.Si);
    double *raw = A.raw4 + 4 * (long long)t;
    raw[0] = psi.x; raw[1] = psi.y; raw[2] = psi.z; raw[3] = th;
    double *Jo = A.J3 + 3 * (long long)t;
    Jo[0] = J.x; Jo[1] = J.y; Jo[2] = J.z;
    if (CLS == kFar) A.P[t] = kInv4Pi * acc.pot;
    if (mode == kAdaptiveRelative) {
        A.stop[t] = kept;
        if (A.level_out) A.level_out[t] = kept;
    }
}

// the level the compat and fixed modes keep for pair t
__device__ __forceinline__ int fixup_kept_level(const ClassArgs &A, int mode, int fixed_level, int t)
{
    if (mode == kFixed) return fixed_level;
    const int L = A.stop[t];
    return ((*A.maxlev - L) & 1) ? (L > 0 ? L - 1 : 0) : L;
}

// Levels deeper than kFixDirect are spread over the GPU: the block that owns a pair stops after
// level kFixDirect, lists the pair (up to ClassArgs::fix_cap pairs; later ones stay in the block)
// with its last sums, and k_fix_spread integrates levels kFixDirect+1..5 in chunks of kFixChunk
// sub-cells, one block per chunk (one sub-cell a thread: 1,024 threads over a level-5 pair);
// k_fix_finish adds the chunks in order and decides.  A needle pair refined to level 5 is
// 17.7 MFLOP of FP64, about 2 ms on one SM, which otherwise sets the length of the whole pass.
// Small blocks keep several resident per SM (chunks of 256 sub-cells measured 0.16 ms slower on
// the 20,480-triangle sphere's batched step).
constexpr int kFixDirect = 3;
constexpr int kFixChunk = 64;
constexpr int kFixSlots = kFixDeepSlots;  // chunks of levels 4 and 5: 4 + 16
static_assert(kFixSlots == 4 + 16 && kFixChunk * 4 == 256, "chunk layout of levels 4 and 5");
__device__ __forceinline__ int fix_slot0(int L) { return L == 4 ? 0 : 4; }
__device__ __forceinline__ int fix_chunks(int L) { return (1 << (2 * L)) / kFixChunk; }

// pair t, by the whole block (red: 5 doubles per warp of shared memory)
template <int CLS>
__device__ void fp64_fixup_item(const ClassArgs &A, const QuadTables &Q, int mode, int fixed_level, double tol, int kmax, int t,
                                double *red)
{
    __shared__ int deep_slot;
    d3 nj, spsi;
    double sth;
    const FixupPair<CLS> p = fixup_pair<CLS>(A, t, nj, spsi, sth);
    acc5 acc;
    int kept;
    if (mode == kAdaptiveRelative) {
        // FP64 refinement with the relative criterion from level 0 (FP32 noise may have kept
        // the mixed pass refining up to the last level); every thread holds the same sums,
        // so the decision is uniform
        acc = fixup_level_sum<CLS>(p, Q, 0, red);
        kept = 0;
        for (int L = 1; L <= kmax; ++L) {
            if (L > kFixDirect && A.fix_deep) {
                if (threadIdx.x == 0) {
                    const int k = atomicAdd(A.cnt + kCntFixDeep, 1);
                    deep_slot = k < A.fix_cap ? k : -1;
                    if (deep_slot >= 0) {
                        A.fix_deep[k] = t;
                        store5(A.fix_base + 5 * (long long)k, acc);
                    }
                }
                __syncthreads();
                const int k = deep_slot;
                __syncthreads();
                if (k >= 0) return;  // k_fix_spread and k_fix_finish take it from here
            }
            const acc5 nxt = fixup_level_sum<CLS>(p, Q, L, red);
            const bool unconv = fixup_unconverged<CLS>(nxt, acc, p, nj, spsi, sth, tol);
            acc = nxt;
            kept = L;
            if (!unconv) break;
        }
    } else {
        kept = fixup_kept_level(A, mode, fixed_level, t);
        if (kept > kFixDirect && A.fix_deep) {
            if (threadIdx.x == 0) {
                const int k = atomicAdd(A.cnt + kCntFixDeep, 1);
                deep_slot = k < A.fix_cap ? k : -1;
                if (deep_slot >= 0) A.fix_deep[k] = t;
            }
            __syncthreads();
            const int k = deep_slot;
            __syncthreads();
            if (k >= 0) return;
        }
        acc = fixup_level_sum<CLS>(p, Q, kept, red);
    }
    if (threadIdx.x == 0) fixup_store<CLS>(A, t, acc, p, nj, spsi, sth, kept, mode);
    __syncthreads();
}

// one chunk of one deep level of listed pair k, by the whole block (kFixChunk threads, one
// sub-cell each); the chunk's sums go to their own slot, so the finish pass adds them in order
template <int CLS>
__device__ void fix_spread_item(const ClassArgs &A, const QuadTables &Q, int mode, int fixed_level, int kmax, int k, int slot, double *red)
{
    const int L = slot < fix_slot0(5) ? 4 : 5;  // slots [fix_slot0(4), fix_slot0(5)) are level 4's chunks
    const int t = A.fix_deep[k];
    const bool wanted = L <= kmax && (mode == kAdaptiveRelative || fixup_kept_level(A, mode, fixed_level, t) == L);
    if (!wanted) return;  // uniform over the block
    d3 nj, spsi;
    double sth;
    const FixupPair<CLS> p = fixup_pair<CLS>(A, t, nj, spsi, sth);
    const int sc = (slot - fix_slot0(L)) * kFixChunk + threadIdx.x;
    const Tri T = subcell(p.Ti, L, sc);
    const double Ssub = p.Si * ldexp(1.0, -2 * L);
    acc5 acc = zero5();
    for (int g = 0; g < Q.npts; ++g) {
        const d3 x = Q.L1[g] * T.a + Q.L2[g] * T.b + Q.L3[g] * T.c;
        d3 psi;
        double th, pot = 0.0;
        if (CLS == kFar) far_integrand(x, p.K, p.F, psi, th, pot);
        else if (CLS == kEdge) edge_integrand(x, p.K, p.E, psi, th);
        else vertex_integrand(x, p.K, p.Vx, psi, th);
        axpy5(acc, Q.w[g], psi, th, pot);
    }
    acc.px *= Ssub; acc.py *= Ssub; acc.pz *= Ssub; acc.th *= Ssub; acc.pot *= Ssub;
    for (int off = 16; off > 0; off >>= 1) {
        acc.px += __shfl_xor_sync(0xffffffffu, acc.px, off);
        acc.py += __shfl_xor_sync(0xffffffffu, acc.py, off);
        acc.pz += __shfl_xor_sync(0xffffffffu, acc.pz, off);
        acc.th += __shfl_xor_sync(0xffffffffu, acc.th, off);
        acc.pot += __shfl_xor_sync(0xffffffffu, acc.pot, off);
    }
    if ((threadIdx.x & 31) == 0) store5(red + 5 * (threadIdx.x >> 5), acc);
    __syncthreads();
    if (threadIdx.x == 0) {
        acc5 tot = zero5();
        for (int w = 0; w < kFixChunk / 32; ++w) {
            const acc5 v = load5(red + 5 * w);
            tot.px += v.px; tot.py += v.py; tot.pz += v.pz; tot.th += v.th; tot.pot += v.pot;
        }
        store5(A.fix_part + 5 * ((long long)k * kFixSlots + slot), tot);
    }
    __syncthreads();
}

template <int CLS>
__device__ __forceinline__ acc5 fix_level_total(const ClassArgs &A, int k, int L)
{
    acc5 tot = zero5();
    for (int c = 0; c < fix_chunks(L); ++c) {
        const acc5 v = load5(A.fix_part + 5 * ((long long)k * kFixSlots + fix_slot0(L) + c));
        tot.px += v.px; tot.py += v.py; tot.pz += v.pz; tot.th += v.th; tot.pot += v.pot;
    }
    return tot;
}

// listed pair k: the deep levels' chunk sums in order, the decision, the outputs (one thread)
template <int CLS>
__device__ void fix_finish_item(const ClassArgs &A, int mode, int fixed_level, double tol, int kmax, int k)
{
    const int t = A.fix_deep[k];
    d3 nj, spsi;
    double sth;
    const FixupPair<CLS> p = fixup_pair<CLS>(A, t, nj, spsi, sth);
    acc5 acc;
    int kept;
    if (mode == kAdaptiveRelative) {
        acc = load5(A.fix_base + 5 * (long long)k);
        kept = kFixDirect;
        for (int L = kFixDirect + 1; L <= kmax; ++L) {
            const acc5 nxt = fix_level_total<CLS>(A, k, L);
            const bool unconv = fixup_unconverged<CLS>(nxt, acc, p, nj, spsi, sth, tol);
            acc = nxt;
            kept = L;
            if (!unconv) break;
        }
    } else {
        kept = fixup_kept_level(A, mode, fixed_level, t);
        acc = fix_level_total<CLS>(A, k, kept);
    }
    fixup_store<CLS>(A, t, acc, p, nj, spsi, sth, kept, mode);
}

template <int CLS>
__global__ void __launch_bounds__(kFixChunk) k_fix_spread(ClassArgs A, QuadTables Q, int mode, int fixed_level, int kmax)
{
    __shared__ double red[5 * (kFixChunk / 32)];
    const long long items = (long long)min(A.cnt[kCntFixDeep], A.fix_cap) * kFixSlots;
    for (long long q = blockIdx.x; q < items; q += gridDim.x) fix_spread_item<CLS>(A, Q, mode, fixed_level, kmax, (int)(q / kFixSlots), (int)(q % kFixSlots), red);
}

template <int CLS>
__global__ void __launch_bounds__(128) k_fix_finish(ClassArgs A, int mode, int fixed_level, double tol, int kmax)
{
    const int count = min(A.cnt[kCntFixDeep], A.fix_cap);
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x)
        fix_finish_item<CLS>(A, mode, fixed_level, tol, kmax, k);
}

template <int CLS>
__global__ void __launch_bounds__(256) k_fp64_fixup(ClassArgs A, QuadTables Q, int mode, int fixed_level, double tol, int kmax,
                                                    const int *__restrict__ list, const int *__restrict__ count)
{
    __shared__ double red[5 * 8];
    const int nbad = *count;
    // one block per gathered pair (grid-stride), so that a few pairs at level 5 spread over the GPU
    for (int q = blockIdx.x; q < nbad; q += gridDim.x) fp64_fixup_item<CLS>(A, Q, mode, fixed_level, tol, kmax, list[q], red);
}

void launch_fp64_fixup(int cls, const ClassArgs &A, const QuadTables &Q, const RunConfig &cfg, int persistent_blocks, cudaStream_t s)
{
    if (A.n <= 0) return;
    // cnt[kCntFixup] counts the gathered pairs (the counters are cleared before every run); the active-list
    // buffer act_a is free after the level chain
    int *list = A.act_a, *count = A.cnt + kCntFixup;
    if (!list) return;  // fixed mode without active lists: nothing to gather into
    if (cls == kFar) k_fixup_collect<kFar><<<persistent_blocks, 256, 0, s>>>(A, list, count);
    else k_fixup_collect<kEdge><<<persistent_blocks, 256, 0, s>>>(A, list, count);
    const int m = cfg.mode, lv = cfg.level, km = cfg.max_level;
    const double tol = cfg.tol;
    const int spread_blocks = persistent_blocks * 4;
    if (cls == kEdge) {
        k_fp64_fixup<kEdge><<<persistent_blocks, 256, 0, s>>>(A, Q, m, lv, tol, km, list, count);
        if (A.fix_deep) {
            k_fix_spread<kEdge><<<spread_blocks, kFixChunk, 0, s>>>(A, Q, m, lv, km);
            k_fix_finish<kEdge><<<8, 128, 0, s>>>(A, m, lv, tol, km);
        }
    } else if (cls == kVertex) {
        k_fp64_fixup<kVertex><<<persistent_blocks, 256, 0, s>>>(A, Q, m, lv, tol, km, list, count);
        if (A.fix_deep) {
            k_fix_spread<kVertex><<<spread_blocks, kFixChunk, 0, s>>>(A, Q, m, lv, km);
            k_fix_finish<kVertex><<<8, 128, 0, s>>>(A, m, lv, tol, km);
        }
    } else if (cls == kFar) {
        k_fp64_fixup<kFar><<<persistent_blocks, 256, 0, s>>>(A, Q, m, lv, tol, km, list, count);
        if (A.fix_deep) {
            k_fix_spread<kFar><<<spread_blocks, kFixChunk, 0, s>>>(A, Q, m, lv, km);
            k_fix_finish<kFar><<<8, 128, 0, s>>>(A, m, lv, tol, km);
        }
    }
}

// ------------------------------------------------------------------ launchers
static int blocks_for_m(long long n, int tpb) { return (int)((n + tpb - 1) / tpb); }

void launch_prepare_panels_f32(int nc, const double *V, const int *C, PanelF *out, cudaStream_t s)
{
    if (nc > 0) k_prepare_panels_f32<<<blocks_for_m(nc, 128), 128, 0, s>>>(nc, V, C, out);
}

// the level passes of one class; finalised on `s` once `join` (when given) has been reached there
template <int CLS>
static void level_chain_mixed(const ClassArgs &A, const QuadTablesF &Qf, const RunConfig &cfg, int persistent_blocks,
                              cudaStream_t s, cudaEvent_t join = nullptr)
{
    const int tpb = 256;
    if (cfg.mode == kFixed) {
        const long long work = (long long)A.n * (cfg.level <= 2 ? (1 << (2 * cfg.level)) : 32);
        k_level_mixed<CLS><<<std::max(1, std::min(blocks_for_m(work, tpb), persistent_blocks * 8)), tpb, 0, s>>>(A, Qf, cfg.level, cfg.mode, cfg.tol,
                                                                                                        cfg.max_level);
        if (join) cudaStreamWaitEvent(s, join, 0);
        launch_finalize(CLS, A, cfg.mode, s);
        return;
    }
    k_level_mixed<CLS><<<blocks_for_m(A.n, tpb), tpb, 0, s>>>(A, Qf, 0, cfg.mode, cfg.tol, cfg.max_level);
    ClassArgs B = A;
    for (int lev = 1; lev <= cfg.max_level; ++lev) {
        if (!level_pass_needed(lev, cfg.mode)) continue;  // level 1 ran inside level 0's pass
        B.act_in = lev == 1 ? nullptr : (lev % 2 ? A.act_b : A.act_a);
        B.cnt_in = lev == 1 ? nullptr : A.cnt + (lev - 1);
        B.act_out = lev % 2 ? A.act_a : A.act_b;
        B.cnt_out = A.cnt + lev;
        k_level_mixed<CLS><<<persistent_blocks, tpb, 0, s>>>(B, Qf, lev, cfg.mode, cfg.tol, cfg.max_level);
    }
    if (join) cudaStreamWaitEvent(s, join, 0);
    launch_finalize(CLS, A, cfg.mode, s);
}

// Adjacent classes: after the closed forms, the potential stages (tier 1, 2, 2b, the adaptive
// rule) run on the side stream while the level chain runs on `s` -- they share nothing until the
// finalisation, which waits for both (the level kernels here are ordinary launches, so the two
// chains' blocks share the SMs).
void launch_class_mixed(int cls, const ClassArgs &A, const QuadTables &Q, const QuadTablesF &Qf, const RunConfig &cfg,
                        int persistent_blocks, cudaStream_t s, const SideStream &side)
{
    if (A.n <= 0) return;
    const int tpb = 128;
    switch (cls) {
    case kSelf:
        launch_self(A, Q, cfg, s);
        break;
    case kEdge:
        k_singular_mixed<kEdge><<<blocks_for_m(A.n, tpb), tpb, 0, s>>>(A, Qf);
        if (A.pot_off) {
            cudaMemsetAsync(A.padj, 0xff, sizeof(double) * (size_t)A.n, s);  // J only: P reads NaN
            level_chain_mixed<kEdge>(A, Qf, cfg, persistent_blocks, s);
        } else {
            cudaEventRecord(side.fork, s);
            cudaStreamWaitEvent(side.stream, side.fork, 0);
            k_tier1_mixed<kEdge><<<blocks_for_m((long long)kTier1Lanes * A.n, tpb), tpb, 0, side.stream>>>(A, Qf);
            if (A.hard_list) {
                k_pot_tier2_mixed<kEdge><<<resident_grid((const void *)k_pot_tier2_mixed<kEdge>, tpb, 0), tpb, 0, side.stream>>>(A, Qf, Q);
                launch_pot_tiers_hard_df(kEdge, A, Q, cfg, persistent_blocks, side.stream);
            }
            cudaEventRecord(side.join, side.stream);
            level_chain_mixed<kEdge>(A, Qf, cfg, persistent_blocks, s, side.join);
        }
        launch_fp64_fixup(kEdge, A, Q, cfg, persistent_blocks, s);
        break;
    case kVertex:
        k_singular_mixed<kVertex><<<blocks_for_m(A.n, tpb), tpb, 0, s>>>(A, Qf);
        if (A.pot_off) {
            cudaMemsetAsync(A.padj, 0xff, sizeof(double) * (size_t)A.n, s);  // J only: P reads NaN
            level_chain_mixed<kVertex>(A, Qf, cfg, persistent_blocks, s);
        } else {
            cudaEventRecord(side.fork, s);
            cudaStreamWaitEvent(side.stream, side.fork, 0);
            k_tier1_mixed<kVertex><<<blocks_for_m((long long)kTier1Lanes * A.n, tpb), tpb, 0, side.stream>>>(A, Qf);
            if (A.hard_list) {
                k_pot_tier2_mixed<kVertex><<<resident_grid((const void *)k_pot_tier2_mixed<kVertex>, tpb, 0), tpb, 0, side.stream>>>(A, Qf, Q);
                launch_pot_tiers_hard_df(kVertex, A, Q, cfg, persistent_blocks, side.stream);
            }
            cudaEventRecord(side.join, side.stream);
            level_chain_mixed<kVertex>(A, Qf, cfg, persistent_blocks, s, side.join);
        }
        launch_fp64_fixup(kVertex, A, Q, cfg, persistent_blocks, s);
        break;
    default:
        level_chain_mixed<kFar>(A, Qf, cfg, persistent_blocks, s);
        launch_fp64_fixup(kFar, A, Q, cfg, persistent_blocks, s);
        break;
    }
}


// ------------------------------------------------------------------ batched persistent kernel
// One cooperative launch runs every refinement level of every (mesh, class) segment of a batch:
// for each level, the whole grid sweeps the segments' active lists (grid-stride, lane groups of
// min(4^L, G_cap) lanes per pair), then a grid-wide barrier; after the last level it finalises
// every pair.  Converged pairs drop out of the lists, so the uneven work left by adaptive
// refinement is spread over the whole GPU at every level, across meshes and classes.
// MINB = 1: registers unconstrained (fewer resident warps); MINB = 2: at most 128 registers per
// thread so that two 256-thread blocks stay resident per SM (some spilling); MINB = 3: at most 85
// registers, three blocks a SM (more spilling; the level kernels are latency-bound at 8-16 warps
// a SM).  The autotuner picks.
template <int MINB, int CLS>
__global__ void __launch_bounds__(256, MINB) k_batch_levels(const BatchSeg *__restrict__ segs, int nseg, QuadTablesF Qf, int mode,
                                                      int level_fixed, double tol, int kmax, int G_cap)
{
    namespace cg = cooperative_groups;
    cg::grid_group grid = cg::this_grid();
    const long long first = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const int lo = mode == kFixed ? level_fixed : 0, hi = mode == kFixed ? level_fixed : kmax;
    for (int level = lo; level <= hi; ++level) {
        if (!level_pass_needed(level, mode)) continue;  // level 1 ran inside level 0's pass (uniform: mode is)
        for (int sgi = 0; sgi < nseg; ++sgi) {
            if (segs[sgi].cls != CLS) continue;
            const ClassArgs &A = segs[sgi].A;  // read in place, no per-thread copy
            if (A.n <= 0) continue;
            level_items_mixed<CLS>(A, level_lists(A, level, mode), Qf, level, mode, tol, kmax, first, stride, G_cap);
        }
        grid.sync();
    }
    for (int sgi = 0; sgi < nseg; ++sgi)
        if (segs[sgi].cls == CLS) finalize_all(CLS, segs[sgi].A, mode, first, stride);
}

namespace {

const void *batch_levels_fn(int variant, int cls)
{
    if (variant == 0) return cls == kFar ? (const void *)k_batch_levels<1, kFar> : cls == kEdge ? (const void *)k_batch_levels<1, kEdge>
                                                                                                 : (const void *)k_batch_levels<1, kVertex>;
    if (variant == 1) return cls == kFar ? (const void *)k_batch_levels<2, kFar> : cls == kEdge ? (const void *)k_batch_levels<2, kEdge>
                                                                                                 : (const void *)k_batch_levels<2, kVertex>;
    return cls == kFar ? (const void *)k_batch_levels<3, kFar> : cls == kEdge ? (const void *)k_batch_levels<3, kEdge>
                                                                              : (const void *)k_batch_levels<3, kVertex>;
}

int batch_levels_occupancy(int threads, int variant, int cls)
{
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, batch_levels_fn(variant, cls), threads, 0) != cudaSuccess) return 0;
    return nb;
}

} // namespace

// the register variant of class cls in a batch's variant code (one base-3 digit per class)
static int class_variant(int code, int cls) { return (code / (cls == kVertex ? 1 : (cls == kEdge ? 3 : 9))) % 3; }

int batch_max_blocks_per_sm(int threads, int variant)
{
    int nb = 0;
    for (int cls : {kVertex, kEdge, kFar}) nb = std::max(nb, batch_levels_occupancy(threads, class_variant(variant, cls), cls));
    return nb;
}

// one cooperative launch per pair class present, each over every segment of that class: a kernel
// holding one class's integrand keeps that class's register footprint (the far-field one fits
// 128 registers without spills; a kernel with all three classes spilled there)
cudaError_t launch_batch_levels(const BatchSeg *segs, int nseg, const bool present[3], const QuadTablesF &Qf, const RunConfig &cfg,
                                int sms, int bps, int threads, int G_cap, int variant, cudaStream_t s)
{
    int mode = cfg.mode, level = cfg.level, kmax = cfg.max_level;
    double tol = cfg.tol;
    QuadTablesF q = Qf;
    void *args[] = {(void *)&segs, (void *)&nseg, (void *)&q, (void *)&mode, (void *)&level, (void *)&tol, (void *)&kmax, (void *)&G_cap};
    for (int cls : {kVertex, kEdge, kFar}) {
        if (!present[cls]) continue;
        const int v = class_variant(variant, cls);
        const int maxb = batch_levels_occupancy(threads, v, cls);
        if (maxb <= 0) return cudaErrorInvalidConfiguration;
        const int blocks = std::max(1, sms) * std::max(1, std::min(bps > 0 ? bps : maxb, maxb));
        const cudaError_t e = cudaLaunchCooperativeKernel(batch_levels_fn(v, cls), dim3(blocks), dim3(threads), args, 0, s);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// ------------------------------------------------------------------ batched stages
// The stages that precede and follow the level sweep, each as one launch over every segment of
// the batch (flattened walks of i2_batch.cuh): counter reset, tier 1 with the singular parts,
// tiers 2 / 2b, the adaptive potential (i2_kernels_fp64.cu), self pairs, and the FP64 fix-up.
// the closed forms of every adjacent pair; before them, thread s clears segment s's counters (the
// stages that count into them run in later launches; the grid has at least one thread a segment)
__global__ void __launch_bounds__(128) k_batch_singular(const BatchSeg *__restrict__ segs, int nseg, QuadTablesF Qf)
{
    extern __shared__ long long prefix[];
    const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid < nseg && segs[gid].A.n > 0) {
        for (int k = 0; k < 16; ++k) segs[gid].A.cnt[k] = 0;
        *segs[gid].A.maxlev = 0;
    }
    const long long total = seg_prefix(segs, nseg, prefix, [](const BatchSeg &S) -> long long { return seg_adjacent(S) ? S.A.n : 0; });
    for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += (long long)gridDim.x * blockDim.x) {
        const int sg = seg_find(prefix, nseg, g);
        const BatchSeg &S = segs[sg];
        if (S.cls == kEdge) singular_mixed_item<kEdge>(S.A, Qf, g - prefix[sg]);
        else singular_mixed_item<kVertex>(S.A, Qf, g - prefix[sg]);
    }
}

// tier 1 of the adjacent pairs' potential (eight lanes a pair) and the self pairs (five to a warp,
// six lanes each) in one launch: global warps [0, w1) take the tier-1 items, warps [w1, w1 + w2)
// the self pairs, so every branch below is uniform over a warp.  prefix holds two prefix-sum
// arrays (tier-1 items, self pairs) of nseg + 1 entries each.
// (at most 128 registers: four blocks per SM, without spills)
__global__ void __launch_bounds__(128, 4) k_batch_tier1_self(const BatchSeg *__restrict__ segs, int nseg, QuadTablesF Qf, QuadTables Q,
                                                          int self_sign)
{
    extern __shared__ long long prefix[];
    long long *p1 = prefix, *ps = prefix + nseg + 1;
    const long long t1 = seg_prefix(segs, nseg, p1, [](const BatchSeg &S) -> long long {
        return seg_adjacent(S) ? (long long)kTier1Lanes * S.A.n : 0;
    });
    const long long ts = seg_prefix(segs, nseg, ps, [](const BatchSeg &S) -> long long { return S.cls == kSelf && S.A.n > 0 ? S.A.n : 0; });
    const long long w1 = (t1 + 31) >> 5, w2 = (ts + kSelfPairsPerWarp - 1) / kSelfPairsPerWarp;
    const int lane = threadIdx.x & 31;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < w1 + w2; w += nwarps) {
        if (w < w1) {
            // a pair's eight items are one aligned group of eight lanes (every count is a multiple of 8)
            const long long g = w * 32 + lane;
            if (g < t1) {
                const int sg = seg_find(p1, nseg, g);
                const BatchSeg &S = segs[sg];
                const long long loc = g - p1[sg];
                if (S.cls == kEdge) tier1_mixed_item<kEdge>(S.A, Qf, loc / kTier1Lanes, (int)(loc % kTier1Lanes));
                else tier1_mixed_item<kVertex>(S.A, Qf, loc / kTier1Lanes, (int)(loc % kTier1Lanes));
            }
        } else {
            const int k = lane / 6;
            const long long g = (w - w1) * kSelfPairsPerWarp + k;
            const bool valid = k < kSelfPairsPerWarp && g < ts;
            int sg = 0;
            long long t = 0;
            double part = 0.0;
            if (valid) {
                sg = seg_find(ps, nseg, g);
                t = g - ps[sg];
                part = self_piece_of(segs[sg].A, Q, t, lane % 6);
            }
            const double sum = self_gather6(part);
            if (valid && lane % 6 == 0) self_store(segs[sg].A, self_sign, t, sum);
        }
    }
}

__global__ void __launch_bounds__(128) k_batch_tier2(const BatchSeg *__restrict__ segs, int nseg, QuadTablesF Qf, QuadTables Q)
{
    extern __shared__ long long prefix[];
    const long long total = seg_prefix(segs, nseg, prefix, [](const BatchSeg &S) -> long long {
        return seg_adjacent(S) && S.A.hard_list ? *S.A.tier2_cnt : 0;
    });
    const int lane = threadIdx.x & 31;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long g = warp_item_index(); g < total; g += nwarps) {
        const int sg = seg_find(prefix, nseg, g);
        const BatchSeg &S = segs[sg];
        if (S.cls == kEdge) tier2_mixed_item<kEdge>(S.A, Qf, Q, (int)(g - prefix[sg]), lane);
        else tier2_mixed_item<kVertex>(S.A, Qf, Q, (int)(g - prefix[sg]), lane);
    }
}

// segments whose pairs the fix-up gathers (into act_a, counted in cnt[kCntFixup])
__device__ __forceinline__ bool seg_fixup(const BatchSeg &S) { return S.A.n > 0 && S.cls != kSelf && S.A.act_a; }

__global__ void __launch_bounds__(256) k_batch_fixup_collect(const BatchSeg *__restrict__ segs, int nseg)
{
    extern __shared__ long long prefix[];
    const long long total = seg_prefix(segs, nseg, prefix, [](const BatchSeg &S) -> long long { return seg_fixup(S) ? S.A.n : 0; });
    for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += (long long)gridDim.x * blockDim.x) {
        const int sg = seg_find(prefix, nseg, g);
        const ClassArgs &A = segs[sg].A;
        if (segs[sg].cls == kFar) fixup_collect_item<kFar>(A, A.act_a, A.cnt + kCntFixup, g - prefix[sg]);
        else fixup_collect_item<kEdge>(A, A.act_a, A.cnt + kCntFixup, g - prefix[sg]);
    }
}

__global__ void __launch_bounds__(256) k_batch_fp64_fixup(const BatchSeg *__restrict__ segs, int nseg, QuadTables Q, int mode,
                                                          int fixed_level, double tol, int kmax)
{
    extern __shared__ long long prefix[];
    __shared__ double red[5 * 8];
    const long long total = seg_prefix(segs, nseg, prefix, [](const BatchSeg &S) -> long long { return seg_fixup(S) ? S.A.cnt[kCntFixup] : 0; });
    // one block per gathered pair
    for (long long g = blockIdx.x; g < total; g += gridDim.x) {
        const int sg = seg_find(prefix, nseg, g);
        const BatchSeg &S = segs[sg];
        const int t = S.A.act_a[g - prefix[sg]];
        if (S.cls == kFar) fp64_fixup_item<kFar>(S.A, Q, mode, fixed_level, tol, kmax, t, red);
        else if (S.cls == kEdge) fp64_fixup_item<kEdge>(S.A, Q, mode, fixed_level, tol, kmax, t, red);
        else fp64_fixup_item<kVertex>(S.A, Q, mode, fixed_level, tol, kmax, t, red);
    }
}

__global__ void __launch_bounds__(kFixChunk) k_batch_fix_spread(const BatchSeg *__restrict__ segs, int nseg, QuadTables Q, int mode,
                                                                 int fixed_level, int kmax)
{
    extern __shared__ long long prefix[];
    __shared__ double red[5 * (kFixChunk / 32)];
    const long long total = seg_prefix(segs, nseg, prefix, [](const BatchSeg &S) -> long long {
        return seg_fixup(S) && S.A.fix_deep ? (long long)min(S.A.cnt[kCntFixDeep], S.A.fix_cap) * kFixSlots : 0;
    });
    for (long long g = blockIdx.x; g < total; g += gridDim.x) {
        const int sg = seg_find(prefix, nseg, g);
        const BatchSeg &S = segs[sg];
        const long long q = g - prefix[sg];
        const int k = (int)(q / kFixSlots), slot = (int)(q % kFixSlots);
        if (S.cls == kFar) fix_spread_item<kFar>(S.A, Q, mode, fixed_level, kmax, k, slot, red);
        else if (S.cls == kEdge) fix_spread_item<kEdge>(S.A, Q, mode, fixed_level, kmax, k, slot, red);
        else fix_spread_item<kVertex>(S.A, Q, mode, fixed_level, kmax, k, slot, red);
    }
}

__global__ void __launch_bounds__(128) k_batch_fix_finish(const BatchSeg *__restrict__ segs, int nseg, int mode, int fixed_level,
                                                          double tol, int kmax)
{
    extern __shared__ long long prefix[];
    const long long total = seg_prefix(segs, nseg, prefix, [](const BatchSeg &S) -> long long {
        return seg_fixup(S) && S.A.fix_deep ? min(S.A.cnt[kCntFixDeep], S.A.fix_cap) : 0;
    });
    for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += (long long)gridDim.x * blockDim.x) {
        const int sg = seg_find(prefix, nseg, g);
        const BatchSeg &S = segs[sg];
        const int k = (int)(g - prefix[sg]);
        if (S.cls == kFar) fix_finish_item<kFar>(S.A, mode, fixed_level, tol, kmax, k);
        else if (S.cls == kEdge) fix_finish_item<kEdge>(S.A, mode, fixed_level, tol, kmax, k);
        else fix_finish_item<kVertex>(S.A, mode, fixed_level, tol, kmax, k);
    }
}

// the adjacent pairs' P from the potential rules (padj), written after them: the batched step runs
// the potential stages beside the needle fix-up, after the level sweep has finalised J
__global__ void __launch_bounds__(256) k_batch_adjacent_potential(const BatchSeg *__restrict__ segs, int nseg)
{
    extern __shared__ long long prefix[];
    const long long total = seg_prefix(segs, nseg, prefix, [](const BatchSeg &S) -> long long { return seg_adjacent(S) ? S.A.n : 0; });
    for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += (long long)gridDim.x * blockDim.x) {
        const int sg = seg_find(prefix, nseg, g);
        const ClassArgs &A = segs[sg].A;
        const long long t = g - prefix[sg];
        A.P[t] = A.padj[t];
    }
}

static size_t seg_smem(int nseg) { return (size_t)(nseg + 1) * sizeof(long long); }

void launch_batch_singular(const BatchSeg *segs, int nseg, const BatchTotals &tot, const QuadTablesF &Qf, cudaStream_t s)
{
    const int tpb = 128;
    // closed forms, with the counter reset in front (always launched: the reset is needed by
    // every segment)
    for (int c0 = 0; c0 < nseg; c0 += kBatchSegChunk) {
        const int nc = std::min(kBatchSegChunk, nseg - c0);
        const int blocks = std::max(blocks_for_m(nc, tpb), std::min(blocks_for_m(tot.adjacent_pairs, tpb), 1 << 16));
        k_batch_singular<<<std::max(1, blocks), tpb, seg_smem(nc), s>>>(segs + c0, nc, Qf);
    }
}

void launch_batch_potential(const BatchSeg *segs, int nseg, const BatchTotals &tot, const QuadTables &Q, const QuadTablesF &Qf,
                            const RunConfig &cfg, int persistent_blocks, cudaStream_t s)
{
    const int tpb = 128;
    // tier 1 with the self pairs, tiers 2 / 2b and the adaptive rule, then the adjacent pairs' P
    const long long warps = (kTier1Lanes * tot.adjacent_pairs + 31) / 32 + (tot.self_pairs + kSelfPairsPerWarp - 1) / kSelfPairsPerWarp;
    if (warps > 0) {
        const int blocks = (int)std::max(1LL, std::min((warps * 32 + tpb - 1) / tpb, 1LL << 16));
        for (int c0 = 0; c0 < nseg; c0 += kBatchSegChunk) {
            const int nc = std::min(kBatchSegChunk, nseg - c0);
            k_batch_tier1_self<<<blocks, tpb, 2 * seg_smem(nc), s>>>(segs + c0, nc, Qf, Q, cfg.self_sign);
        }
    }
    if (tot.adjacent_pairs > 0 && tot.hard_lists) {
        for (int c0 = 0; c0 < nseg; c0 += kBatchSegChunk) {
            const int nc = std::min(kBatchSegChunk, nseg - c0);
            k_batch_tier2<<<resident_grid((const void *)k_batch_tier2, tpb, seg_smem(nc)), tpb, seg_smem(nc), s>>>(segs + c0, nc, Qf, Q);
        }
        launch_batch_pot_df(segs, nseg, Q, cfg.hard_tol, persistent_blocks, s);
    }
    if (tot.adjacent_pairs > 0) {
        const int blocks = std::max(1, std::min(blocks_for_m(tot.adjacent_pairs, 256), 1 << 16));
        for (int c0 = 0; c0 < nseg; c0 += kBatchSegChunk) {
            const int nc = std::min(kBatchSegChunk, nseg - c0);
            k_batch_adjacent_potential<<<blocks, 256, seg_smem(nc), s>>>(segs + c0, nc);
        }
    }
}

void launch_batch_fixup(const BatchSeg *segs, int nseg, const BatchTotals &tot, const QuadTables &Q, const RunConfig &cfg,
                        int persistent_blocks, cudaStream_t s)
{
    if (tot.fixup_pairs <= 0) return;
    const int blocks = std::max(1, std::min(blocks_for_m(tot.fixup_pairs, 256), 1 << 16));
    for (int c0 = 0; c0 < nseg; c0 += kBatchSegChunk) {
        const int nc = std::min(kBatchSegChunk, nseg - c0);
        k_batch_fixup_collect<<<blocks, 256, seg_smem(nc), s>>>(segs + c0, nc);
        k_batch_fp64_fixup<<<persistent_blocks, 256, seg_smem(nc), s>>>(segs + c0, nc, Q, cfg.mode, cfg.level, cfg.tol, cfg.max_level);
        k_batch_fix_spread<<<persistent_blocks * 4, kFixChunk, seg_smem(nc), s>>>(segs + c0, nc, Q, cfg.mode, cfg.level, cfg.max_level);
        k_batch_fix_finish<<<64, 128, seg_smem(nc), s>>>(segs + c0, nc, cfg.mode, cfg.level, cfg.tol, cfg.max_level);
    }
}

} // namespace i2
