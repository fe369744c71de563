// i2_device_f32.cuh -- FP32 geometry and integrands of the mixed-precision form.
//
// Each cell gets a 160-byte FP32 panel record (10 x float4) written once from the FP64 mesh:
//   [0] A_hi.xyz, S     [1] A_lo.xyz, 2S    [2] B_hi.xyz, |C-B|   [3] B_lo.xyz, |A-C|
//   [4] C_hi.xyz, |B-A| [5] C_lo.xyz, 1/sqrt(S)   [6] n.xyz, -
//   [7..9] ta, tb, tc (unit edges C-B, A-C, B-A), each with 1/|edge|
// Vertices are stored as unevaluated float sums hi + lo (double-float), so the offset of a
// point of K_i from a vertex of K_j is formed in FP32 as (a_hi - b_hi) + (a_lo - b_lo) without
// FP64 work and without the cancellation of subtracting two rounded absolute coordinates.
// Edge log terms use a log1p form whose argument is a ratio of sums of positive terms only
// (q_P - q_Q equals the edge length exactly), so no term of the FP32 evaluation cancels.
#pragma once

#include "i2_device.cuh"

namespace i2 {

struct f3 {
    float x, y, z;
};
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return f3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return f3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ f3 operator*(float s, f3 a) { return f3{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ float dotf(f3 a, f3 b) { return fmaf(a.x, b.x, fmaf(a.y, b.y, a.z * b.z)); }
__device__ __forceinline__ f3 crossf(f3 a, f3 b) { return f3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
__device__ __forceinline__ float normf(f3 a) { return sqrtf(dotf(a, a)); }
__device__ __forceinline__ f3 xyzf(float4 v) { return f3{v.x, v.y, v.z}; }
__device__ __forceinline__ f3 to_f3(d3 a) { return f3{(float)a.x, (float)a.y, (float)a.z}; }

struct alignas(16) PanelF {
    float4 v[10];
};
static_assert(sizeof(PanelF) == 160, "FP32 panel record is 160 bytes");

// FP32 view of K_j: offsets are measured from vertex A; B - A and C - A as FP32 vectors
struct PanelJf {
    f3 AB, AC, n, ta, tb, tc;
    float S, lenA, lenB, lenC;
    float rA, rB, rC;  // 1 / lenA, 1 / lenB, 1 / lenC, rounded from FP64
};

__device__ __forceinline__ f3 df_sub(float4 ahi, float4 alo, float4 bhi, float4 blo)
{
    return f3{(ahi.x - bhi.x) + (alo.x - blo.x), (ahi.y - bhi.y) + (alo.y - blo.y), (ahi.z - bhi.z) + (alo.z - blo.z)};
}

// offsets of the three vertices of panel p (cell pi) from vertex k (0..2) of panel q
__device__ __forceinline__ void df_offsets(const PanelF *__restrict__ P, int pi, int qj, int k, f3 &a, f3 &b, f3 &c)
{
    const float4 *u = P[pi].v, *w = P[qj].v;
    const float4 rh = w[2 * k], rl = w[2 * k + 1];
    a = df_sub(u[0], u[1], rh, rl);
    b = df_sub(u[2], u[3], rh, rl);
    c = df_sub(u[4], u[5], rh, rl);
}

// offset of vertex k of panel q from vertex m of panel q
__device__ __forceinline__ f3 df_edge(const PanelF *__restrict__ P, int q, int k, int m)
{
    const float4 *w = P[q].v;
    return df_sub(w[2 * k], w[2 * k + 1], w[2 * m], w[2 * m + 1]);
}

// a - b for a = ah + al, b = bh + bl as an unevaluated sum hi + lo: Knuth's TwoSum gives the
// exact rounding error of ah - bh, the low parts are added to it, and Fast2Sum renormalises
__device__ __forceinline__ void df_diff(float ah, float al, float bh, float bl, float &hi, float &lo)
{
    const float s = ah - bh;
    const float bb = s - ah;
    const float e = (ah - (s - bb)) + (-bh - bb);
    const float t = e + (al - bl);
    hi = s + t;
    lo = t - (hi - s);
}

// vertex k minus vertex m of panel q in double-float
__device__ __forceinline__ void df_edge_pair(const PanelF *__restrict__ P, int q, int k, int m, f3 &hi, f3 &lo)
{
    const float4 *w = P[q].v;
    const float4 kh = w[2 * k], kl = w[2 * k + 1], mh = w[2 * m], ml = w[2 * m + 1];
    df_diff(kh.x, kl.x, mh.x, ml.x, hi.x, lo.x);
    df_diff(kh.y, kl.y, mh.y, ml.y, hi.y, lo.y);
    df_diff(kh.z, kl.z, mh.z, ml.z, hi.z, lo.z);
}

__device__ __forceinline__ PanelJf load_panel_f(const PanelF *__restrict__ P, int c)
{
    const float4 *w = P[c].v;
    PanelJf r;
    r.AB = df_sub(w[2], w[3], w[0], w[1]);
    r.AC = df_sub(w[4], w[5], w[0], w[1]);
    r.S = w[0].w;
    r.lenA = w[2].w;
    r.lenB = w[3].w;
    r.lenC = w[4].w;
    r.n = xyzf(w[6]);
    r.ta = xyzf(w[7]);
    r.tb = xyzf(w[8]);
    r.tc = xyzf(w[9]);
    r.rA = w[7].w;
    r.rB = w[8].w;
    r.rC = w[9].w;
    return r;
}

// n / d from an approximate reciprocal and one correction of the quotient (Markstein's method,
// IBM J. Res. Dev. 34(1), 1990): q0 = n r, e = n - q0 d exactly (one FMA), q = q0 + e r.  Within an
// ulp of the correctly rounded quotient for the normal operands here (|d| < 2^126), at about a
// third of the cost of an IEEE division; an infinite first quotient (d = 0) is returned as it is.
__device__ __forceinline__ float div_q(float n, float d)
{
    const float r = __fdividef(1.0f, d);
    const float q0 = n * r;
    const float q = fmaf(fmaf(-q0, d, n), r, q0);
    return isfinite(q0) ? q : q0;
}

// ln((l_P + q_P) / (l_Q + q_Q)) for the edge P -> Q of length L, q = (x - P).tau, from sums
// and products of positive terms only (q_P - q_Q = L):
//   x beyond Q (q_Q >= 0) or before P (q_P <= 0): log1p(delta) with a positive delta;
//   x projecting inside the edge: the ratio is (l_P + q_P)(l_Q - q_Q) / h^2, h the distance
//   to the edge line, with h^2 = |o x tau|^2 taken from the NEARER endpoint (o_P x tau =
//   o_Q x tau; from the far endpoint the cross product of a long offset cancels down to the
//   short distance).  Close to the line (ratio > 2) log1p(ratio - 1) with ratio - 1 formed as
//   (product - h^2) / h^2 (no cancellation there); farther out log1p of (ratio - 1) from the
//   positive terms keeps small logs accurate.  A point on the line itself (h = 0, where the
//   caller's factor t_e is 0 too) gets a large finite value.
// Every case is log1p(n / d): the cases only select n and d, so the lanes of a warp, which hold
// points in different cases, share one division and one log1pf instead of running each case's.
__device__ __forceinline__ float edge_log_f32(float lP, float qP, f3 oP, float lQ, float qQ, f3 oQ, f3 tau, float L)
{
    const float s = lP + lQ;
    const f3 r = crossf(lP < lQ ? oP : oQ, tau);
    const float h2 = dotf(r, r);
    const float num = (lP + qP) * (lQ - qQ);
    float n, d;
    if (qQ >= 0.0f) {
        n = L * (s + qP + qQ);
        d = s * (lQ + qQ);
    } else if (qP <= 0.0f) {
        n = L * (s - qP - qQ);
        d = s * (lP - qP);
    } else if (num > 2.0f * h2) {
        n = num - h2;
        d = h2;
    } else {
        n = (lP + qP) * L * (s - qP - qQ);
        d = s * h2;
    }
    return log1pf(fminf(div_q(n, d), 3.0e38f));
}

// lambda = ln((l_P + q_P) / (l_Q + q_Q)) / L for the edge P -> Q with rho = 1 / L rounded once
// from FP64: edge_log_f32's cases with the factor L of their numerators moved into the
// denominators as rho, and the result multiplied by rho.  As with L in both places before, the
// rounding of rho enters x = n / d and the final factor alike and cancels to first order (for
// small x, lambda ~ n / (d / rho) rho); it saves the division by L.
__device__ __forceinline__ float edge_lambda_f32(float lP, float qP, f3 oP, float lQ, float qQ, f3 oQ, f3 tau, float rho)
{
    const float s = lP + lQ;
    const f3 r = crossf(lP < lQ ? oP : oQ, tau);
    const float h2 = dotf(r, r);
    const float num = (lP + qP) * (lQ - qQ);
    float n, d;
    if (qQ >= 0.0f) {
        n = s + qP + qQ;
        d = rho * s * (lQ + qQ);
    } else if (qP <= 0.0f) {
        n = s - qP - qQ;
        d = rho * s * (lP - qP);
    } else if (num > 2.0f * h2) {
        n = num - h2;
        d = h2;
    } else {
        n = (lP + qP) * (s - qP - qQ);
        d = rho * s * h2;
    }
    return log1pf(fminf(div_q(n, d), 3.0e38f)) * rho;
}

struct FarCtxF {
    f3 ma, mb, mc;  // unit in-plane edge normals tau_e x n (potential by distances to the edge lines)
    f3 ea, eb;      // edge vectors C - B, A - C (the far-field form below)
};

// theta/psi (a1) and the potential integrand from the offsets to K_j's vertices
__device__ __forceinline__ void far_integrand_f(f3 oa, f3 ob, f3 oc, const PanelJf &K, const FarCtxF &F, f3 &psi, float &th,
                                                float &pot)
{
    const float la = normf(oa), lb = normf(ob), lc = normf(oc);
    const float Lc = edge_log_f32(la, dotf(oa, K.tc), oa, lb, dotf(ob, K.tc), ob, K.tc, K.lenC);  // A -> B
    const float La = edge_log_f32(lb, dotf(ob, K.ta), ob, lc, dotf(oc, K.ta), oc, K.ta, K.lenA);  // B -> C
    const float Lb = edge_log_f32(lc, dotf(oc, K.tb), oc, la, dotf(oa, K.tb), oa, K.tb, K.lenB);  // C -> A
    psi = Lc * K.tc + La * K.ta + Lb * K.tb;
    const float d = dotf(K.n, oa);
    const float den = la * lb * lc + dotf(oa, ob) * lc + dotf(ob, oc) * la + dotf(oc, oa) * lb;
    th = 2.0f * atan2f(2.0f * K.S * d, den);
    const float ta_ = -dotf(F.ma, ob), tb_ = -dotf(F.mb, oc), tc_ = -dotf(F.mc, oa);
    pot = ta_ * La + tb_ * Lb + tc_ * Lc - d * th;
}

// The same three quantities for a point away from K_j (the disjoint class), in a form whose FP32
// errors do not add up into a bias.  With lambda_e = L_e / |e| (edge_lambda_f32: the same rounded
// 1/|e| scales L_e's argument and multiplies the log, so that rounding cancels to first order)
// and e_a + e_b + e_c = 0:
//   Psi = sum_e lambda_e e_e = (lambda_a - lambda_c) e_a + (lambda_b - lambda_c) e_b,
// where the rounding of the edge vectors only multiplies differences of lambda (sum_e tau_e L_e
// with rounded unit tangents cancels down to Psi and keeps their rounding at full size), and
//   sum_e t_e L_e = -(Psi x n).o_A + 2 S lambda_a
// (t_e = distance of the point's projection to edge e's line, e_a x n . (B - A) = 2S,
// e_b x n . (C - A) = 0), whose terms are of the size of the potential instead of cancelling.
// Near K_j's edges lambda grows like a log and the potential's second form would rebuild
// t_e L_e -> 0 from large terms, so the adjacent classes keep far_integrand_f.
__device__ __forceinline__ void far_field_integrand_f(f3 oa, f3 ob, f3 oc, const PanelJf &K, const FarCtxF &F, f3 &psi, float &th,
                                                      float &pot)
{
    const float la = normf(oa), lb = normf(ob), lc = normf(oc);
    const float lam_c = edge_lambda_f32(la, dotf(oa, K.tc), oa, lb, dotf(ob, K.tc), ob, K.tc, K.rC);  // A -> B
    const float lam_a = edge_lambda_f32(lb, dotf(ob, K.ta), ob, lc, dotf(oc, K.ta), oc, K.ta, K.rA);  // B -> C
    const float lam_b = edge_lambda_f32(lc, dotf(oc, K.tb), oc, la, dotf(oa, K.tb), oa, K.tb, K.rB);  // C -> A
    psi = (lam_a - lam_c) * F.ea + (lam_b - lam_c) * F.eb;
    const float d = dotf(K.n, oa);
    const float den = la * lb * lc + dotf(oa, ob) * lc + dotf(ob, oc) * la + dotf(oc, oa) * lb;
    th = 2.0f * atan2f(2.0f * K.S * d, den);
    pot = 2.0f * K.S * lam_a - dotf(crossf(psi, K.n), oa) - d * th;
}

// Kahan-compensated FP32 accumulator of (Psi, Theta, potential)
struct kahan5 {
    float s[5], c[5];
};
__device__ __forceinline__ void kahan_zero(kahan5 &k)
{
#pragma unroll
    for (int i = 0; i < 5; ++i) k.s[i] = k.c[i] = 0.0f;
}
__device__ __forceinline__ void kahan_add(kahan5 &k, int i, float v)
{
    const float y = v - k.c[i];
    const float t = k.s[i] + y;
    k.c[i] = (t - k.s[i]) - y;
    k.s[i] = t;
}

// (s - c) += (s2 - c2) for two Kahan pairs: the rounding error of s + s2 from Knuth's TwoSum
// moves into the compensation, so a sum across lanes keeps about 2^-48 of relative precision with
// no FP64 work on every lane.  TwoSum's error is the exact rounding error, whichever lane forms
// it, so the two lanes of an xor butterfly end with identical pairs.
__device__ __forceinline__ void kahan_pair_add(float &s, float &c, float s2, float c2)
{
    const float t = s + s2;
    const float z = t - s;
    const float err = (s - (t - z)) + (s2 - z);  // (s + s2) - t, exactly
    c = (c + c2) - err;
    s = t;
}

struct QuadTablesF {
    float L1[kMaxGauss], L2[kMaxGauss], L3[kMaxGauss], w[kMaxGauss];
    int npts;
    double pow2p;  // 2^order of the rule (the compat mode's Runge criterion)
    float du_u[kMaxDuffy], du_w[kMaxDuffy], dv_v[kMaxDuffy], dv_w[kMaxDuffy];
    int nu, nv;
    float lo_u[kMaxDuffy], lo_uw[kMaxDuffy], lo_v[kMaxDuffy], lo_vw[kMaxDuffy];
    int lo_nu, lo_nv;
    float hi_u[kMaxDuffy], hi_uw[kMaxDuffy], hi_v[kMaxDuffy], hi_vw[kMaxDuffy];
    int hi_nu, hi_nv;
    float top_u[kDuffyTop], top_uw[kDuffyTop], top_v[kDuffyTop], top_vw[kDuffyTop];
    int top_nu, top_nv;
};

} // namespace i2
