// i2_device.cuh -- device-side geometry and integrands of the pair-integral path.
//
// Layout: every cell of a mesh has one 256-byte "panel" record (8 x 32-byte double4_32a,
// loaded with 256-bit vector loads), written once by k_prepare_panels:
//   [0] A.xyz, S          [1] B.xyz, 2S         [2] C.xyz, 0          [3] n.xyz, 0
//   [4] ta = unit(C-B), |C-B|   [5] tb = unit(A-C), |A-C|   [6] tc = unit(B-A), |B-A|
//   [7] centroid.xyz, longest edge
// Edge naming follows the reference (evaluatorJ3DK.cu:286-288): edge a = B->C, b = C->A,
// c = A->B.
//
// The geometry and integrand functions are templates over the scalar type R.  The forward
// kernels instantiate them with R = double (the names d3, PanelJ, Tri, ... below are those
// instantiations); the adjoint kernels instantiate them with a dual number that carries the
// derivatives with respect to one vertex's coordinates (i2_dual.cuh), so the backward pass
// differentiates exactly the arithmetic of the forward pass.  Math functions are called
// unqualified: for double they resolve to CUDA's, for dual numbers by argument-dependent
// lookup to their own overloads.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace i2 {

constexpr double kPi = 3.14159265358979323846;
constexpr double kTwoPi = 6.28318530717958647692;
constexpr double kInv4Pi = 0.079577471545947667884;
// tolerances of the reference (src/common/constants.h:13-18)
constexpr double kDoubleMin = 2e-6;
constexpr double kEps = 1e-6;
constexpr double kEps2 = 1e-10;
constexpr double kEpsPsi2 = 1e-12;
constexpr double kEpsRunge = 1e-5;
constexpr int kMaxLevel = 5;
constexpr int kMaxGauss = 16;
constexpr int kMaxDuffy = 16;
constexpr int kDuffyTop = 24;  // size of the top Duffy rule of the tiered potential
constexpr int kMaxSelf = 32;

// the value of a scalar (dual numbers provide their own overload)
__host__ __device__ __forceinline__ double value_of(double x) { return x; }
__host__ __device__ __forceinline__ float value_of(float x) { return x; }

// ------------------------------------------------------------------ small vectors
template <class R>
struct V3 {
    R x, y, z;
};
using d3 = V3<double>;

__host__ __device__ __forceinline__ d3 mk(double x, double y, double z) { return d3{x, y, z}; }
template <class R>
__host__ __device__ __forceinline__ V3<R> operator+(V3<R> a, V3<R> b)
{
    return V3<R>{a.x + b.x, a.y + b.y, a.z + b.z};
}
template <class R>
__host__ __device__ __forceinline__ V3<R> operator-(V3<R> a, V3<R> b)
{
    return V3<R>{a.x - b.x, a.y - b.y, a.z - b.z};
}
template <class R>
__host__ __device__ __forceinline__ V3<R> operator-(V3<R> a)
{
    return V3<R>{-a.x, -a.y, -a.z};
}
// scalar times vector; the result takes the type of the product (double x dual -> dual)
template <class S, class R>
__host__ __device__ __forceinline__ auto operator*(S s, V3<R> a) -> V3<decltype(a.x * s)>
{
    return V3<decltype(a.x * s)>{a.x * s, a.y * s, a.z * s};
}
template <class R>
__host__ __device__ __forceinline__ R dot(V3<R> a, V3<R> b)
{
    return a.x * b.x + a.y * b.y + a.z * b.z;
}
template <class R>
__host__ __device__ __forceinline__ V3<R> cross(V3<R> a, V3<R> b)
{
    return V3<R>{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class R>
__host__ __device__ __forceinline__ R norm(V3<R> a)
{
    return sqrt(dot(a, a));
}
template <class R>
__host__ __device__ __forceinline__ V3<R> unit(V3<R> a)
{
    const R inv = 1.0 / norm(a);
    return V3<R>{a.x * inv, a.y * inv, a.z * inv};
}
__device__ __forceinline__ d3 xyz(const double4_32a &v) { return d3{v.x, v.y, v.z}; }

// (Psi.xyz, Theta) accumulator plus the potential channel
struct acc5 {
    double px, py, pz, th, pot;
};
__device__ __forceinline__ acc5 zero5() { return acc5{0, 0, 0, 0, 0}; }
__device__ __forceinline__ void axpy5(acc5 &a, double w, d3 psi, double th, double pot)
{
    a.px += w * psi.x;
    a.py += w * psi.y;
    a.pz += w * psi.z;
    a.th += w * th;
    a.pot += w * pot;
}

// ------------------------------------------------------------------ panels
struct alignas(32) Panel {
    double4_32a v[8];
};
static_assert(sizeof(Panel) == 256, "panel record is 256 bytes");

// a K_j panel held in registers
template <class R>
struct PanelJT {
    V3<R> A, B, C, n, ta, tb, tc;
    R S, lenA, lenB, lenC;  // |C-B|, |A-C|, |B-A|
};
using PanelJ = PanelJT<double>;

__device__ __forceinline__ PanelJ load_panel(const Panel *__restrict__ p, int c)
{
    const double4_32a *q = p[c].v;
    const double4_32a a = q[0], b = q[1], cc = q[2], n = q[3], ta = q[4], tb = q[5], tc = q[6];
    PanelJ r;
    r.A = xyz(a);
    r.S = a.w;
    r.B = xyz(b);
    r.C = xyz(cc);
    r.n = xyz(n);
    r.ta = xyz(ta);
    r.lenA = ta.w;
    r.tb = xyz(tb);
    r.lenB = tb.w;
    r.tc = xyz(tc);
    r.lenC = tc.w;
    return r;
}

// a K_j panel from its vertices (the same quantities k_prepare_panels stores)
template <class R>
__device__ __forceinline__ PanelJT<R> make_panel(V3<R> A, V3<R> B, V3<R> C)
{
    PanelJT<R> r;
    r.A = A;
    r.B = B;
    r.C = C;
    const V3<R> cr = cross(B - A, C - A);
    r.n = unit(cr);
    r.S = 0.5 * norm(cr);
    const V3<R> ea = C - B, eb = A - C, ec = B - A;
    r.lenA = norm(ea);
    r.lenB = norm(eb);
    r.lenC = norm(ec);
    r.ta = unit(ea);
    r.tb = unit(eb);
    r.tc = unit(ec);
    return r;
}

template <class R>
struct TriT {
    V3<R> a, b, c;
};
using Tri = TriT<double>;

__device__ __forceinline__ Tri load_tri(const Panel *__restrict__ p, int c)
{
    const double4_32a *q = p[c].v;
    const double4_32a a = q[0], b = q[1], cc = q[2];
    return Tri{xyz(a), xyz(b), xyz(cc)};
}

// vertex k (0..2) of a panel in its stored order
template <class R>
__device__ __forceinline__ V3<R> panel_vertex(const PanelJT<R> &P, int k)
{
    return k == 0 ? P.A : (k == 1 ? P.B : P.C);
}

// index of this thread's warp when items are dealt warp-major over the grid: item k goes to warp
// k mod (warps in the grid), and consecutive items land in different blocks (hence SMs)
__device__ __forceinline__ long long warp_item_index() { return (long long)(threadIdx.x >> 5) * gridDim.x + blockIdx.x; }

// 1 -> 4 midpoint split in the reference's child order (NumericalIntegrator3d.cu:37-87):
// child 0 = (m_ab, b, m_bc), 1 = (m_bc, c, m_ca), 2 = (m_ca, a, m_ab), 3 = (m_bc, m_ca, m_ab)
template <class R>
__device__ __forceinline__ TriT<R> child(const TriT<R> &t, int k)
{
    const V3<R> mbc = 0.5 * (t.b + t.c), mca = 0.5 * (t.c + t.a), mab = 0.5 * (t.a + t.b);
    switch (k) {
    case 0: return TriT<R>{mab, t.b, mbc};
    case 1: return TriT<R>{mbc, t.c, mca};
    case 2: return TriT<R>{mca, t.a, mab};
    default: return TriT<R>{mbc, mca, mab};
    }
}

// sub-cell s (base-4 digits, most significant = first split) of a level-L refinement
template <class R>
__device__ __forceinline__ TriT<R> subcell(TriT<R> t, int level, int s)
{
    for (int l = level - 1; l >= 0; --l) t = child(t, (s >> (2 * l)) & 3);
    return t;
}

// rotation so that vertex s comes first
template <class R>
__device__ __forceinline__ TriT<R> rotate(const TriT<R> &t, int s)
{
    return s == 0 ? t : (s == 1 ? TriT<R>{t.b, t.c, t.a} : TriT<R>{t.c, t.a, t.b});
}

// ------------------------------------------------------------------ quadrature tables
// Passed by value as kernel parameters (constant bank): per-handle, no process globals.
struct QuadTables {
    double L1[kMaxGauss], L2[kMaxGauss], L3[kMaxGauss], w[kMaxGauss];
    int npts;
    int order;
    double pow2p;
    // graded Duffy rule for the potential of common-edge / common-vertex pairs
    double du_u[kMaxDuffy], du_w[kMaxDuffy];   // radial nodes u = t^g and weights g t^(g-1) w_t
    double dv_v[kMaxDuffy], dv_w[kMaxDuffy];   // angular Gauss-Legendre on [0,1]
    int nu, nv;
    // two more Duffy rules of the tiered potential: a lower-order check (tier 1) and a
    // higher-order rule (tier 2)
    double lo_u[kMaxDuffy], lo_uw[kMaxDuffy], lo_v[kMaxDuffy], lo_vw[kMaxDuffy];
    int lo_nu, lo_nv;
    double hi_u[kMaxDuffy], hi_uw[kMaxDuffy], hi_v[kMaxDuffy], hi_vw[kMaxDuffy];
    int hi_nu, hi_nv;
    // top rule (24 x 24), checked against the higher-order rule before the adaptive rule
    double top_u[kDuffyTop], top_uw[kDuffyTop], top_v[kDuffyTop], top_vw[kDuffyTop];
    int top_nu, top_nv;
    // Gauss-Legendre on [0,1] for the self-pair potential (graded t^2(3-2t) map applied)
    double sx[kMaxSelf], sw[kMaxSelf];
    int nself;
};

// ------------------------------------------------------------------ reference helpers
// angle() with the reference's clamps (src/common/cuda_math.cu:14-26)
template <class R>
__device__ __forceinline__ R angle_ref(V3<R> a, V3<R> b)
{
    const R den = sqrt(dot(a, a) * dot(b, b));
    if (den < kEps) return R(0.0);
    const R c = dot(a, b) / den;
    if (c >= 1.0) return R(0.0);
    if (c <= -1.0) return R(kPi);
    return acos(c);
}
// piecewise constants of the reference: their derivative is 0
template <class R>
__device__ __forceinline__ double sign_ref(R x)
{
    if (fabs(x) < kDoubleMin) return 0.0;
    return x > kDoubleMin ? 1.0 : -1.0;
}
template <class R>
__device__ __forceinline__ double arg_ref(R x)
{
    return x > kDoubleMin ? 0.0 : kPi;
}

// ------------------------------------------------------------------ index shifts
// position in each triangle of the single shared vertex (evaluatorJ3DK.cu:782-795)
__device__ __forceinline__ void shifts_vertex(int3 ti, int3 tj, int &si, int &sj)
{
    const int a[3] = {ti.x, ti.y, ti.z}, b[3] = {tj.x, tj.y, tj.z};
    si = 0;
    sj = 0;
#pragma unroll
    for (int p = 0; p < 3; ++p)
#pragma unroll
        for (int q = 0; q < 3; ++q)
            if (a[p] == b[q]) { si = p; sj = q; }
}
// position in each triangle of the vertex off the shared edge (:797-825)
__device__ __forceinline__ void shifts_edge(int3 ti, int3 tj, int &si, int &sj)
{
    const int a[3] = {ti.x, ti.y, ti.z}, b[3] = {tj.x, tj.y, tj.z};
    bool ina[3] = {false, false, false}, inb[3] = {false, false, false};
#pragma unroll
    for (int p = 0; p < 3; ++p)
#pragma unroll
        for (int q = 0; q < 3; ++q)
            if (a[p] == b[q]) { ina[p] = true; inb[q] = true; }
    si = !ina[0] ? 0 : (!ina[1] ? 1 : 2);
    sj = !inb[0] ? 0 : (!inb[1] ? 1 : 2);
}

// ------------------------------------------------------------------ a1: far-field integrand
// theta/psi of K_j seen from x (evaluatorJ3DK.cu:266-313), written without normalising the
// point-to-vertex vectors:  la (1 + unit(x-A).tc) = la + (x-A).tc, and the solid angle in the
// Van Oosterom-Strackee form with the triple product (x-A).((x-B)x(x-C)) = 2S n.(x-A).
// The collinear fallback of the reference is kept.  The potential integrand
// sum_e t_e L_e - d Theta rides on the same logs (t_e = m_e.(P_e - x), m_e = tau_e x n).
template <class R>
struct FarCtxT {
    V3<R> ma, mb, mc;  // outward in-plane edge normals of K_j
};
using FarCtx = FarCtxT<double>;

template <class R>
__device__ __forceinline__ FarCtxT<R> make_far_ctx(const PanelJT<R> &K)
{
    return FarCtxT<R>{cross(K.ta, K.n), cross(K.tb, K.n), cross(K.tc, K.n)};
}

template <class R>
__device__ __forceinline__ R edge_log_fp64(R l_from, R q_from, R l_to, R q_to)
{
    // q = (x - P).tau ; reference: |1 + unit(x - P_to).tau| < eps^2/2 -> log(l_to / l_from)
    if (fabs(q_to + l_to) < 0.5 * kEpsPsi2 * l_to) return log(l_to / l_from);
    return log((l_from + q_from) / (l_to + q_to));
}

// from the point-to-vertex offsets oa = x - A, ob = x - B, oc = x - C (callers that know a point
// only relative to a nearby vertex form these offsets without cancellation)
template <class R>
__device__ __forceinline__ void far_integrand_o(V3<R> oa, V3<R> ob, V3<R> oc, const PanelJT<R> &K, const FarCtxT<R> &F,
                                                V3<R> &psi, R &th, R &pot)
{
    const R la = norm(oa), lb = norm(ob), lc = norm(oc);
    const R Lc = edge_log_fp64(la, dot(oa, K.tc), lb, dot(ob, K.tc));  // A -> B
    const R La = edge_log_fp64(lb, dot(ob, K.ta), lc, dot(oc, K.ta));  // B -> C
    const R Lb = edge_log_fp64(lc, dot(oc, K.tb), la, dot(oa, K.tb));  // C -> A
    psi = Lc * K.tc + La * K.ta + Lb * K.tb;
    const R d = dot(K.n, oa);
    const R num = 2.0 * K.S * d;
    const R den = la * lb * lc + dot(oa, ob) * lc + dot(ob, oc) * la + dot(oc, oa) * lb;
    th = 2.0 * atan2(num, den);
    // t_e L_e -> 0 on the line of edge e even where L_e itself overflows
    const R ta_ = -dot(F.ma, ob), tb_ = -dot(F.mb, oc), tc_ = -dot(F.mc, oa);
    pot = (ta_ == 0.0 ? R(0.0) : ta_ * La) + (tb_ == 0.0 ? R(0.0) : tb_ * Lb) + (tc_ == 0.0 ? R(0.0) : tc_ * Lc) - d * th;
}

template <class R>
__device__ __forceinline__ void far_integrand(V3<R> x, const PanelJT<R> &K, const FarCtxT<R> &F, V3<R> &psi, R &th, R &pot)
{
    far_integrand_o(x - K.A, x - K.B, x - K.C, K, F, psi, th, pot);
}

// ln((l_P + q_P) / (l_Q + q_Q)) for the edge P -> Q of length L from sums and products of
// positive terms only (q_P - q_Q = L; the squared distance to the edge line is taken from the
// nearer endpoint).  The same form as the FP32 bulk's edge_log_f32, for single-precision scalar
// types (FP32 adjoint) where the reference's form cancels.
template <class R>
__device__ __forceinline__ R edge_log_pos(R lP, R qP, V3<R> oP, R lQ, R qQ, V3<R> oQ, V3<R> tau, R L)
{
    const R s = lP + lQ;
    if (qQ >= 0.0) return log1p(L * (s + qP + qQ) / (s * (lQ + qQ)));
    if (qP <= 0.0) return log1p(L * (s - qP - qQ) / (s * (lP - qP)));
    const V3<R> r = cross(lP < lQ ? oP : oQ, tau);
    const R h2 = dot(r, r);
    const R num = (lP + qP) * (lQ - qQ);
    if (num > 2.0 * h2) return log(num / h2);
    return log1p((lP + qP) * L * (s - qP - qQ) / (s * h2));
}

// far_integrand_o with edge_log_pos (no collinear fallback needed: no term cancels)
template <class R>
__device__ __forceinline__ void far_integrand_pos(V3<R> x, const PanelJT<R> &K, const FarCtxT<R> &F, V3<R> &psi, R &th, R &pot)
{
    const V3<R> oa = x - K.A, ob = x - K.B, oc = x - K.C;
    const R la = norm(oa), lb = norm(ob), lc = norm(oc);
    const R Lc = edge_log_pos(la, dot(oa, K.tc), oa, lb, dot(ob, K.tc), ob, K.tc, K.lenC);  // A -> B
    const R La = edge_log_pos(lb, dot(ob, K.ta), ob, lc, dot(oc, K.ta), oc, K.ta, K.lenA);  // B -> C
    const R Lb = edge_log_pos(lc, dot(oc, K.tb), oc, la, dot(oa, K.tb), oa, K.tb, K.lenB);  // C -> A
    psi = Lc * K.tc + La * K.ta + Lb * K.tb;
    const R d = dot(K.n, oa);
    const R den = la * lb * lc + dot(oa, ob) * lc + dot(ob, oc) * la + dot(oc, oa) * lb;
    th = 2.0 * atan2(2.0 * K.S * d, den);
    pot = -dot(F.ma, ob) * La - dot(F.mb, oc) * Lb - dot(F.mc, oa) * Lc - d * th;
}

// ------------------------------------------------------------------ a2: common-edge regular part
// thetaPsi - singularPartAttached (evaluatorJ3DK.cu:315-350) with K_j rotated so that JA is
// the vertex off the shared edge JB->JC.  The log terms simplify exactly: the shared edge's
// term cancels, and each remaining pair (l + q)(l - q) = rho^2 of one edge line fuses into a
// single well-conditioned log:
//   Psi_reg = log((l_A + o_A.tb) / |BC|) tb + log((l_A - o_A.ta) / |BC|) ta,
// tb = unit(JB-JA), ta = unit(JA-JC).  Theta_reg keeps the reference's three atan2 (branches).
template <class R>
struct EdgeCtxT {
    V3<R> JA, JB, JC, ta, tb, tc;
    R ilvc;
    int sj;
};
using EdgeCtx = EdgeCtxT<double>;

template <class R>
__device__ __forceinline__ EdgeCtxT<R> make_edge_ctx(const PanelJT<R> &K, int sj)
{
    EdgeCtxT<R> e;
    e.sj = sj;
    e.JA = panel_vertex(K, sj);
    e.JB = panel_vertex(K, (sj + 1) % 3);
    e.JC = panel_vertex(K, (sj + 2) % 3);
    e.ta = unit(e.JA - e.JC);
    e.tb = unit(e.JB - e.JA);
    const V3<R> c = e.JC - e.JB;
    e.ilvc = 1.0 / norm(c);
    e.tc = e.ilvc * c;
    return e;
}

template <class R>
__device__ __forceinline__ void edge_integrand(V3<R> x, const PanelJT<R> &K, const EdgeCtxT<R> &E, V3<R> &psi, R &th)
{
    const V3<R> oA = x - E.JA, oB = x - E.JB, oC = x - E.JC;
    const R lA = norm(oA), lB = norm(oB), lC = norm(oC);
    const R l1 = log((lA + dot(oA, E.tb)) * E.ilvc);
    const R l2 = log((lA - dot(oA, E.ta)) * E.ilvc);
    psi = l1 * E.tb + l2 * E.ta;
    // full solid angle (rotation keeps orientation), minus the two asymptotic angles
    const R num = 2.0 * K.S * dot(K.n, oA);
    const R den = lA * lB * lC + dot(oA, oB) * lC + dot(oB, oC) * lA + dot(oC, oA) * lB;
    const R s1 = atan2(dot(cross(oB, E.tb), E.tc), dot(E.tb - E.tc, lB * E.tb + oB));
    const R s2 = atan2(dot(cross(oC, E.ta), E.tc), dot(E.ta - E.tc, lC * E.ta - oC));
    th = 2.0 * atan2(num, den) - 2.0 * (s1 - s2);
}

// ------------------------------------------------------------------ a3: common-vertex regular part
// thetaPsi - singularPartSimple (evaluatorJ3DK.cu:352-407), K_j rotated so JA is the shared
// vertex.  The per-pair direction e (with the reference's two sign flips) is computed once per
// task.  Fused logs: the two edges at JA give log((l_C + o_C.ta) / sqrt(S_i)) ta and
// log((l_B - o_B.tb) / sqrt(S_i)) tb, the opposite edge keeps its thetaPsi term.
template <class R>
struct VertexCtxT {
    V3<R> JA, JB, JC, ta, tb, tbc, e;
    R inv_sqrt_si;
};
using VertexCtx = VertexCtxT<double>;

template <class R>
__device__ __forceinline__ void vertex_deltas(V3<R> ta, V3<R> tb, V3<R> nj, V3<R> e, R &dA, R &dB)
{
    dA = atan2(dot(cross(ta, e), nj), -dot(e, ta));
    dB = atan2(dot(cross(e, tb), nj), dot(e, tb));
}

// intersection direction of the two planes with the reference's flips (:376-399 / :698-723)
template <class R>
__device__ __forceinline__ V3<R> vertex_direction(V3<R> ni, V3<R> nj, V3<R> ta, V3<R> tb, R &dA, R &dB)
{
    V3<R> e = cross(ni, nj);
    if (dot(e, e) < kEps2) e = tb;
    else e = unit(e);
    vertex_deltas(ta, tb, nj, e, dA, dB);
    if ((kPi - fabs(dA) < kEps) || (kPi - fabs(dB) < kEps)) {
        e = -1.0 * e;
        vertex_deltas(ta, tb, nj, e, dA, dB);
    }
    if ((dA * dB < 0.0) && (fabs(dA - dB) > kPi)) {
        e = -1.0 * e;
        vertex_deltas(ta, tb, nj, e, dA, dB);
    }
    return e;
}

template <class R>
__device__ __forceinline__ VertexCtxT<R> make_vertex_ctx(const PanelJT<R> &K, int sj, V3<R> ni, R Si)
{
    VertexCtxT<R> v;
    v.JA = panel_vertex(K, sj);
    v.JB = panel_vertex(K, (sj + 1) % 3);
    v.JC = panel_vertex(K, (sj + 2) % 3);
    v.ta = unit(v.JA - v.JC);
    v.tb = unit(v.JB - v.JA);
    v.tbc = unit(v.JC - v.JB);
    R dA, dB;
    v.e = vertex_direction(ni, K.n, v.ta, v.tb, dA, dB);
    v.inv_sqrt_si = 1.0 / sqrt(Si);
    return v;
}

template <class R>
__device__ __forceinline__ void vertex_integrand(V3<R> x, const PanelJT<R> &K, const VertexCtxT<R> &V, V3<R> &psi, R &th)
{
    const V3<R> oA = x - V.JA, oB = x - V.JB, oC = x - V.JC;
    const R lA = norm(oA), lB = norm(oB), lC = norm(oC);
    const R Lbc = edge_log_fp64(lB, dot(oB, V.tbc), lC, dot(oC, V.tbc));
    const R l1 = log((lC + dot(oC, V.ta)) * V.inv_sqrt_si);
    const R l2 = log((lB - dot(oB, V.tb)) * V.inv_sqrt_si);
    psi = Lbc * V.tbc + l1 * V.ta + l2 * V.tb;
    const R num = 2.0 * K.S * dot(K.n, oA);
    const R den = lA * lB * lC + dot(oA, oB) * lC + dot(oB, oC) * lA + dot(oC, oA) * lB;
    const R s1 = atan2(dot(cross(oA, V.ta), V.e), dot(lA * V.e - oA, V.e - V.ta));
    const R s2 = atan2(dot(cross(oA, V.tb), V.e), dot(lA * V.e - oA, V.e + V.tb));
    th = 2.0 * atan2(num, den) - 2.0 * (s1 + s2);
}

// ------------------------------------------------------------------ a4: common-edge closed form
template <class R>
struct SC2 {
    R s, c;
};
using sc2 = SC2<double>;

template <class R>
__device__ __forceinline__ SC2<R> sc_of(R a)
{
    SC2<R> r;
    sincos(a, &r.s, &r.c);
    return r;
}

// 2 atan2(sin xi sin a sin g, 1 - cos a + cos g + cos l)   (evaluatorJ3DK.cu:418-421)
template <class R>
__device__ __forceinline__ R phi_fn(SC2<R> a, SC2<R> g, R sxi, R cl)
{
    return 2.0 * atan2(sxi * a.s * g.s, 1.0 - a.c + g.c + cl);
}

// q_theta, q_psi of the common-edge closed form (:438-461) and its coplanar limit (:474-481;
// the reference leaves q_theta unset there, its documented value is 0)
template <class R>
__device__ inline void q_edge(SC2<R> a, SC2<R> b, SC2<R> g, SC2<R> n, SC2<R> xi, R cmu, R cla, R &qt, R &qp)
{
    const SC2<R> am{a.s, -a.c}, gm{g.s, -g.c};
    const R p1 = phi_fn(a, g, xi.s, cla);
    const R p2 = phi_fn(am, gm, xi.s, cla);
    const R k = 1.0 / (a.s * (1.0 - cmu * cmu));
    qt = p1 + g.s * n.s * k *
                  ((b.c * g.s - xi.c * b.s * g.c) * p2 +
                   xi.s * b.s *
                       (0.5 * (1.0 + cmu) * log((1.0 + b.c) / (1.0 - n.c)) + 0.5 * (1.0 - cmu) * log((1.0 - b.c) / (1.0 + n.c)) +
                        log((1.0 + cla) / (1.0 - g.c))));
    qp = 1.5 - k * (b.s * (n.c + cmu * cla) * log(1.0 + cla) + n.s * (b.c + cmu * g.c) * log(1.0 - g.c) +
                    b.s * (1.0 - cmu) * (n.c - cla) * log(b.s / n.s) +
                    n.s * b.s * (b.s * g.c - xi.c * g.s * b.c) * log((1.0 - n.c) / (1.0 + b.c)) + p2 * xi.s * g.s * n.s * b.s);
}
template <class R>
__device__ inline void q_edge_coplanar(SC2<R> b, SC2<R> n, R sa, R &qt, R &qp)
{
    qt = R(0.0);
    qp = 1.5 - (n.c * b.s * log(1.0 + n.c) + n.s * b.c * log(1.0 - b.c) + sa - b.s + n.s + b.s * n.c * log(b.s / n.s)) / sa;
}

// integrateSingularPartAttached (:603-672): closed-form integral over K_i of the common-edge
// asymptote; Ti/Tj hold the vertices rotated so that the off-edge vertex comes first.  At the
// scale it is given (see closed_edge for the scale-invariant entry point)
template <class R>
__device__ inline void closed_edge_unit(TriT<R> Ti, TriT<R> Tj, V3<R> ni, V3<R> nj, R Si, V3<R> &psi, R &th)
{
    const V3<R> IA = Ti.a, IB = Ti.b, IC = Ti.c, JA = Tj.a, JB = Tj.b, JC = Tj.c;
    const V3<R> ta = unit(JA - JC), tb = unit(JB - JA), tc = unit(JC - JB);
    const R al = angle_ref(IA - IC, IB - IC);
    const R be = angle_ref(IC - IB, IA - IB);
    const R ga = angle_ref(JC - JB, JA - JB);
    const R de = angle_ref(JB - JC, JA - JC);
    const R nu = kPi - al - be;
    const R xi = atan2(dot(cross(ni, nj), tc), dot(ni, nj));
    const SC2<R> sa = sc_of(al), sb = sc_of(be), sg = sc_of(ga), sd = sc_of(de), sx = sc_of(xi);
    const SC2<R> sn{sa.s * sb.c + sa.c * sb.s, sa.s * sb.s - sa.c * sb.c};
    const R csig = -(sa.c * sd.c + sx.c * sa.s * sd.s);
    const R cmu = -(sb.c * sg.c + sx.c * sb.s * sg.s);
    const R cla = -(sa.c * sg.c - sx.c * sa.s * sg.s);
    const R cth = -(sb.c * sd.c - sx.c * sb.s * sd.s);
    const R qab = sn.s * log(tan(0.5 * al) * tan(0.5 * nu)) / sb.s + sn.s * log(tan(0.5 * be) * tan(0.5 * nu)) / sa.s +
                  log(tan(0.5 * al) * tan(0.5 * be));
    R qAt, qAp, qBt, qBp;
    if (fabs(xi) < kEps && fabs(be - ga) < kEps) q_edge_coplanar(sb, sn, sa.s, qAt, qAp);
    else q_edge(sa, sb, sg, sn, sx, cmu, cla, qAt, qAp);
    if (fabs(xi) < kEps && fabs(al - de) < kEps) q_edge_coplanar(sa, sn, sb.s, qBt, qBp);
    else q_edge(sb, sa, sd, sn, sx, csig, cth, qBt, qBp);
    psi = Si * (qAp * tb + qBp * ta - qab * tc);
    th = Si * (qAt + qBt);
}

// ------------------------------------------------------------------ a5: common-vertex closed form
template <class R>
struct VtxAnglesT {
    SC2<R> xi, mu, nu, psi, nupsi, mupsi;
    R mu_a, nu_a, psi_a, kappa, skappa, lsmu, lsnu;
};

// q_thetaPsi_cont (:511-601): general case plus the reference's four special branches
template <class R>
__device__ inline void q_vertex(const VtxAnglesT<R> &g, R delta, SC2<R> sd, R cla, R cth, R ceta, R csig, R cchi, R &qt, R &qp)
{
    const R mu = g.mu_a, nu = g.nu_a, ps = g.psi_a, sk = g.skappa;
    const SC2<R> xi = g.xi, smu = g.mu, snu = g.nu, sps = g.psi;
    const R lth = log(1.0 + cth), lla = log(1.0 + cla);
    const R Lam1 = lla - lth + g.lsnu - g.lsmu;
    const R Lam2 = log(tan(0.5 * nu) * tan(0.5 * mu));
    const SC2<R> hd = sc_of(R(0.5 * delta));
    const R thd = hd.s / hd.c;
    const SC2<R> hmp = sc_of(R(0.5 * (mu - ps))), hnp = sc_of(R(0.5 * (nu + ps)));
    const R Amu = atan2(thd * hmp.c * xi.s, thd * hmp.c * xi.c + hmp.s);
    const R Anu = atan2(thd * hnp.s * xi.s, thd * hnp.s * xi.c + hnp.c);
    const SC2<R> t1 = sc_of(R(0.5 * (mu - ps) - 0.5 * (nu + ps))), t2 = sc_of(R(0.5 * g.kappa));
    const R W = atan2(sd.s * t2.s * xi.s, t2.c + sd.s * t1.c * xi.c + sd.c * t1.s);
    const SC2<R> t3 = sc_of(R(delta - ps));
    const R D = 1.0 / (t3.s * t3.s + sd.s * sps.s * (1.0 - xi.c) * (t3.c + csig));
    const R G = sps.c * (sd.s * csig * xi.c + sd.c * cchi - sd.s * sd.s / sps.s);
    const double mpsi = sign_ref(R(xi.s * sps.s)), mdel = sign_ref(R(xi.s * sd.s));
    if (fabs(xi.s) < kEps && 1.0 - fabs(csig) < 0.5 * kEps2 && fabs(sps.s) > kEps) {
        const double ara = arg_ref(R(sin(0.5 * (nu + ps)) * csig));
        const double arb = arg_ref(R(cos(0.5 * (mu - ps)) * csig));
        qt = 2.0 * mpsi * csig * xi.c / (sk * sps.s) * (smu.s * g.nupsi.s * ara - snu.s * g.mupsi.s * arb);
        qp = 0.5 * (1.0 - log(2.0)) - 0.5 * log((1.0 - csig * smu.c) * (1.0 + csig * snu.c) / sk) +
             csig * (smu.s - snu.s + 0.5 * sin(mu - nu) * Lam2) / sk;
        return;
    }
    const R gens = 0.5 * (3.0 - log(2.0)) +
                   (smu.s * snu.s / sk) * ((lla - lth) * sps.c / sps.s +
                                           D * (Lam1 * sd.s * ceta / sps.s + Lam2 * cchi - 2.0 * W * sd.s * xi.s -
                                                G * (g.lsnu - g.lsmu))) -
                   (smu.c * snu.s * (lla - g.lsmu) + smu.s * snu.c * (lth - g.lsnu)) / sk - 0.5 * (g.lsmu + g.lsnu - log(sk));
    if (fabs(xi.s) < kEps && fabs(sps.s) > kEps) {
        const double are = arg_ref(R(sin(0.5 * (nu + mu)) + sin(0.5 * (mu - nu) - ps + delta * xi.c)));
        const double arc = arg_ref(R(1.0 / tan(0.5 * (nu + ps)) + tan(0.5 * delta) * xi.c));
        const double ard = arg_ref(R(tan(0.5 * (mu - ps)) + tan(0.5 * delta) * xi.c));
        qt = 2.0 * mdel * (sd.s * smu.s * snu.s / cchi * xi.c * are + smu.s * g.nupsi.s * arc - snu.s * g.mupsi.s * ard) /
             (sk * sps.s);
        qp = gens;
        return;
    }
    if (fabs(sin(ps)) < kEps) {
        if (fabs(delta) > kEps) {
            qt = 2.0 * (smu.s * snu.s * (W * sd.c * xi.c - 0.5 * (Lam1 - Lam2 * csig) * xi.s) / sd.s +
                        (Anu + mdel * arg_ref(R(sin(0.5 * (nu + ps))))) * smu.s * snu.c +
                        (Amu + mdel * arg_ref(R(cos(0.5 * (mu - ps))))) * smu.c * snu.s) /
                 sk;
            qp = 0.5 * (3.0 - log(2.0)) - 0.5 * (log((1.0 + cla) * (1.0 + cth) / sk) - sin(mu - nu) / sk * Lam1) -
                 smu.s * snu.s * ((Lam1 * sd.c - Lam2 * sps.c) * xi.c + 2.0 * W * xi.s) / (sk * sd.s);
        } else {
            qt = R(2.0 * arg_ref(sps.c));
            qp = 0.5 * (1.0 - log(2.0)) - 0.5 * log((1.0 - sps.c * smu.c) * (1.0 + sps.c * snu.c) / sk) +
                 (0.5 * sin(mu - nu) * Lam1 + sps.c * (smu.s - snu.s)) / sk;
        }
        return;
    }
    qt = 2.0 * (Anu * smu.s * g.nupsi.s - Amu * snu.s * g.mupsi.s -
                D * smu.s * snu.s * sd.s * (W * ceta + 0.5 * sps.s * xi.s * (Lam1 - Lam2 * csig))) /
         (sps.s * sk);
    qp = gens;
}

// integrateSingularPartSimple (:674-780); Ti/Tj rotated so that the shared vertex comes first.
// At the scale it is given (see closed_vertex for the scale-invariant entry point)
template <class R>
__device__ inline void closed_vertex_unit(TriT<R> Ti, TriT<R> Tj, V3<R> ni, V3<R> nj, R Si, V3<R> &psi, R &th)
{
    const V3<R> IA = Ti.a, IB = Ti.b, IC = Ti.c, JA = Tj.a, JB = Tj.b, JC = Tj.c;
    const V3<R> ta = unit(JA - JC), tb = unit(JB - JA);
    R dA, dB;
    const V3<R> e = vertex_direction(ni, nj, ta, tb, dA, dB);
    const R xi = atan2(dot(cross(ni, nj), e), dot(ni, nj));
    const SC2<R> sdA = sc_of(dA), sdB = sc_of(dB);
    VtxAnglesT<R> g;
    g.xi = sc_of(xi);
    const V3<R> s = IC - IB;
    g.nu_a = angle_ref(IA - IB, IC - IB);
    g.mu_a = angle_ref(IB - IC, IA - IC);
    g.kappa = angle_ref(IB - IA, IC - IA);
    g.mu = sc_of(g.mu_a);
    g.nu = sc_of(g.nu_a);
    g.lsnu = log(g.nu.s);
    g.lsmu = log(g.mu.s);
    g.skappa = sin(g.kappa);
    g.psi_a = atan2(dot(cross(e, s), ni), dot(e, s));
    g.psi = sc_of(g.psi_a);
    g.nupsi = sc_of(R(g.nu_a + g.psi_a));
    g.mupsi = sc_of(R(g.mu_a - g.psi_a));
    R q[2][2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const SC2<R> d = h == 0 ? sdA : sdB;
        const R csig = d.s * g.psi.s * g.xi.c + d.c * g.psi.c;
        const R cchi = d.s * g.psi.c * g.xi.c - d.c * g.psi.s;
        const R ceta = d.c * g.psi.s * g.xi.c - d.s * g.psi.c;
        const R cth = d.s * g.nupsi.s * g.xi.c + d.c * g.nupsi.c;
        const R cla = d.s * g.mupsi.s * g.xi.c - d.c * g.mupsi.c;
        q_vertex(g, h == 0 ? dA : dB, d, cla, cth, ceta, csig, cchi, q[h][0], q[h][1]);
    }
    psi = Si * (q[0][1] * ta + q[1][1] * tb);
    th = (fabs(xi) < kEps) ? R(0.0) : R(Si * (q[0][0] - q[1][0]));
}

// ------------------------------------------------------------------ scale-invariant closed forms
// The reference's tolerances are absolute (angle() returns 0 below |a||b| = 1e-6,
// src/common/cuda_math.cu:14-26), so its closed forms collapse on meshes far below unit scale.
// The entry points below scale the pair by the power of two 2^k that brings sqrt(S_i) into
// [0.5, 1), evaluate there and scale back: Psi and Theta are S_i times dimensionless functions of
// the angles, the angles of the scaled vertices are bit-identical to the unscaled ones, and a
// power-of-two scaling is exact -- so at ordinary scales the result is unchanged to the last bit,
// and far from unit scale the thresholds act as they do at unit scale.
__device__ __forceinline__ double pow2_normaliser(double len)
{
    int e = 0;
    frexp(len, &e);  // len = m 2^e, m in [0.5, 1)
    return ldexp(1.0, -e);
}

template <class R>
__device__ __forceinline__ TriT<R> scaled_tri(const TriT<R> &t, double s)
{
    return TriT<R>{s * t.a, s * t.b, s * t.c};
}

template <class R>
__device__ inline void closed_edge(TriT<R> Ti, TriT<R> Tj, V3<R> ni, V3<R> nj, R Si, V3<R> &psi, R &th)
{
    const double s = pow2_normaliser(sqrt((double)value_of(Si)));
    closed_edge_unit(scaled_tri(Ti, s), scaled_tri(Tj, s), ni, nj, R((s * s) * Si), psi, th);
    const double inv = 1.0 / (s * s);
    psi = inv * psi;
    th = inv * th;
}

template <class R>
__device__ inline void closed_vertex(TriT<R> Ti, TriT<R> Tj, V3<R> ni, V3<R> nj, R Si, V3<R> &psi, R &th)
{
    const double s = pow2_normaliser(sqrt((double)value_of(Si)));
    closed_vertex_unit(scaled_tri(Ti, s), scaled_tri(Tj, s), ni, nj, R((s * s) * Si), psi, th);
    const double inv = 1.0 / (s * s);
    psi = inv * psi;
    th = inv * th;
}

// ------------------------------------------------------------------ potential helpers
// common-edge potential: subtracted s ln s term along the shared edge (sigma = -2 c s ln(s/h),
// integral over K_i = (5/9) c S_i h)
template <class R>
struct PotEdgeT {
    V3<R> P1, m_in;
    R c, h;
};
using PotEdge = PotEdgeT<double>;

template <class R>
__device__ __forceinline__ R pot_edge_sigma(V3<R> x, const PotEdgeT<R> &p)
{
    const R s = dot(x - p.P1, p.m_in);
    return s > 0.0 ? R(-2.0 * p.c * s * log(s / p.h)) : R(0.0);
}

} // namespace i2
