// i2_device.cuh -- device-side geometry and FP64 integrands of the pair-integral path.
//
// Layout: every cell of a mesh has one 256-byte "panel" record (8 x 32-byte double4_32a,
// loaded with 256-bit vector loads), written once by k_prepare_panels:
//   [0] A.xyz, S          [1] B.xyz, 2S         [2] C.xyz, 0          [3] n.xyz, 0
//   [4] ta = unit(C-B), |C-B|   [5] tb = unit(A-C), |A-C|   [6] tc = unit(B-A), |B-A|
//   [7] centroid.xyz, longest edge
// Edge naming follows the reference (evaluatorJ3DK.cu:286-288): edge a = B->C, b = C->A,
// c = A->B.
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
constexpr int kMaxSelf = 32;

// ------------------------------------------------------------------ small FP64 vectors
struct d3 {
    double x, y, z;
};
__host__ __device__ __forceinline__ d3 mk(double x, double y, double z) { return d3{x, y, z}; }
__host__ __device__ __forceinline__ d3 operator+(d3 a, d3 b) { return d3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__host__ __device__ __forceinline__ d3 operator-(d3 a, d3 b) { return d3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__host__ __device__ __forceinline__ d3 operator-(d3 a) { return d3{-a.x, -a.y, -a.z}; }
__host__ __device__ __forceinline__ d3 operator*(double s, d3 a) { return d3{a.x * s, a.y * s, a.z * s}; }
__host__ __device__ __forceinline__ double dot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ __forceinline__ d3 cross(d3 a, d3 b)
{
    return d3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__host__ __device__ __forceinline__ double norm(d3 a) { return sqrt(dot(a, a)); }
__host__ __device__ __forceinline__ d3 unit(d3 a)
{
    const double inv = 1.0 / norm(a);
    return d3{a.x * inv, a.y * inv, a.z * inv};
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
struct PanelJ {
    d3 A, B, C, n, ta, tb, tc;
    double S, lenA, lenB, lenC;  // |C-B|, |A-C|, |B-A|
};

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

struct Tri {
    d3 a, b, c;
};

__device__ __forceinline__ Tri load_tri(const Panel *__restrict__ p, int c)
{
    const double4_32a *q = p[c].v;
    const double4_32a a = q[0], b = q[1], cc = q[2];
    return Tri{xyz(a), xyz(b), xyz(cc)};
}

// vertex k (0..2) of a panel in its stored order
__device__ __forceinline__ d3 panel_vertex(const PanelJ &P, int k) { return k == 0 ? P.A : (k == 1 ? P.B : P.C); }

// 1 -> 4 midpoint split in the reference's child order (NumericalIntegrator3d.cu:37-87):
// child 0 = (m_ab, b, m_bc), 1 = (m_bc, c, m_ca), 2 = (m_ca, a, m_ab), 3 = (m_bc, m_ca, m_ab)
__device__ __forceinline__ Tri child(const Tri &t, int k)
{
    const d3 mbc = 0.5 * (t.b + t.c), mca = 0.5 * (t.c + t.a), mab = 0.5 * (t.a + t.b);
    switch (k) {
    case 0: return Tri{mab, t.b, mbc};
    case 1: return Tri{mbc, t.c, mca};
    case 2: return Tri{mca, t.a, mab};
    default: return Tri{mbc, mca, mab};
    }
}

// sub-cell s (base-4 digits, most significant = first split) of a level-L refinement
__device__ __forceinline__ Tri subcell(Tri t, int level, int s)
{
    for (int l = level - 1; l >= 0; --l) t = child(t, (s >> (2 * l)) & 3);
    return t;
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
    // Gauss-Legendre on [0,1] for the self-pair potential (graded t^2(3-2t) map applied)
    double sx[kMaxSelf], sw[kMaxSelf];
    int nself;
};

// ------------------------------------------------------------------ reference helpers
// angle() with the reference's clamps (src/common/cuda_math.cu:14-26)
__device__ __forceinline__ double angle_ref(d3 a, d3 b)
{
    const double den = sqrt(dot(a, a) * dot(b, b));
    if (den < kEps) return 0.0;
    const double c = dot(a, b) / den;
    if (c >= 1.0) return 0.0;
    if (c <= -1.0) return kPi;
    return acos(c);
}
__device__ __forceinline__ double sign_ref(double x)
{
    if (fabs(x) < kDoubleMin) return 0.0;
    return x > kDoubleMin ? 1.0 : -1.0;
}
__device__ __forceinline__ double arg_ref(double x) { return x > kDoubleMin ? 0.0 : kPi; }

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
struct FarCtx {
    d3 ma, mb, mc;  // outward in-plane edge normals of K_j
};
__device__ __forceinline__ FarCtx make_far_ctx(const PanelJ &K)
{
    return FarCtx{cross(K.ta, K.n), cross(K.tb, K.n), cross(K.tc, K.n)};
}

__device__ __forceinline__ double edge_log_fp64(double l_from, double q_from, double l_to, double q_to)
{
    // q = (x - P).tau ; reference: |1 + unit(x - P_to).tau| < eps^2/2 -> log(l_to / l_from)
    if (fabs(q_to + l_to) < 0.5 * kEpsPsi2 * l_to) return log(l_to / l_from);
    return log((l_from + q_from) / (l_to + q_to));
}

// from the point-to-vertex offsets oa = x - A, ob = x - B, oc = x - C (callers that know a point
// only relative to a nearby vertex form these offsets without cancellation)
__device__ __forceinline__ void far_integrand_o(d3 oa, d3 ob, d3 oc, const PanelJ &K, const FarCtx &F, d3 &psi, double &th,
                                                double &pot)
{
    const double la = norm(oa), lb = norm(ob), lc = norm(oc);
    const double Lc = edge_log_fp64(la, dot(oa, K.tc), lb, dot(ob, K.tc));  // A -> B
    const double La = edge_log_fp64(lb, dot(ob, K.ta), lc, dot(oc, K.ta));  // B -> C
    const double Lb = edge_log_fp64(lc, dot(oc, K.tb), la, dot(oa, K.tb));  // C -> A
    psi = Lc * K.tc + La * K.ta + Lb * K.tb;
    const double d = dot(K.n, oa);
    const double num = 2.0 * K.S * d;
    const double den = la * lb * lc + dot(oa, ob) * lc + dot(ob, oc) * la + dot(oc, oa) * lb;
    th = 2.0 * atan2(num, den);
    // t_e L_e -> 0 on the line of edge e even where L_e itself overflows
    const double ta_ = -dot(F.ma, ob), tb_ = -dot(F.mb, oc), tc_ = -dot(F.mc, oa);
    pot = (ta_ == 0.0 ? 0.0 : ta_ * La) + (tb_ == 0.0 ? 0.0 : tb_ * Lb) + (tc_ == 0.0 ? 0.0 : tc_ * Lc) - d * th;
}

__device__ __forceinline__ void far_integrand(d3 x, const PanelJ &K, const FarCtx &F, d3 &psi, double &th, double &pot)
{
    far_integrand_o(x - K.A, x - K.B, x - K.C, K, F, psi, th, pot);
}

// ------------------------------------------------------------------ a2: common-edge regular part
// thetaPsi - singularPartAttached (evaluatorJ3DK.cu:315-350) with K_j rotated so that JA is
// the vertex off the shared edge JB->JC.  The log terms simplify exactly: the shared edge's
// term cancels, and each remaining pair (l + q)(l - q) = rho^2 of one edge line fuses into a
// single well-conditioned log:
//   Psi_reg = log((l_A + o_A.tb) / |BC|) tb + log((l_A - o_A.ta) / |BC|) ta,
// tb = unit(JB-JA), ta = unit(JA-JC).  Theta_reg keeps the reference's three atan2 (branches).
struct EdgeCtx {
    d3 JA, JB, JC, ta, tb, tc;
    double ilvc;
    int sj;
};

__device__ __forceinline__ EdgeCtx make_edge_ctx(const PanelJ &K, int sj)
{
    EdgeCtx e;
    e.sj = sj;
    e.JA = panel_vertex(K, sj);
    e.JB = panel_vertex(K, (sj + 1) % 3);
    e.JC = panel_vertex(K, (sj + 2) % 3);
    e.ta = unit(e.JA - e.JC);
    e.tb = unit(e.JB - e.JA);
    const d3 c = e.JC - e.JB;
    e.ilvc = 1.0 / norm(c);
    e.tc = e.ilvc * c;
    return e;
}

__device__ __forceinline__ void edge_integrand(d3 x, const PanelJ &K, const EdgeCtx &E, d3 &psi, double &th)
{
    const d3 oA = x - E.JA, oB = x - E.JB, oC = x - E.JC;
    const double lA = norm(oA), lB = norm(oB), lC = norm(oC);
    const double l1 = log((lA + dot(oA, E.tb)) * E.ilvc);
    const double l2 = log((lA - dot(oA, E.ta)) * E.ilvc);
    psi = l1 * E.tb + l2 * E.ta;
    // full solid angle (rotation keeps orientation), minus the two asymptotic angles
    const double num = 2.0 * K.S * dot(K.n, oA);
    const double den = lA * lB * lC + dot(oA, oB) * lC + dot(oB, oC) * lA + dot(oC, oA) * lB;
    const double s1 = atan2(dot(cross(oB, E.tb), E.tc), dot(E.tb - E.tc, lB * E.tb + oB));
    const double s2 = atan2(dot(cross(oC, E.ta), E.tc), dot(E.ta - E.tc, lC * E.ta - oC));
    th = 2.0 * atan2(num, den) - 2.0 * (s1 - s2);
}

// ------------------------------------------------------------------ a3: common-vertex regular part
// thetaPsi - singularPartSimple (evaluatorJ3DK.cu:352-407), K_j rotated so JA is the shared
// vertex.  The per-pair direction e (with the reference's two sign flips) is computed once per
// task.  Fused logs: the two edges at JA give log((l_C + o_C.ta) / sqrt(S_i)) ta and
// log((l_B - o_B.tb) / sqrt(S_i)) tb, the opposite edge keeps its thetaPsi term.
struct VertexCtx {
    d3 JA, JB, JC, ta, tb, tbc, e;
    double inv_sqrt_si;
};

__device__ __forceinline__ void vertex_deltas(d3 ta, d3 tb, d3 nj, d3 e, double &dA, double &dB)
{
    dA = atan2(dot(cross(ta, e), nj), -dot(e, ta));
    dB = atan2(dot(cross(e, tb), nj), dot(e, tb));
}

// intersection direction of the two planes with the reference's flips (:376-399 / :698-723)
__device__ __forceinline__ d3 vertex_direction(d3 ni, d3 nj, d3 ta, d3 tb, double &dA, double &dB)
{
    d3 e = cross(ni, nj);
    if (dot(e, e) < kEps2) e = tb;
    else e = unit(e);
    vertex_deltas(ta, tb, nj, e, dA, dB);
    if ((kPi - fabs(dA) < kEps) || (kPi - fabs(dB) < kEps)) {
        e = -1.0 * e;
        vertex_deltas(ta, tb, nj, e, dA, dB);
    }
    if ((dA * dB < 0) && (fabs(dA - dB) > kPi)) {
        e = -1.0 * e;
        vertex_deltas(ta, tb, nj, e, dA, dB);
    }
    return e;
}

__device__ __forceinline__ VertexCtx make_vertex_ctx(const PanelJ &K, int sj, d3 ni, double Si)
{
    VertexCtx v;
    v.JA = panel_vertex(K, sj);
    v.JB = panel_vertex(K, (sj + 1) % 3);
    v.JC = panel_vertex(K, (sj + 2) % 3);
    v.ta = unit(v.JA - v.JC);
    v.tb = unit(v.JB - v.JA);
    v.tbc = unit(v.JC - v.JB);
    double dA, dB;
    v.e = vertex_direction(ni, K.n, v.ta, v.tb, dA, dB);
    v.inv_sqrt_si = 1.0 / sqrt(Si);
    return v;
}

__device__ __forceinline__ void vertex_integrand(d3 x, const PanelJ &K, const VertexCtx &V, d3 &psi, double &th)
{
    const d3 oA = x - V.JA, oB = x - V.JB, oC = x - V.JC;
    const double lA = norm(oA), lB = norm(oB), lC = norm(oC);
    const double Lbc = edge_log_fp64(lB, dot(oB, V.tbc), lC, dot(oC, V.tbc));
    const double l1 = log((lC + dot(oC, V.ta)) * V.inv_sqrt_si);
    const double l2 = log((lB - dot(oB, V.tb)) * V.inv_sqrt_si);
    psi = Lbc * V.tbc + l1 * V.ta + l2 * V.tb;
    const double num = 2.0 * K.S * dot(K.n, oA);
    const double den = lA * lB * lC + dot(oA, oB) * lC + dot(oB, oC) * lA + dot(oC, oA) * lB;
    const double s1 = atan2(dot(cross(oA, V.ta), V.e), dot(lA * V.e - oA, V.e - V.ta));
    const double s2 = atan2(dot(cross(oA, V.tb), V.e), dot(lA * V.e - oA, V.e + V.tb));
    th = 2.0 * atan2(num, den) - 2.0 * (s1 + s2);
}

// ------------------------------------------------------------------ a4: common-edge closed form
struct sc2 {
    double s, c;
};
__device__ __forceinline__ sc2 sc_of(double a)
{
    sc2 r;
    sincos(a, &r.s, &r.c);
    return r;
}

// 2 atan2(sin xi sin a sin g, 1 - cos a + cos g + cos l)   (evaluatorJ3DK.cu:418-421)
__device__ __forceinline__ double phi_fn(sc2 a, sc2 g, double sxi, double cl)
{
    return 2.0 * atan2(sxi * a.s * g.s, 1.0 - a.c + g.c + cl);
}

// q_theta, q_psi of the common-edge closed form (:438-461) and its coplanar limit (:474-481;
// the reference leaves q_theta unset there, its documented value is 0)
__device__ inline void q_edge(sc2 a, sc2 b, sc2 g, sc2 n, sc2 xi, double cmu, double cla, double &qt, double &qp)
{
    const sc2 am{a.s, -a.c}, gm{g.s, -g.c};
    const double p1 = phi_fn(a, g, xi.s, cla);
    const double p2 = phi_fn(am, gm, xi.s, cla);
    const double k = 1.0 / (a.s * (1.0 - cmu * cmu));
    qt = p1 + g.s * n.s * k *
                  ((b.c * g.s - xi.c * b.s * g.c) * p2 +
                   xi.s * b.s *
                       (0.5 * (1.0 + cmu) * log((1.0 + b.c) / (1.0 - n.c)) + 0.5 * (1.0 - cmu) * log((1.0 - b.c) / (1.0 + n.c)) +
                        log((1.0 + cla) / (1.0 - g.c))));
    qp = 1.5 - k * (b.s * (n.c + cmu * cla) * log(1.0 + cla) + n.s * (b.c + cmu * g.c) * log(1.0 - g.c) +
                    b.s * (1.0 - cmu) * (n.c - cla) * log(b.s / n.s) +
                    n.s * b.s * (b.s * g.c - xi.c * g.s * b.c) * log((1.0 - n.c) / (1.0 + b.c)) + p2 * xi.s * g.s * n.s * b.s);
}
__device__ inline void q_edge_coplanar(sc2 b, sc2 n, double sa, double &qt, double &qp)
{
    qt = 0.0;
    qp = 1.5 - (n.c * b.s * log(1.0 + n.c) + n.s * b.c * log(1.0 - b.c) + sa - b.s + n.s + b.s * n.c * log(b.s / n.s)) / sa;
}

// integrateSingularPartAttached (:603-672): closed-form integral over K_i of the common-edge
// asymptote; Ti/Tj hold the vertices rotated so that the off-edge vertex comes first
__device__ inline void closed_edge(Tri Ti, Tri Tj, d3 ni, d3 nj, double Si, d3 &psi, double &th)
{
    const d3 IA = Ti.a, IB = Ti.b, IC = Ti.c, JA = Tj.a, JB = Tj.b, JC = Tj.c;
    const d3 ta = unit(JA - JC), tb = unit(JB - JA), tc = unit(JC - JB);
    const double al = angle_ref(IA - IC, IB - IC);
    const double be = angle_ref(IC - IB, IA - IB);
    const double ga = angle_ref(JC - JB, JA - JB);
    const double de = angle_ref(JB - JC, JA - JC);
    const double nu = kPi - al - be;
    const double xi = atan2(dot(cross(ni, nj), tc), dot(ni, nj));
    const sc2 sa = sc_of(al), sb = sc_of(be), sg = sc_of(ga), sd = sc_of(de), sx = sc_of(xi);
    const sc2 sn{sa.s * sb.c + sa.c * sb.s, sa.s * sb.s - sa.c * sb.c};
    const double csig = -(sa.c * sd.c + sx.c * sa.s * sd.s);
    const double cmu = -(sb.c * sg.c + sx.c * sb.s * sg.s);
    const double cla = -(sa.c * sg.c - sx.c * sa.s * sg.s);
    const double cth = -(sb.c * sd.c - sx.c * sb.s * sd.s);
    const double qab = sn.s * log(tan(0.5 * al) * tan(0.5 * nu)) / sb.s + sn.s * log(tan(0.5 * be) * tan(0.5 * nu)) / sa.s +
                       log(tan(0.5 * al) * tan(0.5 * be));
    double qAt, qAp, qBt, qBp;
    if (fabs(xi) < kEps && fabs(be - ga) < kEps) q_edge_coplanar(sb, sn, sa.s, qAt, qAp);
    else q_edge(sa, sb, sg, sn, sx, cmu, cla, qAt, qAp);
    if (fabs(xi) < kEps && fabs(al - de) < kEps) q_edge_coplanar(sa, sn, sb.s, qBt, qBp);
    else q_edge(sb, sa, sd, sn, sx, csig, cth, qBt, qBp);
    psi = Si * (qAp * tb + qBp * ta - qab * tc);
    th = Si * (qAt + qBt);
}

// ------------------------------------------------------------------ a5: common-vertex closed form
struct VtxAngles {
    sc2 xi, mu, nu, psi, nupsi, mupsi;
    double mu_a, nu_a, psi_a, kappa, skappa, lsmu, lsnu;
};

// q_thetaPsi_cont (:511-601): general case plus the reference's four special branches
__device__ inline void q_vertex(const VtxAngles &g, double delta, sc2 sd, double cla, double cth, double ceta, double csig,
                                double cchi, double &qt, double &qp)
{
    const double mu = g.mu_a, nu = g.nu_a, ps = g.psi_a, sk = g.skappa;
    const sc2 xi = g.xi, smu = g.mu, snu = g.nu, sps = g.psi;
    const double lth = log(1.0 + cth), lla = log(1.0 + cla);
    const double Lam1 = lla - lth + g.lsnu - g.lsmu;
    const double Lam2 = log(tan(0.5 * nu) * tan(0.5 * mu));
    const sc2 hd = sc_of(0.5 * delta);
    const double thd = hd.s / hd.c;
    const sc2 hmp = sc_of(0.5 * (mu - ps)), hnp = sc_of(0.5 * (nu + ps));
    const double Amu = atan2(thd * hmp.c * xi.s, thd * hmp.c * xi.c + hmp.s);
    const double Anu = atan2(thd * hnp.s * xi.s, thd * hnp.s * xi.c + hnp.c);
    const sc2 t1 = sc_of(0.5 * (mu - ps) - 0.5 * (nu + ps)), t2 = sc_of(0.5 * g.kappa);
    const double W = atan2(sd.s * t2.s * xi.s, t2.c + sd.s * t1.c * xi.c + sd.c * t1.s);
    const sc2 t3 = sc_of(delta - ps);
    const double D = 1.0 / (t3.s * t3.s + sd.s * sps.s * (1.0 - xi.c) * (t3.c + csig));
    const double G = sps.c * (sd.s * csig * xi.c + sd.c * cchi - sd.s * sd.s / sps.s);
    const double mpsi = sign_ref(xi.s * sps.s), mdel = sign_ref(xi.s * sd.s);
    if (fabs(xi.s) < kEps && 1.0 - fabs(csig) < 0.5 * kEps2 && fabs(sps.s) > kEps) {
        const double ara = arg_ref(sin(0.5 * (nu + ps)) * csig);
        const double arb = arg_ref(cos(0.5 * (mu - ps)) * csig);
        qt = 2.0 * mpsi * csig * xi.c / (sk * sps.s) * (smu.s * g.nupsi.s * ara - snu.s * g.mupsi.s * arb);
        qp = 0.5 * (1.0 - log(2.0)) - 0.5 * log((1.0 - csig * smu.c) * (1.0 + csig * snu.c) / sk) +
             csig * (smu.s - snu.s + 0.5 * sin(mu - nu) * Lam2) / sk;
        return;
    }
    const double gens = 0.5 * (3.0 - log(2.0)) +
                        (smu.s * snu.s / sk) * ((lla - lth) * sps.c / sps.s +
                                                D * (Lam1 * sd.s * ceta / sps.s + Lam2 * cchi - 2.0 * W * sd.s * xi.s -
                                                     G * (g.lsnu - g.lsmu))) -
                        (smu.c * snu.s * (lla - g.lsmu) + smu.s * snu.c * (lth - g.lsnu)) / sk - 0.5 * (g.lsmu + g.lsnu - log(sk));
    if (fabs(xi.s) < kEps && fabs(sps.s) > kEps) {
        const double are = arg_ref(sin(0.5 * (nu + mu)) + sin(0.5 * (mu - nu) - ps + delta * xi.c));
        const double arc = arg_ref(1.0 / tan(0.5 * (nu + ps)) + tan(0.5 * delta) * xi.c);
        const double ard = arg_ref(tan(0.5 * (mu - ps)) + tan(0.5 * delta) * xi.c);
        qt = 2.0 * mdel * (sd.s * smu.s * snu.s / cchi * xi.c * are + smu.s * g.nupsi.s * arc - snu.s * g.mupsi.s * ard) /
             (sk * sps.s);
        qp = gens;
        return;
    }
    if (fabs(sin(ps)) < kEps) {
        if (fabs(delta) > kEps) {
            qt = 2.0 * (smu.s * snu.s * (W * sd.c * xi.c - 0.5 * (Lam1 - Lam2 * csig) * xi.s) / sd.s +
                        (Anu + mdel * arg_ref(sin(0.5 * (nu + ps)))) * smu.s * snu.c +
                        (Amu + mdel * arg_ref(cos(0.5 * (mu - ps)))) * smu.c * snu.s) /
                 sk;
            qp = 0.5 * (3.0 - log(2.0)) - 0.5 * (log((1.0 + cla) * (1.0 + cth) / sk) - sin(mu - nu) / sk * Lam1) -
                 smu.s * snu.s * ((Lam1 * sd.c - Lam2 * sps.c) * xi.c + 2.0 * W * xi.s) / (sk * sd.s);
        } else {
            qt = 2.0 * arg_ref(sps.c);
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

// integrateSingularPartSimple (:674-780); Ti/Tj rotated so that the shared vertex comes first
__device__ inline void closed_vertex(Tri Ti, Tri Tj, d3 ni, d3 nj, double Si, d3 &psi, double &th)
{
    const d3 IA = Ti.a, IB = Ti.b, IC = Ti.c, JA = Tj.a, JB = Tj.b, JC = Tj.c;
    const d3 ta = unit(JA - JC), tb = unit(JB - JA);
    double dA, dB;
    const d3 e = vertex_direction(ni, nj, ta, tb, dA, dB);
    const double xi = atan2(dot(cross(ni, nj), e), dot(ni, nj));
    const sc2 sdA = sc_of(dA), sdB = sc_of(dB);
    VtxAngles g;
    g.xi = sc_of(xi);
    const d3 s = IC - IB;
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
    g.nupsi = sc_of(g.nu_a + g.psi_a);
    g.mupsi = sc_of(g.mu_a - g.psi_a);
    double q[2][2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const sc2 d = h == 0 ? sdA : sdB;
        const double csig = d.s * g.psi.s * g.xi.c + d.c * g.psi.c;
        const double cchi = d.s * g.psi.c * g.xi.c - d.c * g.psi.s;
        const double ceta = d.c * g.psi.s * g.xi.c - d.s * g.psi.c;
        const double cth = d.s * g.nupsi.s * g.xi.c + d.c * g.nupsi.c;
        const double cla = d.s * g.mupsi.s * g.xi.c - d.c * g.mupsi.c;
        q_vertex(g, h == 0 ? dA : dB, d, cla, cth, ceta, csig, cchi, q[h][0], q[h][1]);
    }
    psi = Si * (q[0][1] * ta + q[1][1] * tb);
    th = (fabs(xi) < kEps) ? 0.0 : (Si * (q[0][0] - q[1][0]));
}

// ------------------------------------------------------------------ potential helpers
// potential of K_j seen from x (no 1/4pi): sum_e t_e L_e - d Theta
__device__ __forceinline__ double potential_inner(d3 x, const PanelJ &K, const FarCtx &F)
{
    d3 psi;
    double th, pot;
    far_integrand(x, K, F, psi, th, pot);
    return pot;
}

// common-edge potential: subtracted s ln s term along the shared edge (sigma = -2 c s ln(s/h),
// integral over K_i = (5/9) c S_i h)
struct PotEdge {
    d3 P1, m_in;
    double c, h;
};
__device__ __forceinline__ double pot_edge_sigma(d3 x, const PotEdge &p)
{
    const double s = dot(x - p.P1, p.m_in);
    return s > 0.0 ? -2.0 * p.c * s * log(s / p.h) : 0.0;
}

} // namespace i2
