// i2_rules.cuh -- per-pair integration rules shared by the forward kernels (R = double) and
// the adjoint kernels (R = dual number): the potential of common-edge / common-vertex pairs
// (graded Duffy rule, s ln s term of the shared edge, cells of the adaptive rule), the self-pair
// potential and the finalisation J = (Theta n_j + Psi x n_j)/4pi.
#pragma once

#include "i2_device.cuh"

namespace i2 {

// pair classes (values of the reference's neighbour_type_enum, src/Mesh3d.cuh:18-23, plus self)
enum { kVertex = 0, kEdge = 1, kFar = 2, kSelf = 3 };

// ------------------------------------------------------------------ potential of adjacent pairs
// s ln s term along the shared edge (Ti, Tj rotated: Ti.a / Tj.a off the shared edge); returns
// its integral over K_i, (5/9) c S_i h
template <class R>
__device__ __forceinline__ R make_pot_edge(const TriT<R> &Ti, const TriT<R> &Tj, const PanelJT<R> &K, R Si, PotEdgeT<R> &pe)
{
    const V3<R> tau = unit(Tj.c - Tj.b), m = cross(tau, K.n), w = Ti.a - Tj.b;
    const V3<R> perp = w - dot(w, tau) * tau;
    pe.P1 = Tj.b;
    pe.h = norm(perp);
    pe.m_in = (1.0 / pe.h) * perp;
    pe.c = -dot(m, pe.m_in);
    return (5.0 / 9.0) * pe.c * Si * pe.h;
}

// graded Duffy rule over the pieces of K_i (Ti rotated): one piece with apex at the shared
// vertex (vertex class) or two pieces with apexes at the ends of the shared edge (edge class);
// the edge class integrates g - sigma
template <int CLS, class R>
__device__ R duffy_total(const TriT<R> &Ti, const PanelJT<R> &K, const FarCtxT<R> &F, const PotEdgeT<R> &pe, const double *uu,
                         const double *uw, int nu, const double *vv, const double *vw, int nv)
{
    R total = 0.0;
    const int npieces = CLS == kEdge ? 2 : 1;
    for (int piece = 0; piece < npieces; ++piece) {
        V3<R> Vx, B, Cc;
        if (CLS == kVertex) { Vx = Ti.a; B = Ti.b; Cc = Ti.c; }
        else {
            const V3<R> M = 0.5 * (Ti.b + Ti.c);
            if (piece == 0) { Vx = Ti.b; B = M; Cc = Ti.a; }
            else { Vx = Ti.c; B = Ti.a; Cc = M; }
        }
        const V3<R> eB = B - Vx, eC = Cc - Vx, dA = Vx - K.A, dB = Vx - K.B, dC = Vx - K.C;
        const R area2 = norm(cross(eB, eC));
        R acc = 0.0;
#pragma unroll 1
        for (int a = 0; a < nu; ++a) {
            const double u = uu[a];
            R row = 0.0;
#pragma unroll 1
            for (int b = 0; b < nv; ++b) {
                const V3<R> w = u * ((1.0 - vv[b]) * eB + vv[b] * eC);
                V3<R> psi;
                R th, g;
                far_integrand_o(dA + w, dB + w, dC + w, K, F, psi, th, g);
                if (CLS == kEdge) g -= pot_edge_sigma(Vx + w, pe);
                row += vw[b] * g;
            }
            acc += uw[a] * u * row;
        }
        total += area2 * acc;
    }
    return total;
}

// the same rule's points p = first, first + step, ... of the flattened (piece, radial, angular)
// list, so that a warp can share one rule (step 32)
template <int CLS, class R>
__device__ R duffy_partial(const TriT<R> &Ti, const PanelJT<R> &K, const FarCtxT<R> &F, const PotEdgeT<R> &pe, const double *uu,
                           const double *uw, int nu, const double *vv, const double *vw, int nv, int first, int step)
{
    const int npieces = CLS == kEdge ? 2 : 1;
    const int per = nu * nv;
    R total = 0.0;
#pragma unroll 1
    for (int p = first; p < npieces * per; p += step) {
        const int piece = p / per, q = p - piece * per, a = q / nv, b = q - a * nv;
        V3<R> Vx, B, Cc;
        if (CLS == kVertex) { Vx = Ti.a; B = Ti.b; Cc = Ti.c; }
        else {
            const V3<R> M = 0.5 * (Ti.b + Ti.c);
            if (piece == 0) { Vx = Ti.b; B = M; Cc = Ti.a; }
            else { Vx = Ti.c; B = Ti.a; Cc = M; }
        }
        const V3<R> eB = B - Vx, eC = Cc - Vx;
        const double u = uu[a];
        const V3<R> w = u * ((1.0 - vv[b]) * eB + vv[b] * eC);
        V3<R> psi;
        R th, g;
        far_integrand_o((Vx - K.A) + w, (Vx - K.B) + w, (Vx - K.C) + w, K, F, psi, th, g);
        if (CLS == kEdge) g -= pot_edge_sigma(Vx + w, pe);
        total += (uw[a] * u * vw[b]) * norm(cross(eB, eC)) * g;
    }
    return total;
}

// one cell of the adaptive rule: graded Duffy with the shared vertex (in slot `corner`) as apex,
// or the 13-point rule; offsets to K_j's vertices from vertex differences
template <int CLS, class R>
__device__ R pot_cell(const TriT<R> &T, int corner, const PanelJT<R> &K, const FarCtxT<R> &F, const PotEdgeT<R> &pe,
                      const QuadTables &Q)
{
    R acc = 0.0;
    if (corner >= 0) {
        const V3<R> Vx = corner == 0 ? T.a : (corner == 1 ? T.b : T.c);
        const V3<R> B = corner == 0 ? T.b : (corner == 1 ? T.c : T.a);
        const V3<R> Cc = corner == 0 ? T.c : (corner == 1 ? T.a : T.b);
        const V3<R> eB = B - Vx, eC = Cc - Vx, dA = Vx - K.A, dB = Vx - K.B, dC = Vx - K.C;
        const R area2 = norm(cross(eB, eC));
        for (int a = 0; a < Q.nu; ++a) {
            const double u = Q.du_u[a];
            R row = 0.0;
            for (int b = 0; b < Q.nv; ++b) {
                const double v = Q.dv_v[b];
                const V3<R> w = u * ((1.0 - v) * eB + v * eC);
                V3<R> psi;
                R th, g;
                far_integrand_o(dA + w, dB + w, dC + w, K, F, psi, th, g);
                if (CLS == kEdge) g -= pot_edge_sigma(Vx + w, pe);
                row += Q.dv_w[b] * g;
            }
            acc += Q.du_w[a] * u * row;
        }
        return area2 * acc;
    }
    const V3<R> aA = T.a - K.A, bA = T.b - K.A, cA = T.c - K.A;
    const V3<R> aB = T.a - K.B, bB = T.b - K.B, cB = T.c - K.B;
    const V3<R> aC = T.a - K.C, bC = T.b - K.C, cC = T.c - K.C;
    for (int g = 0; g < Q.npts; ++g) {
        const V3<R> oa = Q.L1[g] * aA + Q.L2[g] * bA + Q.L3[g] * cA;
        const V3<R> ob = Q.L1[g] * aB + Q.L2[g] * bB + Q.L3[g] * cB;
        const V3<R> oc = Q.L1[g] * aC + Q.L2[g] * bC + Q.L3[g] * cC;
        V3<R> psi;
        R th, gx;
        far_integrand_o(oa, ob, oc, K, F, psi, th, gx);
        if (CLS == kEdge) gx -= pot_edge_sigma(oa + K.A, pe);
        acc += Q.w[g] * gx;
    }
    return 0.5 * norm(cross(T.b - T.a, T.c - T.a)) * acc;
}

// corner slot of child k when the parent's corner is in slot c (the shared vertex moves to slot 1)
__device__ __forceinline__ int child_corner(int parent_corner, int k)
{
    if (parent_corner < 0 || k == 3) return -1;
    const int want = parent_corner == 1 ? 0 : (parent_corner == 2 ? 1 : 2);
    return k == want ? 1 : -1;
}

// ------------------------------------------------------------------ self pairs
// J(K_i, K_i): tangential part 0 by antisymmetry; normal part 0 (principal value) or the
// one-sided limit +-(1/4pi) 2 pi S_i n_i.  Potential: with d = 0 the inner potential is
// sum_e t_e L_e; per edge, int_K t_e L_e dS = int_e dl_y int_0^pi sin(phi) R(phi,y)^2/2 dphi
// with the phi integral in closed form on the two sides the ray can hit and the edge integral
// by graded Gauss-Legendre on the pieces on either side of the foot of the altitude.
// ln tan(u/2) from sin u and cos u, in the form that does not cancel on either half of (0, pi)
template <class R>
__device__ __forceinline__ R log_tan_half(R s, R c)
{
    return c >= 0.0 ? R(log(s / (1.0 + c))) : R(log((1.0 - c) / s));
}

// one side of the phi integral, (a^2 sin^2(alpha) / 2) [cos(alpha) ln tan(u/2) + sin(alpha) / sin(u)]
// from u = alpha to u1; sin, cos of alpha and the bracket's value at alpha (F0) come from the caller
template <class R>
__device__ __forceinline__ R ray_side(R a, R sa, R ca, R F0, R u1)
{
    R su, cu;
    sincos(u1, &su, &cu);
    const R F1 = ca * log_tan_half(su, cu) + sa / su;
    return 0.5 * a * a * sa * sa * (F1 - F0);
}

// piece `piece` (0 or 1) of edge e of the self-pair rule for the triangle P[0..2]: the edge
// P[e] -> P[e+1] is split at the foot of the altitude from the third vertex (where the angle to it
// swings fastest) when the foot lies inside the edge; otherwise piece 0 is the whole edge and
// piece 1 is empty
template <class R>
__device__ R self_potential_piece_unit(const V3<R> P[3], int e, int piece, const QuadTables &Q)
{
    const V3<R> P1 = P[e], P2 = P[(e + 1) % 3], P3 = P[(e + 2) % 3];
    const R L = norm(P2 - P1);
    const V3<R> tau = (1.0 / L) * (P2 - P1);
    const R foot = dot(P3 - P1, tau);
    const bool split = foot > 1e-12 * L && foot < (1.0 - 1e-12) * L;
    if (piece == 1 && !split) return R(0.0);
    const R al1 = angle_ref(P2 - P1, P3 - P1);
    const R al2 = angle_ref(P1 - P2, P3 - P2);
    // per-side constants of the phi integral (the lower limit u = alpha)
    R s1, c1, s2, c2;
    sincos(al1, &s1, &c1);
    sincos(al2, &s2, &c2);
    const R F01 = c1 * log_tan_half(s1, c1) + 1.0, F02 = c2 * log_tan_half(s2, c2) + 1.0;
    const R lo = split && piece == 1 ? foot : R(0.0);
    const R span = split ? (piece == 0 ? foot : R(L - foot)) : L;
    R part = 0.0;
#pragma unroll 1
    for (int k = 0; k < Q.nself; ++k) {
        const R b = lo + span * Q.sx[k], a = L - b;
        const V3<R> y = P1 + b * tau;
        const R phis = angle_ref(tau, P3 - y);
        part += Q.sw[k] * (ray_side(a, s2, c2, F02, R(phis + al2)) + ray_side(b, s1, c1, F01, R((kPi - phis) + al1)));
    }
    return span * part;
}

// the same, scale-invariant: evaluated on the triangle scaled by the power of two 2^k that
// brings its longest edge into [0.5, 1) (angle_ref's threshold is absolute), the result scaled
// back by 2^-3k (the potential of a pair of areas is a length cubed); exact at ordinary scales
template <class R>
__device__ R self_potential_piece(const V3<R> P[3], int e, int piece, const QuadTables &Q)
{
    const double lmax = fmax(fmax((double)value_of(norm(P[1] - P[0])), (double)value_of(norm(P[2] - P[1]))),
                             (double)value_of(norm(P[0] - P[2])));
    const double s = pow2_normaliser(lmax);
    const V3<R> Ps[3] = {s * P[0], s * P[1], s * P[2]};
    return (1.0 / (s * s * s)) * self_potential_piece_unit(Ps, e, piece, Q);
}

// int_K int_K 1/|x - y| in closed form: (4 S^2 / 3) sum_s ln(p / (p - 2 s)) / s over the sides s,
// p the perimeter.  Scaling K about the vertex opposite an edge e moves only e, so Euler's relation
// for this integral (homogeneous of degree 3) gives F = (2 H_e / 3) int_e phi ds, H_e the height
// over e and phi the potential of K (both integrals' domains move).  On e, phi is the sum over the
// other two edges of t L (distance to the edge line times the edge log); along e these integrate
// in closed form because d/du ln((r + u + c) / (r + u - c)) = -c / (u r) (u the distance from the
// edge's end, r the distance to its far end, c its length), and the logs combine into the
// symmetric form.  Only the longest side's p - 2s can cancel (a flat cell): the smallest of the
// three is taken from Heron's 16 S^2 = p prod_s (p - 2 s), S from the cross product.  No absolute
// threshold: exact at every scale.
template <class R>
__device__ R self_potential_closed(const V3<R> P[3])
{
    const R a = norm(P[2] - P[1]), b = norm(P[0] - P[2]), c = norm(P[1] - P[0]);
    const V3<R> cr = cross(P[1] - P[0], P[2] - P[0]);
    const R s4 = dot(cr, cr);  // (2S)^2
    const R p = a + b + c;
    R da = (b + c) - a, db = (c + a) - b, dc = (a + b) - c;
    if (value_of(da) <= value_of(db) && value_of(da) <= value_of(dc)) da = 4.0 * s4 / (p * db * dc);
    else if (value_of(db) <= value_of(dc)) db = 4.0 * s4 / (p * da * dc);
    else dc = 4.0 * s4 / (p * da * db);
    return (1.0 / 3.0) * s4 * (log(p / da) / a + log(p / db) / b + log(p / dc) / c);
}

// int_K int_K 1/|x - y| (no 1/4pi) of the triangle (P0, P1, P2): the closed form when the rule
// has no points (Q.nself == 0, the default), else the edge rule above
template <class R>
__device__ R self_potential(V3<R> P0, V3<R> P1v, V3<R> P2v, const QuadTables &Q)
{
    const V3<R> P[3] = {P0, P1v, P2v};
    if (Q.nself == 0) return self_potential_closed(P);
    R total = 0.0;
#pragma unroll 1
    for (int e = 0; e < 3; ++e) total += self_potential_piece(P, e, 0, Q) + self_potential_piece(P, e, 1, Q);
    return total;
}

// ------------------------------------------------------------------ finalisation
// J = (Theta n_j + Psi x n_j)/4pi, with the p-fix of the common-vertex class
// (evaluatorJ3DK.cu:224-264); the shift 2 p 2 pi S_i is a piecewise constant in the geometry
template <class R>
__device__ __forceinline__ V3<R> finalize_j(int cls, V3<R> psi, R th, V3<R> nj, R Si)
{
    if (cls == kVertex) {
        int p = 0;
        const R ref = kTwoPi * Si;
        if (th > ref) p = -((int)trunc(value_of((th - ref) / (2.0 * ref))) + 1);
        else if (th < -ref) p = ((int)trunc(value_of((-ref - th) / (2.0 * ref))) + 1);
        th = th + 2.0 * p * ref;
    }
    return kInv4Pi * (th * nj + cross(psi, nj));
}

} // namespace i2
