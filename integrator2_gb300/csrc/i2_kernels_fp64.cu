// i2_kernels_fp64.cu -- plain FP64 form of the pair-integral path (sm_103a).
//
// Kernel chain per pair class (all launches on one stream, no host synchronisation, so the
// whole chain can be captured into a CUDA graph):
//   k_prepare_panels           once per mesh: 256-byte panel record per cell
//   k_singular<EDGE|VERTEX>    closed-form singular parts + graded-Duffy potential, 1 thread/pair
//   k_self                     self pairs (J convention + closed-form-in-angle potential)
//   k_level<CLS>(L)            regular part at refinement level L; 4^L sub-cells per pair spread
//                              over min(4^L, 32) lanes, warp-shuffle reduction; in adaptive mode
//                              it also runs the convergence test and appends unconverged pairs
//                              to the next level's active list (device-side counter)
//   k_finalize<CLS>            kept level, singular part, J = (Theta n_j + Psi x n_j)/4pi
#include "i2_engine.h"
#include "i2_finalize.cuh"

namespace i2 {

// ------------------------------------------------------------------ mesh preparation
__global__ void k_prepare_panels(int nc, const double *__restrict__ V, const int *__restrict__ C, Panel *__restrict__ out)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    const int ia = C[3 * c], ib = C[3 * c + 1], ic = C[3 * c + 2];
    const d3 A = mk(V[3 * ia], V[3 * ia + 1], V[3 * ia + 2]);
    const d3 B = mk(V[3 * ib], V[3 * ib + 1], V[3 * ib + 2]);
    const d3 Cc = mk(V[3 * ic], V[3 * ic + 1], V[3 * ic + 2]);
    // src/Mesh3d.cu:23-71: n = unit((B-A)x(C-A)), S = |(B-A)x(C-A)|/2
    const d3 cr = cross(B - A, Cc - A);
    const d3 n = unit(cr);
    const double S = norm(cr) * 0.5;
    const d3 ea = Cc - B, eb = A - Cc, ec = B - A;
    const double la = norm(ea), lb = norm(eb), lc = norm(ec);
    const d3 ta = unit(ea), tb = unit(eb), tc = unit(ec);
    const d3 ctr = 0.3333333333333333 * (A + B + Cc);
    // largest cosine of the cell's three angles (a sliver has one close to 1)
    const double cmax = fmax(dot(tc, -1.0 * tb), fmax(dot(ta, -1.0 * tc), dot(tb, -1.0 * ta)));
    Panel p;
    p.v[0] = make_double4_32a(A.x, A.y, A.z, S);
    p.v[1] = make_double4_32a(B.x, B.y, B.z, 2.0 * S);
    p.v[2] = make_double4_32a(Cc.x, Cc.y, Cc.z, cmax);
    p.v[3] = make_double4_32a(n.x, n.y, n.z, 0.0);
    p.v[4] = make_double4_32a(ta.x, ta.y, ta.z, la);
    p.v[5] = make_double4_32a(tb.x, tb.y, tb.z, lb);
    p.v[6] = make_double4_32a(tc.x, tc.y, tc.z, lc);
    p.v[7] = make_double4_32a(ctr.x, ctr.y, ctr.z, fmax(la, fmax(lb, lc)));
    out[c] = p;
}

// ------------------------------------------------------------------ helpers
__device__ __forceinline__ Tri rotate(Tri t, int s)
{
    if (s == 0) return t;
    if (s == 1) return Tri{t.b, t.c, t.a};
    return Tri{t.c, t.a, t.b};
}

__device__ __forceinline__ acc5 shfl_xor5(acc5 a, int off)
{
    acc5 r;
    r.px = __shfl_xor_sync(0xffffffffu, a.px, off);
    r.py = __shfl_xor_sync(0xffffffffu, a.py, off);
    r.pz = __shfl_xor_sync(0xffffffffu, a.pz, off);
    r.th = __shfl_xor_sync(0xffffffffu, a.th, off);
    r.pot = __shfl_xor_sync(0xffffffffu, a.pot, off);
    return r;
}



// Runge criterion of the reference on the regular-part sums (evaluator3d.cu:76-99 with
// divide()/norm1() of cuda_math.cuh:270-300)
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

// ------------------------------------------------------------------ regular part, one level
template <int CLS>
__global__ void __launch_bounds__(128) k_level(ClassArgs A, QuadTables Q, int level, int mode, double tol, int kmax)
{
    const int nsub = 1 << (2 * level);
    const int G = nsub < 32 ? nsub : 32;          // lanes per pair
    const int per_lane = nsub / G;                // sub-cells per lane
    const bool listed = A.act_in != nullptr;
    const int count = listed ? *A.cnt_in : A.n;
    const long long total = (long long)count * G;
    const long long total_r = (total + 31) & ~31LL;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const double sub_scale = ldexp(1.0, -2 * level);  // measure of a sub-cell / measure of K_i
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total_r; idx += stride) {
        const bool valid = idx < total;
        const int slot = (int)(idx / G);
        const int lane_g = (int)(idx % G);
        const int t = valid ? (listed ? A.act_in[slot] : slot) : 0;
        acc5 acc = zero5();
        int2 pr = make_int2(0, 0);
        if (valid) {
            pr = A.pairs[t];
            const PanelJ K = load_panel(A.panels, pr.y);
            const Tri Ti = load_tri(A.panels, pr.x);
            const double Ssub = A.panels[pr.x].v[0].w * sub_scale;
            FarCtx F;
            EdgeCtx E;
            VertexCtx Vx;
            if (CLS == kFar) F = make_far_ctx(K);
            if (CLS == kEdge || CLS == kVertex) {
                const int3 ci = A.cells[pr.x], cj = A.cells[pr.y];
                int si, sj;
                if (CLS == kEdge) {
                    shifts_edge(ci, cj, si, sj);
                    E = make_edge_ctx(K, sj);
                } else {
                    shifts_vertex(ci, cj, si, sj);
                    const double4_32a ni = A.panels[pr.x].v[3];
                    Vx = make_vertex_ctx(K, sj, mk(ni.x, ni.y, ni.z), A.panels[pr.x].v[0].w);
                }
            }
            for (int s = lane_g * per_lane; s < (lane_g + 1) * per_lane; ++s) {
                const Tri T = subcell(Ti, level, s);
                acc5 cell = zero5();
#pragma unroll 1
                for (int g = 0; g < Q.npts; ++g) {
                    const d3 x = Q.L1[g] * T.a + Q.L2[g] * T.b + Q.L3[g] * T.c;
                    d3 psi;
                    double th, pot = 0.0;
                    if (CLS == kFar) far_integrand(x, K, F, psi, th, pot);
                    else if (CLS == kEdge) edge_integrand(x, K, E, psi, th);
                    else vertex_integrand(x, K, Vx, psi, th);
                    axpy5(cell, Q.w[g], psi, th, pot);
                }
                acc.px += Ssub * cell.px;
                acc.py += Ssub * cell.py;
                acc.pz += Ssub * cell.pz;
                acc.th += Ssub * cell.th;
                acc.pot += Ssub * cell.pot;
            }
        }
        // segmented butterfly over the G lanes of this pair (groups never straddle a warp)
        for (int off = 1; off < G; off <<= 1) {
            const acc5 o = shfl_xor5(acc, off);
            acc.px += o.px; acc.py += o.py; acc.pz += o.pz; acc.th += o.th; acc.pot += o.pot;
        }
        if (!valid || lane_g != 0) continue;
        double *cur = A.cur + 5 * (long long)t;
        if (mode == kFixed || level == 0) {
            store5(cur, acc);
            continue;
        }
        const acc5 prev = load5(cur);
        store5(cur, acc);
        bool unconv;
        if (mode == kAdaptiveCompat) {
            unconv = runge_unconverged(acc, prev, Q.pow2p);
        } else {
            const double4_32a nj4 = A.panels[pr.y].v[3];
            const d3 nj = mk(nj4.x, nj4.y, nj4.z);
            const double Si = A.panels[pr.x].v[0].w;
            d3 spsi = mk(0, 0, 0);
            double sth = 0.0;
            if (CLS != kFar) {
                const double *sg = A.sing + 4 * (long long)t;
                spsi = mk(sg[0], sg[1], sg[2]);
                sth = sg[3];
            }
            const d3 Jc = finalize_j(CLS, mk(acc.px, acc.py, acc.pz) + spsi, acc.th + sth, nj, Si);
            const d3 dJ = kInv4Pi * ((acc.th - prev.th) * nj + cross(mk(acc.px - prev.px, acc.py - prev.py, acc.pz - prev.pz), nj));
            unconv = norm(dJ) > tol * norm(Jc);
            if (CLS == kFar) unconv = unconv || fabs(acc.pot - prev.pot) > tol * fabs(acc.pot);
        }
        atomicMax(A.maxlev, level);
        if (!unconv || level >= kmax) {
            A.stop[t] = level;
            store5(A.fin_a + 5 * (long long)t, acc);
            store5(A.fin_b + 5 * (long long)t, prev);
        } else {
            const int pos = atomicAdd(A.cnt_out, 1);
            A.act_out[pos] = t;
        }
    }
}

// ------------------------------------------------------------------ potential of adjacent pairs
// s ln s term along the shared edge (Ti, Tj rotated: Ti.a / Tj.a off the shared edge); returns
// its integral over K_i, (5/9) c S_i h
__device__ __forceinline__ double make_pot_edge(const Tri &Ti, const Tri &Tj, const PanelJ &K, double Si, PotEdge &pe)
{
    const d3 tau = unit(Tj.c - Tj.b), m = cross(tau, K.n), w = Ti.a - Tj.b;
    const d3 perp = w - dot(w, tau) * tau;
    pe.P1 = Tj.b;
    pe.h = norm(perp);
    pe.m_in = (1.0 / pe.h) * perp;
    pe.c = -dot(m, pe.m_in);
    return (5.0 / 9.0) * pe.c * Si * pe.h;
}

// graded Duffy rule over the pieces of K_i (Ti rotated): one piece with apex at the shared
// vertex (vertex class) or two pieces with apexes at the ends of the shared edge (edge class);
// the edge class integrates g - sigma
template <int CLS>
__device__ double duffy_total(const Tri &Ti, const PanelJ &K, const FarCtx &F, const PotEdge &pe, const double *uu,
                              const double *uw, int nu, const double *vv, const double *vw, int nv)
{
    double total = 0.0;
    const int npieces = CLS == kEdge ? 2 : 1;
    for (int piece = 0; piece < npieces; ++piece) {
        d3 Vx, B, Cc;
        if (CLS == kVertex) { Vx = Ti.a; B = Ti.b; Cc = Ti.c; }
        else {
            const d3 M = 0.5 * (Ti.b + Ti.c);
            if (piece == 0) { Vx = Ti.b; B = M; Cc = Ti.a; }
            else { Vx = Ti.c; B = Ti.a; Cc = M; }
        }
        const d3 eB = B - Vx, eC = Cc - Vx, dA = Vx - K.A, dB = Vx - K.B, dC = Vx - K.C;
        const double area2 = norm(cross(eB, eC));
        double acc = 0.0;
#pragma unroll 1
        for (int a = 0; a < nu; ++a) {
            const double u = uu[a];
            double row = 0.0;
#pragma unroll 1
            for (int b = 0; b < nv; ++b) {
                const d3 w = u * ((1.0 - vv[b]) * eB + vv[b] * eC);
                d3 psi;
                double th, g;
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

// ------------------------------------------------------------------ singular parts (edge/vertex)
template <int CLS>
__global__ void __launch_bounds__(128) k_singular(ClassArgs A, QuadTables Q)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= A.n) return;
    const int2 pr = A.pairs[t];
    const int3 ci = A.cells[pr.x], cj = A.cells[pr.y];
    const PanelJ K = load_panel(A.panels, pr.y);
    const Tri Ti0 = load_tri(A.panels, pr.x);
    const Tri Tj0 = Tri{K.A, K.B, K.C};
    const double4_32a ni4 = A.panels[pr.x].v[3];
    const d3 ni = mk(ni4.x, ni4.y, ni4.z);
    const double Si = A.panels[pr.x].v[0].w;
    int si, sj;
    if (CLS == kEdge) shifts_edge(ci, cj, si, sj);
    else shifts_vertex(ci, cj, si, sj);
    const Tri Ti = rotate(Ti0, si), Tj = rotate(Tj0, sj);
    d3 psi;
    double th;
    if (CLS == kEdge) closed_edge(Ti, Tj, ni, K.n, Si, psi, th);
    else closed_vertex(Ti, Tj, ni, K.n, Si, psi, th);
    double *sg = A.sing + 4 * (long long)t;
    sg[0] = psi.x; sg[1] = psi.y; sg[2] = psi.z; sg[3] = th;

    // potential: tier 1 of the tiered rule (graded Duffy, main and lower-order check)
    const FarCtx F = make_far_ctx(K);
    PotEdge pe;
    const double sig = CLS == kEdge ? make_pot_edge(Ti, Tj, K, Si, pe) : 0.0;
    const double pm = duffy_total<CLS>(Ti, K, F, pe, Q.du_u, Q.du_w, Q.nu, Q.dv_v, Q.dv_w, Q.nv) + sig;
    A.padj[t] = kInv4Pi * pm;
    if (A.hard_list) {
        // hard pair (folded: normals more than 60 degrees apart, or a cell with an angle below 10
        // degrees) -> adaptive rule; main and check rules disagree -> higher-order rule
        const double c10 = 0.98480775301220806;
        if (dot(ni, K.n) < 0.5 || A.panels[pr.x].v[2].w > c10 || A.panels[pr.y].v[2].w > c10) {
            A.hard_list[atomicAdd(A.hard_cnt, 1)] = t;
        } else {
            const double pl = duffy_total<CLS>(Ti, K, F, pe, Q.lo_u, Q.lo_uw, Q.lo_nu, Q.lo_v, Q.lo_vw, Q.lo_nv) + sig;
            if (fabs(pm - pl) > A.tier_tol * fabs(pm)) A.tier2_list[atomicAdd(A.tier2_cnt, 1)] = t;
        }
    }
}

// tier 2: higher-order Duffy rule; pairs where it still disagrees with the main rule go on to
// the adaptive rule (tier 3)
template <int CLS>
__global__ void __launch_bounds__(128) k_pot_tier2(ClassArgs A, QuadTables Q)
{
    const int count = *A.tier2_cnt;
    for (int h = blockIdx.x * blockDim.x + threadIdx.x; h < count; h += gridDim.x * blockDim.x) {
        const int t = A.tier2_list[h];
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
        const double ph = duffy_total<CLS>(Ti, K, F, pe, Q.hi_u, Q.hi_uw, Q.hi_nu, Q.hi_v, Q.hi_vw, Q.hi_nv) + sig;
        const double pm = A.padj[t] * (4.0 * kPi);
        A.padj[t] = kInv4Pi * ph;
        if (fabs(ph - pm) > A.tier_tol * fabs(ph)) A.hard_list[atomicAdd(A.hard_cnt, 1)] = t;
    }
}

// ------------------------------------------------------------------ hard adjacent pairs: adaptive potential
// Breadth-first over the cells of ALL hard pairs at once: depth d holds a device list of cells
// (hard-list slot, path, depth, corner slot, value); one thread takes one cell, integrates its
// four children and either accepts their sum (|sum - value| <= tol |P| 2^-d, or d at the depth
// cap) or appends the children to depth d + 1's list.  Cells that hold a shared vertex (always
// in slot 1 of a corner child) use the graded Duffy rule with that vertex as apex, all others
// the 13-point rule; point offsets to K_j's vertices are formed from vertex differences.  The
// whole GPU works on every depth, so one pair that needs thousands of cells no longer runs
// alone on one SM.  Accepted sums are added as 64-bit fixed point (2^40 units per |P| + |sigma
// integral|), so the result does not depend on the order of the atomics.
template <int CLS>
__device__ double pot_cell(const Tri &T, int corner, const PanelJ &K, const FarCtx &F, const PotEdge &pe, const QuadTables &Q)
{
    double acc = 0.0;
    if (corner >= 0) {
        const d3 Vx = corner == 0 ? T.a : (corner == 1 ? T.b : T.c);
        const d3 B = corner == 0 ? T.b : (corner == 1 ? T.c : T.a);
        const d3 Cc = corner == 0 ? T.c : (corner == 1 ? T.a : T.b);
        const d3 eB = B - Vx, eC = Cc - Vx, dA = Vx - K.A, dB = Vx - K.B, dC = Vx - K.C;
        const double area2 = norm(cross(eB, eC));
        for (int a = 0; a < Q.nu; ++a) {
            const double u = Q.du_u[a];
            double row = 0.0;
            for (int b = 0; b < Q.nv; ++b) {
                const double v = Q.dv_v[b];
                const d3 w = u * ((1.0 - v) * eB + v * eC);
                d3 psi;
                double th, g;
                far_integrand_o(dA + w, dB + w, dC + w, K, F, psi, th, g);
                if (CLS == kEdge) g -= pot_edge_sigma(Vx + w, pe);
                row += Q.dv_w[b] * g;
            }
            acc += Q.du_w[a] * u * row;
        }
        return area2 * acc;
    }
    const d3 aA = T.a - K.A, bA = T.b - K.A, cA = T.c - K.A;
    const d3 aB = T.a - K.B, bB = T.b - K.B, cB = T.c - K.B;
    const d3 aC = T.a - K.C, bC = T.b - K.C, cC = T.c - K.C;
    for (int g = 0; g < Q.npts; ++g) {
        const d3 oa = Q.L1[g] * aA + Q.L2[g] * bA + Q.L3[g] * cA;
        const d3 ob = Q.L1[g] * aB + Q.L2[g] * bB + Q.L3[g] * cB;
        const d3 oc = Q.L1[g] * aC + Q.L2[g] * bC + Q.L3[g] * cC;
        d3 psi;
        double th, gx;
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

struct PotPairCtx {
    Tri Ti;
    PanelJ K;
    FarCtx F;
    PotEdge pe;
    double sig_int, tol_abs, scale;
};

template <int CLS>
__device__ __forceinline__ PotPairCtx pot_pair_ctx(const ClassArgs &A, int t, double tol)
{
    PotPairCtx c;
    const int2 pr = A.pairs[t];
    const int3 ci = A.cells[pr.x], cj = A.cells[pr.y];
    c.K = load_panel(A.panels, pr.y);
    c.Ti = load_tri(A.panels, pr.x);
    c.F = make_far_ctx(c.K);
    c.sig_int = 0.0;
    c.pe = PotEdge{};
    if (CLS == kEdge) {
        int si, sj;
        shifts_edge(ci, cj, si, sj);
        c.sig_int = make_pot_edge(rotate(c.Ti, si), rotate(Tri{c.K.A, c.K.B, c.K.C}, sj), c.K, A.panels[pr.x].v[0].w, c.pe);
    }
    const double p_root = A.padj[t] * (4.0 * kPi);  // tier 1/2 value (regular part + sigma integral)
    c.tol_abs = tol * fabs(p_root);
    const double base = fabs(p_root) + fabs(c.sig_int);
    c.scale = base > 0.0 ? ldexp(1.0, 40) / base : 1.0;
    return c;
}

// seed: the root of every hard pair is split once; its four children form depth 1.  Pairs
// beyond a quarter of the list capacity keep their Duffy value and are counted as overflows.
__device__ __forceinline__ int pot_seeded(const ClassArgs &A) { return min(*A.hard_cnt, A.pot_qcap / 4); }

template <int CLS>
__global__ void __launch_bounds__(128) k_pot_seed(ClassArgs A, QuadTables Q, double tol)
{
    const int count = pot_seeded(A);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        // depth 1 holds the roots' children; the deeper lists start empty (the depth kernels
        // run after this one on the same stream)
        A.pot_qcnt[1] = 4 * count;
        for (int d = 2; d <= kHardMaxDepth + 1; ++d) A.pot_qcnt[d] = 0;
        if (*A.hard_cnt > count) atomicAdd(A.hard_overflow, *A.hard_cnt - count);
    }
    for (int h = blockIdx.x * blockDim.x + threadIdx.x; h < count; h += gridDim.x * blockDim.x) {
        const int t = A.hard_list[h];
        const PotPairCtx c = pot_pair_ctx<CLS>(A, t, tol);
        const int3 ci = A.cells[A.pairs[t].x], cj = A.cells[A.pairs[t].y];
        const int ia[3] = {ci.x, ci.y, ci.z};
        bool shared[3];
        for (int k = 0; k < 3; ++k) shared[k] = (ia[k] == cj.x || ia[k] == cj.y || ia[k] == cj.z);
        A.pot_fx[h] = 0;
        // the root's children 0, 1, 2 hold K_i's slots b, c, a in their slot 1
        for (int k = 0; k < 4; ++k) {
            const int corner = k == 3 ? -1 : (shared[k == 0 ? 1 : (k == 1 ? 2 : 0)] ? 1 : -1);
            const double v = pot_cell<CLS>(child(c.Ti, k), corner, c.K, c.F, c.pe, Q);
            A.pot_q_a[4 * (long long)h + k] = PotCellItem{(unsigned long long)k, v, h, corner};
        }
    }
}

template <int CLS>
__global__ void __launch_bounds__(128) k_pot_depth(ClassArgs A, QuadTables Q, double tol, int depth, const PotCellItem *__restrict__ in,
                                                   PotCellItem *__restrict__ out)
{
    const int count = min(A.pot_qcnt[depth], A.pot_qcap);
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < count; idx += gridDim.x * blockDim.x) {
        const PotCellItem it = in[idx];
        if (it.h < 0) continue;
        const int t = A.hard_list[it.h];
        const PotPairCtx c = pot_pair_ctx<CLS>(A, t, tol);
        const Tri T = subcell(c.Ti, depth, (int)it.path);
        double v[4], sum = 0.0;
        for (int k = 0; k < 4; ++k) {
            v[k] = pot_cell<CLS>(child(T, k), child_corner(it.corner, k), c.K, c.F, c.pe, Q);
            sum += v[k];
        }
        bool accept = fabs(sum - it.val) <= ldexp(c.tol_abs, -depth) || depth >= kHardMaxDepth;
        if (!accept) {
            const int pos = atomicAdd(&A.pot_qcnt[depth + 1], 4);
            if (pos + 4 <= A.pot_qcap) {
                for (int k = 0; k < 4; ++k)
                    out[pos + k] = PotCellItem{(it.path << 2) | (unsigned long long)k, v[k], it.h, child_corner(it.corner, k)};
            } else {
                // list full: keep this cell's sum (counted as an overflow) and blank the slots it
                // was given below the capacity, so the next depth skips them
                for (int k = pos; k < A.pot_qcap && k < pos + 4; ++k) out[k] = PotCellItem{0ull, 0.0, -1, -1};
                atomicAdd(A.hard_overflow, 1);
                accept = true;
            }
        }
        if (accept) atomicAdd(reinterpret_cast<unsigned long long *>(&A.pot_fx[it.h]), (unsigned long long)llrint(sum * c.scale));
    }
}

template <int CLS>
__global__ void __launch_bounds__(128) k_pot_final(ClassArgs A, double tol)
{
    const int count = pot_seeded(A);
    for (int h = blockIdx.x * blockDim.x + threadIdx.x; h < count; h += gridDim.x * blockDim.x) {
        const int t = A.hard_list[h];
        const PotPairCtx c = pot_pair_ctx<CLS>(A, t, tol);
        A.padj[t] = kInv4Pi * ((double)A.pot_fx[h] / c.scale + c.sig_int);
    }
}

template <int CLS>
static void pot_adaptive_chain(const ClassArgs &A, const QuadTables &Q, double tol, int persistent_blocks, cudaStream_t s)
{
    k_pot_seed<CLS><<<persistent_blocks, 128, 0, s>>>(A, Q, tol);
    for (int d = 1; d <= kHardMaxDepth; ++d)
        k_pot_depth<CLS><<<persistent_blocks, 128, 0, s>>>(A, Q, tol, d, d % 2 ? A.pot_q_a : A.pot_q_b, d % 2 ? A.pot_q_b : A.pot_q_a);
    k_pot_final<CLS><<<persistent_blocks, 128, 0, s>>>(A, tol);
}
// ------------------------------------------------------------------ self pairs
// J(K_i, K_i): tangential part 0 by antisymmetry; normal part 0 (principal value) or the
// one-sided limit +-(1/4pi) 2 pi S_i n_i.  Potential: with d = 0 the inner potential is
// sum_e t_e L_e; per edge, int_K t_e L_e dS = int_e dl_y int_0^pi sin(phi) R(phi,y)^2/2 dphi
// with the phi integral in closed form on the two sides the ray can hit and the edge integral
// by graded Gauss-Legendre on the pieces on either side of the foot of the altitude.
__device__ __forceinline__ double ray_side(double a, double alpha, double u1)
{
    double sa, ca;
    sincos(alpha, &sa, &ca);
    const double F1 = ca * log(tan(0.5 * u1)) + sa / sin(u1);
    const double F0 = ca * log(tan(0.5 * alpha)) + 1.0;  // lower limit u = alpha
    return 0.5 * a * a * sa * sa * (F1 - F0);
}

__global__ void __launch_bounds__(128) k_self(ClassArgs A, QuadTables Q, int self_sign)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= A.n) return;
    const int i = A.pairs[t].x;
    const PanelJ K = load_panel(A.panels, i);
    const double th = self_sign == 0 ? 0.0 : (self_sign > 0 ? kTwoPi : -kTwoPi) * K.S;
    const d3 J = kInv4Pi * (th * K.n);
    double *raw = A.raw4 + 4 * (long long)t;
    raw[0] = 0.0; raw[1] = 0.0; raw[2] = 0.0; raw[3] = th;
    double *Jo = A.J3 + 3 * (long long)t;
    Jo[0] = J.x; Jo[1] = J.y; Jo[2] = J.z;
    const d3 P[3] = {K.A, K.B, K.C};
    double total = 0.0;
#pragma unroll 1
    for (int e = 0; e < 3; ++e) {
        const d3 P1 = P[e], P2 = P[(e + 1) % 3], P3 = P[(e + 2) % 3];
        const double L = norm(P2 - P1);
        const d3 tau = (1.0 / L) * (P2 - P1);
        const double al1 = angle_ref(P2 - P1, P3 - P1);
        const double al2 = angle_ref(P1 - P2, P3 - P2);
        // split at the foot of the altitude from P3, where the angle to P3 swings fastest
        const double foot = dot(P3 - P1, tau);
        const bool split = foot > 1e-12 * L && foot < (1.0 - 1e-12) * L;
        double acc = 0.0;
#pragma unroll 1
        for (int piece = 0; piece < (split ? 2 : 1); ++piece) {
            const double lo = split && piece == 1 ? foot : 0.0;
            const double span = split ? (piece == 0 ? foot : L - foot) : L;
            double part = 0.0;
#pragma unroll 1
            for (int k = 0; k < Q.nself; ++k) {
                const double b = lo + span * Q.sx[k], a = L - b;
                const d3 y = P1 + b * tau;
                const double phis = angle_ref(tau, P3 - y);
                part += Q.sw[k] * (ray_side(a, al2, phis + al2) + ray_side(b, al1, (kPi - phis) + al1));
            }
            acc += span * part;
        }
        total += acc;
    }
    A.P[t] = kInv4Pi * total;
}

// ------------------------------------------------------------------ finalisation

template <int CLS>
__global__ void __launch_bounds__(128) k_finalize(ClassArgs A, int mode)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < A.n) finalize_item<CLS>(A, mode, t);
}



// ------------------------------------------------------------------ host-side launchers
static int blocks_for(long long n, int tpb) { return (int)((n + tpb - 1) / tpb); }

void launch_prepare_panels(int nc, const double *V, const int *C, Panel *out, cudaStream_t s)
{
    if (nc > 0) k_prepare_panels<<<blocks_for(nc, 128), 128, 0, s>>>(nc, V, C, out);
}

template <int CLS>
static void level_chain(const ClassArgs &A, const QuadTables &Q, const RunConfig &cfg, int persistent_blocks, cudaStream_t s)
{
    const int tpb = 128;
    if (cfg.mode == kFixed) {
        const long long work = (long long)A.n * (cfg.level <= 2 ? (1 << (2 * cfg.level)) : 32);
        k_level<CLS><<<std::max(1, std::min(blocks_for(work, tpb), persistent_blocks * 8)), tpb, 0, s>>>(A, Q, cfg.level, cfg.mode, cfg.tol, cfg.max_level);
        k_finalize<CLS><<<blocks_for(A.n, tpb), tpb, 0, s>>>(A, cfg.mode);
        return;
    }
    // adaptive: level 0 over all pairs, then levels 1..max over device-side active lists
    k_level<CLS><<<blocks_for(A.n, tpb), tpb, 0, s>>>(A, Q, 0, cfg.mode, cfg.tol, cfg.max_level);
    ClassArgs B = A;
    for (int lev = 1; lev <= cfg.max_level; ++lev) {
        B.act_in = lev == 1 ? nullptr : (lev % 2 ? A.act_b : A.act_a);
        B.cnt_in = lev == 1 ? nullptr : A.cnt + (lev - 1);
        B.act_out = lev % 2 ? A.act_a : A.act_b;
        B.cnt_out = A.cnt + lev;
        k_level<CLS><<<persistent_blocks, tpb, 0, s>>>(B, Q, lev, cfg.mode, cfg.tol, cfg.max_level);
    }
    k_finalize<CLS><<<blocks_for(A.n, tpb), tpb, 0, s>>>(A, cfg.mode);
}

void launch_finalize(int cls, const ClassArgs &A, int mode, cudaStream_t s)
{
    const int tpb = 128;
    if (cls == kEdge) k_finalize<kEdge><<<blocks_for(A.n, tpb), tpb, 0, s>>>(A, mode);
    else if (cls == kVertex) k_finalize<kVertex><<<blocks_for(A.n, tpb), tpb, 0, s>>>(A, mode);
    else k_finalize<kFar><<<blocks_for(A.n, tpb), tpb, 0, s>>>(A, mode);
}

void launch_self(const ClassArgs &A, const QuadTables &Q, const RunConfig &cfg, cudaStream_t s)
{
    k_self<<<blocks_for(A.n, 128), 128, 0, s>>>(A, Q, cfg.self_sign);
}

void launch_pot_hard(int cls, const ClassArgs &A, const QuadTables &Q, const RunConfig &cfg, int persistent_blocks, cudaStream_t s)
{
    if (cls == kEdge) pot_adaptive_chain<kEdge>(A, Q, cfg.hard_tol, persistent_blocks, s);
    else pot_adaptive_chain<kVertex>(A, Q, cfg.hard_tol, persistent_blocks, s);
}

void launch_class_fp64(int cls, const ClassArgs &A, const QuadTables &Q, const RunConfig &cfg, int persistent_blocks, cudaStream_t s)
{
    if (A.n <= 0) return;
    const int tpb = 128;
    switch (cls) {
    case kSelf:
        k_self<<<blocks_for(A.n, tpb), tpb, 0, s>>>(A, Q, cfg.self_sign);
        break;
    case kEdge:
        k_singular<kEdge><<<blocks_for(A.n, tpb), tpb, 0, s>>>(A, Q);
        if (A.hard_list) {
            k_pot_tier2<kEdge><<<persistent_blocks, tpb, 0, s>>>(A, Q);
            pot_adaptive_chain<kEdge>(A, Q, cfg.hard_tol, persistent_blocks, s);
        }
        level_chain<kEdge>(A, Q, cfg, persistent_blocks, s);
        break;
    case kVertex:
        k_singular<kVertex><<<blocks_for(A.n, tpb), tpb, 0, s>>>(A, Q);
        if (A.hard_list) {
            k_pot_tier2<kVertex><<<persistent_blocks, tpb, 0, s>>>(A, Q);
            pot_adaptive_chain<kVertex>(A, Q, cfg.hard_tol, persistent_blocks, s);
        }
        level_chain<kVertex>(A, Q, cfg, persistent_blocks, s);
        break;
    default:
        level_chain<kFar>(A, Q, cfg, persistent_blocks, s);
        break;
    }
}

} // namespace i2
