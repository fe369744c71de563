// i2_kernels_df.cu -- the potential stages of the mixed and batched forms that need more than
// FP32, in double-float arithmetic on the FP32 pipe (i2_dfloat.cuh): tier 2b of the adjacent
// pairs' potential (the 16 x 16 graded Duffy rule against the 20 x 20 one) and the breadth-first
// adaptive rule of the hard pairs (seed, twelve depths, final sums).
//
// GB300 executes FP64 at 1/64 of its FP32 rate, and in FP64 these stages were bound by the FP64
// pipe (busy 85-87 % of their cycles, about 40 % of the batched step).  A double-float value
// carries 48 significant bits; with each pair's geometry moved to a local frame -- translated to
// K_j's vertex A and scaled by the power of two that brings K_i's sqrt(S) into [0.5, 1) -- every
// coordinate of the rule is O(1) and stored to 2^-48 of the cell size, which is the precision
// FP64 absolute coordinates give on a mesh of unit size.  The set-up of a pair (the local frame,
// the panel quantities, the shared-edge term) is formed in FP64 once per pair; every quadrature
// point is double-float.  Results go back to true units by the exact factor 2^(-3e) (the
// potential scales with the cube of lengths).
//
// The plain FP64 form keeps its FP64 kernels (i2_kernels_fp64.cu, i2_tiers.cuh): its potential
// is the accuracy reference of the mixed form.
#include "i2_batch.cuh"
#include "i2_dfvec.cuh"
#include "i2_engine.h"
#include "i2_pot.cuh"
#include "i2_rules.cuh"

namespace i2 {

// resident 128-thread blocks per SM the double-float kernels are compiled for (at most 128
// registers a thread, a few spilled; three blocks at 168 registers measured 0.3 % slower on the
// batched C2 step); each warp's pair set-up lives in shared memory, not in registers
constexpr int kDfBlocks = 4;

// ------------------------------------------------------------------ rule tables
struct QuadTablesD {
    dfl L1[kMaxGauss], L2[kMaxGauss], L3[kMaxGauss], w[kMaxGauss];
    dfl du_u[kMaxDuffy], du_w[kMaxDuffy], dv_v[kMaxDuffy], dv_w[kMaxDuffy];
    dfl hi_u[kMaxDuffy], hi_uw[kMaxDuffy], hi_v[kMaxDuffy], hi_vw[kMaxDuffy];
    dfl top_u[kDuffyTop], top_uw[kDuffyTop], top_v[kDuffyTop], top_vw[kDuffyTop];
    int npts, nu, nv, hi_nu, hi_nv, top_nu, top_nv;
};

static QuadTablesD tables_df(const QuadTables &Q)
{
    QuadTablesD D{};
    for (int g = 0; g < kMaxGauss; ++g) {
        D.L1[g] = dfl(Q.L1[g]);
        D.L2[g] = dfl(Q.L2[g]);
        D.L3[g] = dfl(Q.L3[g]);
        D.w[g] = dfl(Q.w[g]);
    }
    for (int a = 0; a < kMaxDuffy; ++a) {
        D.du_u[a] = dfl(Q.du_u[a]);
        D.du_w[a] = dfl(Q.du_w[a]);
        D.dv_v[a] = dfl(Q.dv_v[a]);
        D.dv_w[a] = dfl(Q.dv_w[a]);
        D.hi_u[a] = dfl(Q.hi_u[a]);
        D.hi_uw[a] = dfl(Q.hi_uw[a]);
        D.hi_v[a] = dfl(Q.hi_v[a]);
        D.hi_vw[a] = dfl(Q.hi_vw[a]);
    }
    for (int a = 0; a < kDuffyTop; ++a) {
        D.top_u[a] = dfl(Q.top_u[a]);
        D.top_uw[a] = dfl(Q.top_uw[a]);
        D.top_v[a] = dfl(Q.top_v[a]);
        D.top_vw[a] = dfl(Q.top_vw[a]);
    }
    D.npts = Q.npts;
    D.nu = Q.nu;
    D.nv = Q.nv;
    D.hi_nu = Q.hi_nu;
    D.hi_nv = Q.hi_nv;
    D.top_nu = Q.top_nu;
    D.top_nv = Q.top_nv;
    return D;
}

// ------------------------------------------------------------------ a pair in its local frame
struct PotLocal {
    TriD Ti;       // K_i, stored vertex order
    PanelJD K;     // K_j with A at the origin
    FarCtxD F;
    PotEdgeD pe;   // shared-edge term (edge class)
    double sig;    // integral of the shared-edge term over K_i, true units
    double s3;     // local = true x s3 for the potential (s3 = 2^(3e))
};

template <int CLS>
__device__ PotLocal pot_local(const ClassArgs &A, int t)
{
    const int2 pr = A.pairs[t];
    const PanelJ K = load_panel(A.panels, pr.y);
    const Tri Ti = load_tri(A.panels, pr.x);
    const double Si = A.panels[pr.x].v[0].w;
    const double s = pow2_normaliser(sqrt(Si));
    const d3 o = K.A;
    PanelJ Kl = K;
    Kl.A = mk(0.0, 0.0, 0.0);
    Kl.B = s * (K.B - o);
    Kl.C = s * (K.C - o);
    Kl.S = (s * s) * K.S;
    Kl.lenA = s * K.lenA;
    Kl.lenB = s * K.lenB;
    Kl.lenC = s * K.lenC;
    const Tri Tl{s * (Ti.a - o), s * (Ti.b - o), s * (Ti.c - o)};
    const FarCtx Fl = make_far_ctx(Kl);
    PotEdge pe{};
    double sig_l = 0.0;
    if (CLS == kEdge) {
        int si, sj;
        shifts_edge(A.cells[pr.x], A.cells[pr.y], si, sj);
        sig_l = make_pot_edge(rotate(Tl, si), rotate(Tri{Kl.A, Kl.B, Kl.C}, sj), Kl, (s * s) * Si, pe);
    }
    PotLocal L;
    L.Ti = to_df(Tl);
    L.K.A = to_df(Kl.A);
    L.K.B = to_df(Kl.B);
    L.K.C = to_df(Kl.C);
    L.K.n = to_df(Kl.n);
    L.K.ta = to_df(Kl.ta);
    L.K.tb = to_df(Kl.tb);
    L.K.tc = to_df(Kl.tc);
    L.K.S = dfl(Kl.S);
    L.K.lenA = dfl(Kl.lenA);
    L.K.lenB = dfl(Kl.lenB);
    L.K.lenC = dfl(Kl.lenC);
    L.F = FarCtxD{to_df(Fl.ma), to_df(Fl.mb), to_df(Fl.mc)};
    L.pe = PotEdgeD{to_df(pe.P1), to_df(pe.m_in), dfl(pe.c), dfl(pe.h)};
    L.s3 = s * s * s;
    L.sig = sig_l / L.s3;
    return L;
}

// loads from a warp's shared-memory slot, one field at a time where it is used: the slot's pair
// geometry (some 60 floats) is not held in registers across the point loop
__device__ __forceinline__ dfl ldv(const volatile dfl &x) { return dfl(x.hi, x.lo); }
__device__ __forceinline__ df3 ldv(const volatile df3 &v) { return df3{ldv(v.x), ldv(v.y), ldv(v.z)}; }

// ln((l_from + q_from) / (l_to + q_to)) with the reference's collinear fallback (edge_log_fp64)
// (one division and one logarithm whichever form applies: the lanes of a warp share the call)
__device__ __forceinline__ dfl edge_log_df(dfl l_from, dfl q_from, dfl l_to, dfl q_to)
{
    const dfl s_to = q_to + l_to;
    const bool collinear = fabs(s_to) < (0.5 * kEpsPsi2) * l_to;
    return log((collinear ? l_to : l_from + q_from) / (collinear ? l_from : s_to));
}

// the integrand of the adjacent pairs' potential, sum_e t_e L_e - d Theta (far_integrand_o's
// potential), at a point with offsets oa, ob, oc from K_j's vertices (local frame: oa is the
// point itself), less the shared-edge term for the edge class; evaluated edge by edge so that
// only one edge's quantities are live at a time
template <int CLS>
__device__ __noinline__ dfl pot_point_df(df3 oa, df3 ob, df3 oc, const volatile PanelJD &K, const volatile FarCtxD &F,
                                            const volatile PotEdgeD &pe)
{
    const dfl la = norm(oa), lb = norm(ob), lc = norm(oc);
    dfl pot = dfl(0.0f, 0.0f);
    {
        const df3 tc = ldv(K.tc);
        const dfl t_e = -dot(ldv(F.mc), oa);  // t_e L_e -> 0 on the edge's line even where L_e overflows
        if (!(t_e == 0.0)) pot = t_e * edge_log_df(la, dot(oa, tc), lb, dot(ob, tc));  // A -> B
    }
    {
        const df3 ta = ldv(K.ta);
        const dfl t_e = -dot(ldv(F.ma), ob);
        if (!(t_e == 0.0)) pot += t_e * edge_log_df(lb, dot(ob, ta), lc, dot(oc, ta));  // B -> C
    }
    {
        const df3 tb = ldv(K.tb);
        const dfl t_e = -dot(ldv(F.mb), oc);
        if (!(t_e == 0.0)) pot += t_e * edge_log_df(lc, dot(oc, tb), la, dot(oa, tb));  // C -> A
    }
    const dfl d = dot(ldv(K.n), oa);
    const dfl den = la * lb * lc + dot(oa, ob) * lc + dot(ob, oc) * la + dot(oc, oa) * lb;
    pot -= d * (2.0f * atan2((2.0f * ldv(K.S)) * d, den));
    if (CLS == kEdge) {
        const dfl s = dot(oa - ldv(pe.P1), ldv(pe.m_in));
        if (s > 0.0) pot += ((2.0f * ldv(pe.c)) * s) * log(s / ldv(pe.h));
    }
    return pot;
}

// ------------------------------------------------------------------ tier 2b
// the graded Duffy rule of a pair (pieces with apex at the shared vertex, or at both ends of the
// shared edge) over points p = first, first + step, ... of its flattened (piece, radial, angular)
// list; a piece's geometry is formed once per lane and piece
template <int CLS>
__device__ dfl duffy_partial_df(const TriD &Ti, const volatile PanelJD &K, const volatile FarCtxD &F, const volatile PotEdgeD &pe,
                                const dfl *uu, const dfl *uw, int nu, const dfl *vv, const dfl *vw, int nv, int first, int step)
{
    const int npieces = CLS == kEdge ? 2 : 1;
    const int per = nu * nv;
    dfl total = dfl(0.0f, 0.0f);
    int cur = -1;
    df3 Vx, eB, eC, dB, dC;
    dfl area2;
#pragma unroll 1
    for (int p = first; p < npieces * per; p += step) {
        const int piece = p / per, q = p - piece * per, a = q / nv, b = q - a * nv;
        if (piece != cur) {
            cur = piece;
            df3 B, Cc;
            if (CLS == kVertex) {
                Vx = Ti.a;
                B = Ti.b;
                Cc = Ti.c;
            } else {
                const df3 M = df_half(Ti.b + Ti.c);
                if (piece == 0) {
                    Vx = Ti.b;
                    B = M;
                    Cc = Ti.a;
                } else {
                    Vx = Ti.c;
                    B = Ti.a;
                    Cc = M;
                }
            }
            eB = B - Vx;
            eC = Cc - Vx;
            dB = Vx - ldv(K.B);
            dC = Vx - ldv(K.C);
            area2 = norm(cross(eB, eC));
        }
        const dfl u = uu[a], v = vv[b];
        const df3 w = u * ((1.0f - v) * eB + v * eC);
        const dfl g = pot_point_df<CLS>(Vx + w, dB + w, dC + w, K, F, pe);
        total += ((uw[a] * u) * vw[b]) * area2 * g;
    }
    return total;
}

// listed pair h by one warp: the 16 x 16 and 20 x 20 rules; the pair is settled when they agree
// to A.top_tol, else it goes to the adaptive rule with the 16 x 16 value as its tolerance base
// the pair's local set-up is formed by lane 0 into the warp's shared-memory slot `L` (read by all
// lanes from there rather than held in registers); the caller's next item waits for lane 0
template <int CLS>
__device__ __noinline__ void tier2b_item_df(const ClassArgs &A, const QuadTablesD &Q, int h, int lane, PotLocal &L)
{
    const int t = A.tier2b_list[h];
    const int2 pr = A.pairs[t];
    __syncwarp();
    if (lane == 0) L = pot_local<CLS>(A, t);
    __syncwarp();
    int si, sj;
    if (CLS == kEdge) shifts_edge(A.cells[pr.x], A.cells[pr.y], si, sj);
    else shifts_vertex(A.cells[pr.x], A.cells[pr.y], si, sj);
    const TriD Ti = rotate(L.Ti, si);
    const volatile PotLocal &Lv = L;
    const dfl ph = warp_sum_df(duffy_partial_df<CLS>(Ti, Lv.K, Lv.F, Lv.pe, Q.hi_u, Q.hi_uw, Q.hi_nu, Q.hi_v, Q.hi_vw, Q.hi_nv, lane, 32));
    const dfl pt = warp_sum_df(duffy_partial_df<CLS>(Ti, Lv.K, Lv.F, Lv.pe, Q.top_u, Q.top_uw, Q.top_nu, Q.top_v, Q.top_vw, Q.top_nv, lane, 32));
    if (lane != 0) return;
    const double inv = 1.0 / L.s3;
    const double ph_t = (double)ph * inv + L.sig, pt_t = (double)pt * inv + L.sig;
    if (fabs(pt_t - ph_t) <= A.top_tol * fabs(pt_t)) {
        A.padj[t] = kInv4Pi * pt_t;
    } else {
        A.padj[t] = kInv4Pi * ph_t;  // the adaptive rule's tolerance base
        A.hard_list[atomicAdd(A.hard_cnt, 1)] = t;
    }
}

template <int CLS>
__global__ void __launch_bounds__(128, kDfBlocks) k_pot_tier2b_df(ClassArgs A, QuadTablesD Q)
{
    __shared__ PotLocal slot[4];
    const int count = A.cnt[kCntTier2b];
    const int lane = threadIdx.x & 31;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (long long h = warp_item_index(); h < count; h += nwarps) tier2b_item_df<CLS>(A, Q, (int)h, lane, slot[threadIdx.x >> 5]);
}

// ------------------------------------------------------------------ adaptive rule of hard pairs
// The FP64 form's breadth-first rule (i2_kernels_fp64.cu) with the cells in double-float: the
// same cells, rules, acceptance test (|sum of children - cell| <= tol |P| 2^-depth) and 64-bit
// fixed-point accumulation of accepted sums, in the pair's local frame.
struct PotPairCtxD {
    TriD Ti;  // K_i, stored vertex order, local frame
    PanelJD K;
    FarCtxD F;
    PotEdgeD pe;
    double sig;      // shared-edge integral, true units
    double tol_loc;  // tol |P| in local units
    double scale;    // 2^40 / (|P| + |shared-edge integral|), local units
    double inv_s3;   // local -> true units
};
static_assert(sizeof(PotPairCtxD) <= 8 * kPotCtxDoubles, "cached hard-pair set-up size");

template <int CLS>
__device__ PotPairCtxD pot_pair_ctx_df(const ClassArgs &A, int t, double tol)
{
    const PotLocal L = pot_local<CLS>(A, t);
    PotPairCtxD c;
    c.Ti = L.Ti;
    c.K = L.K;
    c.F = L.F;
    c.pe = L.pe;
    c.sig = L.sig;
    c.inv_s3 = 1.0 / L.s3;
    const double p_loc = A.padj[t] * (4.0 * kPi) * L.s3;  // tier value (regular part + shared-edge integral)
    c.tol_loc = tol * fabs(p_loc);
    const double base = fabs(p_loc) + fabs(L.sig * L.s3);
    c.scale = base > 0.0 ? ldexp(1.0, 40) / base : 1.0;
    return c;
}

// hard pair h's set-up into the warp's shared-memory slot: copied from the cache by the whole
// warp, or recomputed by lane 0 past the cache's capacity
template <int CLS>
__device__ __forceinline__ void pot_ctx_to_slot(const ClassArgs &A, int h, int t, double tol, int lane, PotPairCtxD &slot)
{
    __syncwarp();  // the slot's previous item is done
    if (h < A.pot_ctx_cap) {
        const double *src = A.pot_ctx + (long long)kPotCtxDoubles * h;
        double *dst = reinterpret_cast<double *>(&slot);
        for (int i = lane; i < (int)(sizeof(PotPairCtxD) / 8); i += 32) dst[i] = src[i];
    } else if (lane == 0) {
        slot = pot_pair_ctx_df<CLS>(A, t, tol);
    }
    __syncwarp();
}

// the four children of cell T (corner slot of each in cc[]) by one warp: the flattened (child,
// point) list is cut into 32 contiguous runs, one per lane, so a lane forms a child's geometry
// once for all its points of that child; a butterfly leaves the four sums in every lane
template <int CLS>
__device__ void pot_children_warp_df(const TriD &T, const int cc[4], const volatile PotPairCtxD &c, const QuadTablesD &Q, int lane, dfl v[4])
{
    const int nduffy = Q.nu * Q.nv;
    int start[5];
    start[0] = 0;
    for (int k = 0; k < 4; ++k) start[k + 1] = start[k] + (cc[k] >= 0 ? nduffy : Q.npts);
    const int run = (start[4] + 31) >> 5;
    const int j0 = lane * run, j1 = min(start[4], j0 + run);
    dfl acc0 = dfl(0.0f, 0.0f), acc1 = acc0, acc2 = acc0, acc3 = acc0;
    int kc = -1;
    TriD Tc;
    df3 eB, eC, dB, dC;
    dfl area;
#pragma unroll 1
    for (int j = j0; j < j1; ++j) {
        const int k = j < start[1] ? 0 : (j < start[2] ? 1 : (j < start[3] ? 2 : 3));
        const int p = j - start[k];
        if (k != kc) {
            kc = k;
            Tc = child_df(T, k);
            if (cc[k] >= 0) {
                const int corner = cc[k];
                const df3 Vx = corner == 0 ? Tc.a : (corner == 1 ? Tc.b : Tc.c);
                const df3 B = corner == 0 ? Tc.b : (corner == 1 ? Tc.c : Tc.a);
                const df3 Cc = corner == 0 ? Tc.c : (corner == 1 ? Tc.a : Tc.b);
                Tc.a = Vx;  // the apex, kept for the points
                eB = B - Vx;
                eC = Cc - Vx;
                dB = Vx - ldv(c.K.B);
                dC = Vx - ldv(c.K.C);
                area = norm(cross(eB, eC));
            } else {
                area = df_half(norm(cross(Tc.b - Tc.a, Tc.c - Tc.a)));
            }
        }
        // the point (offsets from K_j's vertices) and its weight by the child's rule; then one
        // integrand call for the whole warp, whichever rules its lanes are on
        df3 oa, ob, oc;
        dfl wgt;
        if (cc[k] >= 0) {
            const int a = p / Q.nv, b = p - a * Q.nv;
            const dfl u = Q.du_u[a], vv = Q.dv_v[b];
            const df3 w = u * ((1.0f - vv) * eB + vv * eC);
            oa = Tc.a + w;
            ob = dB + w;
            oc = dC + w;
            wgt = ((Q.du_w[a] * u) * Q.dv_w[b]) * area;
        } else {
            oa = Q.L1[p] * Tc.a + Q.L2[p] * Tc.b + Q.L3[p] * Tc.c;
            ob = oa - ldv(c.K.B);
            oc = oa - ldv(c.K.C);
            wgt = Q.w[p] * area;
        }
        const dfl g = wgt * pot_point_df<CLS>(oa, ob, oc, c.K, c.F, c.pe);
        if (k == 0) acc0 += g;
        else if (k == 1) acc1 += g;
        else if (k == 2) acc2 += g;
        else acc3 += g;
    }
    v[0] = warp_sum_df(acc0);
    v[1] = warp_sum_df(acc1);
    v[2] = warp_sum_df(acc2);
    v[3] = warp_sum_df(acc3);
}

template <int CLS>
__device__ __noinline__ void pot_seed_item_df(const ClassArgs &A, const QuadTablesD &Q, double tol, int h, int lane, PotPairCtxD &c)
{
    const int t = A.hard_list[h];
    __syncwarp();
    if (lane == 0) c = pot_pair_ctx_df<CLS>(A, t, tol);
    __syncwarp();
    const int3 ci = A.cells[A.pairs[t].x], cj = A.cells[A.pairs[t].y];
    const int ia[3] = {ci.x, ci.y, ci.z};
    bool shared[3];
    for (int k = 0; k < 3; ++k) shared[k] = (ia[k] == cj.x || ia[k] == cj.y || ia[k] == cj.z);
    // the root's children 0, 1, 2 hold K_i's slots b, c, a in their slot 1
    int cc[4];
    for (int k = 0; k < 4; ++k) cc[k] = k == 3 ? -1 : (shared[k == 0 ? 1 : (k == 1 ? 2 : 0)] ? 1 : -1);
    dfl v[4];
    pot_children_warp_df<CLS>(c.Ti, cc, c, Q, lane, v);
    if (lane < 4) {
        const dfl mine = lane == 0 ? v[0] : (lane == 1 ? v[1] : (lane == 2 ? v[2] : v[3]));
        A.pot_q_a[4 * (long long)h + lane] = PotCellItem{(unsigned long long)lane, df_pack(mine), h, cc[lane]};
    }
    if (lane == 0) {
        A.pot_fx[h] = 0;
        if (h < A.pot_ctx_cap) *reinterpret_cast<PotPairCtxD *>(A.pot_ctx + (long long)kPotCtxDoubles * h) = c;
        if (h < A.pot_tri_cap) tri_store_df(pot_tri_list(A, 1) + 9LL * h, c.Ti);  // parent of depth 1's slots 4h..4h+3
    }
}

template <int CLS>
__device__ __noinline__ void pot_depth_item_df(const ClassArgs &A, const QuadTablesD &Q, double tol, int depth, const PotCellItem *__restrict__ in,
                                  PotCellItem *__restrict__ out, int idx, int lane, PotPairCtxD &c)
{
    const PotCellItem it = in[idx];
    if (it.h < 0) return;
    const int t = A.hard_list[it.h];
    pot_ctx_to_slot<CLS>(A, it.h, t, tol, lane, c);
    // siblings sit at 4 consecutive slots, so the parent's triangle is at slot idx / 4
    const TriD T = (idx >> 2) < A.pot_tri_cap ? child_df(tri_load_df(pot_tri_list(A, depth) + 9LL * (idx >> 2)), (int)(it.path & 3))
                                              : subcell_df(c.Ti, depth, it.path);
    int cc[4];
    for (int k = 0; k < 4; ++k) cc[k] = child_corner(it.corner, k);
    dfl v[4];
    pot_children_warp_df<CLS>(T, cc, c, Q, lane, v);
    if (lane != 0) return;
    const dfl sum = (v[0] + v[1]) + (v[2] + v[3]);
    const dfl diff = sum - df_unpack(it.val);
    bool accept = fabsf(diff.hi) <= (float)ldexp(c.tol_loc, -depth) || depth >= kHardMaxDepth;
    if (!accept) {
        const int pos = atomicAdd(&A.pot_qcnt[depth + 1], 4);
        if (pos + 4 <= A.pot_qcap) {
            for (int k = 0; k < 4; ++k) out[pos + k] = PotCellItem{(it.path << 2) | (unsigned long long)k, df_pack(v[k]), it.h, cc[k]};
            if ((pos >> 2) < A.pot_tri_cap) tri_store_df(pot_tri_list(A, depth + 1) + 9LL * (pos >> 2), T);
        } else {
            // list full: keep this cell's sum (counted as an overflow) and blank the slots it
            // was given below the capacity, so the next depth skips them
            for (int k = pos; k < A.pot_qcap && k < pos + 4; ++k) out[k] = PotCellItem{0ull, 0.0, -1, -1};
            atomicAdd(A.hard_overflow, 1);
            accept = true;
        }
    }
    if (accept) {
        const double fx = (double)sum.hi * c.scale + (double)sum.lo * c.scale;
        atomicAdd(reinterpret_cast<unsigned long long *>(&A.pot_fx[it.h]), (unsigned long long)llrint(fx));
    }
}

template <int CLS>
__device__ __forceinline__ void pot_final_item_df(const ClassArgs &A, double tol, int h)
{
    const int t = A.hard_list[h];
    double scale, inv_s3, sig;
    if (h < A.pot_ctx_cap) {
        const PotPairCtxD *c = reinterpret_cast<const PotPairCtxD *>(A.pot_ctx + (long long)kPotCtxDoubles * h);
        scale = c->scale;
        inv_s3 = c->inv_s3;
        sig = c->sig;
    } else {
        const PotPairCtxD c = pot_pair_ctx_df<CLS>(A, t, tol);
        scale = c.scale;
        inv_s3 = c.inv_s3;
        sig = c.sig;
    }
    A.padj[t] = kInv4Pi * ((double)A.pot_fx[h] / scale * inv_s3 + sig);
}

template <int CLS>
__global__ void __launch_bounds__(128, kDfBlocks) k_pot_seed_df(ClassArgs A, QuadTablesD Q, double tol)
{
    __shared__ PotPairCtxD slot[4];
    const int count = pot_seeded(A);
    // the depth kernels run after this one on the same stream
    if (blockIdx.x == 0 && threadIdx.x == 0) pot_seed_init(A);
    const int lane = threadIdx.x & 31;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int h = (int)warp_item_index(); h < count; h += nwarps) pot_seed_item_df<CLS>(A, Q, tol, h, lane, slot[threadIdx.x >> 5]);
}

template <int CLS>
__global__ void __launch_bounds__(128, kDfBlocks) k_pot_depth_df(ClassArgs A, QuadTablesD Q, double tol, int depth, const PotCellItem *__restrict__ in,
                                                                PotCellItem *__restrict__ out)
{
    __shared__ PotPairCtxD slot[4];
    const int count = pot_depth_count(A, depth);
    const int lane = threadIdx.x & 31;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int idx = (int)warp_item_index(); idx < count; idx += nwarps)
        pot_depth_item_df<CLS>(A, Q, tol, depth, in, out, idx, lane, slot[threadIdx.x >> 5]);
}

template <int CLS>
__global__ void __launch_bounds__(128) k_pot_final_df(ClassArgs A, double tol)
{
    const int count = pot_seeded(A);
    for (int h = blockIdx.x * blockDim.x + threadIdx.x; h < count; h += gridDim.x * blockDim.x) pot_final_item_df<CLS>(A, tol, h);
}

// ------------------------------------------------------------------ batched stages
__global__ void __launch_bounds__(128, kDfBlocks) k_batch_tier2b(const BatchSeg *__restrict__ segs, int nseg, QuadTablesD Q)
{
    extern __shared__ long long prefix[];
    __shared__ PotLocal slot[4];
    const long long total = seg_prefix(segs, nseg, prefix, [](const BatchSeg &S) -> long long {
        return seg_adjacent(S) && S.A.hard_list ? S.A.cnt[kCntTier2b] : 0;
    });
    const int lane = threadIdx.x & 31;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long g = warp_item_index(); g < total; g += nwarps) {
        const int sg = seg_find(prefix, nseg, g);
        const BatchSeg &S = segs[sg];
        if (S.cls == kEdge) tier2b_item_df<kEdge>(S.A, Q, (int)(g - prefix[sg]), lane, slot[threadIdx.x >> 5]);
        else tier2b_item_df<kVertex>(S.A, Q, (int)(g - prefix[sg]), lane, slot[threadIdx.x >> 5]);
    }
}

__global__ void __launch_bounds__(128, kDfBlocks) k_batch_pot_seed(const BatchSeg *__restrict__ segs, int nseg, QuadTablesD Q, double tol)
{
    extern __shared__ long long prefix[];
    __shared__ PotPairCtxD slot[4];
    const long long total = seg_prefix(segs, nseg, prefix, [](const BatchSeg &S) -> long long {
        return seg_adjacent(S) && S.A.hard_list ? pot_seeded(S.A) : 0;
    });
    const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid < nseg && seg_adjacent(segs[gid]) && segs[gid].A.hard_list) pot_seed_init(segs[gid].A);
    const int lane = threadIdx.x & 31;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long g = warp_item_index(); g < total; g += nwarps) {
        const int sg = seg_find(prefix, nseg, g);
        const BatchSeg &S = segs[sg];
        const int h = (int)(g - prefix[sg]);
        if (S.cls == kEdge) pot_seed_item_df<kEdge>(S.A, Q, tol, h, lane, slot[threadIdx.x >> 5]);
        else pot_seed_item_df<kVertex>(S.A, Q, tol, h, lane, slot[threadIdx.x >> 5]);
    }
}

__global__ void __launch_bounds__(128, kDfBlocks) k_batch_pot_depth(const BatchSeg *__restrict__ segs, int nseg, QuadTablesD Q, double tol, int depth)
{
    extern __shared__ long long prefix[];
    __shared__ PotPairCtxD slot[4];
    const long long total = seg_prefix(segs, nseg, prefix, [depth](const BatchSeg &S) -> long long {
        return seg_adjacent(S) && S.A.hard_list ? pot_depth_count(S.A, depth) : 0;
    });
    const int lane = threadIdx.x & 31;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long g = warp_item_index(); g < total; g += nwarps) {
        const int sg = seg_find(prefix, nseg, g);
        const BatchSeg &S = segs[sg];
        const int idx = (int)(g - prefix[sg]);
        const PotCellItem *in = depth % 2 ? S.A.pot_q_a : S.A.pot_q_b;
        PotCellItem *out = depth % 2 ? S.A.pot_q_b : S.A.pot_q_a;
        if (S.cls == kEdge) pot_depth_item_df<kEdge>(S.A, Q, tol, depth, in, out, idx, lane, slot[threadIdx.x >> 5]);
        else pot_depth_item_df<kVertex>(S.A, Q, tol, depth, in, out, idx, lane, slot[threadIdx.x >> 5]);
    }
}

__global__ void __launch_bounds__(128) k_batch_pot_final(const BatchSeg *__restrict__ segs, int nseg, double tol)
{
    extern __shared__ long long prefix[];
    const long long total = seg_prefix(segs, nseg, prefix, [](const BatchSeg &S) -> long long {
        return seg_adjacent(S) && S.A.hard_list ? pot_seeded(S.A) : 0;
    });
    for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += (long long)gridDim.x * blockDim.x) {
        const int sg = seg_find(prefix, nseg, g);
        const BatchSeg &S = segs[sg];
        if (S.cls == kEdge) pot_final_item_df<kEdge>(S.A, tol, (int)(g - prefix[sg]));
        else pot_final_item_df<kVertex>(S.A, tol, (int)(g - prefix[sg]));
    }
}

// ------------------------------------------------------------------ host-side launchers
static int blocks_for_d(long long n, int tpb) { return (int)((n + tpb - 1) / tpb); }
static size_t seg_smem_d(int nseg) { return (size_t)(nseg + 1) * sizeof(long long); }

template <int CLS>
static void pot_chain_df(const ClassArgs &A, const QuadTablesD &Qd, double tol, int persistent_blocks, cudaStream_t s)
{
    k_pot_seed_df<CLS><<<resident_grid((const void *)k_pot_seed_df<CLS>, 128, 0), 128, 0, s>>>(A, Qd, tol);
    const int grid = resident_grid((const void *)k_pot_depth_df<CLS>, 128, 0);
    for (int d = 1; d <= kHardMaxDepth; ++d)
        k_pot_depth_df<CLS><<<grid, 128, 0, s>>>(A, Qd, tol, d, d % 2 ? A.pot_q_a : A.pot_q_b, d % 2 ? A.pot_q_b : A.pot_q_a);
    k_pot_final_df<CLS><<<persistent_blocks, 128, 0, s>>>(A, tol);
}

void launch_pot_tiers_hard_df(int cls, const ClassArgs &A, const QuadTables &Q, const RunConfig &cfg, int persistent_blocks, cudaStream_t s)
{
    const QuadTablesD Qd = tables_df(Q);
    if (cls == kEdge) {
        k_pot_tier2b_df<kEdge><<<resident_grid((const void *)k_pot_tier2b_df<kEdge>, 128, 0), 128, 0, s>>>(A, Qd);
        pot_chain_df<kEdge>(A, Qd, cfg.hard_tol, persistent_blocks, s);
    } else {
        k_pot_tier2b_df<kVertex><<<resident_grid((const void *)k_pot_tier2b_df<kVertex>, 128, 0), 128, 0, s>>>(A, Qd);
        pot_chain_df<kVertex>(A, Qd, cfg.hard_tol, persistent_blocks, s);
    }
}

void launch_batch_pot_df(const BatchSeg *segs, int nseg, const QuadTables &Q, double tol, int persistent_blocks, cudaStream_t s)
{
    const QuadTablesD Qd = tables_df(Q);
    for (int c0 = 0; c0 < nseg; c0 += kBatchSegChunk) {
        const int nc = std::min(kBatchSegChunk, nseg - c0);
        k_batch_tier2b<<<resident_grid((const void *)k_batch_tier2b, 128, seg_smem_d(nc)), 128, seg_smem_d(nc), s>>>(segs + c0, nc, Qd);
    }
    for (int c0 = 0; c0 < nseg; c0 += kBatchSegChunk) {
        const int nc = std::min(kBatchSegChunk, nseg - c0);
        // the seed initialises every segment of the chunk: at least one thread per segment
        k_batch_pot_seed<<<std::max(resident_grid((const void *)k_batch_pot_seed, 128, seg_smem_d(nc)), blocks_for_d(nc, 128)), 128,
                           seg_smem_d(nc), s>>>(segs + c0, nc, Qd, tol);
    }
    for (int d = 1; d <= kHardMaxDepth; ++d)
        for (int c0 = 0; c0 < nseg; c0 += kBatchSegChunk) {
            const int nc = std::min(kBatchSegChunk, nseg - c0);
            k_batch_pot_depth<<<resident_grid((const void *)k_batch_pot_depth, 128, seg_smem_d(nc)), 128, seg_smem_d(nc), s>>>(segs + c0, nc, Qd,
                                                                                                                               tol, d);
        }
    for (int c0 = 0; c0 < nseg; c0 += kBatchSegChunk) {
        const int nc = std::min(kBatchSegChunk, nseg - c0);
        k_batch_pot_final<<<persistent_blocks, 128, seg_smem_d(nc), s>>>(segs + c0, nc, tol);
    }
}

} // namespace i2
