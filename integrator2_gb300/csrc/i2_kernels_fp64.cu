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
#include "i2_pot.cuh"
#include "i2_self.cuh"
#include "i2_tiers.cuh"


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



// ------------------------------------------------------------------ regular part, one level
template <int CLS>
__global__ void __launch_bounds__(128) k_level(ClassArgs A, QuadTables Q, int level, int mode, double tol, int kmax)
{
    const int nsub = 1 << (2 * level);
    // lanes per pair: up to a warp, or the whole block once a pair has at least a block's worth
    // of sub-cells (levels 4 and 5: only a few pairs remain, and one warp per pair left each lane
    // hundreds of points in series).  The item count is then a multiple of the block, so every
    // block runs the loop uniformly and reaches the __syncthreads of the reduction below.
    const bool block_group = blockDim.x > 32 && nsub >= (int)blockDim.x;
    const int G = block_group ? (int)blockDim.x : (nsub < 32 ? nsub : 32);  // lanes per pair
    const int per_lane = nsub / G;                // sub-cells per lane
    const bool listed = A.act_in != nullptr;
    const int count = listed ? *A.cnt_in : A.n;
    const long long total = (long long)count * G;
    const long long total_r = block_group ? total : (total + 31) & ~31LL;
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
        for (int off = 1; off < (G < 32 ? G : 32); off <<= 1) {
            const acc5 o = shfl_xor5(acc, off);
            acc.px += o.px; acc.py += o.py; acc.pz += o.pz; acc.th += o.th; acc.pot += o.pot;
        }
        if (block_group) {
            // the warps' sums through shared memory, added in warp order by thread 0 (the
            // kernel's blocks have at most 128 threads, 4 warps)
            __shared__ double grp[4][5];
            const int w = threadIdx.x >> 5;
            if ((threadIdx.x & 31) == 0) store5(grp[w], acc);
            __syncthreads();
            if (threadIdx.x == 0)
                for (int k = 1; k < (int)(blockDim.x >> 5); ++k) {
                    const acc5 o = load5(grp[k]);
                    acc.px += o.px; acc.py += o.py; acc.pz += o.pz; acc.th += o.th; acc.pot += o.pot;
                }
            __syncthreads();
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
            if (mode == kAdaptiveCompat) store5(A.fin_b + 5 * (long long)t, prev);  // read by compat parity only
        } else {
            const int pos = atomicAdd(A.cnt_out, 1);
            A.act_out[pos] = t;
        }
    }
}

// ------------------------------------------------------------------ potential of adjacent pairs
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
    if (A.pot_off) return;  // J only (P was filled with NaN before the launch)

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

// tier 2: higher-order Duffy rule (16 x 16), kept when it agrees with the main rule; otherwise
// the pair is listed for tier 2b (i2_tiers.cuh) with its 16 x 16 value

template <int CLS>
__global__ void __launch_bounds__(128) k_pot_tier2(ClassArgs A, QuadTables Q)
{
    // one warp per listed pair: the lanes share each rule's points, so the FP64 work of the
    // list spreads over every SM
    const int count = *A.tier2_cnt;
    const int lane = threadIdx.x & 31;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int h = (int)warp_item_index(); h < count; h += nwarps) {
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
        const double ph = warp_sum(duffy_partial<CLS>(Ti, K, F, pe, Q.hi_u, Q.hi_uw, Q.hi_nu, Q.hi_v, Q.hi_vw, Q.hi_nv, lane, 32)) + sig;
        const double pm = A.padj[t] * (4.0 * kPi);
        if (lane != 0) continue;
        if (fabs(ph - pm) <= A.tier_tol * fabs(ph)) {
            A.padj[t] = kInv4Pi * ph;
        } else {
            // tier 2b next (the top rule against this one: when the main rule was the inaccurate
            // one, the 16 x 16 and 24 x 24 rules agree and the pair needs no adaptive rule); padj
            // carries the 16 x 16 value, unscaled, until then
            A.padj[t] = ph;
            A.tier2b_list[atomicAdd(A.cnt + kCntTier2b, 1)] = t;
        }
    }
}

// ------------------------------------------------------------------ hard adjacent pairs: adaptive potential
// Breadth-first over the cells of ALL hard pairs at once: depth d holds a device list of cells
// (hard-list slot, path, depth, corner slot, value); one warp takes one cell, integrates its
// four children and either accepts their sum (|sum - value| <= tol |P| 2^-d, or d at the depth
// cap) or appends the children to depth d + 1's list.  Cells that hold a shared vertex (always
// in slot 1 of a corner child) use the graded Duffy rule with that vertex as apex, all others
// the 13-point rule; point offsets to K_j's vertices are formed from vertex differences.  The
// whole GPU works on every depth, so one pair that needs thousands of cells no longer runs
// alone on one SM.  Accepted sums are added as 64-bit fixed point (2^40 units per |P| + |sigma
// integral|), so the result does not depend on the order of the atomics.
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

static_assert(sizeof(PotPairCtx) <= 8 * kPotCtxDoubles, "cached hard-pair set-up size");

// the cached set-up of hard pair h (written by the seed), or the set-up recomputed past the cap
template <int CLS>
__device__ __forceinline__ PotPairCtx pot_ctx_of(const ClassArgs &A, int h, int t, double tol)
{
    if (h < A.pot_ctx_cap) return *reinterpret_cast<const PotPairCtx *>(A.pot_ctx + (long long)kPotCtxDoubles * h);
    return pot_pair_ctx<CLS>(A, t, tol);
}

__device__ __forceinline__ void pot_tri_store(double *dst, const Tri &T)
{
    dst[0] = T.a.x; dst[1] = T.a.y; dst[2] = T.a.z;
    dst[3] = T.b.x; dst[4] = T.b.y; dst[5] = T.b.z;
    dst[6] = T.c.x; dst[7] = T.c.y; dst[8] = T.c.z;
}

__device__ __forceinline__ Tri pot_tri_load(const double *p)
{
    return Tri{mk(p[0], p[1], p[2]), mk(p[3], p[4], p[5]), mk(p[6], p[7], p[8])};
}

// the four children of cell T (corner slot of each in cc[]) integrated by one warp: the lanes
// stride over the flattened (child, quadrature point) list -- the graded Duffy rule for a child
// that holds the shared vertex, the 13-point rule otherwise -- and a butterfly leaves the four
// sums in every lane.  A cell costs 52 to 300 point evaluations, so spreading them over the warp
// is what keeps the GPU busy when a depth holds only a few thousand cells.
template <int CLS>
__device__ void pot_children_warp(const Tri &T, const int cc[4], const PotPairCtx &c, const QuadTables &Q, int lane, double v[4])
{
    const int nduffy = Q.nu * Q.nv;
    int start[5];
    start[0] = 0;
    for (int k = 0; k < 4; ++k) start[k + 1] = start[k] + (cc[k] >= 0 ? nduffy : Q.npts);
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (int j = lane; j < start[4]; j += 32) {
        const int k = j < start[1] ? 0 : (j < start[2] ? 1 : (j < start[3] ? 2 : 3));
        const int p = j - start[k];
        const Tri Tc = child(T, k);
        double g;
        if (cc[k] >= 0) {
            const int corner = cc[k];
            const d3 Vx = corner == 0 ? Tc.a : (corner == 1 ? Tc.b : Tc.c);
            const d3 B = corner == 0 ? Tc.b : (corner == 1 ? Tc.c : Tc.a);
            const d3 Cc = corner == 0 ? Tc.c : (corner == 1 ? Tc.a : Tc.b);
            const d3 eB = B - Vx, eC = Cc - Vx;
            const int a = p / Q.nv, b = p - a * Q.nv;
            const double u = Q.du_u[a], vv = Q.dv_v[b];
            const d3 w = u * ((1.0 - vv) * eB + vv * eC);
            d3 psi;
            double th;
            far_integrand_o((Vx - c.K.A) + w, (Vx - c.K.B) + w, (Vx - c.K.C) + w, c.K, c.F, psi, th, g);
            if (CLS == kEdge) g -= pot_edge_sigma(Vx + w, c.pe);
            g *= Q.du_w[a] * u * Q.dv_w[b] * norm(cross(eB, eC));
        } else {
            const double l1 = Q.L1[p], l2 = Q.L2[p], l3 = Q.L3[p];
            const d3 oa = l1 * (Tc.a - c.K.A) + l2 * (Tc.b - c.K.A) + l3 * (Tc.c - c.K.A);
            const d3 ob = l1 * (Tc.a - c.K.B) + l2 * (Tc.b - c.K.B) + l3 * (Tc.c - c.K.B);
            const d3 oc = l1 * (Tc.a - c.K.C) + l2 * (Tc.b - c.K.C) + l3 * (Tc.c - c.K.C);
            d3 psi;
            double th;
            far_integrand_o(oa, ob, oc, c.K, c.F, psi, th, g);
            if (CLS == kEdge) g -= pot_edge_sigma(oa + c.K.A, c.pe);
            g *= Q.w[p] * 0.5 * norm(cross(Tc.b - Tc.a, Tc.c - Tc.a));
        }
        acc[k] += g;
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        double x = acc[k];
        for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
        v[k] = x;
    }
}

template <int CLS>
__device__ __forceinline__ void pot_seed_item(const ClassArgs &A, const QuadTables &Q, double tol, int h, int lane)
{
    const int t = A.hard_list[h];
    const PotPairCtx c = pot_pair_ctx<CLS>(A, t, tol);
    const int3 ci = A.cells[A.pairs[t].x], cj = A.cells[A.pairs[t].y];
    const int ia[3] = {ci.x, ci.y, ci.z};
    bool shared[3];
    for (int k = 0; k < 3; ++k) shared[k] = (ia[k] == cj.x || ia[k] == cj.y || ia[k] == cj.z);
    // the root's children 0, 1, 2 hold K_i's slots b, c, a in their slot 1
    int cc[4];
    for (int k = 0; k < 4; ++k) cc[k] = k == 3 ? -1 : (shared[k == 0 ? 1 : (k == 1 ? 2 : 0)] ? 1 : -1);
    double v[4];
    pot_children_warp<CLS>(c.Ti, cc, c, Q, lane, v);
    if (lane < 4) A.pot_q_a[4 * (long long)h + lane] = PotCellItem{(unsigned long long)lane, v[lane], h, cc[lane]};
    if (lane == 0) {
        A.pot_fx[h] = 0;
        if (h < A.pot_ctx_cap) *reinterpret_cast<PotPairCtx *>(A.pot_ctx + (long long)kPotCtxDoubles * h) = c;
        if (h < A.pot_tri_cap) pot_tri_store(pot_tri_list(A, 1) + 9LL * h, c.Ti);  // parent of depth 1's slots 4h..4h+3
    }
}

template <int CLS>
__global__ void __launch_bounds__(128) k_pot_seed(ClassArgs A, QuadTables Q, double tol)
{
    const int count = pot_seeded(A);
    // the depth kernels run after this one on the same stream
    if (blockIdx.x == 0 && threadIdx.x == 0) pot_seed_init(A);
    const int lane = threadIdx.x & 31;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int h = (int)warp_item_index(); h < count; h += nwarps) pot_seed_item<CLS>(A, Q, tol, h, lane);
}

// one cell of one depth, by one warp
template <int CLS>
__device__ __forceinline__ void pot_depth_item(const ClassArgs &A, const QuadTables &Q, double tol, int depth,
                                               const PotCellItem *__restrict__ in, PotCellItem *__restrict__ out, int idx, int lane)
{
    const PotCellItem it = in[idx];
    if (it.h < 0) return;
    const int t = A.hard_list[it.h];
    const PotPairCtx c = pot_ctx_of<CLS>(A, it.h, t, tol);
    // siblings sit at 4 consecutive slots, so the parent's triangle is at slot idx / 4
    const Tri T = (idx >> 2) < A.pot_tri_cap ? child(pot_tri_load(pot_tri_list(A, depth) + 9LL * (idx >> 2)), (int)(it.path & 3))
                                             : subcell(c.Ti, depth, (int)it.path);
    int cc[4];
    for (int k = 0; k < 4; ++k) cc[k] = child_corner(it.corner, k);
    double v[4];
    pot_children_warp<CLS>(T, cc, c, Q, lane, v);
    if (lane != 0) return;
    const double sum = v[0] + v[1] + v[2] + v[3];
    bool accept = fabs(sum - it.val) <= ldexp(c.tol_abs, -depth) || depth >= kHardMaxDepth;
    if (!accept) {
        const int pos = atomicAdd(&A.pot_qcnt[depth + 1], 4);
        if (pos + 4 <= A.pot_qcap) {
            for (int k = 0; k < 4; ++k) out[pos + k] = PotCellItem{(it.path << 2) | (unsigned long long)k, v[k], it.h, cc[k]};
            if ((pos >> 2) < A.pot_tri_cap) pot_tri_store(pot_tri_list(A, depth + 1) + 9LL * (pos >> 2), T);
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

// one depth: one warp per cell
template <int CLS>
__global__ void __launch_bounds__(128, 3) k_pot_depth(ClassArgs A, QuadTables Q, double tol, int depth, const PotCellItem *__restrict__ in,
                                                   PotCellItem *__restrict__ out)
{
    const int count = pot_depth_count(A, depth);
    const int lane = threadIdx.x & 31;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int idx = (int)warp_item_index(); idx < count; idx += nwarps)
        pot_depth_item<CLS>(A, Q, tol, depth, in, out, idx, lane);
}

template <int CLS>
__device__ __forceinline__ void pot_final_item(const ClassArgs &A, double tol, int h)
{
    const int t = A.hard_list[h];
    const PotPairCtx c = pot_ctx_of<CLS>(A, h, t, tol);
    A.padj[t] = kInv4Pi * ((double)A.pot_fx[h] / c.scale + c.sig_int);
}

template <int CLS>
__global__ void __launch_bounds__(128) k_pot_final(ClassArgs A, double tol)
{
    const int count = pot_seeded(A);
    for (int h = blockIdx.x * blockDim.x + threadIdx.x; h < count; h += gridDim.x * blockDim.x) pot_final_item<CLS>(A, tol, h);
}

template <int CLS>
static void pot_adaptive_chain(const ClassArgs &A, const QuadTables &Q, double tol, int persistent_blocks, cudaStream_t s)
{
    k_pot_seed<CLS><<<resident_grid((const void *)k_pot_seed<CLS>, 128, 0), 128, 0, s>>>(A, Q, tol);
    const int grid = resident_grid((const void *)k_pot_depth<CLS>, 128, 0);
    for (int d = 1; d <= kHardMaxDepth; ++d)
        k_pot_depth<CLS><<<grid, 128, 0, s>>>(A, Q, tol, d, d % 2 ? A.pot_q_a : A.pot_q_b, d % 2 ? A.pot_q_b : A.pot_q_a);
    k_pot_final<CLS><<<persistent_blocks, 128, 0, s>>>(A, tol);
}
// ------------------------------------------------------------------ self pairs (helpers: i2_self.cuh)
__global__ void __launch_bounds__(128) k_self(ClassArgs A, QuadTables Q, int self_sign)
{
    const int lane = threadIdx.x & 31, k = lane / 6;
    const long long t = (((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * kSelfPairsPerWarp + k;
    const bool valid = k < kSelfPairsPerWarp && t < A.n;
    const double sum = self_gather6(valid ? self_piece_of(A, Q, t, lane % 6) : 0.0);
    if (valid && lane % 6 == 0) self_store(A, self_sign, t, sum);
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

int resident_grid(const void *kernel, int threads, size_t smem)
{
    int dev = 0, sms = 0, nb = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) sms = 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, threads, smem) != cudaSuccess || nb <= 0) nb = 1;
    return std::max(1, sms) * nb;
}

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
    const long long warps = (A.n + kSelfPairsPerWarp - 1) / kSelfPairsPerWarp;
    k_self<<<blocks_for(32 * warps, 128), 128, 0, s>>>(A, Q, cfg.self_sign);
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
        launch_self(A, Q, cfg, s);
        break;
    case kEdge:
        if (A.pot_off) cudaMemsetAsync(A.padj, 0xff, sizeof(double) * (size_t)A.n, s);  // all-ones bytes: NaN
        k_singular<kEdge><<<blocks_for(A.n, tpb), tpb, 0, s>>>(A, Q);
        if (A.hard_list) {
            k_pot_tier2<kEdge><<<resident_grid((const void *)k_pot_tier2<kEdge>, tpb, 0), tpb, 0, s>>>(A, Q);
            k_pot_tier2b<kEdge><<<resident_grid((const void *)k_pot_tier2b<kEdge>, tpb, 0), tpb, 0, s>>>(A, Q, 1);
            pot_adaptive_chain<kEdge>(A, Q, cfg.hard_tol, persistent_blocks, s);
        }
        level_chain<kEdge>(A, Q, cfg, persistent_blocks, s);
        break;
    case kVertex:
        if (A.pot_off) cudaMemsetAsync(A.padj, 0xff, sizeof(double) * (size_t)A.n, s);
        k_singular<kVertex><<<blocks_for(A.n, tpb), tpb, 0, s>>>(A, Q);
        if (A.hard_list) {
            k_pot_tier2<kVertex><<<resident_grid((const void *)k_pot_tier2<kVertex>, tpb, 0), tpb, 0, s>>>(A, Q);
            k_pot_tier2b<kVertex><<<resident_grid((const void *)k_pot_tier2b<kVertex>, tpb, 0), tpb, 0, s>>>(A, Q, 1);
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
