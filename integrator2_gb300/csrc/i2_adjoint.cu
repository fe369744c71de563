// i2_adjoint.cu -- adjoint of the pair integrals with respect to the mesh's vertex coordinates.
//
// Given upstream gradients gJ (dL/dJ_p, 3 per pair) and gP (dL/dP_p), the backward pass adds
//     dL/dV[v] += sum_p gJ_p . dJ_p/dV[v] + gP_p dP_p/dV[v]
// for every vertex v of every pair p.  One thread owns one (pair, vertex) item: it recomputes
// the pair's forward rules -- closed-form singular part, regular part on the refined sub-cells of
// the level the forward pass kept, graded-Duffy / tiered / adaptive potential, self-pair
// potential -- on dual numbers seeded with that vertex's three coordinates (i2_dual.cuh), so
// the derivative includes the singular analytic parts, and nothing of the refinement is stored
// between the passes: the sub-cells are re-derived from their paths.  A vertex shared by K_i and
// K_j is seeded in both triangles at once and handled by a single item.  Coordinates are taken
// relative to K_j's first vertex (a translation, which leaves J and P unchanged) so that the
// FP32 variant keeps the precision of the offsets.  The FP32 variant differentiates the disjoint
// class's regular part in FP32 (with the cancellation-free edge logs of the FP32 bulk) and the
// rest in FP64, as the mixed forward pass splits the work.
#include "i2_dual.cuh"
#include "i2_engine.h"

namespace i2 {

struct AdjointArgs {
    int n;
    const int2 *pairs;
    const int3 *cells;
    const double *V;         // 3 per vertex
    const int *stop;         // refinement level each pair stopped at (nullptr: fixed level)
    const int *maxlev;       // class-wide last level (compat mode's buffer parity)
    int mode, fixed_level;
    const double *gJ, *gP;   // upstream gradients (either may be nullptr)
    double *gradV;           // 3 per vertex, accumulated
    double hard_tol, tier_tol, top_tol;
    int self_sign;
};

template <class R>
__device__ __forceinline__ V3<R> seeded_vertex(const double *V, int vid, int seed, double3 o)
{
    V3<R> p{R(V[3 * vid] - o.x), R(V[3 * vid + 1] - o.y), R(V[3 * vid + 2] - o.z)};
    if (vid == seed) {
        p.x.d[0] = 1;
        p.y.d[1] = 1;
        p.z.d[2] = 1;
    }
    return p;
}

// level whose sums the forward pass kept for this pair (finalize_item's rule)
__device__ __forceinline__ int kept_level(const AdjointArgs &A, int t)
{
    if (A.mode == kFixed || !A.stop) return A.fixed_level;
    const int L = A.stop[t];
    if (A.mode == kAdaptiveCompat && ((*A.maxlev - L) & 1)) return L > 0 ? L - 1 : 0;
    return L;
}

// regular part of (Psi, Theta, potential) over the 4^L sub-cells of K_i
template <int CLS, class R>
__device__ void regular_part(const TriT<R> &Ti, const PanelJT<R> &K, const FarCtxT<R> &F, const EdgeCtxT<R> &E,
                             const VertexCtxT<R> &Vx, R Si, int level, const QuadTables &Q, V3<R> &psi, R &th, R &pot)
{
    psi = V3<R>{R(0.0), R(0.0), R(0.0)};
    th = R(0.0);
    pot = R(0.0);
    const R Ssub = Si * ldexp(1.0, -2 * level);
    const int nsub = 1 << (2 * level);
    for (int s = 0; s < nsub; ++s) {
        const TriT<R> T = subcell(Ti, level, s);
        V3<R> cp{R(0.0), R(0.0), R(0.0)};
        R ct = 0.0, cpot = 0.0;
        for (int g = 0; g < Q.npts; ++g) {
            const V3<R> x = Q.L1[g] * T.a + Q.L2[g] * T.b + Q.L3[g] * T.c;
            V3<R> p;
            R t, pt = 0.0;
            if (CLS == kFar && sizeof(value_of(R())) == sizeof(float)) far_integrand_pos(x, K, F, p, t, pt);
            else if (CLS == kFar) far_integrand(x, K, F, p, t, pt);
            else if (CLS == kEdge) edge_integrand(x, K, E, p, t);
            else vertex_integrand(x, K, Vx, p, t);
            cp = cp + Q.w[g] * p;
            ct += Q.w[g] * t;
            cpot += Q.w[g] * pt;
        }
        psi = psi + Ssub * cp;
        th += Ssub * ct;
        pot += Ssub * cpot;
    }
}

// adaptive potential of a hard pair, depth first with an explicit stack (same acceptance rule
// and depth cap as the forward pass's breadth-first queue)
template <int CLS, class R>
__device__ R adaptive_potential(const TriT<R> &Ti0, const bool shared[3], const PanelJT<R> &K, const FarCtxT<R> &F,
                                const PotEdgeT<R> &pe, const QuadTables &Q, double tol_abs)
{
    struct Item {
        unsigned long long path;
        double val;
        int depth, corner;
    };
    Item st[4 * kHardMaxDepth + 4];
    int top = 0;
    for (int k = 0; k < 4; ++k) {
        const int corner = k == 3 ? -1 : (shared[k == 0 ? 1 : (k == 1 ? 2 : 0)] ? 1 : -1);
        st[top++] = Item{(unsigned long long)k, value_of(pot_cell<CLS>(child(Ti0, k), corner, K, F, pe, Q)), 1, corner};
    }
    R acc = 0.0;
    while (top > 0) {
        const Item it = st[--top];
        const TriT<R> T = subcell(Ti0, it.depth, (int)it.path);
        R v[4];
        R sum = 0.0;
        for (int k = 0; k < 4; ++k) {
            v[k] = pot_cell<CLS>(child(T, k), child_corner(it.corner, k), K, F, pe, Q);
            sum += v[k];
        }
        if (fabs(value_of(sum) - it.val) <= ldexp(tol_abs, -it.depth) || it.depth >= kHardMaxDepth) {
            acc += sum;
        } else {
            for (int k = 0; k < 4; ++k)
                st[top++] = Item{(it.path << 2) | (unsigned long long)k, value_of(v[k]), it.depth + 1, child_corner(it.corner, k)};
        }
    }
    return acc;
}

// largest cosine of a corner angle of a triangle (the forward pass's sliver test)
template <class R>
__device__ __forceinline__ double max_corner_cos(const TriT<R> &T)
{
    const V3<R> P[3] = {T.a, T.b, T.c};
    double m = -1.0;
    for (int k = 0; k < 3; ++k) {
        const V3<R> u = unit(P[(k + 1) % 3] - P[k]), w = unit(P[(k + 2) % 3] - P[k]);
        m = fmax(m, (double)value_of(dot(u, w)));
    }
    return m;
}

template <int CLS, class T>
__global__ void __launch_bounds__(128) k_adjoint(AdjointArgs A, QuadTables Q)
{
    using R = ad::Dual<T, 3>;
    const long long items = 6LL * A.n;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < items; idx += (long long)gridDim.x * blockDim.x) {
        const int t = (int)(idx / 6), slot = (int)(idx % 6);
        const int2 pr = A.pairs[t];
        const int3 ci = A.cells[pr.x], cj = A.cells[pr.y];
        const int vi[3] = {ci.x, ci.y, ci.z}, vj[3] = {cj.x, cj.y, cj.z};
        const int seed = slot < 3 ? vi[slot] : vj[slot - 3];
        // a K_j vertex that K_i also holds is seeded by K_i's item
        if (slot >= 3 && (seed == vi[0] || seed == vi[1] || seed == vi[2])) continue;
        const double3 o = make_double3(A.V[3 * vj[0]], A.V[3 * vj[0] + 1], A.V[3 * vj[0] + 2]);
        const TriT<R> Ti0{seeded_vertex<R>(A.V, vi[0], seed, o), seeded_vertex<R>(A.V, vi[1], seed, o),
                          seeded_vertex<R>(A.V, vi[2], seed, o)};
        const TriT<R> Tj0{seeded_vertex<R>(A.V, vj[0], seed, o), seeded_vertex<R>(A.V, vj[1], seed, o),
                          seeded_vertex<R>(A.V, vj[2], seed, o)};
        const PanelJT<R> K = make_panel(Tj0.a, Tj0.b, Tj0.c);
        const V3<R> cri = cross(Ti0.b - Ti0.a, Ti0.c - Ti0.a);
        const V3<R> ni = unit(cri);
        const R Si = 0.5 * norm(cri);
        V3<R> J;
        R P;
        if (CLS == kSelf) {
            const double sgn = A.self_sign == 0 ? 0.0 : (A.self_sign > 0 ? kTwoPi : -kTwoPi);
            J = kInv4Pi * ((sgn * K.S) * K.n);
            P = kInv4Pi * self_potential(K.A, K.B, K.C, Q);
        } else {
            const int level = kept_level(A, t);
            const FarCtxT<R> F = make_far_ctx(K);
            EdgeCtxT<R> E;
            VertexCtxT<R> Vx;
            V3<R> psi_s{R(0.0), R(0.0), R(0.0)};
            R th_s = 0.0;
            int si = 0, sj = 0;
            if (CLS == kEdge) {
                shifts_edge(ci, cj, si, sj);
                E = make_edge_ctx(K, sj);
                closed_edge(rotate(Ti0, si), rotate(Tj0, sj), ni, K.n, Si, psi_s, th_s);
            } else if (CLS == kVertex) {
                shifts_vertex(ci, cj, si, sj);
                Vx = make_vertex_ctx(K, sj, ni, Si);
                closed_vertex(rotate(Ti0, si), rotate(Tj0, sj), ni, K.n, Si, psi_s, th_s);
            }
            V3<R> psi;
            R th, pot;
            regular_part<CLS>(Ti0, K, F, E, Vx, Si, level, Q, psi, th, pot);
            J = finalize_j(CLS, psi + psi_s, th + th_s, K.n, Si);
            if (CLS == kFar) {
                P = kInv4Pi * pot;
            } else {
                // potential: the forward pass's tiered rule, decided on values
                const TriT<R> Ti = rotate(Ti0, si);
                PotEdgeT<R> pe{};
                const R sig = CLS == kEdge ? make_pot_edge(Ti, rotate(Tj0, sj), K, Si, pe) : R(0.0);
                R pm = duffy_total<CLS>(Ti, K, F, pe, Q.du_u, Q.du_w, Q.nu, Q.dv_v, Q.dv_w, Q.nv) + sig;
                bool adapt = false;
                if (A.hard_tol > 0.0) {
                    const double c10 = 0.98480775301220806;
                    if (value_of(dot(ni, K.n)) < 0.5 || max_corner_cos(Ti0) > c10 || max_corner_cos(Tj0) > c10) {
                        adapt = true;
                    } else {
                        const R pl = duffy_total<CLS>(Ti, K, F, pe, Q.lo_u, Q.lo_uw, Q.lo_nu, Q.lo_v, Q.lo_vw, Q.lo_nv) + sig;
                        if (fabs(value_of(pm) - value_of(pl)) > A.tier_tol * fabs(value_of(pm))) {
                            const R ph = duffy_total<CLS>(Ti, K, F, pe, Q.hi_u, Q.hi_uw, Q.hi_nu, Q.hi_v, Q.hi_vw, Q.hi_nv) + sig;
                            const bool agree = fabs(value_of(ph) - value_of(pm)) <= A.tier_tol * fabs(value_of(ph));
                            pm = ph;
                            if (!agree) {
                                const R pt = duffy_total<CLS>(Ti, K, F, pe, Q.top_u, Q.top_uw, Q.top_nu, Q.top_v, Q.top_vw, Q.top_nv) + sig;
                                adapt = fabs(value_of(pt) - value_of(ph)) > A.top_tol * fabs(value_of(pt));
                                if (!adapt) pm = pt;
                            }
                        }
                    }
                }
                if (adapt) {
                    bool shared[3];
                    for (int k = 0; k < 3; ++k) shared[k] = (vi[k] == vj[0] || vi[k] == vj[1] || vi[k] == vj[2]);
                    const double tol_abs = A.hard_tol * fabs(value_of(pm));
                    pm = adaptive_potential<CLS>(Ti0, shared, K, F, pe, Q, tol_abs) + sig;
                }
                P = kInv4Pi * pm;
            }
        }
        const double gj0 = A.gJ ? A.gJ[3 * (long long)t] : 0.0, gj1 = A.gJ ? A.gJ[3 * (long long)t + 1] : 0.0,
                     gj2 = A.gJ ? A.gJ[3 * (long long)t + 2] : 0.0, gp = A.gP ? A.gP[t] : 0.0;
        for (int k = 0; k < 3; ++k) {
            const double g = gj0 * (double)J.x.d[k] + gj1 * (double)J.y.d[k] + gj2 * (double)J.z.d[k] + gp * (double)P.d[k];
            if (g != 0.0) atomicAdd(A.gradV + 3 * (long long)seed + k, g);
        }
    }
}

template <class T>
static void launch_adjoint_t(int cls, const AdjointArgs &A, const QuadTables &Q, int blocks, cudaStream_t s)
{
    switch (cls) {
    case kVertex: k_adjoint<kVertex, T><<<blocks, 128, 0, s>>>(A, Q); break;
    case kEdge: k_adjoint<kEdge, T><<<blocks, 128, 0, s>>>(A, Q); break;
    case kFar: k_adjoint<kFar, T><<<blocks, 128, 0, s>>>(A, Q); break;
    default: k_adjoint<kSelf, T><<<blocks, 128, 0, s>>>(A, Q); break;
    }
}

void launch_adjoint(int cls, bool fp32, const int2 *pairs, int n, const int3 *cells, const double *V, const int *stop,
                    const int *maxlev, const RunConfig &cfg, double tier_tol, double top_tol, const double *gJ, const double *gP, double *gradV,
                    const QuadTables &Q, int persistent_blocks, cudaStream_t s)
{
    if (n <= 0) return;
    AdjointArgs A;
    A.n = n;
    A.pairs = pairs;
    A.cells = cells;
    A.V = V;
    A.stop = cfg.mode == kFixed ? nullptr : stop;
    A.maxlev = maxlev;
    A.mode = cfg.mode;
    A.fixed_level = cfg.level;
    A.gJ = gJ;
    A.gP = gP;
    A.gradV = gradV;
    A.hard_tol = cfg.hard_tol;
    A.tier_tol = tier_tol;
    A.top_tol = top_tol;
    A.self_sign = cfg.self_sign;
    const long long items = 6LL * n;
    const int blocks = (int)std::min<long long>((items + 127) / 128, (long long)persistent_blocks * 4);
    // the FP32 variant mirrors the mixed forward pass: FP32 for the disjoint class's regular part,
    // FP64 for the closed forms and potential rules of adjacent pairs and for self pairs
    if (fp32 && cls == kFar) k_adjoint<kFar, float><<<std::max(1, blocks), 128, 0, s>>>(A, Q);
    else launch_adjoint_t<double>(cls, A, Q, std::max(1, blocks), s);
}

} // namespace i2
