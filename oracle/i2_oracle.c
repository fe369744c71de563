/*
 * i2_oracle.c -- CPU oracle (TEST INFRASTRUCTURE ONLY, never shipped or measured as the
 * product).  Plain C99, FP64, OpenMP over tasks.  See i2_oracle.h for the parity status.
 *
 * Each function names the reference lines (andreyypopov/integrator2) whose mathematics it
 * restates.  Operation order follows the reference where that keeps the pinning tests
 * tight; device math (log, atan2, sincos, acos, tan) becomes the C library's.
 */
#define _GNU_SOURCE
#include "i2_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* tolerances and constants of the reference (src/common/constants.h:13-26) */
#define O_DOUBLE_MIN 2e-6
#define O_EPS 1e-6
#define O_EPS2 1e-10
#define O_EPS_PSI2 1e-12
#define O_EPS_RUNGE 1e-5
#define O_PI 3.14159265358979323846
#define O_TWO_PI 6.28318530717958647692
#define O_INV_4PI 0.079577471545947667884
#define O_MAX_LEVEL 5

typedef struct { double x, y, z; } v3;

static inline v3 mk(double x, double y, double z) { v3 r = {x, y, z}; return r; }
static inline v3 ld(const double *p) { return mk(p[0], p[1], p[2]); }
static inline v3 add(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 sub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 scl(double s, v3 a) { return mk(a.x * s, a.y * s, a.z * s); }
static inline v3 dvd(v3 a, double s) { return mk(a.x / s, a.y / s, a.z / s); }
static inline double dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 crs(v3 a, v3 b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline double len(v3 a) { return sqrt(dot(a, a)); }
static inline v3 unit(v3 a) { double inv = 1.0 / len(a); return mk(a.x * inv, a.y * inv, a.z * inv); }

typedef struct { double v[4]; } q4; /* (Psi.x, Psi.y, Psi.z, Theta) */

static inline q4 q4zero(void) { q4 r = {{0, 0, 0, 0}}; return r; }
static inline q4 q4add(q4 a, q4 b) { q4 r; for (int k = 0; k < 4; ++k) r.v[k] = a.v[k] + b.v[k]; return r; }
static inline q4 q4sub(q4 a, q4 b) { q4 r; for (int k = 0; k < 4; ++k) r.v[k] = a.v[k] - b.v[k]; return r; }
static inline q4 q4scl(double s, q4 a) { q4 r; for (int k = 0; k < 4; ++k) r.v[k] = a.v[k] * s; return r; }
static inline q4 q4vec(v3 p, double w) { q4 r = {{p.x, p.y, p.z, w}}; return r; }

/* angle between two vectors with the reference's clamps (src/common/cuda_math.cu:14-26) */
static double o_angle(v3 a, v3 b)
{
    double den = sqrt(dot(a, a) * dot(b, b));
    if (den < O_EPS) return 0.0;
    double c = dot(a, b) / den;
    if (c >= 1.0) return 0.0;
    if (c <= -1.0) return O_PI;
    return acos(c);
}

/* sign() and arg() helpers of the reference (src/common/cuda_math.cuh:31-49) */
static inline double o_sign(double x)
{
    if (fabs(x) < O_DOUBLE_MIN) return 0.0;
    return x > O_DOUBLE_MIN ? 1.0 : -1.0;
}
static inline double o_arg(double x) { return x > O_DOUBLE_MIN ? 0.0 : O_PI; }

static inline void tri_of(const double *V, const int *C, int c, v3 *a, v3 *b, v3 *cc)
{
    *a = ld(V + 3 * C[3 * c]);
    *b = ld(V + 3 * C[3 * c + 1]);
    *cc = ld(V + 3 * C[3 * c + 2]);
}

/* ---------------------------------------------------------------- mesh prep */
/* src/Mesh3d.cu:23-71: n = unit((B-A)x(C-A)), S = |(B-A)x(C-A)|/2, centre = (A+B+C)/3 */
void o_cell_geometry(int nc, const double *V, const int *C, double *normals, double *measures, double *centres)
{
    for (int c = 0; c < nc; ++c) {
        v3 a, b, cc;
        tri_of(V, C, c, &a, &b, &cc);
        v3 cr = crs(sub(b, a), sub(cc, a));
        v3 n = unit(cr);
        if (normals) { normals[3 * c] = n.x; normals[3 * c + 1] = n.y; normals[3 * c + 2] = n.z; }
        if (measures) measures[c] = len(cr) * 0.5;
        if (centres) {
            v3 m = scl(0.3333333333333333, add(add(a, b), cc));
            centres[3 * c] = m.x; centres[3 * c + 1] = m.y; centres[3 * c + 2] = m.z;
        }
    }
}

/* ---------------------------------------------------------------- a1: theta / psi */
/* One edge log term: ln of the ratio of (R + x.tau) at the edge's two ends, with the
 * reference's collinear fallback (evaluatorJ3DK.cu:294-307). */
static inline double edge_log(double l_from, double r_from, double l_to, double r_to)
{
    /* r_* = unit(x - P).tau, l_* = |x - P| */
    if (fabs(r_to + 1.0) < 0.5 * O_EPS_PSI2) return log(l_to / l_from);
    return log((l_from * (1.0 + r_from)) / (l_to * (1.0 + r_to)));
}

typedef struct {
    q4 tp;      /* Psi, Theta */
    double L[3]; /* line integrals of 1/R along edges BC (a), CA (b), AB (c) */
} tp_full;

/* theta/psi from the point-to-vertex offsets oa = x - A, ob = x - B, oc = x - C */
static tp_full theta_psi_offsets(v3 oa, v3 ob, v3 oc, v3 A, v3 B, v3 C)
{
    tp_full out;
    double la = len(oa), lb = len(ob), lc = len(oc);
    oa = dvd(oa, la); ob = dvd(ob, lb); oc = dvd(oc, lc);
    v3 ta = unit(sub(C, B)), tb = unit(sub(A, C)), tc = unit(sub(B, A));
    double rac = dot(oa, tc), rbc = dot(ob, tc), rba = dot(ob, ta);
    double rca = dot(oc, ta), rcb = dot(oc, tb), rab = dot(oa, tb);
    double Lc = edge_log(la, rac, lb, rbc); /* edge A->B */
    double La = edge_log(lb, rba, lc, rca); /* edge B->C */
    double Lb = edge_log(lc, rcb, la, rab); /* edge C->A */
    v3 psi = add(add(scl(Lc, tc), scl(La, ta)), scl(Lb, tb));
    double num = dot(crs(oa, ob), oc);
    double den = 1.0 + dot(oa, ob) + dot(ob, oc) + dot(oc, oa);
    out.tp = q4vec(psi, 2.0 * atan2(num, den));
    out.L[0] = La; out.L[1] = Lb; out.L[2] = Lc;
    return out;
}

static tp_full theta_psi_full(v3 x, v3 A, v3 B, v3 C)
{
    return theta_psi_offsets(sub(x, A), sub(x, B), sub(x, C), A, B, C);
}

void o_theta_psi(const double *x, const double *A, const double *B, const double *C, double *out4)
{
    tp_full t = theta_psi_full(ld(x), ld(A), ld(B), ld(C));
    memcpy(out4, t.tp.v, 4 * sizeof(double));
}

/* Potential of the flat triangle seen from x:  int_K 1/|x-y| dS_y = sum_e t_e L_e - d*Theta,
 * t_e the signed in-plane distance from x to edge e (positive inside), L_e the edge line
 * integral of 1/R (the same logs as Psi), d the height of x over the plane (Theta has the
 * sign of d, so d*Theta = |d||Omega|).  No counterpart in the reference. */
static double potential_offsets(v3 oa, v3 ob, v3 oc, v3 A, v3 B, v3 C, const tp_full *t)
{
    v3 n = unit(crs(sub(B, A), sub(C, A)));
    v3 ta = unit(sub(C, B)), tb = unit(sub(A, C)), tc = unit(sub(B, A));
    double sa = -dot(crs(ta, n), ob);
    double sb = -dot(crs(tb, n), oc);
    double sc = -dot(crs(tc, n), oa);
    double d = dot(n, oa);
    /* t_e L_e -> 0 on the edge's line even where L_e overflows */
    double pa = sa == 0.0 ? 0.0 : sa * t->L[0], pb = sb == 0.0 ? 0.0 : sb * t->L[1], pc = sc == 0.0 ? 0.0 : sc * t->L[2];
    return pa + pb + pc - d * t->tp.v[3];
}

static double potential_from(v3 x, v3 A, v3 B, v3 C, const tp_full *t)
{
    return potential_offsets(sub(x, A), sub(x, B), sub(x, C), A, B, C, t);
}

double o_potential_inner(const double *x, const double *A, const double *B, const double *C)
{
    v3 X = ld(x), a = ld(A), b = ld(B), c = ld(C);
    tp_full t = theta_psi_full(X, a, b, c);
    return potential_from(X, a, b, c, &t);
}

/* ---------------------------------------------------------------- a6: index shifts */
/* position (0..2) in each triangle of the single shared vertex (evaluatorJ3DK.cu:782-795):
 * the last match in scan order, as the reference's inner-only break leaves it */
static void shifts_vertex(const int *ti, const int *tj, int *si, int *sj)
{
    *si = 0; *sj = 0;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
            if (ti[a] == tj[b]) { *si = a; *sj = b; break; }
}

/* position in each triangle of the vertex that is NOT on the shared edge (:797-825) */
static void shifts_edge(const int *ti, const int *tj, int *si, int *sj)
{
    int mi[2] = {-1, -1}, mj[2] = {-1, -1}, k = 0;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
            if (ti[a] == tj[b] && k < 2) { mi[k] = a; mj[k] = b; ++k; }
    *si = 0; *sj = 0;
    for (int a = 0; a < 3; ++a) if (mi[0] != a && mi[1] != a) { *si = a; break; }
    for (int b = 0; b < 3; ++b) if (mj[0] != b && mj[1] != b) { *sj = b; break; }
}

/* cyclic rotation so that position s comes first (:827-847) */
static void rotated(const int *t, int s, int *out)
{
    for (int k = 0; k < 3; ++k) out[k] = t[(k + s) % 3];
}

/* ---------------------------------------------------------------- a2/a3: asymptotes */
typedef struct {     /* per-task constants of the common-edge asymptote */
    v3 JB, JC, ta, tb, tc;
    double ilvc;
} edge_ctx;

static edge_ctx make_edge_ctx(int i, int j, const double *V, const int *C)
{
    edge_ctx e;
    int si, sj, rj[3];
    shifts_edge(C + 3 * i, C + 3 * j, &si, &sj);
    rotated(C + 3 * j, sj, rj);
    v3 JA = ld(V + 3 * rj[0]);
    e.JB = ld(V + 3 * rj[1]);
    e.JC = ld(V + 3 * rj[2]);
    e.ta = unit(sub(JA, e.JC));
    e.tb = unit(sub(e.JB, JA));
    v3 c = sub(e.JC, e.JB);
    e.ilvc = 1.0 / len(c);
    e.tc = scl(e.ilvc, c);
    return e;
}

/* evaluatorJ3DK.cu:315-350 */
static q4 sing_edge(v3 x, const edge_ctx *e)
{
    v3 va = sub(x, e->JB), vb = sub(x, e->JC);
    double la = len(va), lb = len(vb);
    va = dvd(va, la); vb = dvd(vb, lb);
    double l1 = log((lb * dot(e->tc, sub(e->tc, vb))) / (la * dot(e->tc, sub(e->tc, va))));
    double l2 = log(la * dot(e->tb, add(e->tb, va)) * e->ilvc);
    double l3 = log(lb * dot(e->ta, sub(e->ta, vb)) * e->ilvc);
    v3 psi = sub(sub(scl(l1, e->tc), scl(l2, e->tb)), scl(l3, e->ta));
    double th = 2.0 * (atan2(dot(crs(va, e->tb), e->tc), dot(sub(e->tb, e->tc), add(e->tb, va))) -
                       atan2(dot(crs(vb, e->ta), e->tc), dot(sub(e->ta, e->tc), sub(e->ta, vb))));
    return q4vec(psi, th);
}

typedef struct {     /* per-task constants of the common-vertex asymptote */
    v3 JA, ta, tb, e;
    double inv_sqrt_si;
} vertex_ctx;

static void vertex_deltas(v3 ta, v3 tb, v3 nj, v3 e, double *dA, double *dB)
{
    *dA = atan2(dot(crs(ta, e), nj), -dot(e, ta));
    *dB = atan2(dot(crs(e, tb), nj), dot(e, tb));
}

/* direction of the planes' intersection line with the reference's two sign flips
 * (evaluatorJ3DK.cu:376-399, repeated at :698-723) */
static v3 vertex_direction(v3 ni, v3 nj, v3 ta, v3 tb, double *dA, double *dB)
{
    v3 e = crs(ni, nj);
    if (dot(e, e) < O_EPS2) e = tb;
    else e = unit(e);
    vertex_deltas(ta, tb, nj, e, dA, dB);
    if ((O_PI - fabs(*dA) < O_EPS) || (O_PI - fabs(*dB) < O_EPS)) {
        e = scl(-1.0, e);
        vertex_deltas(ta, tb, nj, e, dA, dB);
    }
    if ((*dA * *dB < 0) && (fabs(*dA - *dB) > O_PI)) {
        e = scl(-1.0, e);
        vertex_deltas(ta, tb, nj, e, dA, dB);
    }
    return e;
}

static vertex_ctx make_vertex_ctx(int i, int j, const double *V, const int *C, const double *N, const double *S)
{
    vertex_ctx c;
    int si, sj, rj[3];
    shifts_vertex(C + 3 * i, C + 3 * j, &si, &sj);
    rotated(C + 3 * j, sj, rj);
    c.JA = ld(V + 3 * rj[0]);
    v3 JB = ld(V + 3 * rj[1]), JC = ld(V + 3 * rj[2]);
    c.ta = unit(sub(c.JA, JC));
    c.tb = unit(sub(JB, c.JA));
    double dA, dB;
    c.e = vertex_direction(ld(N + 3 * i), ld(N + 3 * j), c.ta, c.tb, &dA, &dB);
    c.inv_sqrt_si = 1.0 / sqrt(S[i]);
    return c;
}

/* evaluatorJ3DK.cu:352-407 */
static q4 sing_vertex(v3 x, const vertex_ctx *c)
{
    v3 oc = sub(x, c->JA);
    double lc = len(oc);
    oc = dvd(oc, lc);
    double l1 = log((lc * (1 + dot(c->ta, oc))) * c->inv_sqrt_si);
    double l2 = log((lc * (1 - dot(c->tb, oc))) * c->inv_sqrt_si);
    v3 psi = scl(-1.0, add(scl(l1, c->ta), scl(l2, c->tb)));
    double th = 2.0 * (atan2(dot(crs(oc, c->ta), c->e), dot(sub(c->e, oc), sub(c->e, c->ta))) +
                       atan2(dot(crs(oc, c->tb), c->e), dot(sub(c->e, oc), add(c->e, c->tb))));
    return q4vec(psi, th);
}

void o_sing_edge(const double *x, int i, int j, const double *V, const int *C, double *out4)
{
    edge_ctx e = make_edge_ctx(i, j, V, C);
    q4 r = sing_edge(ld(x), &e);
    memcpy(out4, r.v, sizeof r.v);
}

void o_sing_vertex(const double *x, int i, int j, const double *V, const int *C, const double *N, const double *S, double *out4)
{
    vertex_ctx c = make_vertex_ctx(i, j, V, C, N, S);
    q4 r = sing_vertex(ld(x), &c);
    memcpy(out4, r.v, sizeof r.v);
}

/* ---------------------------------------------------------------- a4: common-edge closed form */
typedef struct { double s, c; } sc2;
static inline sc2 sincos2(double a) { sc2 r; sincos(a, &r.s, &r.c); return r; }

/* 2 atan2(sin xi sin a sin g, 1 - cos a + cos g + cos l)  (evaluatorJ3DK.cu:418-421) */
static inline double phi_fn(sc2 a, sc2 g, double sxi, double cl)
{
    return 2.0 * atan2(sxi * a.s * g.s, 1.0 - a.c + g.c + cl);
}

/* (q_theta, q_psi) of the general common-edge case (:438-461) */
static void q_edge(sc2 a, sc2 b, sc2 g, sc2 n, sc2 xi, double cmu, double cla, double *qt, double *qp)
{
    sc2 am = {a.s, -a.c}, gm = {g.s, -g.c};
    double p1 = phi_fn(a, g, xi.s, cla);
    double p2 = phi_fn(am, gm, xi.s, cla);
    double k = 1.0 / (a.s * (1.0 - cmu * cmu));
    *qt = p1 + g.s * n.s * k * ((b.c * g.s - xi.c * b.s * g.c) * p2 +
            xi.s * b.s * (0.5 * (1.0 + cmu) * log((1.0 + b.c) / (1.0 - n.c)) +
                          0.5 * (1.0 - cmu) * log((1.0 - b.c) / (1.0 + n.c)) +
                          log((1.0 + cla) / (1.0 - g.c))));
    *qp = 1.5 - k * (b.s * (n.c + cmu * cla) * log(1.0 + cla) +
                     n.s * (b.c + cmu * g.c) * log(1.0 - g.c) +
                     b.s * (1.0 - cmu) * (n.c - cla) * log(b.s / n.s) +
                     n.s * b.s * (b.s * g.c - xi.c * g.s * b.c) * log((1.0 - n.c) / (1.0 + b.c)) +
                     p2 * xi.s * g.s * n.s * b.s);
}

/* coplanar limit (:474-481).  The reference leaves q_theta unset here; its documented value
 * (and the limit of the general formula) is 0. */
static void q_edge_coplanar(sc2 b, sc2 n, double sa, double *qt, double *qp)
{
    *qt = 0.0;
    *qp = 1.5 - (n.c * b.s * log(1.0 + n.c) + n.s * b.c * log(1.0 - b.c) + sa - b.s + n.s +
                 b.s * n.c * log(b.s / n.s)) / sa;
}

static q4 closed_edge(int i, int j, const double *V, const int *C, const double *N, const double *S)
{
    int si, sj, ri[3], rj[3];
    shifts_edge(C + 3 * i, C + 3 * j, &si, &sj);
    rotated(C + 3 * i, si, ri);
    rotated(C + 3 * j, sj, rj);
    v3 IA = ld(V + 3 * ri[0]), IB = ld(V + 3 * ri[1]), IC = ld(V + 3 * ri[2]);
    v3 JA = ld(V + 3 * rj[0]), JB = ld(V + 3 * rj[1]), JC = ld(V + 3 * rj[2]);
    v3 ta = unit(sub(JA, JC)), tb = unit(sub(JB, JA)), tc = unit(sub(JC, JB));
    double al = o_angle(sub(IA, IC), sub(IB, IC));
    double be = o_angle(sub(IC, IB), sub(IA, IB));
    double ga = o_angle(sub(JC, JB), sub(JA, JB));
    double de = o_angle(sub(JB, JC), sub(JA, JC));
    double nu = O_PI - al - be;
    v3 ni = ld(N + 3 * i), nj = ld(N + 3 * j);
    double xi = atan2(dot(crs(ni, nj), tc), dot(ni, nj));
    sc2 sa = sincos2(al), sb = sincos2(be), sg = sincos2(ga), sd = sincos2(de), sx = sincos2(xi);
    sc2 sn = {sa.s * sb.c + sa.c * sb.s, sa.s * sb.s - sa.c * sb.c};
    double csig = -(sa.c * sd.c + sx.c * sa.s * sd.s);
    double cmu = -(sb.c * sg.c + sx.c * sb.s * sg.s);
    double cla = -(sa.c * sg.c - sx.c * sa.s * sg.s);
    double cth = -(sb.c * sd.c - sx.c * sb.s * sd.s);
    double qab = sn.s * log(tan(0.5 * al) * tan(0.5 * nu)) / sb.s +
                 sn.s * log(tan(0.5 * be) * tan(0.5 * nu)) / sa.s +
                 log(tan(0.5 * al) * tan(0.5 * be));
    double qAt, qAp, qBt, qBp;
    if (fabs(xi) < O_EPS && fabs(be - ga) < O_EPS) q_edge_coplanar(sb, sn, sa.s, &qAt, &qAp);
    else q_edge(sa, sb, sg, sn, sx, cmu, cla, &qAt, &qAp);
    if (fabs(xi) < O_EPS && fabs(al - de) < O_EPS) q_edge_coplanar(sa, sn, sb.s, &qBt, &qBp);
    else q_edge(sb, sa, sd, sn, sx, csig, cth, &qBt, &qBp);
    double si_ = S[i];
    v3 psi = scl(si_, sub(add(scl(qAp, tb), scl(qBp, ta)), scl(qab, tc)));
    return q4vec(psi, si_ * (qAt + qBt));
}

void o_closed_edge(int i, int j, const double *V, const int *C, const double *N, const double *S, double *out4)
{
    q4 r = closed_edge(i, j, V, C, N, S);
    memcpy(out4, r.v, sizeof r.v);
}

/* ---------------------------------------------------------------- a5: common-vertex closed form */
typedef struct {  /* angle data shared by the two halves A and B */
    sc2 xi, mu, nu, psi, nupsi, mupsi;
    double mu_a, nu_a, psi_a, kappa, skappa, lsmu, lsnu;
} vtx_angles;

/* (q_theta, q_psi) for one of the two edges of K_j at the shared vertex (:511-601) */
static void q_vertex(const vtx_angles *g, double delta, sc2 sd, double cla, double cth,
                     double ceta, double csig, double cchi, double *qt, double *qp)
{
    const double mu = g->mu_a, nu = g->nu_a, ps = g->psi_a, sk = g->skappa;
    const sc2 xi = g->xi, smu = g->mu, snu = g->nu, sps = g->psi;
    double lth = log(1.0 + cth), lla = log(1.0 + cla);
    double Lam1 = lla - lth + g->lsnu - g->lsmu;
    double Lam2 = log(tan(0.5 * nu) * tan(0.5 * mu));
    sc2 hd = sincos2(0.5 * delta);
    double thd = hd.s / hd.c;
    sc2 hmp = sincos2(0.5 * (mu - ps)), hnp = sincos2(0.5 * (nu + ps));
    double Amu = atan2(thd * hmp.c * xi.s, thd * hmp.c * xi.c + hmp.s);
    double Anu = atan2(thd * hnp.s * xi.s, thd * hnp.s * xi.c + hnp.c);
    sc2 t1 = sincos2(0.5 * (mu - ps) - 0.5 * (nu + ps)), t2 = sincos2(0.5 * g->kappa);
    double W = atan2(sd.s * t2.s * xi.s, t2.c + sd.s * t1.c * xi.c + sd.c * t1.s);
    sc2 t3 = sincos2(delta - ps);
    double D = 1.0 / (t3.s * t3.s + sd.s * sps.s * (1.0 - xi.c) * (t3.c + csig));
    double G = sps.c * (sd.s * csig * xi.c + sd.c * cchi - sd.s * sd.s / sps.s);
    double gent = 2.0 * (Anu * smu.s * g->nupsi.s - Amu * snu.s * g->mupsi.s -
                         D * smu.s * snu.s * sd.s * (W * ceta + 0.5 * sps.s * xi.s * (Lam1 - Lam2 * csig))) /
                  (sps.s * sk);
    double gens = 0.5 * (3.0 - log(2.0)) +
                  (smu.s * snu.s / sk) * ((lla - lth) * sps.c / sps.s +
                                          D * (Lam1 * sd.s * ceta / sps.s + Lam2 * cchi - 2.0 * W * sd.s * xi.s -
                                               G * (g->lsnu - g->lsmu))) -
                  (smu.c * snu.s * (lla - g->lsmu) + smu.s * snu.c * (lth - g->lsnu)) / sk -
                  0.5 * (g->lsmu + g->lsnu - log(sk));
    double mpsi = o_sign(xi.s * sps.s), mdel = o_sign(xi.s * sd.s);

    if (fabs(xi.s) < O_EPS && 1.0 - fabs(csig) < 0.5 * O_EPS2 && fabs(sps.s) > O_EPS) {
        double ara = o_arg(sin(0.5 * (nu + ps)) * csig);
        double arb = o_arg(cos(0.5 * (mu - ps)) * csig);
        *qt = 2.0 * mpsi * csig * xi.c / (sk * sps.s) * (smu.s * g->nupsi.s * ara - snu.s * g->mupsi.s * arb);
        *qp = 0.5 * (1.0 - log(2.0)) - 0.5 * log((1.0 - csig * smu.c) * (1.0 + csig * snu.c) / sk) +
              csig * (smu.s - snu.s + 0.5 * sin(mu - nu) * Lam2) / sk;
        return;
    }
    if (fabs(xi.s) < O_EPS && fabs(sps.s) > O_EPS) {
        double are = o_arg(sin(0.5 * (nu + mu)) + sin(0.5 * (mu - nu) - ps + delta * xi.c));
        double arc = o_arg(1.0 / tan(0.5 * (nu + ps)) + tan(0.5 * delta) * xi.c);
        double ard = o_arg(tan(0.5 * (mu - ps)) + tan(0.5 * delta) * xi.c);
        *qt = 2.0 * mdel * (sd.s * smu.s * snu.s / cchi * xi.c * are + smu.s * g->nupsi.s * arc -
                            snu.s * g->mupsi.s * ard) / (sk * sps.s);
        *qp = gens;
        return;
    }
    if (fabs(sin(ps)) < O_EPS) {
        if (fabs(delta) > O_EPS) {
            *qt = 2.0 * (smu.s * snu.s * (W * sd.c * xi.c - 0.5 * (Lam1 - Lam2 * csig) * xi.s) / sd.s +
                         (Anu + mdel * o_arg(sin(0.5 * (nu + ps)))) * smu.s * snu.c +
                         (Amu + mdel * o_arg(cos(0.5 * (mu - ps)))) * smu.c * snu.s) / sk;
            *qp = 0.5 * (3.0 - log(2.0)) - 0.5 * (log((1.0 + cla) * (1.0 + cth) / sk) - sin(mu - nu) / sk * Lam1) -
                  smu.s * snu.s * ((Lam1 * sd.c - Lam2 * sps.c) * xi.c + 2.0 * W * xi.s) / (sk * sd.s);
        } else {
            *qt = 2.0 * o_arg(sps.c);
            *qp = 0.5 * (1.0 - log(2.0)) - 0.5 * log((1.0 - sps.c * smu.c) * (1.0 + sps.c * snu.c) / sk) +
                  (0.5 * sin(mu - nu) * Lam1 + sps.c * (smu.s - snu.s)) / sk;
        }
        return;
    }
    *qt = gent;
    *qp = gens;
}

static q4 closed_vertex(int i, int j, const double *V, const int *C, const double *N, const double *S)
{
    int si, sj, ri[3], rj[3];
    shifts_vertex(C + 3 * i, C + 3 * j, &si, &sj);
    rotated(C + 3 * i, si, ri);
    rotated(C + 3 * j, sj, rj);
    v3 IA = ld(V + 3 * ri[0]), IB = ld(V + 3 * ri[1]), IC = ld(V + 3 * ri[2]);
    v3 JA = ld(V + 3 * rj[0]), JB = ld(V + 3 * rj[1]), JC = ld(V + 3 * rj[2]);
    v3 ta = unit(sub(JA, JC)), tb = unit(sub(JB, JA));
    v3 ni = ld(N + 3 * i), nj = ld(N + 3 * j);
    double dA, dB;
    v3 e = vertex_direction(ni, nj, ta, tb, &dA, &dB);
    double xi = atan2(dot(crs(ni, nj), e), dot(ni, nj));
    sc2 sdA = sincos2(dA), sdB = sincos2(dB);
    vtx_angles g;
    g.xi = sincos2(xi);
    v3 s = sub(IC, IB);
    g.nu_a = o_angle(sub(IA, IB), sub(IC, IB));
    g.mu_a = o_angle(sub(IB, IC), sub(IA, IC));
    g.kappa = o_angle(sub(IB, IA), sub(IC, IA));
    g.mu = sincos2(g.mu_a);
    g.nu = sincos2(g.nu_a);
    g.lsnu = log(g.nu.s);
    g.lsmu = log(g.mu.s);
    g.skappa = sin(g.kappa);
    g.psi_a = atan2(dot(crs(e, s), ni), dot(e, s));
    g.psi = sincos2(g.psi_a);
    g.nupsi = sincos2(g.nu_a + g.psi_a);
    g.mupsi = sincos2(g.mu_a - g.psi_a);
    const sc2 ps = g.psi, x = g.xi, np = g.nupsi, mp = g.mupsi;
    double qAt, qAp, qBt, qBp;
    {
        sc2 d = sdA;
        double csig = d.s * ps.s * x.c + d.c * ps.c;
        double cchi = d.s * ps.c * x.c - d.c * ps.s;
        double ceta = d.c * ps.s * x.c - d.s * ps.c;
        double cth = d.s * np.s * x.c + d.c * np.c;
        double cla = d.s * mp.s * x.c - d.c * mp.c;
        q_vertex(&g, dA, d, cla, cth, ceta, csig, cchi, &qAt, &qAp);
    }
    {
        sc2 d = sdB;
        double csig = d.s * ps.s * x.c + d.c * ps.c;
        double cchi = d.s * ps.c * x.c - d.c * ps.s;
        double ceta = d.c * ps.s * x.c - d.s * ps.c;
        double cth = d.s * np.s * x.c + d.c * np.c;
        double cla = d.s * mp.s * x.c - d.c * mp.c;
        q_vertex(&g, dB, d, cla, cth, ceta, csig, cchi, &qBt, &qBp);
    }
    double si_ = S[i];
    v3 psi = scl(si_, add(scl(qAp, ta), scl(qBp, tb)));
    double th = (fabs(xi) < O_EPS) ? 0.0 : (si_ * (qAt - qBt));
    (void)JA;
    return q4vec(psi, th);
}

void o_closed_vertex(int i, int j, const double *V, const int *C, const double *N, const double *S, double *out4)
{
    q4 r = closed_vertex(i, j, V, C, N, S);
    memcpy(out4, r.v, sizeof r.v);
}

/* ---------------------------------------------------------------- potential: singular pieces */
/* Common-edge pair: the potential integrand carries -2 c s ln s along the shared edge (s the
 * distance to the edge inside K_i, c s the in-plane distance t_E of x to the edge in K_j's
 * plane).  sigma(x) = -2 c s ln(s/h_i) is subtracted and integrated in closed form:
 * int_{K_i} s ln(s/h) dS = -(5/18) S_i h_i. */
typedef struct { v3 P1, tau, m_in; double c, h, area; } pot_edge_ctx;

static pot_edge_ctx make_pot_edge_ctx(int i, int j, const double *V, const int *C, const double *N, const double *S)
{
    pot_edge_ctx p;
    int si, sj, ri[3], rj[3];
    shifts_edge(C + 3 * i, C + 3 * j, &si, &sj);
    rotated(C + 3 * i, si, ri);
    rotated(C + 3 * j, sj, rj);
    v3 IA = ld(V + 3 * ri[0]);
    v3 JB = ld(V + 3 * rj[1]), JC = ld(V + 3 * rj[2]);
    p.P1 = JB;
    p.tau = unit(sub(JC, JB));
    v3 nj = ld(N + 3 * j);
    v3 m = crs(p.tau, nj);               /* outward normal of the edge in K_j's plane */
    v3 w = sub(IA, JB);
    v3 perp = sub(w, scl(dot(w, p.tau), p.tau));
    p.h = len(perp);                      /* height of K_i over the shared edge */
    p.m_in = scl(1.0 / p.h, perp);        /* unit direction into K_i, normal to the edge */
    p.c = -dot(m, p.m_in);                /* t_E(x) = c s */
    p.area = S[i];
    return p;
}

static inline double pot_edge_sigma(v3 x, const pot_edge_ctx *p)
{
    double s = dot(sub(x, p->P1), p->m_in);
    if (s <= 0.0) return 0.0;
    return -2.0 * p->c * s * log(s / p->h);
}

static inline double pot_edge_sigma_integral(const pot_edge_ctx *p)
{
    return (5.0 / 9.0) * p->c * p->area * p->h;
}

/* Self potential, int_K int_K 1/|x-y| / 4pi.  With d = 0 the inner integral is
 * sum_e t_e(x) L_e(x); swapping the order per edge gives
 *   int_K t_e L_e dS = int_e dl_y int_0^pi sin(phi) R(phi, y)^2 / 2 dphi,
 * R the distance from y to the boundary along direction phi; the phi integral is done in
 * closed form on each of the two sides the ray can hit, the edge integral by Gauss-Legendre. */
static void gauss_legendre(int n, double *x, double *w)
{
    for (int k = 0; k < n; ++k) {
        double z = cos(O_PI * (k + 0.75) / (n + 0.5)), dp = 0.0;
        for (int it = 0; it < 100; ++it) {
            double p0 = 1.0, p1 = 0.0;
            for (int m = 1; m <= n; ++m) { double p2 = p1; p1 = p0; p0 = ((2.0 * m - 1.0) * z * p1 - (m - 1.0) * p2) / m; }
            dp = n * (z * p0 - p1) / (z * z - 1.0);
            double dz = p0 / dp;
            z -= dz;
            if (fabs(dz) < 1e-16) break;
        }
        x[k] = z; w[k] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
}

static inline double ray_side(double a, double alpha, double u1)
{
    /* (a^2 sin^2(alpha)/2) [cos(alpha) ln tan(u/2) + sin(alpha)/sin(u)]_{alpha}^{u1} */
    double sa = sin(alpha), ca = cos(alpha);
    double F1 = ca * log(tan(0.5 * u1)) + sa / sin(u1);
    double F0 = ca * log(tan(0.5 * alpha)) + sa / sin(alpha);
    return 0.5 * a * a * sa * sa * (F1 - F0);
}

/* Gauss-Legendre points per piece of the self-pair rule used by o_integrate_class (default 96);
 * 0 selects the closed form below (the library's default) */
static int g_self_nquad = 96;
void o_set_self_rule(int nquad) { g_self_nquad = nquad < 0 ? 0 : nquad; }

/* Self potential in closed form, the library's default self rule:
 *   int_K int_K 1/|x-y| = (4 S^2 / 3) sum over the sides s of ln(p / (p - 2 s)) / s,
 * p the perimeter.  Scaling K about the vertex opposite edge e moves only e, so Euler's relation
 * (the integral is homogeneous of degree 3) gives (2 H_e / 3) int_e phi ds, phi the potential of K;
 * on e, phi = sum of t L over the other two edges, and d/du ln((r + u + c) / (r + u - c)) =
 * -c / (u r) makes those edge integrals elementary.  The smallest p - 2 s (the longest side, which
 * cancels in a flat cell) is taken from Heron's 16 S^2 = p prod (p - 2 s).  Checked against the
 * 96-point edge rule (o_self_potential) in the CPU tests. */
double o_self_potential_closed(const double *Ap, const double *Bp, const double *Cp)
{
    v3 A = ld(Ap), B = ld(Bp), C = ld(Cp);
    double a = len(sub(C, B)), b = len(sub(A, C)), c = len(sub(B, A));
    v3 cr = crs(sub(B, A), sub(C, A));
    double s4 = dot(cr, cr); /* (2S)^2 */
    double p = a + b + c;
    double da = (b + c) - a, db = (c + a) - b, dc = (a + b) - c;
    if (da <= db && da <= dc) da = 4.0 * s4 / (p * db * dc);
    else if (db <= dc) db = 4.0 * s4 / (p * da * dc);
    else dc = 4.0 * s4 / (p * da * db);
    return O_INV_4PI * (s4 / 3.0) * (log(p / da) / a + log(p / db) / b + log(p / dc) / c);
}

double o_self_potential(const double *Ap, const double *Bp, const double *Cp, int nquad)
{
    v3 P[3] = {ld(Ap), ld(Bp), ld(Cp)};
    double gx[256], gw[256];
    if (nquad > 256) nquad = 256;
    if (nquad < 2) nquad = 2;
    gauss_legendre(nquad, gx, gw);
    double total = 0.0;
    for (int e = 0; e < 3; ++e) {
        v3 P1 = P[e], P2 = P[(e + 1) % 3], P3 = P[(e + 2) % 3];
        double L = len(sub(P2, P1));
        v3 tau = scl(1.0 / L, sub(P2, P1));
        double al1 = o_angle(sub(P2, P1), sub(P3, P1));
        double al2 = o_angle(sub(P1, P2), sub(P3, P2));
        /* split at the foot of the altitude from P3 (the angle to P3 swings fastest there) */
        double foot = dot(sub(P3, P1), tau);
        double cuts[3] = {0.0, L, L};
        int nseg = 1;
        if (foot > 1e-12 * L && foot < (1.0 - 1e-12) * L) { cuts[1] = foot; cuts[2] = L; nseg = 2; }
        double acc = 0.0;
        for (int sgi = 0; sgi < nseg; ++sgi) {
            double lo = cuts[sgi], span = cuts[sgi + 1] - cuts[sgi];
            for (int k = 0; k < nquad; ++k) {
                /* graded map t -> t^2(3-2t) clusters nodes at both ends of the piece */
                double t = 0.5 * (gx[k] + 1.0), wt = 0.5 * gw[k];
                double tt = t * t * (3.0 - 2.0 * t), jac = 6.0 * t * (1.0 - t);
                double b = lo + span * tt, a = L - b;      /* b from P1, a from P2 */
                v3 y = add(P1, scl(b, tau));
                double phis = o_angle(tau, sub(P3, y));
                double f = ray_side(a, al2, phis + al2) + ray_side(b, al1, (O_PI - phis) + al1);
                acc += wt * jac * span * f;
            }
        }
        total += acc;
    }
    return O_INV_4PI * total;
}

/* Potential of common-edge and common-vertex pairs: graded Duffy rule around each shared
 * vertex.  A piece (V, B, C) of K_i with the singular corner V is mapped from the unit square,
 * x = V + u[(1-v)(B-V) + v(C-V)], dS = 2|piece| u du dv, with u = t^g graded towards V and
 * Gauss-Legendre in t and v.  A common-vertex pair uses K_i as one piece; a common-edge pair
 * splits K_i at the shared edge's midpoint M into (P1, M, A) and (P2, A, M) and also subtracts
 * the s ln s term along the shared edge (pot_edge_sigma), added back in closed form. */
static int g_pot_nu = 40, g_pot_nv = 32, g_pot_grade = 3;

void o_set_potential_rule(int nu, int nv, int grade)
{
    g_pot_nu = nu < 2 ? 2 : (nu > 256 ? 256 : nu);
    g_pot_nv = nv < 2 ? 2 : (nv > 256 ? 256 : nv);
    g_pot_grade = grade < 1 ? 1 : grade;
}

static double duffy_piece_rule(v3 Vx, v3 B, v3 Cc, v3 JA, v3 JB, v3 JC, const pot_edge_ctx *pe, int nu, int nv)
{
    double tu[256], wu[256], tv[256], wv[256];
    gauss_legendre(nu, tu, wu);
    gauss_legendre(nv, tv, wv);
    double area2 = len(crs(sub(B, Vx), sub(Cc, Vx)));
    double acc = 0.0;
    for (int a = 0; a < nu; ++a) {
        double t = 0.5 * (tu[a] + 1.0), wt = 0.5 * wu[a];
        double u = pow(t, g_pot_grade), du = g_pot_grade * pow(t, g_pot_grade - 1) * wt;
        for (int b = 0; b < nv; ++b) {
            double v = 0.5 * (tv[b] + 1.0), wvv = 0.5 * wv[b];
            v3 w = scl(u, add(scl(1.0 - v, sub(B, Vx)), scl(v, sub(Cc, Vx))));
            v3 oa = add(sub(Vx, JA), w), ob = add(sub(Vx, JB), w), oc = add(sub(Vx, JC), w);
            tp_full f = theta_psi_offsets(oa, ob, oc, JA, JB, JC);
            double g = potential_offsets(oa, ob, oc, JA, JB, JC, &f);
            if (pe) g -= pot_edge_sigma(add(Vx, w), pe);
            acc += du * wvv * area2 * u * g;
        }
    }
    return acc;
}

static double duffy_piece(v3 Vx, v3 B, v3 Cc, v3 JA, v3 JB, v3 JC, const pot_edge_ctx *pe)
{
    return duffy_piece_rule(Vx, B, Cc, JA, JB, JC, pe, g_pot_nu, g_pot_nv);
}

/* Hard adjacent pairs (folded: n_i.n_j < 0.5, or a cell with an angle below 10 degrees) get a
 * locally adaptive rule: a cell is compared with the sum of its four children and split again
 * where they differ by more than tol x |P| x 2^-depth; cells holding a shared vertex use the
 * Duffy rule with that vertex as apex, all others the 13-point rule. */
static double g_pot_adapt_tol = 1e-10;   /* 0 disables the adaptive route */
static int g_pot_adapt_depth = 18;
static int g_pot_adapt_all = 0;   /* 1: adaptive rule for every adjacent pair, not only hard ones */
static double g_pot_tier_tol = 0;  /* > 0: tiered rule (main vs check, then 16x16, then adaptive) */

void o_set_potential_adaptive(double tol) { g_pot_adapt_tol = tol; }
void o_set_potential_adaptive_depth(int d) { g_pot_adapt_depth = d; }
void o_set_potential_adaptive_all(int on) { g_pot_adapt_all = on; }
void o_set_potential_tiered(double tol) { g_pot_tier_tol = tol; }

static const double Q13[13][3] = {
    {0.333333333333333, 0.333333333333333, -0.149570044467670},
    {0.479308067841923, 0.260345966079038, 0.175615257433204}, {0.260345966079038, 0.479308067841923, 0.175615257433204},
    {0.260345966079038, 0.260345966079038, 0.175615257433204},
    {0.869739794195598, 0.065130102902216, 0.053347235608839}, {0.065130102902216, 0.869739794195598, 0.053347235608839},
    {0.065130102902216, 0.065130102902216, 0.053347235608839},
    {0.638444188569809, 0.312865496004875, 0.077113760890257}, {0.312865496004875, 0.638444188569809, 0.077113760890257},
    {0.638444188569809, 0.048690315425316, 0.077113760890257}, {0.048690315425316, 0.638444188569809, 0.077113760890257},
    {0.312865496004875, 0.048690315425316, 0.077113760890257}, {0.048690315425316, 0.312865496004875, 0.077113760890257}};

typedef struct { v3 JA, JB, JC; const pot_edge_ctx *pe; } pot_ctx;

static double pot_cell(const pot_ctx *c, v3 a, v3 b, v3 cc, int corner)
{
    if (corner >= 0) { /* apex at the shared vertex, held in slot 'corner' */
        v3 t[3] = {a, b, cc};
        return duffy_piece(t[corner], t[(corner + 1) % 3], t[(corner + 2) % 3], c->JA, c->JB, c->JC, c->pe);
    }
    double acc = 0.0;
    for (int g = 0; g < 13; ++g) {
        double l3 = 1.0 - Q13[g][0] - Q13[g][1];
        v3 oa = add(add(scl(Q13[g][0], sub(a, c->JA)), scl(Q13[g][1], sub(b, c->JA))), scl(l3, sub(cc, c->JA)));
        v3 ob = add(add(scl(Q13[g][0], sub(a, c->JB)), scl(Q13[g][1], sub(b, c->JB))), scl(l3, sub(cc, c->JB)));
        v3 oc = add(add(scl(Q13[g][0], sub(a, c->JC)), scl(Q13[g][1], sub(b, c->JC))), scl(l3, sub(cc, c->JC)));
        tp_full f = theta_psi_offsets(oa, ob, oc, c->JA, c->JB, c->JC);
        double gx = potential_offsets(oa, ob, oc, c->JA, c->JB, c->JC, &f);
        if (c->pe) gx -= pot_edge_sigma(add(oa, c->JA), c->pe);
        acc += Q13[g][2] * gx;
    }
    return 0.5 * len(crs(sub(b, a), sub(cc, a))) * acc;
}

/* children in the reference's split order; a parent corner in slot k moves to child
 * (k==1 ? 0 : k==2 ? 1 : 2) at slot 1 */
/* cells split by the adaptive rule, per depth (work statistics for sizing the device queues) */
static long long g_adapt_cells[32];
void o_adapt_stats(long long *out32, int reset)
{
    for (int k = 0; k < 32; ++k) {
        if (out32) out32[k] = g_adapt_cells[k];
        if (reset) g_adapt_cells[k] = 0;
    }
}

static double pot_adapt(const pot_ctx *c, v3 a, v3 b, v3 cc, int corner, double val, double tol_abs, int depth)
{
#pragma omp atomic
    g_adapt_cells[depth < 31 ? depth : 31]++;
    v3 mbc = scl(0.5, add(b, cc)), mca = scl(0.5, add(cc, a)), mab = scl(0.5, add(a, b));
    v3 ch[4][3] = {{mab, b, mbc}, {mbc, cc, mca}, {mca, a, mab}, {mbc, mca, mab}};
    int cc_[4] = {-1, -1, -1, -1};
    if (corner == 1) cc_[0] = 1;
    else if (corner == 2) cc_[1] = 1;
    else if (corner == 0) cc_[2] = 1;
    double v[4], sum = 0.0;
    for (int k = 0; k < 4; ++k) { v[k] = pot_cell(c, ch[k][0], ch[k][1], ch[k][2], cc_[k]); sum += v[k]; }
    if (fabs(sum - val) <= tol_abs || depth >= g_pot_adapt_depth) return sum;
    double out = 0.0;
    for (int k = 0; k < 4; ++k) out += pot_adapt(c, ch[k][0], ch[k][1], ch[k][2], cc_[k], v[k], 0.5 * tol_abs, depth + 1);
    return out;
}

/* tiered potential rule of the library: the main Duffy rule is kept when a lower-order check
 * (two fewer nodes per direction) agrees within the tier tolerance; otherwise a 16 x 16 rule is
 * kept when it agrees with the main rule; otherwise a 24 x 24 rule is kept when it agrees with the
 * 16 x 16 one to a tenth of the tolerance; otherwise the adaptive rule runs.  Returns 1 when the adaptive rule must run (*acc
 * then holds the 16 x 16 value, the adaptive rule's tolerance base), and stores the kept Duffy
 * value in *acc otherwise. */
static int tier_select(int npieces, const v3 P[2][3], v3 JA, v3 JB, v3 JC, const pot_edge_ctx *pe, double sig, double *acc)
{
    double lo = 0.0, hi = 0.0;
    for (int k = 0; k < npieces; ++k)
        lo += duffy_piece_rule(P[k][0], P[k][1], P[k][2], JA, JB, JC, pe, g_pot_nu > 4 ? g_pot_nu - 2 : 2, g_pot_nv > 4 ? g_pot_nv - 2 : 2);
    if (fabs((*acc + sig) - (lo + sig)) <= g_pot_tier_tol * fabs(*acc + sig)) return 0;
    for (int k = 0; k < npieces; ++k) hi += duffy_piece_rule(P[k][0], P[k][1], P[k][2], JA, JB, JC, pe, 16, 16);
    if (fabs((hi + sig) - (*acc + sig)) <= g_pot_tier_tol * fabs(hi + sig)) { *acc = hi; return 0; }
    /* tier 2b: 24 x 24 against 16 x 16 (the main rule was the inaccurate one) */
    double top = 0.0;
    for (int k = 0; k < npieces; ++k) top += duffy_piece_rule(P[k][0], P[k][1], P[k][2], JA, JB, JC, pe, 24, 24);
    if (fabs((top + sig) - (hi + sig)) <= 0.1 * g_pot_tier_tol * fabs(top + sig)) { *acc = top; return 0; }
    *acc = hi;
    return 1;
}

static int pair_is_hard(int i, int j, const double *V, const int *C, const double *N)
{
    if (dot(ld(N + 3 * i), ld(N + 3 * j)) < 0.5) return 1;
    const double c10 = 0.98480775301220806; /* cos 10 degrees */
    for (int q = 0; q < 2; ++q) {
        v3 a, b, cc;
        tri_of(V, C, q ? j : i, &a, &b, &cc);
        v3 P[3] = {a, b, cc};
        for (int k = 0; k < 3; ++k) {
            v3 u = unit(sub(P[(k + 1) % 3], P[k])), w = unit(sub(P[(k + 2) % 3], P[k]));
            if (dot(u, w) > c10) return 1;
        }
    }
    return 0;
}

int o_pair_is_hard(int i, int j, const double *V, const int *C)
{
    int nc = (i > j ? i : j) + 1;
    double *N = (double *)malloc(sizeof(double) * 3 * nc);
    o_cell_geometry(nc, V, C, N, NULL, NULL);
    int r = pair_is_hard(i, j, V, C, N);
    free(N);
    return r;
}

static double potential_adjacent(int cls, int i, int j, const double *V, const int *C, const double *N, const double *S)
{
    v3 JA, JB, JC;
    tri_of(V, C, j, &JA, &JB, &JC);
    if (cls == O_VERTEX) {
        int si, sj, ri[3];
        shifts_vertex(C + 3 * i, C + 3 * j, &si, &sj);
        rotated(C + 3 * i, si, ri);
        double acc = duffy_piece(ld(V + 3 * ri[0]), ld(V + 3 * ri[1]), ld(V + 3 * ri[2]), JA, JB, JC, NULL);
        int go_adapt = g_pot_adapt_tol > 0 && (g_pot_adapt_all || pair_is_hard(i, j, V, C, N));
        if (!go_adapt && g_pot_tier_tol > 0) {
            const v3 P[2][3] = {{ld(V + 3 * ri[0]), ld(V + 3 * ri[1]), ld(V + 3 * ri[2])}, {ld(V), ld(V), ld(V)}};
            go_adapt = tier_select(1, P, JA, JB, JC, NULL, 0.0, &acc);
        }
        if (go_adapt) {
            pot_ctx c = {JA, JB, JC, NULL};
            v3 a, b, cc;
            tri_of(V, C, i, &a, &b, &cc);
            /* shared vertex in slot si of K_i: it is corner (slot 1) of child 0 (b), 1 (c) or 2 (a) */
            v3 mbc = scl(0.5, add(b, cc)), mca = scl(0.5, add(cc, a)), mab = scl(0.5, add(a, b));
            v3 ch[4][3] = {{mab, b, mbc}, {mbc, cc, mca}, {mca, a, mab}, {mbc, mca, mab}};
            int corner_of_child[4] = {si == 1 ? 1 : -1, si == 2 ? 1 : -1, si == 0 ? 1 : -1, -1};
            double tol_abs = g_pot_adapt_tol * fabs(acc);
            double sum = 0.0;
            for (int k = 0; k < 4; ++k) {
                double v = pot_cell(&c, ch[k][0], ch[k][1], ch[k][2], corner_of_child[k]);
                sum += pot_adapt(&c, ch[k][0], ch[k][1], ch[k][2], corner_of_child[k], v, 0.5 * tol_abs, 1);
            }
            acc = sum;
        }
        return O_INV_4PI * acc;
    }
    int si, sj, ri[3];
    shifts_edge(C + 3 * i, C + 3 * j, &si, &sj);
    rotated(C + 3 * i, si, ri);
    v3 A = ld(V + 3 * ri[0]), P1 = ld(V + 3 * ri[1]), P2 = ld(V + 3 * ri[2]);
    v3 M = scl(0.5, add(P1, P2));
    pot_edge_ctx pe = make_pot_edge_ctx(i, j, V, C, N, S);
    double acc = duffy_piece(P1, M, A, JA, JB, JC, &pe) + duffy_piece(P2, A, M, JA, JB, JC, &pe);
    int go_adapt = g_pot_adapt_tol > 0 && (g_pot_adapt_all || pair_is_hard(i, j, V, C, N));
    if (!go_adapt && g_pot_tier_tol > 0) {
        const v3 P[2][3] = {{P1, M, A}, {P2, A, M}};
        go_adapt = tier_select(2, P, JA, JB, JC, &pe, pot_edge_sigma_integral(&pe), &acc);
    }
    if (go_adapt) {
        pot_ctx c = {JA, JB, JC, &pe};
        v3 a, b, cc;
        tri_of(V, C, i, &a, &b, &cc);
        /* root: both ends of the shared edge are corners; its value is the two-piece Duffy rule */
        v3 mbc = scl(0.5, add(b, cc)), mca = scl(0.5, add(cc, a)), mab = scl(0.5, add(a, b));
        v3 ch[4][3] = {{mab, b, mbc}, {mbc, cc, mca}, {mca, a, mab}, {mbc, mca, mab}};
        int in_i[3];
        for (int k = 0; k < 3; ++k) in_i[k] = (C[3 * i + k] == C[3 * j] || C[3 * i + k] == C[3 * j + 1] || C[3 * i + k] == C[3 * j + 2]);
        int corner_of_child[4] = {in_i[1] ? 1 : -1, in_i[2] ? 1 : -1, in_i[0] ? 1 : -1, -1};
        double tol_abs = g_pot_adapt_tol * fabs(acc + pot_edge_sigma_integral(&pe));
        double sum = 0.0;
        for (int k = 0; k < 4; ++k) {
            double v = pot_cell(&c, ch[k][0], ch[k][1], ch[k][2], corner_of_child[k]);
            sum += pot_adapt(&c, ch[k][0], ch[k][1], ch[k][2], corner_of_child[k], v, 0.5 * tol_abs, 1);
        }
        acc = sum;
    }
    return O_INV_4PI * (acc + pot_edge_sigma_integral(&pe));
}

/* ---------------------------------------------------------------- quadrature + refinement */
typedef struct { v3 a, b, c; } tri3;

/* 1 -> 4 midpoint split in the reference's child order (NumericalIntegrator3d.cu:37-87) */
static void split4(tri3 t, tri3 *ch)
{
    v3 mbc = scl(0.5, add(t.b, t.c)), mca = scl(0.5, add(t.c, t.a)), mab = scl(0.5, add(t.a, t.b));
    ch[0].a = mab; ch[0].b = t.b; ch[0].c = mbc;
    ch[1].a = mbc; ch[1].b = t.c; ch[1].c = mca;
    ch[2].a = mca; ch[2].b = t.a; ch[2].c = mab;
    ch[3].a = mbc; ch[3].b = mca; ch[3].c = mab;
}

typedef struct {
    int cls, i, j;
    v3 JA, JB, JC;       /* K_j */
    edge_ctx ectx;
    vertex_ctx vctx;
    pot_edge_ctx pctx;
    int npts;
    const double *L1, *L2, *L3, *w;
} task_ctx;

typedef struct { q4 r; double p; } qp5;

/* quadrature over one (sub-)cell: sum_g w_g f(x_g), times the cell measure
 * (NumericalIntegrator3d.cu:560-585, evaluatorJ3DK.cu:87-205) */
static qp5 cell_integral(const task_ctx *t, tri3 c, double measure)
{
    q4 acc = q4zero();
    double pacc = 0.0;
    for (int g = 0; g < t->npts; ++g) {
        v3 x = add(add(scl(t->L1[g], c.a), scl(t->L2[g], c.b)), scl(t->L3[g], c.c));
        tp_full f = theta_psi_full(x, t->JA, t->JB, t->JC);
        double pot = potential_from(x, t->JA, t->JB, t->JC, &f);
        q4 val = f.tp;
        if (t->cls == O_VERTEX) val = q4sub(val, sing_vertex(x, &t->vctx));
        else if (t->cls == O_EDGE) {
            val = q4sub(val, sing_edge(x, &t->ectx));
            pot -= pot_edge_sigma(x, &t->pctx);
        }
        acc = q4add(acc, q4scl(t->w[g], val));
        pacc += t->w[g] * pot;
    }
    qp5 out;
    out.r = q4scl(measure, acc);
    out.p = measure * pacc;
    return out;
}

/* uniform level-L refinement of K_i: sum over the 4^L sub-cells in tree order */
static qp5 level_integral(const task_ctx *t, tri3 root, double measure, int level)
{
    if (level == 0) return cell_integral(t, root, measure);
    tri3 ch[4];
    split4(root, ch);
    qp5 acc = {q4zero(), 0.0};
    for (int k = 0; k < 4; ++k) {
        qp5 r = level_integral(t, ch[k], 0.25 * measure, level - 1);
        acc.r = q4add(acc.r, r.r);
        acc.p += r.p;
    }
    return acc;
}

/* Runge criterion of the reference (evaluator3d.cu:76-99, cuda_math.cuh:270-300) */
static int runge_unconverged(q4 cur, q4 prev, double pow2p)
{
    double crit = 0.0;
    for (int k = 0; k < 4; ++k) {
        double num = cur.v[k] - prev.v[k];
        double den = pow2p * prev.v[k] - cur.v[k];
        double lim = (k < 3) ? O_DOUBLE_MIN : O_EPS2;
        double d = (fabs(num) < lim && fabs(den) < lim) ? 0.0 : num / den;
        crit += fabs(d);
    }
    return crit > O_EPS_RUNGE;
}

/* p-fix of the vertex class and J = (Theta n_j + Psi x n_j)/4pi (evaluatorJ3DK.cu:224-264) */
static v3 finalize_j(int cls, q4 r, v3 nj, double si)
{
    v3 psi = mk(r.v[0], r.v[1], r.v[2]);
    double th = r.v[3];
    if (cls == O_VERTEX) {
        int p = 0;
        double ref = O_TWO_PI * si;
        if (th > ref) p = -((int)trunc((th - ref) / (2.0 * ref)) + 1);
        else if (th < -ref) p = ((int)trunc((-ref - th) / (2.0 * ref)) + 1);
        th = th + 2.0 * p * ref;
    }
    return scl(O_INV_4PI, add(scl(th, nj), crs(psi, nj)));
}

/* scale-invariant change between two refinement levels: max of |dJ|_2/|J|_2 and |dP|/|P|,
 * both measured on the complete values (regular part + closed-form singular part) */
static v3 finalize_j(int cls, q4 r, v3 nj, double si);
static double rel_change(int cls, q4 cur, q4 prev, q4 sing, double pc, double pp, v3 nj, double si)
{
    v3 jc = finalize_j(cls, q4add(cur, sing), nj, si), jp = finalize_j(cls, q4add(prev, sing), nj, si);
    double nn = len(jc), dn = len(sub(jc, jp));
    double a = nn > 0 ? dn / nn : dn;
    double b = fabs(pc) > 0 ? fabs(pc - pp) / fabs(pc) : fabs(pc - pp);
    return a > b ? a : b;
}

int o_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

static void build_task(task_ctx *t, int cls, int i, int j, const double *V, const int *C,
                       const double *N, const double *S)
{
    t->cls = cls; t->i = i; t->j = j;
    tri_of(V, C, j, &t->JA, &t->JB, &t->JC);
    if (cls == O_EDGE) {
        t->ectx = make_edge_ctx(i, j, V, C);
        t->pctx = make_pot_edge_ctx(i, j, V, C, N, S);
    } else if (cls == O_VERTEX) {
        t->vctx = make_vertex_ctx(i, j, V, C, N, S);
    }
}

void o_task_integrand(int cls, int i, int j, const double *V, const int *C, int npts, const double *pts, double *out5)
{
    int nc = (i > j ? i : j) + 1;
    double *N = (double *)malloc(sizeof(double) * 3 * nc), *S = (double *)malloc(sizeof(double) * nc);
    o_cell_geometry(nc, V, C, N, S, NULL);
    task_ctx t;
    build_task(&t, cls, i, j, V, C, N, S);
    for (int k = 0; k < npts; ++k) {
        v3 x = ld(pts + 3 * k);
        tp_full f = theta_psi_full(x, t.JA, t.JB, t.JC);
        double pot = potential_from(x, t.JA, t.JB, t.JC, &f);
        q4 val = f.tp;
        if (cls == O_VERTEX) val = q4sub(val, sing_vertex(x, &t.vctx));
        else if (cls == O_EDGE) { val = q4sub(val, sing_edge(x, &t.ectx)); pot -= pot_edge_sigma(x, &t.pctx); }
        memcpy(out5 + 5 * k, val.v, 4 * sizeof(double));
        out5[5 * k + 4] = pot;
    }
    free(N); free(S);
}

double o_antisymmetry(const double *a, const double *b)
{
    double s = fabs(a[0] + b[0]) + fabs(a[1] + b[1]) + fabs(a[2] + b[2]);
    double na = fabs(a[0]) + fabs(a[1]) + fabs(a[2]);
    double nb = fabs(b[0]) + fabs(b[1]) + fabs(b[2]);
    return s / (na > nb ? na : nb);
}


int o_integrate_class(int cls, int ntasks, const int *ti, const int *tj,
                      int nv, const double *V, int nc, const int *C,
                      int npts, const double *qf_coords, const double *qf_w, int order,
                      int mode, int level, double tol, int self_sign,
                      double *raw4, double *J3, double *P, int *levels, int nthreads)
{
    if (ntasks < 0 || nv <= 0 || nc <= 0 || npts <= 0 || npts > 64) return 1;
    if (mode == O_FIXED && (level < 0 || level > 8)) return 1;
    for (int t = 0; t < ntasks; ++t)
        if (ti[t] < 0 || ti[t] >= nc || tj[t] < 0 || tj[t] >= nc) return 2;
    double L1[64], L2[64], L3[64], W[64];
    for (int g = 0; g < npts; ++g) {
        L1[g] = qf_coords[2 * g];
        L2[g] = qf_coords[2 * g + 1];
        L3[g] = 1.0 - qf_coords[2 * g] - qf_coords[2 * g + 1];
        W[g] = qf_w[g];
    }
    double *N = (double *)malloc(sizeof(double) * 3 * nc);
    double *S = (double *)malloc(sizeof(double) * nc);
    o_cell_geometry(nc, V, C, N, S, NULL);
    const double pow2p = (double)(1 << order);

    /* adaptive compat mode: per-task level histories, then the class-wide loop end K */
    int *conv = (int *)calloc(ntasks > 0 ? ntasks : 1, sizeof(int));
    qp5 *hist = NULL;
    if (mode != O_FIXED) hist = (qp5 *)malloc(sizeof(qp5) * (ntasks > 0 ? ntasks : 1) * (O_MAX_LEVEL + 1));

#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 16)
#endif
    for (int t = 0; t < ntasks; ++t) {
        int i = ti[t], j = tj[t];
        v3 nj = ld(N + 3 * j);
        if (cls == O_SELF) {
            v3 a, b, c;
            tri_of(V, C, i, &a, &b, &c);
            double th = self_sign == 0 ? 0.0 : (self_sign > 0 ? O_TWO_PI : -O_TWO_PI) * S[i];
            q4 r = q4vec(mk(0, 0, 0), th);
            v3 J = finalize_j(O_FAR, r, nj, S[i]);
            if (raw4) memcpy(raw4 + 4 * t, r.v, sizeof r.v);
            if (J3) { J3[3 * t] = J.x; J3[3 * t + 1] = J.y; J3[3 * t + 2] = J.z; }
            if (P) P[t] = g_self_nquad > 0 ? o_self_potential(&a.x, &b.x, &c.x, g_self_nquad) : o_self_potential_closed(&a.x, &b.x, &c.x);
            if (levels) levels[t] = 0;
            continue;
        }
        task_ctx ctx;
        build_task(&ctx, cls, i, j, V, C, N, S);
        ctx.npts = npts; ctx.L1 = L1; ctx.L2 = L2; ctx.L3 = L3; ctx.w = W;
        tri3 root;
        tri_of(V, C, i, &root.a, &root.b, &root.c);
        qp5 val;
        int used = 0;
        if (mode == O_FIXED) {
            val = level_integral(&ctx, root, S[i], level);
            used = level;
        } else {
            qp5 *h = hist + (size_t)t * (O_MAX_LEVEL + 1);
            q4 sing = q4zero();
            if (mode == O_ADAPTIVE_RELATIVE) {
                if (cls == O_EDGE) sing = closed_edge(i, j, V, C, N, S);
                else if (cls == O_VERTEX) sing = closed_vertex(i, j, V, C, N, S);
            }
            h[0] = level_integral(&ctx, root, S[i], 0);
            int k = 1;
            for (; k <= O_MAX_LEVEL; ++k) {
                h[k] = level_integral(&ctx, root, S[i], k);
                int unconv;
                if (mode == O_ADAPTIVE_COMPAT) unconv = runge_unconverged(h[k].r, h[k - 1].r, pow2p);
                else if (cls == O_FAR) unconv = rel_change(cls, h[k].r, h[k - 1].r, sing, h[k].p, h[k - 1].p, nj, S[i]) > tol;
                else unconv = rel_change(cls, h[k].r, h[k - 1].r, sing, 1.0, 1.0, nj, S[i]) > tol;
                if (!unconv) break;
            }
            if (k > O_MAX_LEVEL) k = O_MAX_LEVEL;
            conv[t] = k;
            continue;  /* finalised below, once the class-wide loop end is known */
        }
        q4 r = val.r;
        if (cls == O_EDGE) { r = q4add(r, closed_edge(i, j, V, C, N, S)); val.p = 4.0 * O_PI * potential_adjacent(cls, i, j, V, C, N, S); }
        else if (cls == O_VERTEX) { r = q4add(r, closed_vertex(i, j, V, C, N, S)); val.p = 4.0 * O_PI * potential_adjacent(cls, i, j, V, C, N, S); }
        v3 J = finalize_j(cls, r, nj, S[i]);
        if (raw4) memcpy(raw4 + 4 * t, r.v, sizeof r.v);
        if (J3) { J3[3 * t] = J.x; J3[3 * t + 1] = J.y; J3[3 * t + 2] = J.z; }
        if (P) P[t] = O_INV_4PI * val.p;
        if (levels) levels[t] = used;
    }

    if (mode != O_FIXED && cls != O_SELF) {
        int K = 0;
        for (int t = 0; t < ntasks; ++t) if (conv[t] > K) K = conv[t];
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
        for (int t = 0; t < ntasks; ++t) {
            int i = ti[t], j = tj[t];
            int L = conv[t];
            int keep = L;
            /* compat: the reference swaps its two result buffers every iteration but rewrites
             * only unconverged entries (evaluatorJ3DK.cu:966-1011), so a task that converged
             * at iteration L keeps I_L if the loop ran an even number of further iterations,
             * else I_{L-1}. */
            if (mode == O_ADAPTIVE_COMPAT && ((K - L) & 1)) keep = L - 1;
            qp5 val = hist[(size_t)t * (O_MAX_LEVEL + 1) + keep];
            q4 r = val.r;
            if (cls == O_EDGE) {
                r = q4add(r, closed_edge(i, j, V, C, N, S));
                val.p = 4.0 * O_PI * potential_adjacent(cls, i, j, V, C, N, S);
            } else if (cls == O_VERTEX) {
                r = q4add(r, closed_vertex(i, j, V, C, N, S));
                val.p = 4.0 * O_PI * potential_adjacent(cls, i, j, V, C, N, S);
            }
            v3 J = finalize_j(cls, r, ld(N + 3 * j), S[i]);
            if (raw4) memcpy(raw4 + 4 * t, r.v, sizeof r.v);
            if (J3) { J3[3 * t] = J.x; J3[3 * t + 1] = J.y; J3[3 * t + 2] = J.z; }
            if (P) P[t] = O_INV_4PI * val.p;
            if (levels) levels[t] = keep;
        }
    }
    free(conv);
    free(hist);
    free(N);
    free(S);
    return 0;
}
