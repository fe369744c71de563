/*
 * i2_oracle.h -- CPU oracle for the pair-integral hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C FP64 restatement of the
 * reference's formulas (andreyypopov/integrator2), used as the checker by
 * tests/, by __graft_entry__.smoke() and as the timed CPU baseline in
 * bench.py.  The shipped library never links, loads or calls it.
 *
 * Parity status: the functions that restate reference code (theta/psi,
 * singular asymptotes, closed-form singular integrals, quadrature,
 * refinement, Runge rule, finalisation) are pinned against golden vectors
 * produced by the reference's own source compiled for the host
 * (oracle/ref_build.sh + oracle/ref_driver.cu, tests/golden/).  The
 * potential channel and the self class have no counterpart in the
 * reference: they are checked against independent quadrature (mpmath /
 * brute force) only and are "parity unpinned".
 *
 * Conventions (same as the reference):
 *   vertices  double[3*nv], cells int[3*nc] (0-based),
 *   a task is (i, j): K_i is integrated numerically (and refined),
 *   K_j analytically; the raw per-task result is (Psi.x, Psi.y, Psi.z, Theta).
 */
#ifndef I2_ORACLE_H
#define I2_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum { O_VERTEX = 0, O_EDGE = 1, O_FAR = 2, O_SELF = 3 };          /* pair classes */
enum { O_FIXED = 0, O_ADAPTIVE_COMPAT = 1, O_ADAPTIVE_RELATIVE = 2 }; /* refinement modes */

/* normals (3*nc), measures (nc), centres (3*nc) of every cell */
void o_cell_geometry(int nc, const double *V, const int *C,
                     double *normals, double *measures, double *centres);

/* (Psi, Theta) of triangle (A,B,C) seen from point x -- evaluatorJ3DK.cu:266-313 */
void o_theta_psi(const double *x, const double *A, const double *B, const double *C, double *out4);

/* integral over triangle (A,B,C) of 1/|x-y| dS_y (no 1/4pi) -- new channel */
double o_potential_inner(const double *x, const double *A, const double *B, const double *C);

/* singular asymptotes -- evaluatorJ3DK.cu:315-350 and :352-407 */
void o_sing_edge(const double *x, int i, int j, const double *V, const int *C, double *out4);
void o_sing_vertex(const double *x, int i, int j, const double *V, const int *C,
                   const double *N, const double *S, double *out4);

/* closed-form integrals of the asymptotes over K_i -- evaluatorJ3DK.cu:603-672 and :674-780 */
void o_closed_edge(int i, int j, const double *V, const int *C, const double *N, const double *S, double *out4);
void o_closed_vertex(int i, int j, const double *V, const int *C, const double *N, const double *S, double *out4);

/* graded Duffy rule used for the potential of common-edge / common-vertex pairs
 * (nu radial x nv angular Gauss-Legendre points per piece, radial grading u = t^grade);
 * default 40 x 32, grade 3 */
void o_set_potential_rule(int nu, int nv, int grade);

/* locally adaptive potential rule for hard common-edge / common-vertex pairs (folded, n_i.n_j <
 * 0.5, or a cell with an angle below 10 degrees): relative tolerance, 0 disables (default 1e-10) */
void o_set_potential_adaptive(double tol);
void o_set_potential_adaptive_depth(int depth); /* default 18 */
void o_set_potential_adaptive_all(int on);     /* 1: adaptive rule for every adjacent pair */
/* > 0: the library's tiered rule (Duffy main vs check, then 16 x 16, then adaptive); 0 off */
void o_set_potential_tiered(double tier_tol);
int o_pair_is_hard(int i, int j, const double *V, const int *C);

/* potential of a self pair (1/4pi included) */
double o_self_potential(const double *A, const double *B, const double *C, int nquad);
double o_self_potential_closed(const double *A, const double *B, const double *C);

/*
 * Integrate one class of tasks.
 *   cls          O_VERTEX / O_EDGE / O_FAR / O_SELF
 *   qf_coords    2*npts barycentric (L1, L2) pairs, qf_w npts weights, order = Runge order p
 *   mode, level  O_FIXED with refinement level, or an adaptive mode (max level 5)
 *   tol          relative tolerance for O_ADAPTIVE_RELATIVE (ignored otherwise)
 *   raw4         out, 4 per task: (Psi, Theta) after singular closed forms (before finalisation)
 *   J3           out, 3 per task: finalised gradient integral J
 *   P            out, 1 per task: potential integral (1/4pi included)
 *   levels       out (may be NULL): refinement level whose value was kept, per task
 *   self_sign    self-class normal convention: 0 principal value, +1/-1 one-sided limit
 *   nthreads     OpenMP threads (<=0: library default)
 * Returns 0 on success, nonzero on bad arguments.
 */
int o_integrate_class(int cls, int ntasks, const int *ti, const int *tj,
                      int nv, const double *V, int nc, const int *C,
                      int npts, const double *qf_coords, const double *qf_w, int order,
                      int mode, int level, double tol, int self_sign,
                      double *raw4, double *J3, double *P, int *levels, int nthreads);

/* point samples of the regular integrand of a task (raw (Psi,Theta) minus asymptote) and of
 * the potential integrand, for quadrature experiments: out5 = 5 doubles per point */
void o_task_integrand(int cls, int i, int j, const double *V, const int *C,
                      int npts, const double *pts, double *out5);

/* antisymmetry check of the reference: delta = |J_ij + J_ji|_1 / max(|J_ij|_1, |J_ji|_1) */
double o_antisymmetry(const double *Jij, const double *Jji);

int o_max_threads(void);
/* Gauss-Legendre points per piece of the self-pair potential in o_integrate_class (default 96) */
void o_set_self_rule(int nquad);
/* cells visited by the adaptive potential rule per depth since the last reset */
void o_adapt_stats(long long *out32, int reset);

#ifdef __cplusplus
}
#endif
#endif
