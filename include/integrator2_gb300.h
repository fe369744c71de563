/*
 * integrator2_gb300.h -- C-ABI of the GB300 (sm_103a) pair-integral library.
 *
 * Computes, for ordered pairs (i, j) of triangles K_i, K_j of a surface mesh, the gradient
 * integral of the Newtonian kernel
 *     J(K_i, K_j) = int_{K_i} int_{K_j} grad_y 1/(4 pi |x - y|) dS_y dS_x
 *                 = (1/4pi) (Theta n_j + Psi x n_j)      (Theta, Psi integrated over K_i)
 * and the potential integral P(K_i, K_j) = int_{K_i} int_{K_j} 1/(4 pi |x - y|) dS_y dS_x,
 * for the four pair classes: common vertex ("simple neighbours" in the reference's naming),
 * common edge ("attached neighbours"), disjoint ("not neighbours"; a near-field subset when
 * the pair lists are built with a distance cutoff) and self.
 *
 * It is a drop-in for the pair-integral path of andreyypopov/integrator2 (Mesh3D,
 * NumericalIntegrator3D, Evaluator3D, EvaluatorJ3DK).  Each entry point names the reference
 * interface it replaces (paths relative to the reference's repository).  Differences:
 *   - every call returns an i2_status instead of calling exit() on CUDA errors;
 *   - quadrature state is per integrator handle (the reference keeps it in process-global
 *     __constant__ memory, src/NumericalIntegrator3d.cu:9-11);
 *   - results can be read at full precision (the reference exposes them only through a
 *     6-significant-digit text export, src/evaluators/evaluator3d.cu:354-457);
 *   - pair lists are plain (i, j[, k]) rows; the result index is the row index (the reference
 *     requires k == row index, src/evaluators/evaluatorJ3DK.cu:94);
 *   - the potential channel and the self class are additions.
 *
 * Threading: handles are not thread-safe; distinct handles may be used from distinct threads.
 * All device work of an evaluator is ordered on its stream (i2_evaluator_set_stream): the mixed
 * form forks an adjacent class's potential stages onto a second stream the evaluator owns and joins
 * them back by an event before the class's results are written, so work enqueued on the
 * evaluator's stream afterwards, and a graph captured from it, see the finished class.  A batch
 * does the same with its own second stream.
 */
#ifndef INTEGRATOR2_GB300_H
#define INTEGRATOR2_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif
#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

typedef struct i2_mesh i2_mesh_t;
typedef struct i2_integrator i2_integrator_t;
typedef struct i2_evaluator i2_evaluator_t;

typedef enum i2_status {
    I2_OK = 0,
    I2_ERR_INVALID_ARGUMENT = 1,
    I2_ERR_CUDA = 2,
    I2_ERR_OUT_OF_MEMORY = 3,
    I2_ERR_IO = 4,
    I2_ERR_STATE = 5,       /* call out of order, e.g. run before prepare */
    I2_ERR_UNSUPPORTED = 6
} i2_status;

/* values 0..2 are the reference's neighbour_type_enum (src/Mesh3d.cuh:18-23) */
typedef enum i2_pair_class {
    I2_SIMPLE_NEIGHBORS = 0,    /* one shared vertex */
    I2_ATTACHED_NEIGHBORS = 1,  /* one shared edge */
    I2_NOT_NEIGHBORS = 2,       /* no shared vertex */
    I2_SELF = 3                 /* i == j (not in the reference) */
} i2_pair_class;

/* values 0..1 are the reference's error_control_type_enum (src/NumericalIntegrator3d.cuh:16-19) */
typedef enum i2_error_control {
    I2_FIXED_REFINEMENT_LEVEL = 0,
    I2_AUTOMATIC_ERROR_CONTROL = 1,  /* the reference's Runge loop, including its buffer parity */
    I2_RELATIVE_ERROR_CONTROL = 2    /* scale-invariant: |J_L - J_{L-1}| <= tol |J_L| */
} i2_error_control;

/* FP64: every stage in FP64 (matches the reference's CUDA build to 1e-12).  MIXED: the regular-part
 * quadrature in FP32 with compensated sums; the closed forms, the potential's tier 2b and adaptive
 * rule in double-float arithmetic on the FP32 pipe (about 2^-44 relative); the estimator's level
 * differences, pairs holding a needle cell (a corner below 5 degrees), adjacent pairs whose
 * closed-form part exceeds J 48-fold, and self pairs in FP64.  MIXED holds 1e-6 against FP64
 * (normwise, 99.9th percentile per pair) on well-conditioned meshes; on pairs whose sensitivity to
 * relative coordinate perturbations (kappa) runs into the thousands its error is about
 * kappa x 1e-8, the FP32 rounding of the quadrature points: use FP64 there */
typedef enum i2_precision { I2_PRECISION_FP64 = 0, I2_PRECISION_MIXED = 1 } i2_precision;

typedef enum i2_channel {
    I2_CHANNEL_J = 0,      /* 3 doubles per pair */
    I2_CHANNEL_P = 1,      /* 1 double per pair */
    I2_CHANNEL_RAW = 2,    /* (Psi, Theta) before finalisation, 4 doubles per pair */
    I2_CHANNEL_ERROR = 3,  /* antisymmetry delta after run_all_pairs(check=1), 1 double per pair */
    I2_CHANNEL_LEVEL = 4   /* refinement level kept per pair (as double), -1 in fixed mode */
} i2_channel;

/* values of the reference's output_format_enum (src/evaluators/evaluator3d.cuh:19-22) + full precision */
typedef enum i2_output_format { I2_PLAIN_TEXT = 0, I2_CSV = 1, I2_CSV_FULL_PRECISION = 2 } i2_output_format;

const char *i2_status_string(i2_status s);
/* message of the last failed call on this thread ("" if none) */
const char *i2_last_error(void);
int32_t i2_version(void);

/* ------------------------------------------------------------------ Mesh3D */
i2_status i2_mesh_create(i2_mesh_t **out);
void i2_mesh_destroy(i2_mesh_t *mesh);
/* Mesh3D::loadMeshFromFile (src/Mesh3d.cuh:55, src/Mesh3d.cu:159-217): reference .dat format */
i2_status i2_mesh_load_file(i2_mesh_t *mesh, const char *path, double scale);
/* host arrays: vertices 3*nv doubles, cells 3*nc 0-based ints (no reference counterpart) */
i2_status i2_mesh_set_geometry(i2_mesh_t *mesh, const double *vertices, int32_t nv, const int32_t *cells, int32_t nc);
/* Mesh3D::prepareMesh (src/Mesh3d.cuh:63, src/Mesh3d.cu:219-262): cell normals, measures,
 * centres and the pair lists.  near_factor > 0 keeps disjoint pairs whose centroid distance is
 * below near_factor x mean edge length; near_factor <= 0 keeps every disjoint pair, as the
 * reference's all-pairs classifier does.  Lists are built in O(N) (vertex incidence + a
 * uniform grid over centroids) instead of the reference's O(N^2) kernel. */
i2_status i2_mesh_prepare(i2_mesh_t *mesh, double near_factor);
/* Mesh3D::prepareMesh with the pair lists built on the GPU (the reference's prepareMesh
 * classifies pairs on the GPU, src/Mesh3d.cu:93-142 and 243-262, by an O(N^2) shared-vertex
 * count).  Same cell data and the same lists, in the same order, as i2_mesh_prepare: O(N)
 * through vertex incidence and a sorted centroid grid.  Also uploads the mesh.  host_copy = 0
 * keeps the lists on the device only (they are copied to the host the first time a host-side
 * call needs them); i2_mesh_device_pairs hands them out.  Synchronises the device. */
i2_status i2_mesh_prepare_device(i2_mesh_t *mesh, double near_factor, int32_t host_copy);
/* device copy of a class's unordered list: *d_rows = n int2 (i, j) rows (i < j, sorted; the
 * self class (i, i)), owned by the mesh and valid until it is prepared again or destroyed.  A
 * mesh prepared on the host has its lists uploaded on the first call. */
i2_status i2_mesh_device_pairs(const i2_mesh_t *mesh, i2_pair_class cls, const int32_t **d_rows, int64_t *n);
i2_status i2_mesh_sizes(const i2_mesh_t *mesh, int32_t *nv, int32_t *nc);
/* Mesh3D::getSimpleNeighbors / getAttachedNeighbors / getNotNeighbors ().size: unordered
 * (i < j) pairs of a class; the self class has nc entries */
i2_status i2_mesh_pair_count(const i2_mesh_t *mesh, i2_pair_class cls, int64_t *n);
/* copies the unordered list as int3 rows (i, j, k = row index), the reference's layout */
i2_status i2_mesh_copy_pairs(const i2_mesh_t *mesh, i2_pair_class cls, int32_t *rows, int64_t n);
/* Mesh3D::getCellNormals / getCellMeasures (src/Mesh3d.cuh:110-126); any pointer may be NULL */
i2_status i2_mesh_copy_cell_data(const i2_mesh_t *mesh, double *normals, double *measures, double *centres);
/* Mesh3D::getVertices / getCells (src/Mesh3d.cuh:70-126) as host copies: 3 nv doubles, 3 nc int32
 * (0-based); either pointer may be NULL */
i2_status i2_mesh_copy_geometry(const i2_mesh_t *mesh, double *vertices, int32_t *cells);

/* ------------------------------------------------------------------ QuadratureFormula3D */
/* the reference's built-in rules qf3D1, qf3D3, qf3D4, qf3D6, qf3D7, qf3D9, qf3D12, qf3D13
 * (src/QuadratureFormula3d.cuh:34-213): npoints selects the rule; coords receives 2*npoints
 * barycentric (L1, L2) pairs, weights npoints values, order the Runge order */
i2_status i2_quadrature_builtin(int32_t npoints, double *coords, double *weights, int32_t *order);

/* ------------------------------------------------------------------ NumericalIntegrator3D */
/* NumericalIntegrator3D(mesh, qf) (src/NumericalIntegrator3d.cuh:73, .cu:197-222);
 * default: automatic error control as in the reference */
i2_status i2_integrator_create(const i2_mesh_t *mesh, const double *coords, const double *weights, int32_t npoints,
                               int32_t order, i2_integrator_t **out);
void i2_integrator_destroy(i2_integrator_t *it);
/* NumericalIntegrator3D::setFixedRefinementLevel (src/NumericalIntegrator3d.cu:225-229) */
i2_status i2_integrator_set_fixed_refinement_level(i2_integrator_t *it, int32_t level);
/* error control: mode, relative tolerance (relative mode), maximum level (1..5) */
i2_status i2_integrator_set_error_control(i2_integrator_t *it, i2_error_control mode, double rel_tol, int32_t max_level);
i2_status i2_integrator_get_error_control(const i2_integrator_t *it, i2_error_control *mode, int32_t *level);
i2_status i2_integrator_set_precision(i2_integrator_t *it, i2_precision precision);
/* potential rule of common-edge / common-vertex pairs (graded Duffy, n_radial x n_angular per
 * piece, radial grading exponent) and of self pairs (n_self points per edge piece of the graded
 * edge rule; 0 = the closed form, exact, the default in both precisions) */
i2_status i2_integrator_set_potential_rule(i2_integrator_t *it, int32_t n_radial, int32_t n_angular, int32_t grading,
                                           int32_t n_self);
/* relative tolerance of the locally adaptive potential rule used for hard common-edge /
 * common-vertex pairs (folded: normals more than 60 degrees apart, or a cell with an angle
 * below 10 degrees); 0 keeps the plain Duffy rule for them too.  Default 1e-8. */
i2_status i2_integrator_set_hard_pair_tolerance(i2_integrator_t *it, double rel_tol);
/* No counterpart in the reference, which computes J only: enabled = 0 computes J only here too.
 * The potential rule of the adjacent classes (graded Duffy tiers, adaptive rule) is skipped and
 * their P reads NaN; the disjoint and self classes keep P (it costs them almost nothing).
 * Default 1.  The batched form and the adjoint need the potential (I2_ERR_UNSUPPORTED). */
i2_status i2_integrator_set_potential(i2_integrator_t *it, int32_t enabled);
/* self-class normal convention: 0 principal value (J = 0), +1 / -1 one-sided limit */
i2_status i2_integrator_set_self_convention(i2_integrator_t *it, int32_t sign);

/* ------------------------------------------------------------------ EvaluatorJ3DK */
/* EvaluatorJ3DK(mesh, integrator) (src/evaluators/evaluatorJ3DK.cuh:140-211) */
i2_status i2_evaluator_create(const i2_mesh_t *mesh, i2_integrator_t *it, i2_evaluator_t **out);
void i2_evaluator_destroy(i2_evaluator_t *ev);
/* cudaStream_t passed as void* (default: the legacy default stream) */
i2_status i2_evaluator_set_stream(i2_evaluator_t *ev, void *stream);
/* Evaluator3D::runAllPairs (src/evaluators/evaluator3d.cu:120-204): every pair of the mesh's
 * lists in both orders (rows 0..n-1 = (i,j), rows n..2n-1 = (j,i)), self class included;
 * check_correctness != 0 also computes the antisymmetry delta of each (i,j)/(j,i) pair */
i2_status i2_evaluator_run_all_pairs(i2_evaluator_t *ev, int32_t check_correctness);
/* Evaluator3D::runPairs (src/evaluators/evaluator3d.cu:213-288): host int3 rows per class */
i2_status i2_evaluator_run_pairs(i2_evaluator_t *ev, const int32_t *simple, int64_t n_simple, const int32_t *attached,
                                 int64_t n_attached, const int32_t *not_neighbors, int64_t n_not);
/* one class from host rows (row_stride 2 or 3 int32 per row), self class included */
i2_status i2_evaluator_run_class(i2_evaluator_t *ev, i2_pair_class cls, const int32_t *rows, int64_t n, int32_t row_stride);
/* device-resident hot path: d_pairs = n int2 (i, j) rows in device memory; outputs are device
 * buffers (d_raw4: 4n, d_J: 3n, d_P: n doubles; any may be NULL to keep them in the
 * evaluator).  Enqueues the class's kernel chain on the evaluator's stream and returns without
 * synchronising.  Scratch memory is owned by the evaluator and reused across calls. */
i2_status i2_evaluator_run_class_device(i2_evaluator_t *ev, i2_pair_class cls, const int32_t *d_pairs, int64_t n,
                                        double *d_raw4, double *d_J, double *d_P);
i2_status i2_evaluator_synchronize(i2_evaluator_t *ev);
/* number of results held for a class after the last run */
i2_status i2_evaluator_result_count(const i2_evaluator_t *ev, i2_pair_class cls, int64_t *n);
/* statistics of the last run of a class (the reference prints per-cell refinement counts,
 * src/NumericalIntegrator3d.cu:494): out[0] pairs; out[1] pairs whose tier-1 potential check
 * failed; out[2] pairs that reached tier 2b; out[3] pairs given the adaptive potential rule;
 * out[4] adaptive-rule cells kept because a depth's list was full; out[5] pairs recomputed in
 * FP64 by the mixed form (a needle cell, or a closed-form part 48 times J); out[6] the class's last
 * refinement level; out[6 + L] pairs still unconverged after level L (L = 1..7, adaptive modes);
 * out[14] of the out[5] pairs, those whose levels 4-5 were spread over the GPU.  Synchronises the evaluator's stream. */
#define I2_RUN_STATS 15
i2_status i2_evaluator_run_stats(const i2_evaluator_t *ev, i2_pair_class cls, int64_t *out, int32_t n);
/* full-precision copy of a result channel (replaces subclassing for d_*Results) */
i2_status i2_evaluator_copy_results(const i2_evaluator_t *ev, i2_pair_class cls, i2_channel channel, double *out,
                                    int64_t n);
/* Evaluator3D::outputResultsToFile (src/evaluators/evaluator3d.cu:354-457) to a given path */
i2_status i2_evaluator_output_results(const i2_evaluator_t *ev, i2_pair_class cls, i2_output_format format,
                                      const char *path);

/* ------------------------------------------------------------------ adjoint */
/* Backward pass of the pair integrals (no reference counterpart): adds to d_gradV (3 doubles
 * per vertex, device) the vector-Jacobian product
 *     sum_p d_gJ[p] . dJ_p/dV + d_gP[p] dP_p/dV
 * for the pairs of one class, with the refinement the forward pass kept frozen (sub-cells are
 * recomputed, not stored).  It must follow the forward run of the same class with the same device
 * pairs on this evaluator (i2_evaluator_run_class / run_class_device).  d_gJ (3 per pair) or d_gP
 * (1 per pair) may be NULL.  FP64 dual numbers after an FP64 forward, FP32 after a mixed one.
 * Asynchronous on the evaluator's stream; accumulation uses atomics. */
i2_status i2_evaluator_backward_class(i2_evaluator_t *ev, i2_pair_class cls, const int32_t *d_pairs, int64_t n,
                                      const double *d_gJ, const double *d_gP, double *d_gradV);

/* ------------------------------------------------------------------ batched form */
/* Many (mesh, pair class) segments integrated together (no reference counterpart): the
 * refinement levels of all segments of one pair class run in ONE persistent cooperative kernel
 * (three in all), a fixed number of launches whatever the number of segments; the whole run is
 * captured into a CUDA graph on the first i2_batch_run and replayed afterwards.  Settings
 * (rule, error control, potential rule) come from the integrator given at creation; the
 * batched form computes in mixed precision (FP32 bulk; double-float closed forms, tier 2b and
 * adaptive potential; FP64 estimator differences, needle and high-ratio pairs) whatever the integrator's
 * precision. */
typedef struct i2_batch i2_batch_t;
i2_status i2_batch_create(const i2_integrator_t *settings, i2_batch_t **out);
void i2_batch_destroy(i2_batch_t *batch);
i2_status i2_batch_set_stream(i2_batch_t *batch, void *stream);
/* adds one segment (host rows, stride 2 or 3 int32); returns its index in *segment */
i2_status i2_batch_add(i2_batch_t *batch, const i2_mesh_t *mesh, i2_pair_class cls, const int32_t *rows, int64_t n,
                       int32_t row_stride, int32_t *segment);
/* times the candidate launch shapes (threads per block, resident blocks per SM, lanes per pair,
 * register variant of each pair class's level kernel: 0 unconstrained, 1 capped at 128 per thread,
 * 2 capped at 85) on the batch and keeps the fastest; the chosen shape is returned in shape[4] (may
 * be NULL), the variants as one code v_vertex + 3 v_edge + 9 v_disjoint in shape[3] */
i2_status i2_batch_autotune(i2_batch_t *batch, int32_t *shape);
/* enqueues the batch on its stream (graph replay after the first call); asynchronous */
i2_status i2_batch_run(i2_batch_t *batch);
/* 1 if the last run replayed a CUDA graph, 0 if it used direct launches */
i2_status i2_batch_uses_graph(const i2_batch_t *batch, int32_t *uses_graph);
i2_status i2_batch_result_count(const i2_batch_t *batch, int32_t segment, int64_t *n);
i2_status i2_batch_copy_results(const i2_batch_t *batch, int32_t segment, i2_channel channel, double *out, int64_t n);

/* ------------------------------------------------------------------ without allocation */
/* No counterpart in the reference.  For callers that cannot allocate device memory (plugins in
 * a host application that reserves the GPU's memory for its own pool; loops where cudaMalloc /
 * cudaFree, which may synchronise the device, are not allowed): the disjoint class with
 * relative error control and the 13-point rule, as i2_evaluator_run_class_device with
 * I2_RELATIVE_ERROR_CONTROL, with every scratch buffer in one static device array of about
 * 4.6 MB that each GPU loading the library holds until exit.  The caller passes device
 * buffers: vertices (3 nv doubles), cells (3 nc int32, 0-based), pairs (2 n int32, 8-byte
 * aligned, indices valid: they are read on the device only), J (3 n doubles) and P (n
 * doubles).  Limits: nc <= I2_NOALLOC_MAX_CELLS, n <= I2_NOALLOC_MAX_PAIRS; larger inputs are
 * rejected with I2_ERR_INVALID_ARGUMENT before any launch.  Asynchronous on `stream`.  The
 * first call in each CUDA context (normally one per device) looks up the array's device
 * address in that context (make it before any stream capture).  Every call shares the array:
 * calls that overlap on the GPU race. */
#define I2_NOALLOC_MAX_CELLS 8192
#define I2_NOALLOC_MAX_PAIRS 16384
i2_status i2_not_neighbors_noalloc(const double *d_vertices, int32_t nv, const int32_t *d_cells, int32_t nc,
                                   const int32_t *d_pairs, int64_t n, double rel_tol, int32_t max_level, double *d_J,
                                   double *d_P, void *stream);

/* ------------------------------------------------------------------ measurement */
/* measured pipe peaks of the current GPU for the kernels' roofline (no reference counterpart):
 * out[0] FP64 FMA TFLOP/s, out[1] FP32 FMA TFLOP/s, out[2..7] time of one FP64 sqrt, divide,
 * log, atan2, sincos, acos in units of one FP64 FMA, out[8..12] time of one FP32 sqrtf,
 * divide, log1pf, atan2f, logf in units of one FP32 FMA (out holds 13 doubles) */
i2_status i2_calibrate_pipes(double *out);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif
#ifdef __cplusplus
}
#endif
#endif
