/*
 * ref_driver.cu -- host driver around the reference's own routines.  TEST INFRASTRUCTURE ONLY.
 *
 * Built by oracle/ref_build.sh together with the unmodified reference sources (compiled for
 * the host through oracle/ref_shim.h) into oracle/_ref/libi2ref.so.  It is used only to
 * generate the golden vectors under tests/golden/ and to cross-check the oracle here; the
 * GPU tests never load it.
 *
 * The per-task bodies below mirror the reference's kernels one thread at a time and call the
 * reference's own device functions (thetaPsi, singularPart*, integrateSingularPart*,
 * calculateQuadraturePoints, integrate4D, divide, norm1, normalize, cross, ...).  The host
 * orchestration mirrors prepareTasksAndMesh / refineMesh / updateTasks / gatherResults /
 * compareIntegrationResults and the adaptive loop of EvaluatorJ3DK::numericalIntegration,
 * executed sequentially (cell and task order = thread order).
 */
#include "NumericalIntegrator3d.cuh"
#include "evaluators/evaluatorJ3DK.cuh"

#include <cstdio>
#include <cstring>
#include <vector>

extern __constant__ Point3 c_GaussPointsCoordinates[CONSTANTS::MAX_GAUSS_POINTS];
extern __constant__ double c_GaussPointsWeights[CONSTANTS::MAX_GAUSS_POINTS];
extern __constant__ int c_GaussPointsNumber;

namespace {

int g_npts = 0;
double g_pow2p = 128.0;

struct HostMesh {
    std::vector<Point3> V;
    std::vector<int3> C;
    std::vector<Point3> N;
    std::vector<double> S;
};

struct RefinedMesh {
    std::vector<Point3> V;
    std::vector<int3> C;
    std::vector<double> S;
    std::vector<int> orig;
    std::vector<int> parent;
};

HostMesh make_mesh(int nv, const double *V, int nc, const int *C)
{
    HostMesh m;
    m.V.resize(nv);
    m.C.resize(nc);
    for (int k = 0; k < nv; ++k) m.V[k] = make_double3(V[3 * k], V[3 * k + 1], V[3 * k + 2]);
    for (int k = 0; k < nc; ++k) m.C[k] = make_int3(C[3 * k], C[3 * k + 1], C[3 * k + 2]);
    m.N.resize(nc);
    m.S.resize(nc);
    for (int c = 0; c < nc; ++c) { /* kCalculateCellNormal / kCalculateCellMeasure bodies */
        const int3 t = m.C[c];
        const Point3 v12 = m.V[t.y] - m.V[t.x];
        const Point3 v13 = m.V[t.z] - m.V[t.x];
        m.N[c] = normalize(cross(v12, v13));
        m.S[c] = vector_length(cross(v12, v13)) * 0.5;
    }
    return m;
}

/* kSplitCell body over all cells of src, thread order */
void split_cells(const RefinedMesh &src, RefinedMesh &dst, const std::vector<unsigned char> *flags, bool parents)
{
    dst.V = src.V;
    dst.C.clear(); dst.S.clear(); dst.orig.clear(); dst.parent.clear();
    for (int idx = 0; idx < (int)src.C.size(); ++idx) {
        const int oc = src.orig[idx];
        if (flags && !(*flags)[oc]) continue;
        const int3 tri = src.C[idx];
        const Point3 A = src.V[tri.x], B = src.V[tri.y], Cc = src.V[tri.z];
        const int vi = (int)dst.V.size();
        dst.V.push_back(0.5 * (B + Cc));
        dst.V.push_back(0.5 * (Cc + A));
        dst.V.push_back(0.5 * (A + B));
        dst.C.push_back(make_int3(vi + 2, tri.y, vi));
        dst.C.push_back(make_int3(vi, tri.z, vi + 1));
        dst.C.push_back(make_int3(vi + 1, tri.x, vi + 2));
        dst.C.push_back(make_int3(vi, vi + 1, vi + 2));
        const double m = 0.25 * src.S[idx];
        for (int k = 0; k < 4; ++k) {
            dst.S.push_back(m);
            dst.orig.push_back(oc);
            if (parents) dst.parent.push_back(idx);
        }
    }
}

/* kIntegrateRegularPart{Simple,Attached} / kIntegrateNotNeighbors body */
double4 regular_task(int cls, int3 task, int3 orig_task, const HostMesh &m, const RefinedMesh &r)
{
    const int3 triI = r.C[task.x];
    const int3 triJ = m.C[task.y];
    Point3 q[CONSTANTS::MAX_GAUSS_POINTS];
    double4 f[CONSTANTS::MAX_GAUSS_POINTS];
    calculateQuadraturePoints(q, r.V.data(), triI);
    for (int g = 0; g < g_npts; ++g) {
        if (cls == 0)
            f[g] = thetaPsi(q[g], m.V.data(), triJ) -
                   singularPartSimple(q[g], orig_task.x, task.y, m.V.data(), m.C.data(), m.N.data(), m.S.data());
        else if (cls == 1)
            f[g] = thetaPsi(q[g], m.V.data(), triJ) - singularPartAttached(q[g], orig_task.x, task.y, m.V.data(), m.C.data());
        else
            f[g] = thetaPsi(q[g], m.V.data(), triJ);
    }
    const double4 res = integrate4D(f);
    return r.S[task.x] * res;
}

/* kFinalizeSimpleNeighborsResults / kFinalizeNonSimpleResults bodies */
Point3 finalize(int cls, int3 task, double4 integral, const HostMesh &m)
{
    const Point3 normal = m.N[task.y];
    if (cls == 0) {
        int p = 0;
        const double refTheta = CONSTANTS::TWO_PI * m.S[task.x];
        if (integral.w > refTheta)
            p = -((int)trunc((integral.w - refTheta) / (2.0 * refTheta)) + 1);
        else if (integral.w < -refTheta)
            p = ((int)trunc((-refTheta - integral.w) / (2.0 * refTheta)) + 1);
        return CONSTANTS::RECIPROCAL_FOUR_PI * ((integral.w + 2.0 * p * refTheta) * normal + cross(extract_vector_part(integral), normal));
    }
    return CONSTANTS::RECIPROCAL_FOUR_PI * (integral.w * normal + cross(extract_vector_part(integral), normal));
}

RefinedMesh original_as_refined(const HostMesh &m)
{
    RefinedMesh r;
    r.V = m.V; r.C = m.C; r.S = m.S;
    r.orig.resize(m.C.size());
    for (size_t k = 0; k < m.C.size(); ++k) r.orig[k] = (int)k;
    return r;
}

} // namespace

extern "C" {

/* NumericalIntegrator3D constructor + Evaluator3D constructor: quadrature and 2^order */
void refd_set_qf(const double *coords, const double *weights, int n, int order)
{
    for (int i = 0; i < n; ++i) {
        Point3 p = make_double3(coords[2 * i], coords[2 * i + 1], 1.0 - coords[2 * i] - coords[2 * i + 1]);
        memcpy((void *)(c_GaussPointsCoordinates + i), &p, sizeof p);
        memcpy((void *)(c_GaussPointsWeights + i), weights + i, sizeof(double));
    }
    memcpy((void *)&c_GaussPointsNumber, &n, sizeof n);
    g_npts = n;
    g_pow2p = (double)(1 << order);
}

void refd_theta_psi(const double *x, const double *A, const double *B, const double *C, double *out4)
{
    Point3 v[3] = {make_double3(A[0], A[1], A[2]), make_double3(B[0], B[1], B[2]), make_double3(C[0], C[1], C[2])};
    const double4 r = thetaPsi(make_double3(x[0], x[1], x[2]), v, make_int3(0, 1, 2));
    out4[0] = r.x; out4[1] = r.y; out4[2] = r.z; out4[3] = r.w;
}

void refd_geometry(int nv, const double *V, int nc, const int *C, double *N, double *S)
{
    HostMesh m = make_mesh(nv, V, nc, C);
    for (int c = 0; c < nc; ++c) { N[3 * c] = m.N[c].x; N[3 * c + 1] = m.N[c].y; N[3 * c + 2] = m.N[c].z; S[c] = m.S[c]; }
}

void refd_singular_parts(int cls, const double *x, int i, int j, int nv, const double *V, int nc, const int *C, double *out4)
{
    HostMesh m = make_mesh(nv, V, nc, C);
    const Point3 p = make_double3(x[0], x[1], x[2]);
    double4 r = cls == 0 ? singularPartSimple(p, i, j, m.V.data(), m.C.data(), m.N.data(), m.S.data())
                         : singularPartAttached(p, i, j, m.V.data(), m.C.data());
    out4[0] = r.x; out4[1] = r.y; out4[2] = r.z; out4[3] = r.w;
}

void refd_closed_forms(int cls, int i, int j, int nv, const double *V, int nc, const int *C, double *out4)
{
    HostMesh m = make_mesh(nv, V, nc, C);
    double4 r = cls == 0 ? integrateSingularPartSimple(i, j, m.V.data(), m.C.data(), m.N.data(), m.S.data())
                         : integrateSingularPartAttached(i, j, m.V.data(), m.C.data(), m.N.data(), m.S.data());
    out4[0] = r.x; out4[1] = r.y; out4[2] = r.z; out4[3] = r.w;
}

/*
 * One class of tasks through the reference pipeline.  cls: 0 simple (common vertex),
 * 1 attached (common edge), 2 not-neighbours.  level >= 0: setFixedRefinementLevel(level)
 * (levels 0 and 1 only: see below); level < 0: automatic error control.
 * Outputs per task: raw4 (Psi, Theta after the singular part), J3, and for the adaptive mode
 * iters (the iteration at which the task stopped being refined).
 */
int refd_run_class(int cls, int ntasks, const int *ti, const int *tj, int nv, const double *V, int nc, const int *C,
                   int level, double *raw4, double *J3, int *iters)
{
    if (level > 1) return 1; /* fixed levels >= 2 look up tempOriginalCells with an original cell index
                                (NumericalIntegrator3d.cu:120 via :292-301) and are not reproduced */
    HostMesh m = make_mesh(nv, V, nc, C);
    std::vector<int3> tasks(ntasks);
    for (int t = 0; t < ntasks; ++t) tasks[t] = make_int3(ti[t], tj[t], t);

    std::vector<double4> integrals(ntasks, make_double4(0, 0, 0, 0));

    if (level >= 0) {
        RefinedMesh r = original_as_refined(m), prev;
        std::vector<int3> refined = tasks;
        if (level == 1) {
            prev = r;
            split_cells(prev, r, nullptr, false);
            refined.clear();
            for (const int3 &ot : tasks) {                   /* kCountOrCreateTasks, no parents */
                const int oci = prev.orig[ot.x];
                for (int c = 0; c < (int)r.C.size(); ++c)
                    if (oci == r.orig[c]) refined.push_back(make_int3(c, ot.y, ot.z));
            }
        }
        for (const int3 &rt : refined) integrals[rt.z] += regular_task(cls, rt, tasks[rt.z], m, r); /* gather */
        if (iters) for (int t = 0; t < ntasks; ++t) iters[t] = level;
    } else {
        /* automatic error control: EvaluatorJ3DK::numericalIntegration (evaluatorJ3DK.cu:949-1011) */
        std::vector<double4> temp(ntasks, make_double4(0, 0, 0, 0));
        std::vector<unsigned char> converged(ntasks, 0);
        std::vector<int> rest(ntasks), stop(ntasks, 0);
        for (int t = 0; t < ntasks; ++t) rest[t] = t;
        RefinedMesh r = original_as_refined(m);
        r.parent.assign(r.C.size(), -1);
        std::vector<int3> refined = tasks;
        for (const int3 &rt : refined) integrals[rt.z] += regular_task(cls, rt, tasks[rt.z], m, r);
        std::vector<double4> *cur = &integrals, *old = &temp;
        int remaining = ntasks, iteration = 0;
        std::vector<unsigned char> flags(nc, 0);
        for (int t : rest) flags[tasks[t].x] = 1;                   /* determineCellsToBeRefined */
        while (remaining && iteration < CONSTANTS::MAX_REFINE_LEVEL) {
            ++iteration;
            RefinedMesh prev = r;                                   /* refineMesh */
            split_cells(prev, r, &flags, true);
            std::vector<int3> next;                                 /* updateTasks */
            for (const int3 &ot : refined) {
                if (converged[ot.z]) continue;
                const int oci = prev.orig[ot.x];
                for (int c = 0; c < (int)r.C.size(); ++c)
                    if (oci == r.orig[c] && r.parent[c] == ot.x) next.push_back(make_int3(c, ot.y, ot.z));
            }
            refined.swap(next);
            std::swap(cur, old);                                    /* integrals->swap(*tempIntegrals) */
            std::vector<double4> res(refined.size());
            for (size_t k = 0; k < refined.size(); ++k) res[k] = regular_task(cls, refined[k], tasks[refined[k].z], m, r);
            for (int k = 0; k < remaining; ++k) (*cur)[rest[k]] = make_double4(0, 0, 0, 0);
            for (size_t k = 0; k < refined.size(); ++k) (*cur)[refined[k].z] += res[k];
            /* compareIntegrationResults / kCompareIntegrationResults */
            std::vector<int> check;
            if (iteration == 1) { check.resize(ntasks); for (int t = 0; t < ntasks; ++t) check[t] = t; }
            else check = rest;
            std::vector<int> newrest;
            for (int idx : check) {
                const double4 a = (*cur)[idx], b = (*old)[idx];
                const double4 num = a - b;
                const double4 den = g_pow2p * b - a;
                const double crit = norm1(divide(num, den));
                if (crit > CONSTANTS::EPS_INTEGRATION) { newrest.push_back(idx); converged[idx] = 0; }
                else { converged[idx] = 1; stop[idx] = iteration; }
            }
            rest.swap(newrest);
            remaining = (int)rest.size();
            if (remaining) {
                std::fill(flags.begin(), flags.end(), 0);
                for (int t : rest) flags[tasks[t].x] = 1;
            }
        }
        for (int t : rest) stop[t] = iteration;
        if (iters) for (int t = 0; t < ntasks; ++t) iters[t] = stop[t];
        if (cur != &integrals) integrals = *cur;
    }

    for (int t = 0; t < ntasks; ++t) {                               /* singular parts + finalisation */
        if (cls == 0) integrals[t] += integrateSingularPartSimple(tasks[t].x, tasks[t].y, m.V.data(), m.C.data(), m.N.data(), m.S.data());
        else if (cls == 1) integrals[t] += integrateSingularPartAttached(tasks[t].x, tasks[t].y, m.V.data(), m.C.data(), m.N.data(), m.S.data());
        const Point3 J = finalize(cls, tasks[t], integrals[t], m);
        raw4[4 * t] = integrals[t].x; raw4[4 * t + 1] = integrals[t].y;
        raw4[4 * t + 2] = integrals[t].z; raw4[4 * t + 3] = integrals[t].w;
        J3[3 * t] = J.x; J3[3 * t + 1] = J.y; J3[3 * t + 2] = J.z;
    }
    return 0;
}

} // extern "C"
