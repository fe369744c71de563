// NumericalIntegrator3d.cuh -- NumericalIntegrator3D with the reference's interface
// (src/NumericalIntegrator3d.cuh): constructed from a mesh and a quadrature rule, fixed
// refinement level or automatic (Runge) error control, the rule's size and order, the refined
// mesh of a fixed-level run (getRefinedVertices / Cells / CellMeasures) and, after an adaptive
// run, the number of refinements each cell needed per pair class (getRefinementsRequired).
// The integrator's settings live in a library handle (integrator2_gb300.h); the library refines
// per pair without building a refined mesh, so the refined mesh is made on request: every cell
// split refinementLevel times at its edge midpoints in the reference's child order (kSplitCell,
// src/NumericalIntegrator3d.cu:37-87), the midpoints appended per cell, as many vertices and cells
// as the reference keeps (nv + nc (4^L - 1) and 4^L nc).
// Additions: setErrorControl (relative, scale-free criterion), setPrecision (mixed FP32/FP64),
// setPotential, setPotentialRule, setHardPairTolerance, setSelfConvention, handle().
#ifndef I2_DROPIN_NUMERICAL_INTEGRATOR_3D_CUH
#define I2_DROPIN_NUMERICAL_INTEGRATOR_3D_CUH

#include "Mesh3d.cuh"
#include "QuadratureFormula3d.cuh"
#include "common/constants.h"

// src/NumericalIntegrator3d.cuh:16-19; relative_error_control is the library's scale-free mode
enum class error_control_type_enum { fixed_refinement_level = 0, automatic_error_control = 1, relative_error_control = 2 };

class Evaluator3D;

class NumericalIntegrator3D {
public:
    NumericalIntegrator3D(const Mesh3D &mesh_, const QuadratureFormula3D &qf_) : mesh(mesh_), qf(qf_), GaussPointsNum((int)qf_.weights.size())
    {
        i2dropin::check(i2_integrator_create(mesh.handle(), &qf.coordinates[0].x, qf.weights.data(), GaussPointsNum, qf.order, &h_),
                        "i2_integrator_create");
    }
    virtual ~NumericalIntegrator3D() { i2_integrator_destroy(h_); }
    NumericalIntegrator3D(const NumericalIntegrator3D &) = delete;
    NumericalIntegrator3D &operator=(const NumericalIntegrator3D &) = delete;

    void setFixedRefinementLevel(int refinementLevel = 0)
    {
        i2dropin::check(i2_integrator_set_fixed_refinement_level(h_, refinementLevel), "i2_integrator_set_fixed_refinement_level");
        meshRefinementLevel = refinementLevel;
        refinedLevel = -1;
    }
    int getGaussPointsNumber() const { return GaussPointsNum; }
    int getQuadratureFormulaOrder() const { return qf.order; }
    error_control_type_enum getErrorControlType() const
    {
        i2_error_control m;
        int32_t lv = 0;
        i2dropin::check(i2_integrator_get_error_control(h_, &m, &lv), "i2_integrator_get_error_control");
        return (error_control_type_enum)m;
    }

    // the mesh refined uniformly refinementLevel times (the original mesh in an adaptive run)
    const deviceVector<Point3> &getRefinedVertices() const { refine(); return refinedVertices; }
    const deviceVector<int3> &getRefinedCells() const { refine(); return refinedCells; }
    const deviceVector<double> &getRefinedCellMeasures() const { refine(); return refinedCellMeasures; }
    // per original cell, how often it was refined for pairs of a class in the last adaptive run
    deviceVector<unsigned char> *getRefinementsRequired(neighbour_type_enum t)
    {
        const int k = (int)t;
        return k >= 0 && k < 3 ? &refinementsRequired[k] : nullptr;
    }

    void setErrorControl(error_control_type_enum mode, double rel_tol = 1e-6, int max_level = CONSTANTS::MAX_REFINE_LEVEL)
    {
        i2dropin::check(i2_integrator_set_error_control(h_, (i2_error_control)mode, rel_tol, max_level), "i2_integrator_set_error_control");
    }
    void setPrecision(i2_precision p) { i2dropin::check(i2_integrator_set_precision(h_, p), "i2_integrator_set_precision"); }
    void setPotential(bool enabled) { i2dropin::check(i2_integrator_set_potential(h_, enabled ? 1 : 0), "i2_integrator_set_potential"); }
    void setPotentialRule(int n_radial, int n_angular, int grading, int n_self = 0)
    {
        i2dropin::check(i2_integrator_set_potential_rule(h_, n_radial, n_angular, grading, n_self), "i2_integrator_set_potential_rule");
    }
    void setHardPairTolerance(double rel_tol) { i2dropin::check(i2_integrator_set_hard_pair_tolerance(h_, rel_tol), "i2_integrator_set_hard_pair_tolerance"); }
    void setSelfConvention(int sign) { i2dropin::check(i2_integrator_set_self_convention(h_, sign), "i2_integrator_set_self_convention"); }
    i2_integrator_t *handle() const { return h_; }

private:
    friend class Evaluator3D;

    void refine() const
    {
        const int L = getErrorControlType() == error_control_type_enum::fixed_refinement_level ? meshRefinementLevel : 0;
        if (refinedLevel == L && refinedCells.size == (1 << (2 * L)) * mesh.getCells().size) return;
        const int nv = mesh.getVertices().size, nc = mesh.getCells().size;
        std::vector<Point3> V(nv);
        std::vector<int3> C(nc);
        copy_d2h(mesh.getVertices().data, V.data(), nv);
        copy_d2h(mesh.getCells().data, C.data(), nc);
        std::vector<double> S(nc);
        for (int c = 0; c < nc; ++c) S[c] = 0.5 * vector_length(cross(V[C[c].y] - V[C[c].x], V[C[c].z] - V[C[c].x]));
        for (int l = 0; l < L; ++l) {
            std::vector<int3> C2;
            std::vector<double> S2;
            C2.reserve(4 * C.size());
            S2.reserve(4 * C.size());
            for (size_t c = 0; c < C.size(); ++c) {
                const int3 t = C[c];
                const int m = (int)V.size();  // midpoints of BC, CA, AB
                V.push_back(0.5 * (V[t.y] + V[t.z]));
                V.push_back(0.5 * (V[t.z] + V[t.x]));
                V.push_back(0.5 * (V[t.x] + V[t.y]));
                C2.push_back(make_int3(m + 2, t.y, m));
                C2.push_back(make_int3(m, t.z, m + 1));
                C2.push_back(make_int3(m + 1, t.x, m + 2));
                C2.push_back(make_int3(m, m + 1, m + 2));
                for (int k = 0; k < 4; ++k) S2.push_back(0.25 * S[c]);
            }
            C.swap(C2);
            S.swap(S2);
        }
        i2dropin::upload(refinedVertices, V);
        i2dropin::upload(refinedCells, C);
        i2dropin::upload(refinedCellMeasures, S);
        refinedLevel = L;
    }

    const Mesh3D &mesh;
    const QuadratureFormula3D &qf;
    const int GaussPointsNum;
    int meshRefinementLevel = 0;
    i2_integrator_t *h_ = nullptr;
    mutable int refinedLevel = -1;
    mutable deviceVector<Point3> refinedVertices;
    mutable deviceVector<int3> refinedCells;
    mutable deviceVector<double> refinedCellMeasures;
    deviceVector<unsigned char> refinementsRequired[3];
};

#endif
