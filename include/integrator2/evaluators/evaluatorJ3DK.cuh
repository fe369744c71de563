// evaluatorJ3DK.cuh -- EvaluatorJ3DK, the reference's evaluator of
// J(K_i, K_j) = (1/4 pi) int_{K_i} int_{K_j} grad_y 1/|x - y| dS_y dS_x (src/evaluators/
// evaluatorJ3DK.cuh:140-211) over the library: each integrateOver<Class>() integrates that class's
// tasks (regular part with the integrator's rule and refinement, closed-form singular parts,
// finalisation) into the protected result vectors of Evaluator3D.  numericalIntegration(type)
// is that whole class run (the library does not split the regular and singular parts into
// separate calls).
#ifndef I2_DROPIN_EVALUATOR_J3DK_CUH
#define I2_DROPIN_EVALUATOR_J3DK_CUH

#include "evaluator3d.cuh"

class EvaluatorJ3DK : public Evaluator3D {
public:
    EvaluatorJ3DK(const Mesh3D &mesh_, NumericalIntegrator3D &numIntegrator_) : Evaluator3D(mesh_, numIntegrator_) {}

    virtual void integrateOverSimpleNeighbors() override { numericalIntegration(neighbour_type_enum::simple_neighbors); }
    virtual void integrateOverAttachedNeighbors() override { numericalIntegration(neighbour_type_enum::attached_neighbors); }
    virtual void integrateOverNotNeighbors() override { numericalIntegration(neighbour_type_enum::not_neighbors); }

    void numericalIntegration(neighbour_type_enum neighborType)
    {
        const deviceVector<int3> *T = getTasks(neighborType);
        std::printf("\nIntegrating over %s (%d pairs)...\n", neighborTypeString(neighborType).c_str(), T ? T->size : 0);
        runClass(neighborType);
    }
};

#endif
