// evaluator3d.cuh -- Evaluator3D, the reference's abstract evaluator (src/evaluators/
// evaluator3d.cuh, evaluator3d.cu): runAllPairs builds the task lists of the three classes (the
// mesh's (i, j) rows followed by the reversed rows, as kAddReversedPairs does) and calls the
// virtual integrateOver<Class>() of each, timing each with a GpuTimer as the reference does;
// runPairs does the same for user lists; outputResultsToFile writes the reference's plain-text or
// CSV files.  A subclass sees the reference's protected vectors: the tasks (int3), the integrals
// (double4: Psi, Theta), the results J (Point3) and, after runAllPairs(true), the (i,j)/(j,i)
// antisymmetry errors.  runClass() integrates one class's tasks through the library into those
// vectors; EvaluatorJ3DK's overrides call it.
// Additions: the potential P per pair (d_*Potentials), setStream, getLevels, handle().
#ifndef I2_DROPIN_EVALUATOR3D_CUH
#define I2_DROPIN_EVALUATOR3D_CUH

#include "../Mesh3d.cuh"
#include "../NumericalIntegrator3d.cuh"
#include "../common/gpu_timer.cuh"

#include <algorithm>
#include <iomanip>
#include <vector>

// src/evaluators/evaluator3d.cuh:19-22; csvFullPrecision writes 17 significant digits
enum class output_format_enum { plainText = 1, csv = 2, csvFullPrecision = 3 };

class Evaluator3D {
public:
    Evaluator3D(const Mesh3D &mesh_, NumericalIntegrator3D &numIntegrator_) : mesh(mesh_), numIntegrator(numIntegrator_)
    {
        i2dropin::check(i2_evaluator_create(mesh.handle(), numIntegrator.handle(), &h_), "i2_evaluator_create");
    }
    virtual ~Evaluator3D() { i2_evaluator_destroy(h_); }
    Evaluator3D(const Evaluator3D &) = delete;
    Evaluator3D &operator=(const Evaluator3D &) = delete;

    virtual void integrateOverSimpleNeighbors() = 0;
    virtual void integrateOverAttachedNeighbors() = 0;
    virtual void integrateOverNotNeighbors() = 0;

    // src/evaluators/evaluator3d.cu:120-204
    virtual void runAllPairs(bool checkCorrectness = false)
    {
        with_reversed(mesh.getSimpleNeighbors(), simpleNeighborsTasks);
        with_reversed(mesh.getAttachedNeighbors(), attachedNeighborsTasks);
        with_reversed(mesh.getNotNeighbors(), notNeighborsTasks);
        for (int k = 0; k < 3; ++k) size_outputs((neighbour_type_enum)k);
        timed(&Evaluator3D::integrateOverSimpleNeighbors, "Simple neighbors integration");
        timed(&Evaluator3D::integrateOverAttachedNeighbors, "Attached neighbors integration");
        timed(&Evaluator3D::integrateOverNotNeighbors, "Non-neighbors integration");
        if (checkCorrectness)
            for (int k = 0; k < 3; ++k) antisymmetry((neighbour_type_enum)k);
    }
    // src/evaluators/evaluator3d.cu:213-288: (i, j, index) rows per class; empty lists are skipped
    void runPairs(const std::vector<int3> &userSimpleNeighborsTasks, const std::vector<int3> &userAttachedNeighborsTasks,
                  const std::vector<int3> &userNotNeighborsTasks)
    {
        const std::vector<int3> *user[3] = {&userSimpleNeighborsTasks, &userAttachedNeighborsTasks, &userNotNeighborsTasks};
        for (int k = 0; k < 3; ++k) {
            if (user[k]->empty()) continue;
            i2dropin::upload(*tasks_of((neighbour_type_enum)k), *user[k]);
            size_outputs((neighbour_type_enum)k);
            errors_of((neighbour_type_enum)k)->allocate(0);
        }
        if (!userSimpleNeighborsTasks.empty()) timed(&Evaluator3D::integrateOverSimpleNeighbors, "Simple neighbors integration");
        if (!userAttachedNeighborsTasks.empty()) timed(&Evaluator3D::integrateOverAttachedNeighbors, "Attached neighbors integration");
        if (!userNotNeighborsTasks.empty()) timed(&Evaluator3D::integrateOverNotNeighbors, "Non-neighbors integration");
    }
    // src/evaluators/evaluator3d.cu:354-457: <Class>.dat ("(i, j): [x, y, z]" lines) or <Class>.csv
    // (";"-separated with a header), with the error column after runAllPairs(true)
    bool outputResultsToFile(neighbour_type_enum neighborType, output_format_enum outputFormat) const
    {
        const int k = (int)neighborType;
        if (k < 0 || k > 2) return false;
        const deviceVector<int3> &T = *getTasks(neighborType);
        if (!T.size) return false;
        const int n = T.size;
        std::vector<int3> tasks(n);
        std::vector<Point3> J(n);
        std::vector<double> err;
        copy_d2h(T.data, tasks.data(), n);
        copy_d2h(results_of(neighborType)->data, J.data(), n);
        const deviceVector<double> &E = *const_cast<Evaluator3D *>(this)->errors_of(neighborType);
        if (E.size == n) {
            err.resize(n);
            copy_d2h(E.data, err.data(), n);
        }
        const std::string name = neighborTypeString(neighborType) + (outputFormat == output_format_enum::plainText ? ".dat" : ".csv");
        std::ofstream f(name.c_str());
        if (!f.is_open()) return false;
        if (outputFormat == output_format_enum::csvFullPrecision) f << std::setprecision(17);
        if (outputFormat != output_format_enum::plainText) f << "\"TaskI\";\"TaskJ\";\"IntegralX\";\"IntegralY\";\"IntegralZ\"" << (err.empty() ? "" : ";\"Error\"") << "\n";
        for (int i = 0; i < n; ++i) {
            if (outputFormat == output_format_enum::plainText) {
                f << "(" << tasks[i].x << ", " << tasks[i].y << "): [" << J[i].x << ", " << J[i].y << ", " << J[i].z << "]";
                if (!err.empty()) f << ", error = " << err[i];
            } else {
                f << tasks[i].x << ";" << tasks[i].y << ";" << J[i].x << ";" << J[i].y << ";" << J[i].z;
                if (!err.empty()) f << ";" << err[i];
            }
            f << "\n";
        }
        return true;
    }
    const deviceVector<int3> *getTasks(neighbour_type_enum neighborType) const
    {
        return const_cast<Evaluator3D *>(this)->tasks_of(neighborType);
    }

    // additions: the evaluator's stream (cudaStream_t; default the legacy default stream), the
    // refinement level each pair of a class kept (-1 in fixed mode), the library handle
    void setStream(cudaStream_t s)
    {
        stream_ = s;
        i2dropin::check(i2_evaluator_set_stream(h_, (void *)s), "i2_evaluator_set_stream");
    }
    std::vector<int> getLevels(neighbour_type_enum neighborType) const
    {
        int64_t n = 0;
        i2dropin::check(i2_evaluator_result_count(h_, (i2_pair_class)neighborType, &n), "i2_evaluator_result_count");
        std::vector<double> lv((size_t)n);
        if (n) i2dropin::check(i2_evaluator_copy_results(h_, (i2_pair_class)neighborType, I2_CHANNEL_LEVEL, lv.data(), n), "i2_evaluator_copy_results");
        return std::vector<int>(lv.begin(), lv.end());
    }
    i2_evaluator_t *handle() const { return h_; }

protected:
    // integrates the tasks of one class through the library: J into d_<Class>Results, (Psi, Theta)
    // into d_<Class>Integrals, P into d_<Class>Potentials; after an adaptive run, the integrator's
    // per-cell refinement counts of the class
    void runClass(neighbour_type_enum neighborType)
    {
        const deviceVector<int3> &T = *tasks_of(neighborType);
        const int n = T.size;
        if (!n) return;
        pairs2_.resize(n);
        // (i, j, index) rows to the library's (i, j) rows: a strided device-to-device copy
        checkCudaErrors(cudaMemcpy2DAsync(pairs2_.data, sizeof(int2), T.data, sizeof(int3), sizeof(int2), n, cudaMemcpyDeviceToDevice, stream_));
        i2dropin::check(i2_evaluator_run_class_device(h_, (i2_pair_class)neighborType, &pairs2_.data[0].x, n, &integrals_of(neighborType)->data[0].x,
                                                      &results_of(neighborType)->data[0].x, potentials_of(neighborType)->data),
                        "i2_evaluator_run_class_device");
        if (numIntegrator.getErrorControlType() != error_control_type_enum::fixed_refinement_level) refinements(neighborType, T);
    }

    deviceVector<int3> simpleNeighborsTasks, attachedNeighborsTasks, notNeighborsTasks;
    deviceVector<double4> d_simpleNeighborsIntegrals, d_attachedNeighborsIntegrals, d_notNeighborsIntegrals;
    deviceVector<Point3> d_simpleNeighborsResults, d_attachedNeighborsResults, d_notNeighborsResults;
    deviceVector<double> d_simpleNeighborsPotentials, d_attachedNeighborsPotentials, d_notNeighborsPotentials;
    deviceVector<double> simpleNeighborsErrors, attachedNeighborsErrors, notNeighborsErrors;
    const Mesh3D &mesh;
    NumericalIntegrator3D &numIntegrator;
    GpuTimer timer;

private:
    deviceVector<int3> *tasks_of(neighbour_type_enum t)
    {
        return t == neighbour_type_enum::simple_neighbors ? &simpleNeighborsTasks
             : t == neighbour_type_enum::attached_neighbors ? &attachedNeighborsTasks
             : t == neighbour_type_enum::not_neighbors ? &notNeighborsTasks : nullptr;
    }
    deviceVector<double4> *integrals_of(neighbour_type_enum t)
    {
        return t == neighbour_type_enum::simple_neighbors ? &d_simpleNeighborsIntegrals
             : t == neighbour_type_enum::attached_neighbors ? &d_attachedNeighborsIntegrals : &d_notNeighborsIntegrals;
    }
    const deviceVector<Point3> *results_of(neighbour_type_enum t) const
    {
        return t == neighbour_type_enum::simple_neighbors ? &d_simpleNeighborsResults
             : t == neighbour_type_enum::attached_neighbors ? &d_attachedNeighborsResults : &d_notNeighborsResults;
    }
    deviceVector<Point3> *results_of(neighbour_type_enum t) { return const_cast<deviceVector<Point3> *>(static_cast<const Evaluator3D *>(this)->results_of(t)); }
    deviceVector<double> *potentials_of(neighbour_type_enum t)
    {
        return t == neighbour_type_enum::simple_neighbors ? &d_simpleNeighborsPotentials
             : t == neighbour_type_enum::attached_neighbors ? &d_attachedNeighborsPotentials : &d_notNeighborsPotentials;
    }
    deviceVector<double> *errors_of(neighbour_type_enum t)
    {
        return t == neighbour_type_enum::simple_neighbors ? &simpleNeighborsErrors
             : t == neighbour_type_enum::attached_neighbors ? &attachedNeighborsErrors : &notNeighborsErrors;
    }
    void size_outputs(neighbour_type_enum t)
    {
        const int n = tasks_of(t)->size;
        integrals_of(t)->allocate(n);
        results_of(t)->allocate(n);
        potentials_of(t)->allocate(n);
    }
    // rows (i, j, k) of the mesh's list, then (j, i, n + k) (kAddReversedPairs, evaluator3d.cu:22-31)
    void with_reversed(const deviceVector<int3> &list, deviceVector<int3> &tasks)
    {
        const int n = list.size;
        std::vector<int3> rows(2 * (size_t)n);
        if (n) copy_d2h(list.data, rows.data(), n);
        for (int k = 0; k < n; ++k) rows[n + k] = make_int3(rows[k].y, rows[k].x, n + k);
        i2dropin::upload(tasks, rows);
    }
    void timed(void (Evaluator3D::*f)(), const char *what)
    {
        timer.start(stream_);
        (this->*f)();
        timer.stop(what, stream_);
    }
    // delta = |J_ij + J_ji|_1 / max(|J_ij|_1, |J_ji|_1) for rows k and n + k, both rows
    // (kCalculateIntegrationError, evaluator3d.cu:45-57)
    void antisymmetry(neighbour_type_enum t)
    {
        const int n2 = results_of(t)->size, n = n2 / 2;
        std::vector<Point3> J(n2);
        std::vector<double> d(n2);
        if (n2) copy_d2h(results_of(t)->data, J.data(), n2, stream_);
        for (int k = 0; k < n; ++k) {
            const double e = norm1(J[k] + J[n + k]) / std::max(norm1(J[k]), norm1(J[n + k]));
            d[k] = d[n + k] = e;
        }
        i2dropin::upload(*errors_of(t), d);
    }
    // per original cell i: the deepest refinement level kept by a pair (i, .) of the class
    void refinements(neighbour_type_enum t, const deviceVector<int3> &T)
    {
        const std::vector<int> lv = getLevels(t);
        std::vector<int3> rows(T.size);
        copy_d2h(T.data, rows.data(), T.size, stream_);
        std::vector<unsigned char> r(mesh.getCells().size, 0);
        for (size_t k = 0; k < rows.size() && k < lv.size(); ++k)
            r[rows[k].x] = (unsigned char)std::max((int)r[rows[k].x], std::max(lv[k], 0));
        i2dropin::upload(numIntegrator.refinementsRequired[(int)t], r);
    }

    i2_evaluator_t *h_ = nullptr;
    cudaStream_t stream_ = nullptr;
    deviceVector<int2> pairs2_;
};

#endif
