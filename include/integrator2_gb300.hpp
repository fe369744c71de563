// integrator2_gb300.hpp -- C++ classes with the reference's names and call pattern
// (andreyypopov/integrator2: src/Mesh3d.cuh, src/QuadratureFormula3d.cuh,
// src/NumericalIntegrator3d.cuh, src/evaluators/evaluator3d.cuh, evaluatorJ3DK.cuh), implemented
// header-only over the C-ABI of integrator2_gb300.h.  A program written against the reference
//
//     Mesh3D mesh;  mesh.loadMeshFromFile(file, scale);  mesh.prepareMesh();
//     NumericalIntegrator3D integrator(mesh, qf3D13);  integrator.setFixedRefinementLevel(r);
//     EvaluatorJ3DK evaluator(mesh, integrator);  evaluator.runAllPairs(check);
//     evaluator.outputResultsToFile(neighbour_type_enum::simple_neighbors, output_format_enum::csv);
//
// compiles against this header unchanged in those calls.  Differences: results are read with
// getResults()/getPotentials() (full precision, host vectors) instead of protected device
// vectors; CUDA failures throw i2::Error instead of exit(); prepareMesh(near_factor) can restrict
// the disjoint class to near-field pairs.
#pragma once

#include "integrator2_gb300.h"

#include <array>
#include <stdexcept>
#include <string>
#include <vector>

namespace i2 {

struct Error : std::runtime_error {
    i2_status code;
    Error(i2_status c, const std::string &where)
        : std::runtime_error(where + ": " + i2_status_string(c) + ": " + i2_last_error()), code(c)
    {
    }
};

inline void check(i2_status s, const char *where)
{
    if (s != I2_OK) throw Error(s, where);
}

} // namespace i2

// src/Mesh3d.cuh:18-23 (plus the self class)
enum class neighbour_type_enum { simple_neighbors = 0, attached_neighbors = 1, not_neighbors = 2, self = 3, undefined = -1 };
// src/NumericalIntegrator3d.cuh:16-19 (plus the scale-invariant mode)
enum class error_control_type_enum { fixed_refinement_level = 0, automatic_error_control = 1, relative_error_control = 2 };
// src/evaluators/evaluator3d.cuh:19-22 (plus full precision CSV)
enum class output_format_enum { plainText = 0, csv = 1, csvFullPrecision = 2 };

struct Int3 {
    int x, y, z;
};

// src/QuadratureFormula3d.cuh:20-31: a rule is (barycentric coordinates, weights, order)
struct QuadratureFormula3D {
    std::vector<std::array<double, 2>> coordinates;
    std::vector<double> weights;
    int order;

    static QuadratureFormula3D builtin(int npoints)
    {
        QuadratureFormula3D q;
        std::vector<double> c(2 * npoints), w(npoints);
        int32_t order = 0;
        i2::check(i2_quadrature_builtin(npoints, c.data(), w.data(), &order), "i2_quadrature_builtin");
        for (int k = 0; k < npoints; ++k) q.coordinates.push_back({c[2 * k], c[2 * k + 1]});
        q.weights = w;
        q.order = order;
        return q;
    }
};

// the reference's built-in rules (src/QuadratureFormula3d.cuh:34-213)
inline const QuadratureFormula3D qf3D1 = QuadratureFormula3D::builtin(1);
inline const QuadratureFormula3D qf3D3 = QuadratureFormula3D::builtin(3);
inline const QuadratureFormula3D qf3D4 = QuadratureFormula3D::builtin(4);
inline const QuadratureFormula3D qf3D6 = QuadratureFormula3D::builtin(6);
inline const QuadratureFormula3D qf3D7 = QuadratureFormula3D::builtin(7);
inline const QuadratureFormula3D qf3D9 = QuadratureFormula3D::builtin(9);
inline const QuadratureFormula3D qf3D12 = QuadratureFormula3D::builtin(12);
inline const QuadratureFormula3D qf3D13 = QuadratureFormula3D::builtin(13);

inline std::string neighborTypeString(neighbour_type_enum t)
{
    switch (t) {
    case neighbour_type_enum::simple_neighbors: return "SimpleNeighbors";
    case neighbour_type_enum::attached_neighbors: return "AttachedNeighbors";
    case neighbour_type_enum::not_neighbors: return "NotNeighbors";
    case neighbour_type_enum::self: return "Self";
    default: return std::string();
    }
}

class Mesh3D {
public:
    Mesh3D() { i2::check(i2_mesh_create(&h_), "i2_mesh_create"); }
    ~Mesh3D() { i2_mesh_destroy(h_); }
    Mesh3D(const Mesh3D &) = delete;
    Mesh3D &operator=(const Mesh3D &) = delete;

    // src/Mesh3d.cuh:55
    bool loadMeshFromFile(const std::string &filename, double scale = 1.0)
    {
        return i2_mesh_load_file(h_, filename.c_str(), scale) == I2_OK;
    }
    void setGeometry(const std::vector<double> &vertices, const std::vector<int> &cells)
    {
        i2::check(i2_mesh_set_geometry(h_, vertices.data(), (int32_t)(vertices.size() / 3), cells.data(), (int32_t)(cells.size() / 3)),
                  "i2_mesh_set_geometry");
    }
    // src/Mesh3d.cuh:63; near_factor <= 0: every disjoint pair, as the reference
    void prepareMesh(double near_factor = 0.0) { i2::check(i2_mesh_prepare(h_, near_factor), "i2_mesh_prepare"); }
    // prepareMesh with the lists built on the GPU (same lists, same order)
    void prepareMeshDevice(double near_factor = 0.0, bool host_copy = true)
    {
        i2::check(i2_mesh_prepare_device(h_, near_factor, host_copy ? 1 : 0), "i2_mesh_prepare_device");
    }
    // device rows (i, j) of a class's unordered list (2 int32 per row), owned by the mesh
    const int32_t *devicePairs(i2_pair_class cls, int64_t &n) const
    {
        const int32_t *p = nullptr;
        i2::check(i2_mesh_device_pairs(h_, cls, &p, &n), "i2_mesh_device_pairs");
        return p;
    }

    std::vector<Int3> getSimpleNeighbors() const { return pairs(I2_SIMPLE_NEIGHBORS); }
    std::vector<Int3> getAttachedNeighbors() const { return pairs(I2_ATTACHED_NEIGHBORS); }
    std::vector<Int3> getNotNeighbors() const { return pairs(I2_NOT_NEIGHBORS); }
    std::vector<Int3> getSelfPairs() const { return pairs(I2_SELF); }
    std::vector<double> getCellMeasures() const
    {
        int32_t nv = 0, nc = 0;
        i2::check(i2_mesh_sizes(h_, &nv, &nc), "i2_mesh_sizes");
        std::vector<double> m(nc);
        i2::check(i2_mesh_copy_cell_data(h_, nullptr, m.data(), nullptr), "i2_mesh_copy_cell_data");
        return m;
    }
    // src/Mesh3d.cuh:70-126 (host copies)
    std::vector<double> getVertices() const
    {
        int32_t nv = 0, nc = 0;
        i2::check(i2_mesh_sizes(h_, &nv, &nc), "i2_mesh_sizes");
        std::vector<double> v(3 * (size_t)nv);
        i2::check(i2_mesh_copy_geometry(h_, v.data(), nullptr), "i2_mesh_copy_geometry");
        return v;
    }
    std::vector<Int3> getCells() const
    {
        int32_t nv = 0, nc = 0;
        i2::check(i2_mesh_sizes(h_, &nv, &nc), "i2_mesh_sizes");
        std::vector<Int3> c(nc);
        if (nc) i2::check(i2_mesh_copy_geometry(h_, nullptr, &c[0].x), "i2_mesh_copy_geometry");
        return c;
    }
    std::vector<double> getCellNormals() const
    {
        int32_t nv = 0, nc = 0;
        i2::check(i2_mesh_sizes(h_, &nv, &nc), "i2_mesh_sizes");
        std::vector<double> n(3 * (size_t)nc);
        i2::check(i2_mesh_copy_cell_data(h_, n.data(), nullptr, nullptr), "i2_mesh_copy_cell_data");
        return n;
    }
    i2_mesh_t *handle() const { return h_; }

private:
    std::vector<Int3> pairs(i2_pair_class cls) const
    {
        int64_t n = 0;
        i2::check(i2_mesh_pair_count(h_, cls, &n), "i2_mesh_pair_count");
        std::vector<Int3> rows(n);
        if (n) i2::check(i2_mesh_copy_pairs(h_, cls, &rows[0].x, n), "i2_mesh_copy_pairs");
        return rows;
    }
    i2_mesh_t *h_ = nullptr;
};

class NumericalIntegrator3D {
public:
    // src/NumericalIntegrator3d.cuh:73
    NumericalIntegrator3D(const Mesh3D &mesh, const QuadratureFormula3D &qf) : qf_(qf)
    {
        std::vector<double> c;
        for (const auto &p : qf.coordinates) {
            c.push_back(p[0]);
            c.push_back(p[1]);
        }
        i2::check(i2_integrator_create(mesh.handle(), c.data(), qf.weights.data(), (int32_t)qf.weights.size(), qf.order, &h_),
                  "i2_integrator_create");
    }
    ~NumericalIntegrator3D() { i2_integrator_destroy(h_); }
    NumericalIntegrator3D(const NumericalIntegrator3D &) = delete;
    NumericalIntegrator3D &operator=(const NumericalIntegrator3D &) = delete;

    void setFixedRefinementLevel(int refinementLevel = 0)
    {
        i2::check(i2_integrator_set_fixed_refinement_level(h_, refinementLevel), "i2_integrator_set_fixed_refinement_level");
    }
    void setErrorControl(error_control_type_enum mode, double rel_tol = 1e-6, int max_level = 5)
    {
        i2::check(i2_integrator_set_error_control(h_, (i2_error_control)mode, rel_tol, max_level), "i2_integrator_set_error_control");
    }
    void setPrecision(i2_precision p) { i2::check(i2_integrator_set_precision(h_, p), "i2_integrator_set_precision"); }
    error_control_type_enum getErrorControlType() const
    {
        i2_error_control m;
        int32_t lv;
        i2::check(i2_integrator_get_error_control(h_, &m, &lv), "i2_integrator_get_error_control");
        return (error_control_type_enum)m;
    }
    int getGaussPointsNumber() const { return (int)qf_.weights.size(); }
    int getQuadratureFormulaOrder() const { return qf_.order; }
    i2_integrator_t *handle() const { return h_; }

private:
    QuadratureFormula3D qf_;
    i2_integrator_t *h_ = nullptr;
};

class EvaluatorJ3DK {
public:
    // src/evaluators/evaluatorJ3DK.cuh:140-146
    EvaluatorJ3DK(const Mesh3D &mesh, NumericalIntegrator3D &integrator)
    {
        i2::check(i2_evaluator_create(mesh.handle(), integrator.handle(), &h_), "i2_evaluator_create");
    }
    ~EvaluatorJ3DK() { i2_evaluator_destroy(h_); }
    EvaluatorJ3DK(const EvaluatorJ3DK &) = delete;
    EvaluatorJ3DK &operator=(const EvaluatorJ3DK &) = delete;

    // src/evaluators/evaluator3d.cu:120-204
    void runAllPairs(bool checkCorrectness = false)
    {
        i2::check(i2_evaluator_run_all_pairs(h_, checkCorrectness ? 1 : 0), "i2_evaluator_run_all_pairs");
    }
    // src/evaluators/evaluator3d.cu:213-288
    void runPairs(const std::vector<Int3> &simple, const std::vector<Int3> &attached, const std::vector<Int3> &notNeighbors)
    {
        i2::check(i2_evaluator_run_pairs(h_, simple.empty() ? nullptr : &simple[0].x, (int64_t)simple.size(),
                                         attached.empty() ? nullptr : &attached[0].x, (int64_t)attached.size(),
                                         notNeighbors.empty() ? nullptr : &notNeighbors[0].x, (int64_t)notNeighbors.size()),
                  "i2_evaluator_run_pairs");
    }
    // src/evaluators/evaluator3d.cu:354-457 (file name as in the reference unless given)
    bool outputResultsToFile(neighbour_type_enum type, output_format_enum format, std::string path = std::string()) const
    {
        if (path.empty()) path = neighborTypeString(type) + (format == output_format_enum::plainText ? ".dat" : ".csv");
        return i2_evaluator_output_results(h_, (i2_pair_class)type, (i2_output_format)format, path.c_str()) == I2_OK;
    }
    std::vector<double> getResults(neighbour_type_enum type) const { return channel(type, I2_CHANNEL_J, 3); }
    std::vector<double> getIntegrals(neighbour_type_enum type) const { return channel(type, I2_CHANNEL_RAW, 4); }
    std::vector<double> getPotentials(neighbour_type_enum type) const { return channel(type, I2_CHANNEL_P, 1); }
    // refinement level kept per pair (-1 in fixed mode) and the (i,j)/(j,i) check (after runAllPairs(true))
    std::vector<double> getLevels(neighbour_type_enum type) const { return channel(type, I2_CHANNEL_LEVEL, 1); }
    std::vector<double> getErrors(neighbour_type_enum type) const { return channel(type, I2_CHANNEL_ERROR, 1); }

private:
    std::vector<double> channel(neighbour_type_enum type, i2_channel ch, int width) const
    {
        int64_t n = 0;
        i2::check(i2_evaluator_result_count(h_, (i2_pair_class)type, &n), "i2_evaluator_result_count");
        std::vector<double> out((size_t)n * width);
        if (n) i2::check(i2_evaluator_copy_results(h_, (i2_pair_class)type, ch, out.data(), n), "i2_evaluator_copy_results");
        return out;
    }
    i2_evaluator_t *h_ = nullptr;
};
