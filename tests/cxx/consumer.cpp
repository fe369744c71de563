// A program written against the reference's C++ interface (the header set include/integrator2/,
// which keeps the reference's file names: Mesh3d.cuh, NumericalIntegrator3d.cuh,
// evaluators/evaluatorJ3DK.cuh), linked with libi2gb300.so.  It follows the reference's test
// program (load, prepareMesh, fixed level or automatic error control, runAllPairs with the check,
// result files, refined-mesh and refinement-count exports) and adds a harness subclass of
// EvaluatorJ3DK that reads the protected result vectors at full precision, the way a user of the
// reference reads its results.
//
// usage: consumer <mesh.dat> <level | -1 for automatic error control> <out.txt>
// out.txt: one line per task, "class i j Jx Jy Jz error" (17 significant digits).
#include "integrator2/Mesh3d.cuh"
#include "integrator2/NumericalIntegrator3d.cuh"
#include "integrator2/evaluators/evaluatorJ3DK.cuh"

#include <array>
#include <cstdio>
#include <cstdlib>
#include <vector>

class Harness : public EvaluatorJ3DK {
public:
    Harness(const Mesh3D &m, NumericalIntegrator3D &it) : EvaluatorJ3DK(m, it) {}

    void dump(const char *path) const
    {
        FILE *f = std::fopen(path, "w");
        if (!f) std::exit(3);
        const deviceVector<int3> *T[3] = {&simpleNeighborsTasks, &attachedNeighborsTasks, &notNeighborsTasks};
        const deviceVector<Point3> *R[3] = {&d_simpleNeighborsResults, &d_attachedNeighborsResults, &d_notNeighborsResults};
        const deviceVector<double> *E[3] = {&simpleNeighborsErrors, &attachedNeighborsErrors, &notNeighborsErrors};
        for (int k = 0; k < 3; ++k) {
            const int n = T[k]->size;
            std::vector<int3> t(n);
            std::vector<Point3> r(n);
            std::vector<double> e(n, -1.0);
            copy_d2h(T[k]->data, t.data(), n);
            copy_d2h(R[k]->data, r.data(), n);
            if (E[k]->size == n) copy_d2h(E[k]->data, e.data(), n);
            for (int i = 0; i < n; ++i) std::fprintf(f, "%d %d %d %.17g %.17g %.17g %.17g\n", k, t[i].x, t[i].y, r[i].x, r[i].y, r[i].z, e[i]);
        }
        std::fclose(f);
    }
};

int main(int argc, char **argv)
{
    if (argc < 4) {
        std::printf("usage: consumer <mesh.dat> <level | -1> <out.txt>\n");
        return 2;
    }
    const int level = std::atoi(argv[2]);
    Mesh3D mesh;
    if (!mesh.loadMeshFromFile(argv[1], 1.0)) return 1;
    mesh.prepareMesh();
    std::printf("pairs %d %d %d\n", mesh.getSimpleNeighbors().size, mesh.getAttachedNeighbors().size, mesh.getNotNeighbors().size);

    NumericalIntegrator3D numIntegrator(mesh, qf3D13);
    if (level >= 0) numIntegrator.setFixedRefinementLevel(level);
    Harness evaluator(mesh, numIntegrator);
    evaluator.runAllPairs(true);
    evaluator.outputResultsToFile(neighbour_type_enum::attached_neighbors, output_format_enum::csv);
    evaluator.dump(argv[3]);

    // the reference's exports: the refined mesh of a fixed-level run, the per-cell refinement
    // counts of an adaptive one
    std::vector<Point3> vertices(numIntegrator.getRefinedVertices().size);
    copy_d2h(numIntegrator.getRefinedVertices().data, vertices.data(), vertices.size());
    std::vector<int3> cells(numIntegrator.getRefinedCells().size);
    copy_d2h(numIntegrator.getRefinedCells().data, cells.data(), cells.size());
    exportMeshToObj("RefinedMesh.obj", vertices, cells);
    std::array<std::vector<unsigned char>, 3> refinements;
    if (level < 0)
        for (int k = 0; k < 3; ++k) {
            const auto *r = numIntegrator.getRefinementsRequired(neighbour_type_enum(k));
            refinements[k].resize(r->size);
            if (r->size) copy_d2h(r->data, refinements[k].data(), r->size);
        }
    exportMeshToVtk("RefinedMesh.vtp", vertices, cells, refinements);
    std::printf("refined %zu %zu\n", vertices.size(), cells.size());
    return 0;
}
