// A consumer written in the reference's call pattern (tests/integrator3D/main.cu of the
// reference), compiled against include/integrator2_gb300.hpp and linked with libi2gb300.so.
// Mode "host": mesh loading, preparation and pair lists only (no GPU needed).
// Mode "run": also integrates (needs a GPU) and prints the number of results per class.
#include "integrator2_gb300.hpp"

#include <cstdio>
#include <cstring>

int main(int argc, char **argv)
{
    if (argc < 3) {
        std::printf("usage: consumer <mesh.dat> host|run [scale]\n");
        return 2;
    }
    const double scale = argc > 3 ? std::atof(argv[3]) : 1.0;
    Mesh3D mesh;
    if (!mesh.loadMeshFromFile(argv[1], scale)) {
        std::printf("cannot load %s\n", argv[1]);
        return 1;
    }
    mesh.prepareMesh();
    std::printf("pairs %zu %zu %zu %zu\n", mesh.getSimpleNeighbors().size(), mesh.getAttachedNeighbors().size(),
                mesh.getNotNeighbors().size(), mesh.getSelfPairs().size());
    NumericalIntegrator3D numIntegrator(mesh, qf3D13);
    numIntegrator.setFixedRefinementLevel(0);
    if (std::strcmp(argv[2], "run") == 0) {
        EvaluatorJ3DK evaluator(mesh, numIntegrator);
        evaluator.runAllPairs(true);
        std::printf("results %zu %zu %zu\n", evaluator.getResults(neighbour_type_enum::simple_neighbors).size() / 3,
                    evaluator.getResults(neighbour_type_enum::attached_neighbors).size() / 3,
                    evaluator.getResults(neighbour_type_enum::not_neighbors).size() / 3);
        evaluator.outputResultsToFile(neighbour_type_enum::attached_neighbors, output_format_enum::csv);
    }
    return 0;
}
