// integrator2test3D -- command-line driver with the options of the reference's test program
// (tests/integrator3D/main.cu: -f/--meshfile, -s/--scale, -r/--refine, -c/--checkresults,
// --exporttoobj, --exporttovtk, --exporttocsv, --exportresults), written over the C++ drop-in
// headers of this library (include/integrator2/).  Additions: --near=<factor> (disjoint pairs with
// centroid distance < factor x mean edge length only; default: every disjoint pair, as the
// reference), --relative=<tol> (scale-invariant error control), --mixed (mixed precision),
// --fullprecision (CSV with 17 significant digits).
//
// Output files have the reference's names: SimpleNeighbors / AttachedNeighbors / NotNeighbors
// .dat (plain text) or .csv, OriginalMesh.obj / RefinedMesh.obj, OriginalMesh.vtp / RefinedMesh.vtp.
// The VTK export of an adaptive run carries, per cell and per pair class, the refinement level
// the cell's pairs (the cell as K_i) needed: the largest kept level over those pairs.  The
// refined mesh of a fixed-level run is the reference's (every cell split at its own edge
// midpoints, NumericalIntegrator3D::getRefinedVertices / getRefinedCells).
#include "integrator2/Mesh3d.cuh"
#include "integrator2/NumericalIntegrator3d.cuh"
#include "integrator2/evaluators/evaluatorJ3DK.cuh"

#include <array>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {

void usage()
{
    std::printf("USAGE: integrator2test3D [options]\n\n"
                "Options:\n"
                "  -h, --help             Print usage and exit.\n"
                "  -f <arg>, --meshfile=<arg>  Input mesh file name.\n"
                "  -s <arg>, --scale=<arg>     Mesh scale factor.\n"
                "  --exporttoobj          Export original and refined meshes to OBJ files.\n"
                "  --exporttovtk          Export original and refined meshes to VTK (VTP) files.\n"
                "  --exporttocsv          Export results of integration to csv files.\n"
                "  --exportresults        Export results of integration to text files.\n"
                "  -r <arg>, --refine=<arg>    Refine the whole mesh N times.\n"
                "  -c, --checkresults     Check correctness of pairs of results.\n"
                "  --near=<arg>           Disjoint pairs closer than <arg> x mean edge length only.\n"
                "  --relative=<arg>       Relative (scale-invariant) error control with tolerance <arg>.\n"
                "  --mixed                Mixed precision (FP32 bulk, FP64 singular parts).\n"
                "  --fullprecision        Full precision CSV output.\n");
}

bool numeric(const char *s)
{
    char *end = nullptr;
    std::strtod(s, &end);
    return end != s && *end == 0;
}

// the evaluator with the largest (i,j)/(j,i) difference per class after runAllPairs(true)
class Evaluator : public EvaluatorJ3DK {
public:
    Evaluator(const Mesh3D &m, NumericalIntegrator3D &it) : EvaluatorJ3DK(m, it) {}
    double largestError(neighbour_type_enum t) const
    {
        const deviceVector<double> &e = t == neighbour_type_enum::simple_neighbors ? simpleNeighborsErrors
                                      : t == neighbour_type_enum::attached_neighbors ? attachedNeighborsErrors : notNeighborsErrors;
        std::vector<double> h(e.size);
        if (e.size) copy_d2h(e.data, h.data(), h.size());
        double mx = 0.0;
        for (double x : h) mx = x > mx ? x : mx;
        return mx;
    }
};

template <class T> std::vector<T> host_copy(const deviceVector<T> &d)
{
    std::vector<T> h(d.size);
    if (d.size) copy_d2h(d.data, h.data(), h.size());
    return h;
}

} // namespace

int main(int argc, char **argv)
{
    std::string meshfile;
    double scale = 1.0, near = 0.0, rel = 0.0;
    int refineLevel = -1;
    bool check = false, obj = false, vtk = false, csv = false, plain = false, mixed = false, full = false;
    if (argc <= 1) {
        usage();
        return EXIT_SUCCESS;
    }
    for (int k = 1; k < argc; ++k) {
        std::string a = argv[k], val;
        const size_t eq = a.find('=');
        if (a.rfind("--", 0) == 0 && eq != std::string::npos) {
            val = a.substr(eq + 1);
            a = a.substr(0, eq);
        }
        auto need = [&](const char *what) -> std::string {
            if (!val.empty()) return val;
            if (k + 1 < argc) return argv[++k];
            std::fprintf(stderr, "Option '%s' requires an argument\n", what);
            std::exit(EXIT_FAILURE);
        };
        if (a == "-h" || a == "--help") {
            usage();
            return EXIT_SUCCESS;
        } else if (a == "-f" || a == "--meshfile") meshfile = need(a.c_str());
        else if (a == "-s" || a == "--scale" || a == "-r" || a == "--refine" || a == "--near" || a == "--relative") {
            const std::string v = need(a.c_str());
            if (!numeric(v.c_str())) {
                std::fprintf(stderr, "Option '%s' requires a numeric argument\n", a.c_str());
                return EXIT_FAILURE;
            }
            if (a == "-s" || a == "--scale") scale = std::stod(v);
            else if (a == "-r" || a == "--refine") refineLevel = std::stoi(v);
            else if (a == "--near") near = std::stod(v);
            else rel = std::stod(v);
        } else if (a == "-c" || a == "--checkresults") check = true;
        else if (a == "--exporttoobj") obj = true;
        else if (a == "--exporttovtk") vtk = true;
        else if (a == "--exporttocsv") csv = true;
        else if (a == "--exportresults") plain = true;
        else if (a == "--mixed") mixed = true;
        else if (a == "--fullprecision") full = true;
        else {
            std::fprintf(stderr, "Unknown option '%s'\n", a.c_str());
            return EXIT_FAILURE;
        }
    }
    if (meshfile.empty()) {
        std::printf("No input file with mesh specified. Exiting\n");
        return EXIT_FAILURE;
    }
    try {
        Mesh3D mesh;
        if (!mesh.loadMeshFromFile(meshfile, scale)) return EXIT_FAILURE;
        mesh.prepareMesh(near);
        NumericalIntegrator3D integrator(mesh, qf3D13);
        if (refineLevel >= 0) {
            integrator.setFixedRefinementLevel(refineLevel);
            if (refineLevel) std::printf("Using fixed refinement level equal to %d\n", refineLevel);
            else std::printf("Using original mesh without refinement\n");
        } else if (rel > 0.0) {
            integrator.setErrorControl(error_control_type_enum::relative_error_control, rel, 5);
            std::printf("Using relative error control with tolerance %g\n", rel);
        } else {
            std::printf("Using adaptive error control procedure\n");
        }
        if (mixed) integrator.setPrecision(I2_PRECISION_MIXED);
        const std::vector<Point3> V = host_copy(mesh.getVertices());
        const std::vector<int3> C = host_copy(mesh.getCells());
        const std::array<std::vector<unsigned char>, 3> none;
        if (obj) exportMeshToObj("OriginalMesh.obj", V, C);
        if (vtk && refineLevel >= 0) exportMeshToVtk("OriginalMesh.vtp", V, C, none);

        Evaluator evaluator(mesh, integrator);
        const auto t0 = std::chrono::steady_clock::now();
        evaluator.runAllPairs(check);
        const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        const neighbour_type_enum types[3] = {neighbour_type_enum::simple_neighbors, neighbour_type_enum::attached_neighbors,
                                              neighbour_type_enum::not_neighbors};
        const size_t counts[3] = {(size_t)mesh.getSimpleNeighbors().size, (size_t)mesh.getAttachedNeighbors().size,
                                  (size_t)mesh.getNotNeighbors().size};
        std::printf("Integration of %zu ordered pairs (simple %zu, attached %zu, not neighbours %zu): %.3f ms\n",
                    2 * (counts[0] + counts[1] + counts[2]), 2 * counts[0], 2 * counts[1], 2 * counts[2], ms);
        if (check)
            for (int k = 0; k < 3; ++k)
                if (counts[k])
                    std::printf("%s: largest (i,j)/(j,i) difference %.3e\n", neighborTypeString(types[k]).c_str(), evaluator.largestError(types[k]));
        if (plain || csv) {
            const output_format_enum fmt = plain && !csv ? output_format_enum::plainText
                                                         : (full ? output_format_enum::csvFullPrecision : output_format_enum::csv);
            for (int k = 0; k < 3; ++k)
                if (counts[k]) evaluator.outputResultsToFile(types[k], fmt);
        }
        if ((obj || vtk) && refineLevel > 0) {
            const std::vector<Point3> Vr = host_copy(integrator.getRefinedVertices());
            const std::vector<int3> Cr = host_copy(integrator.getRefinedCells());
            if (obj) exportMeshToObj("RefinedMesh.obj", Vr, Cr);
            if (vtk) exportMeshToVtk("RefinedMesh.vtp", Vr, Cr, none);
        }
        if (vtk && refineLevel < 0) {
            std::array<std::vector<unsigned char>, 3> ref;
            for (int k = 0; k < 3; ++k)
                if (counts[k]) ref[k] = host_copy(*integrator.getRefinementsRequired(types[k]));
            exportMeshToVtk("OriginalMesh.vtp", V, C, ref);
        }
    } catch (const i2dropin::Error &e) {
        std::fprintf(stderr, "%s\n", e.what());
        return EXIT_FAILURE;
    }
    return EXIT_SUCCESS;
}
