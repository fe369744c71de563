// integrator2test3D -- command-line driver with the options of the reference's test program
// (tests/integrator3D/main.cu: -f/--meshfile, -s/--scale, -r/--refine, -c/--checkresults,
// --exporttoobj, --exporttovtk, --exporttocsv, --exportresults), written over the C++ layer of
// this library (include/integrator2_gb300.hpp).  Additions: --near=<factor> (disjoint pairs with
// centroid distance < factor x mean edge length only; default: every disjoint pair, as the
// reference), --relative=<tol> (scale-invariant error control), --mixed (mixed precision),
// --fullprecision (CSV with 17 significant digits).
//
// Output files have the reference's names: SimpleNeighbors / AttachedNeighbors / NotNeighbors
// .dat (plain text) or .csv, OriginalMesh.obj / RefinedMesh.obj, OriginalMesh.vtp / RefinedMesh.vtp.
// The VTK export of an adaptive run carries, per cell and per pair class, the refinement level
// the cell's pairs (the cell as K_i) needed: the largest kept level over those pairs.
#include "integrator2_gb300.hpp"

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <string>
#include <utility>
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

void write_obj(const std::string &name, const std::vector<double> &V, const std::vector<Int3> &C)
{
    std::ofstream f(name);
    for (size_t k = 0; k < V.size() / 3; ++k) f << "v " << V[3 * k] << " " << V[3 * k + 1] << " " << V[3 * k + 2] << "\n";
    for (const Int3 &c : C) f << "f " << c.x + 1 << " " << c.y + 1 << " " << c.z + 1 << "\n";
    std::printf("Mesh saved to %s\n", name.c_str());
}

void write_vtp(const std::string &name, const std::vector<double> &V, const std::vector<Int3> &C,
               const std::vector<std::vector<int>> &refinements)
{
    std::ofstream f(name);
    f << "<?xml version=\"1.0\" ?>\n<VTKFile type=\"PolyData\" version=\"0.1\" byte_order=\"LittleEndian\">\n  <PolyData>\n";
    f << "    <Piece NumberOfPoints=\"" << V.size() / 3 << "\" NumberOfPolys=\"" << C.size() << "\">\n";
    f << "      <Points>\n        <DataArray type=\"Float32\" NumberOfComponents=\"3\" Format=\"ascii\">\n        ";
    for (double x : V) f << x << " ";
    f << "\n        </DataArray>\n      </Points>\n      <Polys>\n";
    f << "        <DataArray type=\"Int32\" Name=\"connectivity\" Format=\"ascii\">\n          ";
    for (const Int3 &c : C) f << c.x << " " << c.y << " " << c.z << " ";
    f << "\n        </DataArray>\n        <DataArray type=\"Int32\" Name=\"offsets\" Format=\"ascii\">\n          ";
    for (size_t k = 0; k < C.size(); ++k) f << 3 * (k + 1) << " ";
    f << "\n        </DataArray>\n      </Polys>\n";
    bool any = false;
    for (const auto &r : refinements) any = any || !r.empty();
    if (any) {
        f << "      <CellData>\n";
        const neighbour_type_enum types[3] = {neighbour_type_enum::simple_neighbors, neighbour_type_enum::attached_neighbors,
                                              neighbour_type_enum::not_neighbors};
        for (int k = 0; k < 3; ++k) {
            if (refinements[k].empty()) continue;
            f << "        <DataArray type=\"Int32\" Name=\"" << neighborTypeString(types[k]) << "Refinements\" Format=\"ascii\">\n          ";
            for (int v : refinements[k]) f << v << " ";
            f << "\n        </DataArray>\n";
        }
        f << "      </CellData>\n";
    }
    f << "    </Piece>\n  </PolyData>\n</VTKFile>\n";
    std::printf("Mesh saved to %s\n", name.c_str());
}

// every cell split `level` times by midpoints in the reference's child order; vertices at edge
// midpoints are shared between the cells on both sides
void refine(std::vector<double> &V, std::vector<Int3> &C, int level)
{
    for (int l = 0; l < level; ++l) {
        std::map<std::pair<int, int>, int> mid;
        auto midpoint = [&](int a, int b) {
            const std::pair<int, int> key(std::min(a, b), std::max(a, b));
            auto it = mid.find(key);
            if (it != mid.end()) return it->second;
            const int id = (int)(V.size() / 3);
            for (int k = 0; k < 3; ++k) V.push_back(0.5 * (V[3 * a + k] + V[3 * b + k]));
            mid[key] = id;
            return id;
        };
        std::vector<Int3> out;
        out.reserve(4 * C.size());
        for (const Int3 &c : C) {
            const int mab = midpoint(c.x, c.y), mbc = midpoint(c.y, c.z), mca = midpoint(c.z, c.x);
            out.push_back({mab, c.y, mbc});
            out.push_back({mbc, c.z, mca});
            out.push_back({mca, c.x, mab});
            out.push_back({mbc, mca, mab});
        }
        C.swap(out);
    }
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
        if (!mesh.loadMeshFromFile(meshfile, scale)) {
            std::fprintf(stderr, "%s\n", i2_last_error());
            return EXIT_FAILURE;
        }
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
        const std::vector<double> V = mesh.getVertices();
        const std::vector<Int3> C = mesh.getCells();
        if (obj) write_obj("OriginalMesh.obj", V, C);
        if (vtk && refineLevel >= 0) write_vtp("OriginalMesh.vtp", V, C, {{}, {}, {}});

        EvaluatorJ3DK evaluator(mesh, integrator);
        const auto t0 = std::chrono::steady_clock::now();
        evaluator.runAllPairs(check);
        const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        const neighbour_type_enum types[3] = {neighbour_type_enum::simple_neighbors, neighbour_type_enum::attached_neighbors,
                                              neighbour_type_enum::not_neighbors};
        const size_t counts[3] = {mesh.getSimpleNeighbors().size(), mesh.getAttachedNeighbors().size(), mesh.getNotNeighbors().size()};
        std::printf("Integration of %zu ordered pairs (simple %zu, attached %zu, not neighbours %zu): %.3f ms\n",
                    2 * (counts[0] + counts[1] + counts[2]), 2 * counts[0], 2 * counts[1], 2 * counts[2], ms);
        if (check) {
            for (int k = 0; k < 3; ++k) {
                if (!counts[k]) continue;
                const std::vector<double> e = evaluator.getErrors(types[k]);
                double mx = 0.0;
                for (double x : e) mx = x > mx ? x : mx;
                std::printf("%s: largest (i,j)/(j,i) difference %.3e\n", neighborTypeString(types[k]).c_str(), mx);
            }
        }
        if (plain || csv) {
            const output_format_enum fmt = plain && !csv ? output_format_enum::plainText
                                                         : (full ? output_format_enum::csvFullPrecision : output_format_enum::csv);
            for (int k = 0; k < 3; ++k)
                if (counts[k]) evaluator.outputResultsToFile(types[k], fmt);
        }
        if ((obj || vtk) && refineLevel > 0) {
            std::vector<double> Vr = V;
            std::vector<Int3> Cr = C;
            refine(Vr, Cr, refineLevel);
            if (obj) write_obj("RefinedMesh.obj", Vr, Cr);
            if (vtk) write_vtp("RefinedMesh.vtp", Vr, Cr, {{}, {}, {}});
        }
        if (vtk && refineLevel < 0) {
            std::vector<std::vector<int>> ref(3);
            const std::vector<std::vector<Int3>> lists = {mesh.getSimpleNeighbors(), mesh.getAttachedNeighbors(), mesh.getNotNeighbors()};
            for (int k = 0; k < 3; ++k) {
                if (lists[k].empty()) continue;
                ref[k].assign(C.size(), 0);
                const std::vector<double> lev = evaluator.getLevels(types[k]);
                const size_t n = lists[k].size();
                for (size_t p = 0; p < lev.size(); ++p) {
                    const Int3 &pr = lists[k][p % n];
                    const int i = p < n ? pr.x : pr.y;  // rows n..2n-1 are the reversed pairs
                    ref[k][i] = std::max(ref[k][i], (int)lev[p]);
                }
            }
            write_vtp("OriginalMesh.vtp", V, C, ref);
        }
    } catch (const i2::Error &e) {
        std::fprintf(stderr, "%s\n", e.what());
        return EXIT_FAILURE;
    }
    return EXIT_SUCCESS;
}
