// Mesh3d.cuh -- Mesh3D with the reference's interface (andreyypopov/integrator2, src/Mesh3d.cuh:
// loadMeshFromFile, prepareMesh, getters returning deviceVector<T> references, the OBJ / VTK
// export functions and neighborTypeString), implemented over the library's C-ABI
// (integrator2_gb300.h).  The mesh is loaded and its pair lists are built by the library (an O(N)
// builder in place of the reference's O(N^2) one); the getters hand out device copies in the
// reference's layout: vertices Point3, cells int3, normals Point3, measures double, and the three
// neighbour lists as int3 (i, j, position) rows with i < j.
// Additions: prepareMesh(near_factor) keeps only the disjoint pairs closer than near_factor x the
// mean edge length; setGeometry; getSelfPairs and getCellCenters; handle() for the C-ABI.
#ifndef I2_DROPIN_MESH3D_CUH
#define I2_DROPIN_MESH3D_CUH

#include "../integrator2_gb300.h"
#include "common/cuda_math.cuh"
#include "common/device_vector.cuh"

#include <array>
#include <cstdio>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

// src/Mesh3d.cuh:18-23; self (pairs (i, i)) is the library's fourth class
enum class neighbour_type_enum { simple_neighbors = 0, attached_neighbors = 1, not_neighbors = 2, undefined = -1, self = 3 };

namespace i2dropin {

struct Error : std::runtime_error {
    i2_status code;
    Error(i2_status c, const std::string &where) : std::runtime_error(where + ": " + i2_status_string(c) + ": " + i2_last_error()), code(c) {}
};
// library failures throw i2dropin::Error (the reference ends the program on CUDA failures)
inline void check(i2_status s, const char *where)
{
    if (s != I2_OK) throw Error(s, where);
}

template <class T> void upload(deviceVector<T> &dv, const std::vector<T> &host)
{
    dv.allocate((int)host.size());
    copy_h2d(host.data(), dv.data, host.size());
}

} // namespace i2dropin

class Mesh3D {
public:
    Mesh3D() { i2dropin::check(i2_mesh_create(&h_), "i2_mesh_create"); }
    virtual ~Mesh3D() { i2_mesh_destroy(h_); }
    Mesh3D(const Mesh3D &) = delete;
    Mesh3D &operator=(const Mesh3D &) = delete;

    // src/Mesh3d.cuh:55: the reference's .dat format, coordinates multiplied by scale
    bool loadMeshFromFile(const std::string &filename, double scale = 1.0)
    {
        if (i2_mesh_load_file(h_, filename.c_str(), scale) != I2_OK) {
            std::printf("Error loading mesh from %s: %s\n", filename.c_str(), i2_last_error());
            return false;
        }
        upload_geometry();
        std::printf("Loaded mesh with %d vertices and %d cells\n", vertices.size, cells.size);
        return true;
    }
    // src/Mesh3d.cuh:63: cell normals, measures and the three neighbour lists (every disjoint pair)
    void prepareMesh() { prepare(0.0); }
    void prepareMesh(double near_factor) { prepare(near_factor); }
    void setGeometry(const std::vector<Point3> &v, const std::vector<int3> &c)
    {
        i2dropin::check(i2_mesh_set_geometry(h_, &v[0].x, (int32_t)v.size(), &c[0].x, (int32_t)c.size()), "i2_mesh_set_geometry");
        upload_geometry();
    }

    // src/Mesh3d.cuh:70-126
    const auto &getSimpleNeighbors() const { return simpleNeighbors; }
    const auto &getAttachedNeighbors() const { return attachedNeighbors; }
    const auto &getNotNeighbors() const { return notNeighbors; }
    const auto &getVertices() const { return vertices; }
    const auto &getCells() const { return cells; }
    const auto &getCellNormals() const { return cellNormals; }
    const auto &getCellMeasures() const { return cellMeasures; }
    const auto &getCellCenters() const { return cellCenters; }
    const auto &getSelfPairs() const { return selfPairs; }
    i2_mesh_t *handle() const { return h_; }

private:
    void upload_geometry()
    {
        int32_t nv = 0, nc = 0;
        i2dropin::check(i2_mesh_sizes(h_, &nv, &nc), "i2_mesh_sizes");
        std::vector<Point3> v(nv);
        std::vector<int3> c(nc);
        i2dropin::check(i2_mesh_copy_geometry(h_, nv ? &v[0].x : nullptr, nc ? &c[0].x : nullptr), "i2_mesh_copy_geometry");
        i2dropin::upload(vertices, v);
        i2dropin::upload(cells, c);
    }
    void prepare(double near_factor)
    {
        i2dropin::check(i2_mesh_prepare(h_, near_factor), "i2_mesh_prepare");
        const int nc = cells.size;
        std::vector<Point3> n(nc), ctr(nc);
        std::vector<double> s(nc);
        if (nc) i2dropin::check(i2_mesh_copy_cell_data(h_, &n[0].x, s.data(), &ctr[0].x), "i2_mesh_copy_cell_data");
        i2dropin::upload(cellNormals, n);
        i2dropin::upload(cellMeasures, s);
        i2dropin::upload(cellCenters, ctr);
        list(I2_SIMPLE_NEIGHBORS, simpleNeighbors);
        list(I2_ATTACHED_NEIGHBORS, attachedNeighbors);
        list(I2_NOT_NEIGHBORS, notNeighbors);
        list(I2_SELF, selfPairs);
    }
    void list(i2_pair_class cls, deviceVector<int3> &out)
    {
        int64_t n = 0;
        i2dropin::check(i2_mesh_pair_count(h_, cls, &n), "i2_mesh_pair_count");
        std::vector<int3> rows((size_t)n);
        if (n) i2dropin::check(i2_mesh_copy_pairs(h_, cls, &rows[0].x, n), "i2_mesh_copy_pairs");
        i2dropin::upload(out, rows);
    }

    i2_mesh_t *h_ = nullptr;
    deviceVector<Point3> vertices;
    deviceVector<int3> cells;
    deviceVector<Point3> cellNormals;
    deviceVector<Point3> cellCenters;
    deviceVector<double> cellMeasures;
    deviceVector<int3> simpleNeighbors;
    deviceVector<int3> attachedNeighbors;
    deviceVector<int3> notNeighbors;
    deviceVector<int3> selfPairs;
};

// src/Mesh3d.cuh:188-209
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

// Wavefront OBJ: "v x y z" lines, then "f a b c" with 1-based vertex indices
inline void exportMeshToObj(const std::string &filename, const std::vector<Point3> &vertices, const std::vector<int3> &cells)
{
    std::ofstream f(filename.c_str());
    for (const Point3 &p : vertices) f << "v " << p.x << " " << p.y << " " << p.z << "\n";
    for (const int3 &c : cells) f << "f " << c.x + 1 << " " << c.y + 1 << " " << c.z + 1 << "\n";
    std::printf("Mesh saved to %s\n", filename.c_str());
}

// VTK XML PolyData (ASCII) with, when given, an Int32 cell array "<Class>Refinements" per class
inline void exportMeshToVtk(const std::string &filename, const std::vector<Point3> &vertices, const std::vector<int3> &cells,
                            const std::array<std::vector<unsigned char>, 3> &refinementsRequired)
{
    std::ofstream f(filename.c_str());
    f << "<?xml version=\"1.0\" ?> \n<VTKFile type=\"PolyData\" version=\"0.1\" byte_order=\"LittleEndian\">\n  <PolyData>\n";
    f << "    <Piece NumberOfPoints=\"" << vertices.size() << "\" NumberOfPolys=\"" << cells.size() << "\">\n";
    f << "      <Points>\n        <DataArray type=\"Float32\" NumberOfComponents=\"3\" Format=\"ascii\">\n        ";
    for (const Point3 &p : vertices) f << p.x << " " << p.y << " " << p.z << " ";
    f << "\n        </DataArray>\n      </Points>\n      <Polys>\n";
    f << "        <DataArray type=\"Int32\" Name=\"connectivity\" Format=\"ascii\">\n          ";
    for (const int3 &c : cells) f << c.x << " " << c.y << " " << c.z << " ";
    f << "\n        </DataArray>\n        <DataArray type=\"Int32\" Name=\"offsets\" Format=\"ascii\">\n          ";
    for (size_t k = 0; k < cells.size(); ++k) f << 3 * (k + 1) << " ";
    f << "\n        </DataArray>\n      </Polys>\n";
    if (!refinementsRequired[0].empty() || !refinementsRequired[1].empty() || !refinementsRequired[2].empty()) {
        f << "      <CellData>\n";
        for (int k = 0; k < 3; ++k) {
            if (refinementsRequired[k].empty()) continue;
            f << "        <DataArray type=\"Int32\" Name=\"" << neighborTypeString(neighbour_type_enum(k)) << "Refinements\" Format=\"ascii\">\n          ";
            for (size_t i = 0; i < cells.size(); ++i) f << (int)refinementsRequired[k][i] << " ";
            f << "\n        </DataArray>\n";
        }
        f << "      </CellData>\n";
    }
    f << "    </Piece>\n  </PolyData>\n</VTKFile>\n";
    std::printf("Mesh saved to %s\n", filename.c_str());
}

#endif
