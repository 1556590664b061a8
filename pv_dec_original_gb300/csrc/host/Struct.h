// Plain data types of the host layer, named after the reference's Struct.h
// (Struct.h:117-134) so that code written against the reference's headers
// reads the same.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

struct Triangle {
    double x1, y1, z1;
    double x2, y2, z2;
    double x3, y3, z3;
    double nx, ny, nz;  // the STL file's own facet normal (used by the ray test)
};

struct BoundingBox {
    double min_x, max_x, min_y, max_y, min_z, max_z;
};

struct Point {
    double x, y, z;
};

// Node classes of the lattice (the reference's NodeType / BoundaryType pair,
// Struct.h:15-29, collapsed into one byte per point).
enum class NodeClass : uint8_t { Solid = 0, Fluid = 1, Wall = 2, Boundary0 = 3 };

// Flattens triangles into the C ABI's 12-doubles-per-facet rows.
inline std::vector<double> triangles_to_rows(const std::vector<Triangle>& t) {
    std::vector<double> r;
    r.reserve(t.size() * 12);
    for (const Triangle& a : t) {
        const double v[12] = {a.x1, a.y1, a.z1, a.x2, a.y2, a.z2, a.x3, a.y3, a.z3, a.nx, a.ny, a.nz};
        r.insert(r.end(), v, v + 12);
    }
    return r;
}
