// Geometry: STL -> lattice with the reference's constructor
// Geometry(FileName, velSet, spacing, raydirection) (ComplexGeometry.h:91).
//
// The reference's constructor runs the whole pipeline: bounding box and
// lattice size (ComplexGeometry.cpp:133-214), point generation (:318-351),
// +z ray-parity labelling (:978-1053), boundary points (:1259-1300) and the
// PV.stl-specific inlet/outlet classification (:1369-1429).  Here the
// bounding box is computed on the host and labelling runs on the GPU
// (lbm_voxelize, bit-identical mask); boundary points and their
// classification are built on the device when the lattice is handed to a
// Simulation, from the rules collected in `boundaryRules`.
// UsePVPreset() installs the reference's own PV.stl coordinates.
// The reference always casts rays along +z whatever `raydirection` says
// (labelPoints sets directionSwitch = 0); so does this class.
#pragma once
#include <memory>
#include <string>
#include <vector>

#include "GeometryReader.h"
#include "LatticeModel.h"
#include "Struct.h"
#include "lbm_gb300.h"

class Geometry {
public:
    Reader Reader_;
    std::vector<Triangle> globalTriangles;
    std::string stlFileName;
    BoundingBox boundingbox{};
    double spacing = 1.0;
    char raydirection = 'z';
    int nx = 0, ny = 0, nz = 0;
    double origin[3] = {0, 0, 0};
    std::vector<uint8_t> mask;  // [(k*ny + j)*nx + i], 1 = Fluid
    int64_t fluidCount = 0;
    int64_t rayTests = 0;
    std::vector<lbm_bc_spec> boundaryRules;
    std::shared_ptr<VelocitySet> m_velSet;

    Geometry() = default;
    Geometry(const std::string& FileName, std::shared_ptr<VelocitySet> velSet, double spacing, char raydirection);
    // Lattice of a given size and origin; `rayBox` is the box the ray
    // adjustment compares against (the reference uses the STL's bbox).
    Geometry(const std::vector<Triangle>& tris, std::shared_ptr<VelocitySet> velSet, double spacing,
             const BoundingBox& rayBox, const double origin[3], const int dims[3]);

    void GetSubBoundingBox();
    void labelPoints();
    // Fluid points with a lattice neighbour that is NotFluid or outside the box.
    std::vector<Point> findBoundaryPoints() const;

    // Boundary rules (first match wins; unmatched boundary points are walls).
    void AddBoundaryRule(const lbm_bc_spec& rule) { boundaryRules.push_back(rule); }
    void AddInlet(int face, int plane, double scale = 1.0);
    void AddParabolicInlet(int face, int plane, double c1, double c2, double R, double scale = 1.0);
    void AddPressureOutlet(int face, int plane, double density = 1.0);
    // The reference's classifyBoundaryPoints coordinates for PV.stl.
    void UsePVPreset();
    void classifyBoundaryPoints() {}

    bool IsFluid(int i, int j, int k) const {
        return i >= 0 && j >= 0 && k >= 0 && i < nx && j < ny && k < nz &&
               mask[((size_t)k * ny + j) * nx + i] != 0;
    }
    Point PointAt(int i, int j, int k) const {
        return Point{origin[0] + i * spacing, origin[1] + j * spacing, origin[2] + k * spacing};
    }

private:
    BoundingBox rayBox_{};
    bool referenceBox_ = true;
};
