// Output writers with the reference's names (OutputFile.h:61-84).
//   WriteVTK_Collective:   Fluid_Variables/<idx>.vtu -- every active node as a
//     point at its lattice index (x, y, z) with Velocity, Density and
//     VelocityMagnitude, and a hexahedron for every lattice cube whose eight
//     corners are active (OutputFile.cpp:259-429).  VTK is not linked: the
//     XML UnstructuredGrid file is written directly.  The values are the
//     moments of the post-boundary distributions.
//   WriteSurfaceAttribute: FlowHemodynamics/<iter>_FlowHemodynamics.csv with
//     "X,Y,Z,WSS,OSI,TAWSS" per next-to-wall node (OutputFile.cpp:867-938),
//     rows in increasing lattice index.
//   InterpolateAttributesToSTLVertices / WriteSTLVertexAttribute: the
//     reference's commented-out surface read-out (OutputFile.cpp:431-488):
//     every STL triangle vertex takes WSS, OSI and TAWSS from its nearest
//     next-to-wall node (lbm_nearest_next_to_wall); written as
//     STL_Vertices/<iter>_Vertices.csv, "X,Y,Z,WSS,OSI,TAWSS", three rows per
//     triangle in file order.
#pragma once
#include <string>
#include <vector>

#include "Struct.h"

class Simulation;

// WSS, OSI, TAWSS at the three vertices of a triangle.
struct VertexAttributes {
    double wss[3], osi[3], tawss[3];
};

class OutputFile {
public:
    OutputFile() = default;
    explicit OutputFile(int outputIdx) : m_outputIdx(outputIdx) {}
    std::string root = ".";
    bool WriteVTK_Collective(Simulation& sim);
    bool WriteSurfaceAttribute(Simulation& sim, int iter);
    static std::vector<VertexAttributes> InterpolateAttributesToSTLVertices(Simulation& sim,
                                                                            const std::vector<Triangle>& tris);
    bool WriteSTLVertexAttribute(Simulation& sim, const std::vector<Triangle>& tris, int iter);

private:
    int m_outputIdx = 0;
};
