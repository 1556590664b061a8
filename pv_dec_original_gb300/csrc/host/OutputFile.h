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
#pragma once
#include <string>

class Simulation;

class OutputFile {
public:
    OutputFile() = default;
    explicit OutputFile(int outputIdx) : m_outputIdx(outputIdx) {}
    std::string root = ".";
    bool WriteVTK_Collective(Simulation& sim);
    bool WriteSurfaceAttribute(Simulation& sim, int iter);

private:
    int m_outputIdx = 0;
};
