#include "OutputFile.h"

#include <sys/stat.h>

#include <cmath>
#include <fstream>
#include <iostream>
#include <limits>
#include <stdexcept>
#include <vector>

#include "Simulation.h"

namespace {

std::string join(const std::string& a, const std::string& b) { return a.empty() || a == "." ? b : a + "/" + b; }

}  // namespace

bool OutputFile::WriteVTK_Collective(Simulation& sim) {
    const std::string folder = join(root, "Fluid_Variables");
    mkdir(folder.c_str(), 0777);
    const std::string name = folder + "/" + std::to_string(m_outputIdx) + ".vtu";
    const Geometry& g = sim.SubDomain_.Geometry_;
    std::vector<uint8_t> cls = sim.Classes();
    std::vector<double> rho, u;
    sim.Macro(rho, u);
    const int64_t nx = g.nx, ny = g.ny, nz = g.nz;
    std::vector<int64_t> pid(cls.size(), -1);
    int64_t np = 0;
    for (size_t n = 0; n < cls.size(); ++n)
        if (cls[n]) pid[n] = np++;
    std::ofstream out(name);
    if (!out) {
        std::cerr << "Unable to open file " << name << std::endl;
        return false;
    }
    // hexahedra over cubes with all eight corners active (corner order of OutputFile.cpp:384-393)
    std::vector<int64_t> conn;
    for (int64_t z = 0; z + 1 < nz; ++z)
        for (int64_t y = 0; y + 1 < ny; ++y)
            for (int64_t x = 0; x + 1 < nx; ++x) {
                const int64_t c[8][3] = {{x, y, z},         {x + 1, y, z},         {x + 1, y + 1, z},
                                         {x, y + 1, z},     {x, y, z + 1},         {x + 1, y, z + 1},
                                         {x + 1, y + 1, z + 1}, {x, y + 1, z + 1}};
                int64_t ids[8];
                bool ok = true;
                for (int i = 0; i < 8 && ok; ++i) {
                    ids[i] = pid[(c[i][2] * ny + c[i][1]) * nx + c[i][0]];
                    ok = ids[i] >= 0;
                }
                if (ok) conn.insert(conn.end(), ids, ids + 8);
            }
    const int64_t ncell = (int64_t)conn.size() / 8;
    out << "<?xml version=\"1.0\"?>\n<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\">\n"
        << "<UnstructuredGrid>\n<Piece NumberOfPoints=\"" << np << "\" NumberOfCells=\"" << ncell << "\">\n";
    out.precision(17);
    out << "<PointData>\n<DataArray type=\"Float64\" Name=\"Velocity\" NumberOfComponents=\"3\" format=\"ascii\">\n";
    for (int64_t a = 0; a < np; ++a) out << u[3 * a] << ' ' << u[3 * a + 1] << ' ' << u[3 * a + 2] << '\n';
    out << "</DataArray>\n<DataArray type=\"Float64\" Name=\"Density\" format=\"ascii\">\n";
    for (int64_t a = 0; a < np; ++a) out << rho[a] << '\n';
    out << "</DataArray>\n<DataArray type=\"Float64\" Name=\"VelocityMagnitude\" format=\"ascii\">\n";
    for (int64_t a = 0; a < np; ++a)
        out << std::sqrt(u[3 * a] * u[3 * a] + u[3 * a + 1] * u[3 * a + 1] + u[3 * a + 2] * u[3 * a + 2]) << '\n';
    out << "</DataArray>\n</PointData>\n<Points>\n<DataArray type=\"Float64\" NumberOfComponents=\"3\" format=\"ascii\">\n";
    for (size_t n = 0; n < cls.size(); ++n)
        if (cls[n]) out << (int64_t)(n % nx) << ' ' << (int64_t)((n / nx) % ny) << ' ' << (int64_t)(n / (nx * ny)) << '\n';
    out << "</DataArray>\n</Points>\n<Cells>\n<DataArray type=\"Int64\" Name=\"connectivity\" format=\"ascii\">\n";
    for (int64_t c = 0; c < ncell; ++c) {
        for (int i = 0; i < 8; ++i) out << conn[8 * c + i] << (i == 7 ? '\n' : ' ');
    }
    out << "</DataArray>\n<DataArray type=\"Int64\" Name=\"offsets\" format=\"ascii\">\n";
    for (int64_t c = 0; c < ncell; ++c) out << 8 * (c + 1) << '\n';
    out << "</DataArray>\n<DataArray type=\"UInt8\" Name=\"types\" format=\"ascii\">\n";
    for (int64_t c = 0; c < ncell; ++c) out << "12\n";
    out << "</DataArray>\n</Cells>\n</Piece>\n</UnstructuredGrid>\n</VTKFile>\n";
    return (bool)out;
}

bool OutputFile::WriteSurfaceAttribute(Simulation& sim, int iter) {
    const std::string folder = join(root, "FlowHemodynamics");
    mkdir(folder.c_str(), 0777);
    const std::string name = folder + "/" + std::to_string(iter) + "_FlowHemodynamics.csv";
    const Geometry& g = sim.SubDomain_.Geometry_;
    std::vector<int64_t> pt;
    std::vector<double> wss, osi, tawss;
    sim.WallShearStress(pt, wss, osi, tawss);
    std::ofstream outfile(name);
    if (!outfile.is_open()) {
        std::cerr << "Unable to open file " << name << std::endl;
        return false;
    }
    outfile << "X,Y,Z,WSS,OSI,TAWSS\n";
    for (size_t p = 0; p < pt.size(); ++p) {
        const int64_t n = pt[p];
        const Point x = g.PointAt((int)(n % g.nx), (int)((n / g.nx) % g.ny), (int)(n / ((int64_t)g.nx * g.ny)));
        outfile << x.x << "," << x.y << "," << x.z << "," << wss[p] << "," << osi[p] << "," << tawss[p] << "\n";
    }
    return (bool)outfile;
}

std::vector<VertexAttributes> OutputFile::InterpolateAttributesToSTLVertices(Simulation& sim,
                                                                            const std::vector<Triangle>& tris) {
    std::vector<double> xyz(9 * tris.size());
    for (size_t t = 0; t < tris.size(); ++t) {
        const Triangle& T = tris[t];
        const double v[9] = {T.x1, T.y1, T.z1, T.x2, T.y2, T.z2, T.x3, T.y3, T.z3};
        for (int k = 0; k < 9; ++k) xyz[9 * t + k] = v[k];
    }
    std::vector<int64_t> idx(3 * tris.size());
    if (lbm_nearest_next_to_wall(sim.handle(), xyz.data(), (int64_t)idx.size(), 32, idx.data(), nullptr) != LBM_OK)
        throw std::runtime_error(std::string("lbm_nearest_next_to_wall: ") + lbm_last_error(sim.handle()));
    std::vector<int64_t> pt;
    std::vector<double> wss, osi, tawss;
    sim.WallShearStress(pt, wss, osi, tawss);
    const double nan = std::numeric_limits<double>::quiet_NaN();
    std::vector<VertexAttributes> out(tris.size());
    for (size_t t = 0; t < tris.size(); ++t)
        for (int k = 0; k < 3; ++k) {
            const int64_t e = idx[3 * t + k];
            out[t].wss[k] = e >= 0 ? wss[e] : nan;
            out[t].osi[k] = e >= 0 ? osi[e] : nan;
            out[t].tawss[k] = e >= 0 ? tawss[e] : nan;
        }
    return out;
}

bool OutputFile::WriteSTLVertexAttribute(Simulation& sim, const std::vector<Triangle>& tris, int iter) {
    const std::string folder = join(root, "STL_Vertices");
    mkdir(folder.c_str(), 0777);
    const std::string name = folder + "/" + std::to_string(iter) + "_Vertices.csv";
    const std::vector<VertexAttributes> va = InterpolateAttributesToSTLVertices(sim, tris);
    std::ofstream outfile(name);
    if (!outfile.is_open()) {
        std::cerr << "Unable to open file " << name << std::endl;
        return false;
    }
    outfile << "X,Y,Z,WSS,OSI,TAWSS\n";
    for (size_t t = 0; t < tris.size(); ++t) {
        const Triangle& T = tris[t];
        const double p[3][3] = {{T.x1, T.y1, T.z1}, {T.x2, T.y2, T.z2}, {T.x3, T.y3, T.z3}};
        for (int k = 0; k < 3; ++k)
            outfile << p[k][0] << "," << p[k][1] << "," << p[k][2] << "," << va[t].wss[k] << "," << va[t].osi[k]
                    << "," << va[t].tawss[k] << "\n";
    }
    return (bool)outfile;
}
