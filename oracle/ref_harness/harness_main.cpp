// Oracle harness around the reference's own C++ (test infrastructure only).
//
// Links the reference's Geometry / SubDomain / Simulation objects, compiled
// unchanged from their sources, and drives them step by step so that their
// outputs can be dumped as golden vectors:
//
//   ref_harness vox <stl> <spacing> <out.bin>
//       Geometry pipeline up to findBoundaryPoints (ComplexGeometry.cpp:8-36,
//       minus the PV-specific classifyBoundaryPoints and the unused
//       CalculateWallDistances). Dumps the +z ray-parity mask.
//
//   ref_harness sim <stl> <spacing> <bc.txt> <tau> <dt> <nsteps> <inlet.txt> <out.bin>
//       Builds the node graph (Subdomain.cpp:3-32) and advances the
//       reference step methods in Iterate()'s order (Simulation.cpp:569-601).
//
//   ref_harness pulse <dt> <nsteps> <out.bin>
//       The pulsatile inlet waveform at the times Iterate() visits.
//
// Harness differences from the reference's main() (LBM.cpp:20-85), all
// outside the arithmetic under test:
//   * boundary points are split into inlet / outlet1..3 by the plane rules of
//     <bc.txt> instead of the hard-coded PV.stl coordinates
//     (ComplexGeometry.cpp:1369-1429); priority inlet > outlet1 > outlet2 >
//     outlet3 > wall, as in SubDomain::CreateNodes (Subdomain.cpp:124-151);
//   * the Simulation constructor always runs Iterate() once; the harness
//     hands it empty node lists for that call, so it touches no node, and
//     restores the lists afterwards;
//   * the inlet amplitude of step s is line s of <inlet.txt>; a parabolic
//     profile calls Boundary::ApplyBc per node with amplitude * profile.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <chrono>
#include <string>
#include <vector>
#include <fstream>
#include <sstream>
#include <algorithm>

#include "LatticeModel.h"
#include "ComplexGeometry.h"
#include "Subdomain.h"
#include "Simulation.h"

namespace {

struct PlaneRule {
    int kind;      // 1 inlet, 2 outlet1, 3 outlet2, 4 outlet3
    int axis;      // 0 x, 1 y, 2 z
    int index;     // lattice index on that axis
};

struct BcSpec {
    std::vector<PlaneRule> rules;
    int profile = 0;          // 0 uniform, 1 parabolic about (c1, c2) with radius R
    double c1 = 0, c2 = 0, R = 1;
};

BcSpec read_bc(const char* path) {
    BcSpec s;
    std::ifstream in(path);
    std::string line;
    while (std::getline(in, line)) {
        if (line.empty() || line[0] == '#') continue;
        std::istringstream ss(line);
        std::string key;
        ss >> key;
        if (key == "profile") {
            ss >> s.profile >> s.c1 >> s.c2 >> s.R;
            continue;
        }
        PlaneRule r{};
        std::string ax;
        if (key == "inlet") r.kind = 1;
        else if (key == "outlet1") r.kind = 2;
        else if (key == "outlet2") r.kind = 3;
        else if (key == "outlet3") r.kind = 4;
        else { std::fprintf(stderr, "bad bc key %s\n", key.c_str()); std::exit(2); }
        ss >> ax >> r.index;
        r.axis = ax == "x" ? 0 : ax == "y" ? 1 : 2;
        s.rules.push_back(r);
    }
    return s;
}

// Inlet profile factor; the product computes the identical expression.
double profile_factor(const BcSpec& s, double y, double z) {
    if (s.profile == 0) return 1.0;
    double dy = y - s.c1, dz = z - s.c2;
    double p = 1.0 - (dy * dy + dz * dz) / (s.R * s.R);
    return p > 0.0 ? p : 0.0;
}

void setup_geometry(Geometry& g, const char* stl, double spacing, std::shared_ptr<LatticeModel> vs) {
    g.stlFileName = stl;
    g.m_velSet = vs;
    g.spacing = spacing;
    g.raydirection = 'z';
    g.Create_cart_comm();
    g.GetSubBoundingBox();
    g.Add_Ghost();
    g.generatePointsInSubBox();
    g.labelPoints();
    g.Comm_Ghost();
    g.findBoundaryPoints();
}

template <class T>
void put(std::FILE* f, const T& v) { std::fwrite(&v, sizeof(T), 1, f); }

int run_vox(int argc, char** argv) {
    if (argc != 5) return 2;
    auto vs = std::make_shared<LatticeModel>();
    Geometry g;
    auto t0 = std::chrono::steady_clock::now();
    setup_geometry(g, argv[2], std::atof(argv[3]), vs);
    auto t1 = std::chrono::steady_clock::now();
    int nx = g.pointsBox.size(), ny = g.pointsBox[0].size(), nz = g.pointsBox[0][0].size();
    std::FILE* f = std::fopen(argv[4], "wb");
    put<int32_t>(f, 0x584f5652);  // "RVOX"
    put<int32_t>(f, nx); put<int32_t>(f, ny); put<int32_t>(f, nz);
    put<double>(f, g.boundingbox.min_x); put<double>(f, g.boundingbox.max_x);
    put<double>(f, g.boundingbox.min_y); put<double>(f, g.boundingbox.max_y);
    put<double>(f, g.boundingbox.min_z); put<double>(f, g.boundingbox.max_z);
    put<int64_t>(f, (int64_t)g.globalTriangles.size());
    put<double>(f, std::chrono::duration<double>(t1 - t0).count());
    // mask, x fastest: index = (k*ny + j)*nx + i
    std::vector<uint8_t> mask((size_t)nx * ny * nz);
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k)
                mask[((size_t)k * ny + j) * nx + i] = g.pointsBox[i][j][k]->NodeType == NodeType::Fluid ? 1 : 0;
    std::fwrite(mask.data(), 1, mask.size(), f);
    put<int64_t>(f, (int64_t)g.boundaryIndices.size());
    for (auto& t : g.boundaryIndices) {
        put<int32_t>(f, std::get<0>(t)); put<int32_t>(f, std::get<1>(t)); put<int32_t>(f, std::get<2>(t));
    }
    std::fclose(f);
    std::fprintf(stderr, "vox %dx%dx%d tris=%zu boundary=%zu %.3fs\n", nx, ny, nz,
                 g.globalTriangles.size(), g.boundaryIndices.size(),
                 std::chrono::duration<double>(t1 - t0).count());
    return 0;
}

int run_sim(int argc, char** argv) {
    if (argc != 10) return 2;
    const char* stl = argv[2];
    double spacing = std::atof(argv[3]);
    BcSpec bc = read_bc(argv[4]);
    double tau = std::atof(argv[5]);
    double dt = std::atof(argv[6]);
    int nsteps = std::atoi(argv[7]);
    std::vector<double> amp;
    {
        std::ifstream in(argv[8]);
        double v;
        while (in >> v) amp.push_back(v);
        if (amp.empty()) amp.push_back(0.0);
    }

    auto vs = std::make_shared<LatticeModel>();
    Geometry g;
    setup_geometry(g, stl, spacing, vs);

    // Plane-rule classification of the boundary points (replaces the PV.stl
    // coordinates of classifyBoundaryPoints, keeping its list structure).
    std::vector<int> cls(g.boundaryPoints.size(), 0);
    for (size_t b = 0; b < g.boundaryPoints.size(); ++b) {
        int idx[3] = {std::get<0>(g.boundaryIndices[b]), std::get<1>(g.boundaryIndices[b]),
                      std::get<2>(g.boundaryIndices[b])};
        for (auto& r : bc.rules) {
            if (idx[r.axis] == r.index) { cls[b] = r.kind; break; }
        }
        switch (cls[b]) {
            case 1: g.InletboundaryPoints.push_back(g.boundaryPoints[b]); break;
            case 2: g.OutletboundaryPoints1.push_back(g.boundaryPoints[b]); break;
            case 3: g.OutletboundaryPoints2.push_back(g.boundaryPoints[b]); break;
            case 4: g.OutletboundaryPoints3.push_back(g.boundaryPoints[b]); break;
            default:
                g.WallboundaryPoints.push_back(g.boundaryPoints[b]);
                g.wallBoundaryIndices.push_back(g.boundaryIndices[b]);
        }
    }

    auto t0 = std::chrono::steady_clock::now();
    SubDomain sd(g);
    auto t1 = std::chrono::steady_clock::now();

    // Hand the constructor's mandatory Iterate() empty lists.
    auto inv = sd.Involved_Lat_, inl = sd.InletBoundaryNode_, o1 = sd.OutletBoundaryNode1_,
         o2 = sd.OutletBoundaryNode2_, o3 = sd.OutletBoundaryNode3_, wall = sd.WallBoundaryNode_,
         nw = sd.nextToTheWall;
    sd.Involved_Lat_.clear(); sd.InletBoundaryNode_.clear(); sd.OutletBoundaryNode1_.clear();
    sd.OutletBoundaryNode2_.clear(); sd.OutletBoundaryNode3_.clear(); sd.WallBoundaryNode_.clear();
    sd.nextToTheWall.clear();
    std::FILE* saved_stdout = stdout;
    (void)saved_stdout;
    Simulation sim(sd, tau, 1.0, 1e9);  // dt > 2.7: exactly one (empty) iteration
    sim.SubDomain_.Involved_Lat_ = inv; sim.SubDomain_.InletBoundaryNode_ = inl;
    sim.SubDomain_.OutletBoundaryNode1_ = o1; sim.SubDomain_.OutletBoundaryNode2_ = o2;
    sim.SubDomain_.OutletBoundaryNode3_ = o3; sim.SubDomain_.WallBoundaryNode_ = wall;
    sim.SubDomain_.nextToTheWall = nw;
    sim.m_dt = dt;
    sim.InitializeShearStressAccumulators();

    auto t2 = std::chrono::steady_clock::now();
    for (int s = 0; s < nsteps; ++s) {
        double a = amp[s % amp.size()];
        sim.Collision();
        sim.FaceCommunicate(s);
        sim.Streaming();
        if (bc.profile == 0) {
            sim.InletVelocity_ = a;
            sim.ApplyZouHeBc();
        } else {
            for (auto& node : sim.SubDomain_.InletBoundaryNode_) {
                auto& p = g.pointsBox[node->x_position][node->y_position][node->z_position];
                double v = a * profile_factor(bc, p->y, p->z);
                node->ApplyBc(v);
            }
        }
        sim.ApplyOutletBc();
        sim.ApplyWallBc();
        sim.ComputeWallShearStress(s);
        sim.ComputeOSIAndTAWSS(s);
    }
    auto t3 = std::chrono::steady_clock::now();

    int nx = sd.my_Nx, ny = sd.my_Ny, nz = sd.my_Nz;
    std::FILE* f = std::fopen(argv[9], "wb");
    put<int32_t>(f, 0x4d495352);  // "RSIM"
    put<int32_t>(f, nx); put<int32_t>(f, ny); put<int32_t>(f, nz);
    put<int32_t>(f, _nLatNodes); put<int32_t>(f, nsteps);
    put<double>(f, std::chrono::duration<double>(t1 - t0).count());
    put<double>(f, std::chrono::duration<double>(t3 - t2).count());
    put<int64_t>(f, (int64_t)inv.size());
    for (auto& n : inv) {
        int t = 0;
        if (n->NodeType_ == NodeType::Boundary) {
            if (n->BoundaryType_ == BoundaryType::Wall) t = 5;
            else if (std::find(inl.begin(), inl.end(), n) != inl.end()) t = 1;
            else if (std::find(o1.begin(), o1.end(), n) != o1.end()) t = 2;
            else if (std::find(o2.begin(), o2.end(), n) != o2.end()) t = 3;
            else t = 4;
        }
        put<int32_t>(f, n->x_position); put<int32_t>(f, n->y_position); put<int32_t>(f, n->z_position);
        put<int32_t>(f, t);
        std::fwrite(n->m_distributions.data(), sizeof(double), _nLatNodes, f);
        std::fwrite(n->m_newDistributions.data(), sizeof(double), _nLatNodes, f);
        std::fwrite(n->m_eqdistributions.data(), sizeof(double), _nLatNodes, f);
        put<double>(f, n->density);
        put<double>(f, n->velocity[0]); put<double>(f, n->velocity[1]); put<double>(f, n->velocity[2]);
    }
    put<int64_t>(f, (int64_t)nw.size());
    for (auto& n : nw) {
        put<int32_t>(f, n->x_position); put<int32_t>(f, n->y_position); put<int32_t>(f, n->z_position);
        put<double>(f, n->normal[0]); put<double>(f, n->normal[1]); put<double>(f, n->normal[2]);
        put<double>(f, n->wall_shear_stress);
        put<double>(f, n->accumulated_shear_stress[0]); put<double>(f, n->accumulated_shear_stress[1]);
        put<double>(f, n->accumulated_shear_stress[2]);
        put<double>(f, n->accumulated_shear_stress_magnitude);
        put<double>(f, n->osi); put<double>(f, n->tawss);
    }
    put<int64_t>(f, (int64_t)wall.size());
    for (auto& n : wall) {
        put<int32_t>(f, n->x_position); put<int32_t>(f, n->y_position); put<int32_t>(f, n->z_position);
        put<double>(f, n->normal[0]); put<double>(f, n->normal[1]); put<double>(f, n->normal[2]);
    }
    std::fclose(f);
    std::fprintf(stderr, "sim %dx%dx%d active=%zu inlet=%zu out=%zu/%zu/%zu wall=%zu nw=%zu steps=%d %.3fs\n",
                 nx, ny, nz, inv.size(), inl.size(), o1.size(), o2.size(), o3.size(), wall.size(),
                 nw.size(), nsteps, std::chrono::duration<double>(t3 - t2).count());
    return 0;
}

// ref_harness pulse <dt> <nsteps> <out.bin>: Simulation::getInletVelocity
// (Simulation.cpp:548-563) at the times Iterate() visits (t += dt from 0).
int run_pulse(int argc, char** argv) {
    if (argc != 5) return 2;
    double dt = std::atof(argv[2]);
    int n = std::atoi(argv[3]);
    SubDomain sd;
    sd.my_left = sd.my_right = sd.my_front = sd.my_back = sd.my_up = sd.my_down = MPI_PROC_NULL;
    Simulation sim(sd, 1.0, 1.0, 1e9);
    std::FILE* f = std::fopen(argv[4], "wb");
    double t = 0.0;
    for (int s = 0; s < n; ++s) {
        double v = sim.getInletVelocity(t, 0.9);
        std::fwrite(&t, sizeof(double), 1, f);
        std::fwrite(&v, sizeof(double), 1, f);
        t += dt;
    }
    std::fclose(f);
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: ref_harness vox|sim ...\n");
        return 2;
    }
    std::string mode = argv[1];
    int rc = 2;
    if (mode == "vox") rc = run_vox(argc, argv);
    else if (mode == "sim") rc = run_sim(argc, argv);
    else if (mode == "pulse") rc = run_pulse(argc, argv);
    if (rc == 2) std::fprintf(stderr, "bad arguments for %s\n", mode.c_str());
    return rc;
}
