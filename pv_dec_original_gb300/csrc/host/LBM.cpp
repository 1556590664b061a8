// lbm_run: the reference's driver (LBM.cpp:20-85) on the GPU engine.
//
//   lbm_run <config>
//
// The reference hard-codes PV.stl, spacing 0.05, tau 1.5, dt 8e-6 and runs to
// t = 2.7 s.  Here those are config keys ("key value" lines, ConfigReader):
//   stl <path>         spacing <s>        tau <tau>         dt <dt>
//   end_time <t>       output_every <n>   output_dir <dir>  lattice 19|27
//   precision 0..3 (f64, f32, f16, bf16)  mode 0|1 (parity, physics)
//   pv_preset 1        (the reference's PV.stl inlet / outlet coordinates)
//   write_output 0|1   write_vertices 0|1 (WSS / OSI / TAWSS at the STL's vertices)
//   interpolated_walls 1 (physics mode: Bouzidi bounce-back from the STL's wall distances)
//   graph_steps <n>    (even: steps replayed from one captured CUDA graph; 0 = direct launches)
//   persistent_steps <k> (even: steps per persistent launch, a divisor of graph_steps; 0 = off)
//   inlet_face <f> inlet_plane <p>  outlet_face <f> outlet_plane <p>
// Defaults reproduce the reference: FP64, parity semantics, D3Q19.
#include <chrono>
#include <iomanip>
#include <iostream>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>

#include "ComplexGeometry.h"
#include "ConfigReader.h"
#include "LatticeModel.h"
#include "Simulation.h"
#include "Subdomain.h"

int main(int argc, char** argv) {
    if (argc < 2) {
        std::cerr << "usage: lbm_run <config>\n";
        return 2;
    }
    auto start = std::chrono::high_resolution_clock::now();
    ConfigReader reader(argv[1]);
    std::map<std::string, std::string> sv;
    if (!reader.readConfigStrings(sv)) {
        std::cerr << reader.lastError() << "\n";
        return 2;
    }
    auto num = [&](const char* k, double def) { return sv.count(k) ? std::stod(sv[k]) : def; };
    const std::string stl = sv.count("stl") ? sv["stl"] : "PV.stl";
    const double spacing = num("spacing", 0.05);
    const double tau = num("tau", 1.5);
    const double dt = num("dt", 8e-6);
    LbmOptions opt;
    opt.Q = (int)num("lattice", 19);
    opt.precision = (int)num("precision", LBM_F64);
    opt.mode = (int)num("mode", LBM_PARITY);
    using clk = std::chrono::high_resolution_clock;
    auto secs = [](clk::time_point a, clk::time_point b) { return std::chrono::duration<double>(b - a).count(); };
    try {
        auto velSet = std::make_shared<LatticeModel>(opt.Q);
        const auto t0 = clk::now();
        Geometry geometry(stl, velSet, spacing, 'z');
        const auto t1 = clk::now();
        if (num("pv_preset", 0) != 0) geometry.UsePVPreset();
        if (sv.count("inlet_face")) geometry.AddInlet((int)num("inlet_face", 0), (int)num("inlet_plane", -1));
        if (sv.count("outlet_face"))
            geometry.AddPressureOutlet((int)num("outlet_face", 1), (int)num("outlet_plane", -1), 1.0);
        std::cout << "lattice " << geometry.nx << "x" << geometry.ny << "x" << geometry.nz << ", "
                  << geometry.fluidCount << " fluid points\n";
        SubDomain subdomain(geometry, opt);
        Simulation sim(subdomain, tau, 1.0, dt, false);
        sim.end_time = num("end_time", 2.7);
        sim.output_every = (int)num("output_every", 100);
        sim.output_root = sv.count("output_dir") ? sv["output_dir"] : ".";
        sim.write_output = num("write_output", 1) != 0;
        sim.write_vertices = num("write_vertices", 0) != 0;
        if (num("interpolated_walls", 0) != 0) sim.UseInterpolatedWalls(true);
        auto ck = [&](lbm_status rc, const char* what) {
            if (rc != LBM_OK) throw std::runtime_error(std::string(what) + ": " + lbm_last_error(sim.handle()));
        };
        if (sv.count("persistent_steps"))
            ck(lbm_set_persistent(sim.handle(), (int)num("persistent_steps", 0)), "persistent_steps");
        if (sv.count("graph_steps")) ck(lbm_set_graph_steps(sim.handle(), (int)num("graph_steps", 0)), "graph_steps");
        lbm_counts c{};
        if (lbm_get_counts(sim.handle(), &c) != LBM_OK) throw std::runtime_error("lbm_get_counts failed");
        const auto t2 = clk::now();
        sim.Iterate();
        const auto t3 = clk::now();
        const int64_t n = sim.steps();
        std::cout << "steps " << n << "\n";
        std::cout << "active " << c.active << " next_to_wall " << c.next_to_wall << "\n";
        std::cout << std::setprecision(4) << "geometry " << secs(t0, t1) << " s, set-up " << secs(t1, t2)
                  << " s, iterate " << secs(t2, t3) << " s = "
                  << (n > 0 ? (double)c.active * (double)n / secs(t2, t3) / 1e6 : 0.0)
                  << " MLUPS (output included)\n";
    } catch (const std::exception& e) {
        std::cerr << "lbm_run: " << e.what() << "\n";
        return 1;
    }
    std::chrono::duration<double> el = std::chrono::high_resolution_clock::now() - start;
    std::cout << "\nTotal Elapsed time: " << std::fixed << std::setprecision(2) << std::setw(8) << el.count()
              << " seconds." << std::endl;
    return 0;
}
