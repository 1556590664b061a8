#include "Simulation.h"

#include <cmath>
#include <iostream>
#include <stdexcept>

Simulation::Simulation(SubDomain& sd, double tau, double pressure, double del_t)
    : Simulation(sd, tau, pressure, del_t, true) {}

Simulation::Simulation(SubDomain& sd, double tau, double pressure, double del_t, bool run) : SubDomain_(sd) {
    SetRelaxation(tau);
    pressure_ = pressure;
    m_dt = del_t;
    m_omega = 1.0 / m_relaxation;
    InitializeShearStressAccumulators();
    if (run) Iterate();
}

Simulation::~Simulation() {
    if (h_) lbm_destroy(h_);
}

void Simulation::check(lbm_status rc, const char* what) {
    if (rc != LBM_OK) throw std::runtime_error(std::string(what) + ": " + lbm_last_error(h_));
}

void Simulation::ensure() {
    if (h_) return;
    const Geometry& g = SubDomain_.Geometry_;
    lbm_desc d{};
    d.Q = SubDomain_.options.Q;
    d.precision = SubDomain_.options.precision;
    d.mode = SubDomain_.options.mode;
    d.tau = m_relaxation;
    d.spacing = g.spacing;
    d.origin[0] = g.origin[0]; d.origin[1] = g.origin[1]; d.origin[2] = g.origin[2];
    // ComputeWallShearStress's constant (Simulation.cpp:880-881), same evaluation order
    double phys_den = 1060;
    double dtdt = m_dt * m_dt;
    double dxdx = g.spacing * g.spacing * 1e-6;
    d.wss_scale = phys_den * dtdt / dxdx;
    d.tawss_div = Pulsatile_.period;
    d.device = SubDomain_.options.device;
    if (lbm_create(&d, &h_) != LBM_OK) {
        h_ = nullptr;
        throw std::runtime_error(std::string("lbm_create: ") + lbm_last_global_error());
    }
    const int dims[3] = {g.nx, g.ny, g.nz};
    check(lbm_set_geometry(h_, g.mask.data(), dims, g.boundaryRules.data(), (int)g.boundaryRules.size()),
          "lbm_set_geometry");
    std::vector<double> rows = triangles_to_rows(g.globalTriangles);
    check(lbm_set_normals_from_surface(h_, rows.data(), (int64_t)g.globalTriangles.size()),
          "lbm_set_normals_from_surface");
}

lbm_handle* Simulation::handle() {
    ensure();
    return h_;
}

void Simulation::UseInterpolatedWalls(bool on) {
    ensure();
    const Geometry& g = SubDomain_.Geometry_;
    std::vector<double> rows = triangles_to_rows(g.globalTriangles);
    check(lbm_set_wall_distances(h_, on ? rows.data() : nullptr, on ? (int64_t)g.globalTriangles.size() : 0),
          "lbm_set_wall_distances");
}

int64_t Simulation::steps() {
    lbm_counts c{};
    check(lbm_get_counts(handle(), &c), "lbm_get_counts");
    return c.steps;
}

void Simulation::InitializeShearStressAccumulators() {
    // accumulators live on the device; a fresh state starts from f = w with
    // cleared accumulators (Simulation.cpp:32-38)
    if (h_) check(lbm_init_equilibrium(h_), "lbm_init_equilibrium");
}

void Simulation::SetRelaxation(double tau) {
    if (h_ && tau != m_relaxation)
        throw std::logic_error("SetRelaxation: tau is fixed once the lattice is on the device");
    m_relaxation = tau;
    m_omega = 1.0 / tau;
}

double Simulation::getInletVelocity(double x, double period) {
    // Simulation.cpp:548-563
    double vel = 0.0;
    double normalizedX = std::fmod(x, period);
    if (normalizedX >= 0 && normalizedX < (0.1 * period)) vel = Pulsatile_.InletVelequation1(normalizedX);
    else if (normalizedX >= (0.1 * period) && normalizedX < (0.3 * period)) vel = Pulsatile_.InletVelequation2(normalizedX);
    else if (normalizedX >= (0.3 * period) && normalizedX < (0.9 * period)) vel = Pulsatile_.InletVelequation3(normalizedX);
    return vel;
}

void Simulation::expect_phase(int p, const char* name) {
    if (phase_ != p)
        throw std::logic_error(std::string(name) +
                               ": the fused GPU step needs the phases in Iterate()'s order "
                               "(Collision, Streaming, ApplyZouHeBc, ApplyOutletBc, ApplyWallBc, "
                               "ComputeWallShearStress, ComputeOSIAndTAWSS)");
    phase_ = p + 1;
}

void Simulation::Collision() { expect_phase(0, "Collision"); }
void Simulation::Streaming() { expect_phase(1, "Streaming"); }
void Simulation::ApplyZouHeBc() {
    expect_phase(2, "ApplyZouHeBc");
    pending_inlet_ = InletVelocity_;
}
void Simulation::ApplyOutletBc() { expect_phase(3, "ApplyOutletBc"); }
void Simulation::ApplyWallBc() { expect_phase(4, "ApplyWallBc"); }
void Simulation::ComputeWallShearStress(int) { expect_phase(5, "ComputeWallShearStress"); }
void Simulation::ComputeOSIAndTAWSS(int) {
    expect_phase(6, "ComputeOSIAndTAWSS");
    phase_ = 0;
    Step(1, pending_inlet_);
}

void Simulation::Step(int nsteps, double inlet_velocity) {
    ensure();
    check(lbm_set_inlet_table(h_, &inlet_velocity, 1), "lbm_set_inlet_table");
    check(lbm_step(h_, nsteps), "lbm_step");
}

void Simulation::SetInletTable(const std::vector<double>& amp) {
    ensure();
    check(lbm_set_inlet_table(h_, amp.data(), (int64_t)amp.size()), "lbm_set_inlet_table");
}

void Simulation::StepTable(int nsteps) {
    ensure();
    check(lbm_step(h_, nsteps), "lbm_step");
}

void Simulation::Iterate() {
    ensure();
    // the inlet value of every iteration, at the times the reference visits
    // (t from 0, t += dt, while t <= end_time); step s reads table[s % N]
    const int64_t s0 = steps();
    std::vector<double> amp;
    std::vector<double> times;
    for (double t = 0.0; t <= end_time; t += m_dt) {
        times.push_back(t);
        amp.push_back(getInletVelocity(t, 0.9));
    }
    const int64_t N = (int64_t)amp.size();
    if (N == 0) return;
    std::vector<double> table(N);
    for (int64_t k = 0; k < N; ++k) table[(s0 + k) % N] = amp[k];
    SetInletTable(table);
    int64_t iter = 0;
    while (iter < N) {
        // up to and including the next iteration that writes output
        int64_t next = output_every > 0 ? ((iter + output_every - 1) / output_every) * output_every : N - 1;
        if (next >= N) next = N - 1;
        const int64_t n = next - iter + 1;
        StepTable((int)n);
        iter = next;
        total_runtime = times[iter];
        InletVelocity_ = amp[iter];
        if (output_every > 0 && iter % output_every == 0 && write_output) WriteOutput((int)iter);
        if (verbose && myrank_ == 0)
            std::cout << "\nIteration " << iter << " has been performed successfully" << std::endl;
        iter++;
    }
    total_runtime = times[N - 1] + m_dt;
}

void Simulation::WriteOutput(int iter) {
    OutputFile file(iter);
    file.root = output_root;
    file.WriteVTK_Collective(*this);
    file.WriteSurfaceAttribute(*this, iter);
    if (write_vertices) file.WriteSTLVertexAttribute(*this, SubDomain_.Geometry_.globalTriangles, iter);
}

void Simulation::Macro(std::vector<double>& rho, std::vector<double>& u3) {
    lbm_counts c{};
    check(lbm_get_counts(handle(), &c), "lbm_get_counts");
    rho.resize((size_t)c.active);
    u3.resize(3 * (size_t)c.active);
    check(lbm_get_macro(h_, rho.data(), u3.data()), "lbm_get_macro");
}

void Simulation::Distributions(std::vector<double>& f) {
    lbm_counts c{};
    check(lbm_get_counts(handle(), &c), "lbm_get_counts");
    f.resize((size_t)c.active * SubDomain_.options.Q);
    check(lbm_get_distributions(h_, f.data()), "lbm_get_distributions");
}

void Simulation::WallShearStress(std::vector<int64_t>& pt, std::vector<double>& wss, std::vector<double>& osi,
                                 std::vector<double>& tawss) {
    lbm_counts c{};
    check(lbm_get_counts(handle(), &c), "lbm_get_counts");
    const size_t n = (size_t)c.next_to_wall;
    pt.resize(n); wss.resize(n); osi.resize(n); tawss.resize(n);
    check(lbm_get_wss(h_, pt.data(), nullptr, wss.data(), nullptr, nullptr, osi.data(), tawss.data()), "lbm_get_wss");
    wall_shear_stress = wss;
}

std::vector<uint8_t> Simulation::Classes() {
    const Geometry& g = SubDomain_.Geometry_;
    std::vector<uint8_t> cls((size_t)g.nx * g.ny * g.nz);
    check(lbm_get_classes(handle(), cls.data()), "lbm_get_classes");
    return cls;
}
