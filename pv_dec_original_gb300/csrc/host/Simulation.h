// Simulation with the reference's constructor and step methods
// (Simulation.h:10-51).  Like the reference, the four-argument constructor
// runs Iterate() to the end time (t <= 2.7 s, Simulation.cpp:569-601); the
// five-argument form with run = false leaves stepping to the caller.
//
// The per-phase methods keep the reference's names and order.  On the GPU
// the phases of one step are a single fused launch (collide, stream, inlet,
// outlets, wall rule, WSS), so the phase methods must be called in
// Iterate()'s order; the last one, ComputeOSIAndTAWSS, runs the step with
// the inlet velocity in effect at ApplyZouHeBc.  Calling them out of order
// throws std::logic_error.  FaceCommunicate is a no-op: the lattice is one
// device-resident domain with no halo (the reference's MPI face exchange,
// Simulation.cpp:258-543).
#pragma once
#include <string>
#include <vector>

#include "OutputFile.h"
#include "Subdomain.h"
#include "lbm_gb300.h"
#include "pulsatile.h"

class Simulation {
public:
    OutputFile file1;
    int myrank_ = 0, num_procs_ = 1;
    SubDomain SubDomain_;
    Pulsatile Pulsatile_;
    double pressure_ = 1.0;
    double m_relaxation = 1.0;
    double m_omega = 1.0;
    double m_dt = 1.0;
    double total_runtime = 0.0;
    double Cs = 0.0;
    std::vector<double> wall_shear_stress;
    double InletVelocity_ = 0.0;

    // driver settings (not in the reference, which hard-codes them)
    double end_time = 2.7;      // Iterate(): while (total_runtime <= end_time)
    int output_every = 100;     // WriteOutput cadence (Simulation.cpp:589)
    bool write_output = true;
    bool write_vertices = false;  // also STL_Vertices/<iter>_Vertices.csv (WSS at the STL's vertices)
    bool verbose = false;
    std::string output_root = ".";

    Simulation(SubDomain& sd, double tau, double pressure, double del_t);
    Simulation(SubDomain& sd, double tau, double pressure, double del_t, bool run);
    ~Simulation();
    Simulation(const Simulation&) = delete;
    Simulation& operator=(const Simulation&) = delete;

    void InitializeShearStressAccumulators();
    void Collision();
    void Streaming();
    void ApplyZouHeBc();
    void ApplyOutletBc();
    void ApplyWallBc();
    void ComputeWallShearStress(int iteration);
    void ComputeOSIAndTAWSS(int iteration);
    void FaceCommunicate(int iter) { (void)iter; }
    double getInletVelocity(double x, double period);
    void Iterate();
    void SetRelaxation(double tau);
    void WriteOutput(int iter);

    // GPU-native additions
    void Step(int nsteps, double inlet_velocity);  // nsteps full steps at a fixed inlet velocity
    void SetInletTable(const std::vector<double>& amp);
    void StepTable(int nsteps);                    // nsteps steps reading the inlet table
    lbm_handle* handle();
    int64_t steps();
    void Macro(std::vector<double>& rho, std::vector<double>& u3);
    void Distributions(std::vector<double>& f);
    void WallShearStress(std::vector<int64_t>& pt, std::vector<double>& wss, std::vector<double>& osi,
                         std::vector<double>& tawss);
    std::vector<uint8_t> Classes();
    // Interpolated (Bouzidi) bounce-back with wall distances from the
    // geometry's triangles (physics mode; off: half-way bounce-back).
    void UseInterpolatedWalls(bool on = true);

private:
    lbm_handle* h_ = nullptr;
    int phase_ = 0;
    double pending_inlet_ = 0.0;
    void ensure();
    void check(lbm_status rc, const char* what);
    void expect_phase(int p, const char* name);
};
