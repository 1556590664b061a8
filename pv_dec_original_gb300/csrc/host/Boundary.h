// Boundary condition handle with the reference's method names
// (Boundary.h:6-27).  In the reference every inlet / outlet / wall point is
// a Boundary node and Simulation::ApplyZouHeBc calls ApplyBc(vel) on each
// inlet node with the step's inlet velocity (Simulation.cpp:614-622).  Here
// the boundary nodes live on the device; a Boundary object names one rule of
// the Geometry and ApplyBc(vel) sets the inlet velocity its nodes get in the
// next step.
#pragma once
#include <vector>

#include "lbm_gb300.h"

class Simulation;

class Boundary {
public:
    Boundary(Simulation& sim, int rule_index);
    void SetInletVel(double ux, double uy, double uz);
    double Density() const { return 1.0; }  // Boundary::Density (Boundary.cpp:19-22)
    std::vector<double> Velocity() const { return m_inletVel; }
    void ApplyBc(double& vel);

private:
    Simulation* sim_;
    int rule_;
    std::vector<double> m_inletVel{0.0, 0.0, 0.0};
};
