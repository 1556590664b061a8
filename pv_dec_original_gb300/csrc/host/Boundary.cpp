#include "Boundary.h"

#include "Simulation.h"

Boundary::Boundary(Simulation& sim, int rule_index) : sim_(&sim), rule_(rule_index) {}

void Boundary::SetInletVel(double ux, double uy, double uz) { m_inletVel = {ux, uy, uz}; }

void Boundary::ApplyBc(double& vel) {
    // the velocity every inlet node of the lattice gets in the next step
    m_inletVel = {vel, 0.0, 0.0};
    sim_->InletVelocity_ = vel;
}
