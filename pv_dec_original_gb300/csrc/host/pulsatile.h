// Pulsatile inlet waveform (pulsatile.h:8-30 of the reference): three
// piecewise polynomials of the phase over a 0.9 s period, zero on
// [0.81, 0.9).  Simulation::getInletVelocity selects the piece.
#pragma once

class Pulsatile {
public:
    double period = 0.9;
    double InletVelequation1(double x) const;
    double InletVelequation2(double x) const;
    double InletVelequation3(double x) const;
};
