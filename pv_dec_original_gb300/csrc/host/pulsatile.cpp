#include "pulsatile.h"

#include <cmath>

double Pulsatile::InletVelequation1(double x) const {
    return (-8.579e+08 * std::pow(x, 8) + 4.059e+08 * std::pow(x, 7) - 7.817e+07 * std::pow(x, 6) +
            7.994e+06 * std::pow(x, 5) - 4.835e+05 * std::pow(x, 4) + 1.782e+04 * std::pow(x, 3) -
            321.6 * std::pow(x, 2) + 3.215 * x + 0.1423);
}

double Pulsatile::InletVelequation2(double x) const {
    return (-4.32e+06 * std::pow(x, 8) + 7.94e+06 * std::pow(x, 7) - 6.298e+06 * std::pow(x, 6) +
            2.82e+06 * std::pow(x, 5) - 7.809e+05 * std::pow(x, 4) + 1.37e+05 * std::pow(x, 3) -
            1.484e+04 * std::pow(x, 2) + 901.9 * x - 22.87);
}

double Pulsatile::InletVelequation3(double x) const {
    return (-5.123 * std::pow(x, 4) + 14.15 * std::pow(x, 3) - 14.21 * std::pow(x, 2) + 5.865 * x - 0.5696);
}
