// Shadow of the reference's Math/Constants.h used only when the reference's own
// sources are compiled into the checker library (oracle/Makefile puts this
// directory first on the include path).  It keeps every name the reference
// uses, with the same values, except the gravitational constant, which is 1 so
// that the reference runs in the G = 1 code units of the CUDA path.
#pragma once

namespace Constants
{
    constexpr double C = 299792458.0;         // speed of light [m/s]
    constexpr double G = 1.0;                 // code units (the reference uses SI: 6.67430e-11)
    constexpr double PI = 3.14159265358979323846;
    constexpr double E = 2.71828182845904523536;
    constexpr double PHI = 1.61803398874989484820;
    constexpr double GAMMA = 5.0 / 3.0;       // adiabatic index
    constexpr double k_b = 1.38064852e-23;    // Boltzmann constant [J/K]
    constexpr double h_p = 6.62607015e-34;    // Planck constant [J s]
    constexpr double prtn = 1.6726219e-27;    // proton mass [kg]
    const double X_H = 0.76;                  // hydrogen mass fraction
    const double X_He = 0.24;                 // helium mass fraction
};
