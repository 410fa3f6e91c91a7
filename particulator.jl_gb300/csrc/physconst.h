// Physical constants in SI, the CODATA-2014 values the reference uses
// (src/constants.jl:6-164, generated from scipy.constants), and the derived
// device unit system.
//
// Device units: momentum in m_e c, energy in m_e c^2, time in ns, length in m.
// SI momenta (~5e-22 kg m/s at 1 MeV) square to ~1e-43, below FP32's normal
// range, so the device never sees SI momenta.
#pragma once

namespace pcl {
namespace si {
constexpr double c            = 299792458.0;
constexpr double e            = 1.6021766208e-19;
constexpr double eV           = 1.6021766208e-19;
constexpr double m_e          = 9.10938356e-31;
constexpr double hbar         = 1.0545718001391127e-34;
constexpr double epsilon_0    = 8.854187817620389e-12;
constexpr double alpha        = 0.0072973525664;
constexpr double N_A          = 6.022140857e+23;
constexpr double k_B          = 1.38064852e-23;
constexpr double kilo         = 1000.0;
constexpr double centi        = 0.01;
constexpr double pi           = 3.141592653589793;
constexpr double mc2          = m_e * (c * c);        // constants.jl:163
constexpr double mc           = m_e * c;              // constants.jl:164
// classical electron radius r_e = e^2 / (m_e c^2) / (4 pi eps0)  (constants.jl:157)
constexpr double r_e          = e * e / (m_e * (c * c)) / (4.0 * pi * epsilon_0);
// Bohr radius a_0 = hbar / (m_e c alpha)  (constants.jl:160)
constexpr double a_0          = hbar / (m_e * c * alpha);
}  // namespace si

// Conversions SI <-> device units.
constexpr double NS            = 1e-9;                // s per device time unit
constexpr double C_M_PER_NS    = si::c * NS;          // speed of light in m/ns
inline double p_to_dev(double p_si) { return p_si / si::mc; }
inline double p_to_si(double p_dev) { return p_dev * si::mc; }
inline double e_to_dev(double e_si) { return e_si / si::mc2; }
inline double e_to_si(double e_dev) { return e_dev * si::mc2; }
inline double t_to_dev(double t_si) { return t_si / NS; }
inline double t_to_si(double t_dev) { return t_dev * NS; }
inline double rate_to_dev(double nu_si) { return nu_si * NS; }   // 1/s -> 1/ns
// force (N) -> device momentum per ns
inline double force_to_dev(double f_si) { return f_si / si::mc * NS; }
}  // namespace pcl
