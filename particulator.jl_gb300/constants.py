"""Physical constants (SI), the CODATA-2014 values of the reference
(src/constants.jl:6-164, generated from scipy.constants), and derived values."""
import math

c = 299792458.0
elementary_charge = e = eV = 1.6021766208e-19
electron_mass = m_e = 9.10938356e-31
hbar = 1.0545718001391127e-34
epsilon_0 = 8.854187817620389e-12
fine_structure = alpha = 0.0072973525664
N_A = Avogadro = 6.022140857e+23
k = Boltzmann = 1.38064852e-23
kilo = 1000.0
centi = 0.01
atm = 101325.0
nair = 2.6867811e+25          # constants.jl:149 (273.15 K)
Td = 1e-21                    # constants.jl:150
pi = math.pi

electron_mc2 = electron_mass * c ** 2
electron_mc = electron_mass * c
r_e = elementary_charge ** 2 / (electron_mass * c ** 2) / (4 * math.pi * epsilon_0)
a_0 = hbar / (electron_mass * c * fine_structure)
