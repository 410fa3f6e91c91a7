"""Physical data the processes of air (N, O) need.

These are data tables, carried as published:
  * Seltzer-Berger bremsstrahlung tables ``data/brem_SB/br7``, ``br8``
    (S.M. Seltzer, M.J. Berger, At. Data Nucl. Data Tables 35 (1986) 345, in the
    G4Physics2DVector text format of the Geant4 G4EMLOW set; the same files the
    reference reads, src/seltzer.jl:64).
  * SANDIA photo-absorption fit coefficients for Z = 7, 8 (F. Biggs, R. Lighthill,
    SAND-0070 (1990), as tabulated by Geant4's G4StaticSandiaData.hh; the rows the
    reference uses, src/static_sandia_data.jl:134-154) and the Z/A ratios
    (static_sandia_data.jl:1405-1414).
  * Atomic shell binding energies for Z = 7, 8 (src/atomic_shells.jl:35-39).
Only Z = 7 and 8 are carried: air is the only material of the hot path.
"""
from __future__ import annotations

import os

import numpy as np

from . import constants as co

DATA_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")

# (left energy keV, a1..a4 in cm^2 keV^i / g) per interval
SANDIA_TABLE = {
    7: [(0.01, 0.1010E+05, 0.0000E+00, 0.0000E+00, 0.0000E+00),
        (0.0404, -0.3622E+03, 0.3873E+03, 0.1244E+02, -0.4452E+00),
        (0.4016, -0.2338E+04, 0.5732E+04, -0.2082E+03, 0.1482E+03),
        (0.8, -0.4940E+01, -0.8442E+02, 0.4620E+04, -0.1186E+04),
        (4.0, 0.2019E+01, -0.1249E+03, 0.4609E+04, -0.9421E+03),
        (20.0, 0.1709E-01, -0.8196E+01, 0.2345E+04, 0.1369E+05),
        (100.0, 0.1872E-02, -0.6732E+00, 0.1282E+04, 0.5700E+05),
        (500.0, 0.8122E-03, 0.8364E+00, 0.4410E+03, 0.2358E+06)],
    8: [(0.01, 9.343E+03, 9.026E+02, -2.467E+01, 1.505E-01),
        (0.02, 6.034E+03, 7.319E+02, -2.677E+01, 2.842E-01),
        (0.0483, -0.2863E+03, 0.4085E+03, 0.4436E+02, -0.1782E+01),
        (0.532, -0.7181E+02, 0.4748E+03, 0.5542E+04, -0.1363E+04),
        (4.0, 0.2745E+01, -0.1747E+03, 0.7159E+04, -0.2213E+04),
        (20.0, 0.3774E-01, -0.1559E+02, 0.4045E+04, 0.1810E+05),
        (100.0, 0.3169E-02, -0.1146E+01, 0.2194E+04, 0.9131E+05),
        (500.0, 0.1367E-02, 0.1473E+01, 0.7214E+03, 0.4048E+06)],
}
Z_TO_A_RATIO = {7: 0.4998, 8: 0.5}
ATOMIC_SHELLS_EV = {7: (403.0, 37.3, 20.33, 14.53), 8: (543.1, 41.6, 28.48, 13.62)}


def binding_energies(Z: int) -> np.ndarray:
    """binding_energies(Z) (atomic_shells.jl:481-486), in J."""
    return np.array(ATOMIC_SHELLS_EV[Z], dtype=np.float64) * co.eV


def sandia(Z: int):
    """Left energies (J) and coefficients [n][4] (m^2 J^i per atom) as built by
    PhotoElectric(T, Z) (photo_electric.jl:19-31)."""
    rows = SANDIA_TABLE[Z]
    A = Z / Z_TO_A_RATIO[Z]
    s = (co.kilo * co.eV) ** np.arange(1, 5)
    left = np.array([r[0] for r in rows], dtype=np.float64) * (co.kilo * co.eV)
    coeffs = np.array([np.array(r[1:]) * s for r in rows], dtype=np.float64) * (co.centi ** 2 * A / co.N_A)
    return left, np.ascontiguousarray(coeffs)


def read_g4_2dvector(path: str):
    """RawG4Physics2DVector (util.jl:165-190): header 'k nx ny', x[nx], y[ny],
    then value[ny][nx]."""
    with open(path) as f:
        k, nx, ny = (int(v) for v in f.readline().split())
        x = np.array(f.readline().split(), dtype=np.float64)
        y = np.array(f.readline().split(), dtype=np.float64)
        rest = np.array(f.read().split(), dtype=np.float64)
    assert len(x) == nx and len(y) == ny and rest.size == nx * ny
    return k, x, y, rest.reshape(ny, nx)


def sb_path(Z: int) -> str:
    return os.path.join(DATA_DIR, "brem_SB", f"br{Z}")
