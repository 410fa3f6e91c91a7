"""Collision processes: the closed set the device samples.

Each class carries the fields of its reference struct and converts itself to
the C descriptor ``pcl_process``.  ``totalcs(proc, E)`` evaluates the
reference's cross-section formula through the library's host builder.
Arbitrary user-defined processes are not accepted: the device has no
`collide` for them (PCL_ERR_UNSUPPORTED).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from . import constants as co
from . import data


class _Proc:
    kind = 0
    Z = 0

    def _fill(self, p: _lib.Process):
        pass

    def to_c(self, coef: float = 1.0) -> _lib.Process:
        p = _lib.Process()
        p.kind = self.kind
        p.Z = int(self.Z) if float(self.Z).is_integer() else 0
        p.coef = float(coef)
        self._fill(p)
        self._keep = p  # keep aux arrays alive with the descriptor
        return p


class Moller(_Proc):
    """Moller(Z, tcut) (moller.jl:8-11)."""
    kind = _lib.PROC_MOLLER

    def __init__(self, Z: int, tcut: float):
        self.Z, self.tcut = Z, float(tcut)

    def _fill(self, p):
        p.param[0] = self.tcut
        p.nparam = 1


class Bhaba(_Proc):
    """Bhaba(Z, tcut) (bhaba.jl:4-7)."""
    kind = _lib.PROC_BHABHA

    def __init__(self, Z: int, tcut: float):
        self.Z, self.tcut = Z, float(tcut)

    def _fill(self, p):
        p.param[0] = self.tcut
        p.nparam = 1


Bhabha = Bhaba


class RBEB(_Proc):
    """RBEB(B, U, N) orbital (rbeb.jl:5-14)."""
    kind = _lib.PROC_RBEB

    def __init__(self, B: float, U: float, N: int):
        self.B, self.U, self.N = float(B), float(U), int(N)

    def _fill(self, p):
        p.param[0], p.param[1], p.param[2] = self.B, self.U, float(self.N)
        p.nparam = 3

    def __repr__(self):
        return f"RBEB(B = {self.B / co.eV} eV, U = {self.U / co.eV} eV, N = {self.N})"


# Molecular orbitals (rbeb.jl:25-52): K shells from Santos et al. (2003),
# valence orbitals from Hwang et al. (1996).
N2_ORBITALS = [RBEB(0.4095e3 * co.eV, 0.6033e3 * co.eV, 4), RBEB(41.72 * co.eV, 71.13 * co.eV, 2),
               RBEB(21.00 * co.eV, 63.18 * co.eV, 2), RBEB(17.07 * co.eV, 44.30 * co.eV, 4),
               RBEB(15.58 * co.eV, 54.91 * co.eV, 2)]
O2_ORBITALS = [RBEB(0.5438e3 * co.eV, 0.7962e3 * co.eV, 4), RBEB(46.19 * co.eV, 79.73 * co.eV, 2),
               RBEB(29.82 * co.eV, 90.92 * co.eV, 2), RBEB(19.64 * co.eV, 59.89 * co.eV, 4),
               RBEB(19.79 * co.eV, 71.84 * co.eV, 2), RBEB(12.07 * co.eV, 84.88 * co.eV, 2)]
ORBITALS = {"N2": N2_ORBITALS, "O2": O2_ORBITALS}


class RelativisticCoulomb(_Proc):
    """RelativisticCoulomb(Z) screened elastic scattering (relativistic_coulomb.jl:5-8)."""
    kind = _lib.PROC_REL_COULOMB

    def __init__(self, Z):
        self.Z = Z

    def _fill(self, p):
        p.param[0] = float(self.Z)
        p.nparam = 1


class Compton(_Proc):
    """Compton(Z), Geant4 empirical cross section (compton.jl:1-3, 59-112)."""
    kind = _lib.PROC_COMPTON

    def __init__(self, Z: int):
        self.Z = Z


class KleinNishinaCompton(Compton):
    """KleinNishinaCompton(Z) (compton.jl:5-7, 34-47)."""
    kind = _lib.PROC_KN_COMPTON


class BetheHeitler(_Proc):
    """BetheHeitler(Z) pair production (bethe_heitler.jl:1-3)."""
    kind = _lib.PROC_BETHE_HEITLER

    def __init__(self, Z: int):
        self.Z = Z


class PositronAnihilation(_Proc):
    """PositronAnihilation(Z) in flight (anihilation.jl:1-4); Z may be fractional."""
    kind = _lib.PROC_ANNIHILATION

    def __init__(self, Z):
        self.Z = Z

    def _fill(self, p):
        p.param[0] = float(self.Z)
        p.nparam = 1


PositronAnnihilation = PositronAnihilation


class PhotoElectric(_Proc):
    """PhotoElectric(Z) (photo_electric.jl:7-35): SANDIA cross section, single
    binding energy per photon energy."""
    kind = _lib.PROC_PHOTOELECTRIC

    def __init__(self, Z: int):
        self.Z = Z
        self.left_energy, self.coeffs = data.sandia(Z)
        self.binding = data.binding_energies(Z)

    def _fill(self, p):
        nb = min(8, len(self.binding))
        for m in range(nb):
            p.param[m] = float(self.binding[m])
        p.nparam = nb
        p.naux = len(self.left_energy)
        p.aux0 = _lib.dptr(self.left_energy)
        p.aux1 = _lib.dptr(self.coeffs)


class SeltzerBerger(_Proc):
    """SeltzerBerger(Z; ncum, gamma_min, gamma_max, energy_scale)
    (seltzer.jl:9-64): inverse-CDF table of log(k/T) over (pcum, log T) and the
    total cross section, built by the library from the G4 ``brZ`` file."""
    kind = _lib.PROC_SELTZER_BERGER

    def __init__(self, Z: int, ncum: int = 1000, gamma_min: float = 1e2 * co.eV,
                 gamma_max: float = 5e7 * co.eV, energy_scale: float = 1e6 * co.eV, path: str | None = None):
        self.Z = Z
        _, x, y, value = data.read_g4_2dvector(path or data.sb_path(Z))
        ne = len(y)
        self.ncum = ncum
        self.pcum = np.linspace(0.0, 1.0, ncum)
        self.log_energy = np.zeros(ne)
        self.totalcs = np.zeros(ne)
        self.data = np.zeros(ncum * ne)  # column-major [ncum][ne], pcum fastest
        x = np.ascontiguousarray(x)
        y = np.ascontiguousarray(y)
        value = np.ascontiguousarray(value)
        rc = _lib.lib().pcl_sb_build(Z, len(x), ne, _lib.dptr(x), _lib.dptr(y), _lib.dptr(value), ncum,
                                     float(gamma_min), float(gamma_max), float(energy_scale),
                                     _lib.dptr(self.log_energy), _lib.dptr(self.totalcs), _lib.dptr(self.data))
        _lib.check(rc, None, "pcl_sb_build")

    def table(self) -> np.ndarray:
        """data[i_pcum, j_energy] as a (ncum, ne) array."""
        return self.data.reshape(len(self.log_energy), self.ncum).T

    def _fill(self, p):
        p.naux = len(self.log_energy)
        p.aux0 = _lib.dptr(self.log_energy)
        p.aux1 = _lib.dptr(self.totalcs)
        p.aux2 = _lib.dptr(self.data)
        p.naux2 = self.ncum


class Elastic(_Proc):
    """Elastic(mass_ratio) (slow-electron.jl:82-84, 133-139): isotropic scattering
    in the centre of mass frame of an electron and a target of mass m / mass_ratio."""
    kind = _lib.PROC_ELASTIC

    def __init__(self, mass_ratio: float):
        self.mass_ratio = float(mass_ratio)

    def _fill(self, p):
        p.param[0] = self.mass_ratio
        p.nparam = 1


class Excitation(_Proc):
    """Excitation(threshold) (slow-electron.jl:70-72, 108-114): the electron loses
    `threshold` and leaves isotropically."""
    kind = _lib.PROC_EXCITATION

    def __init__(self, threshold: float):
        self.threshold = float(threshold)

    def _fill(self, p):
        p.param[0] = self.threshold
        p.nparam = 1


class Ionization(_Proc):
    """Ionization(threshold) (slow-electron.jl:74-76, 117-127): two electrons
    share the energy above the threshold equally, both isotropic."""
    kind = _lib.PROC_IONIZATION

    def __init__(self, threshold: float):
        self.threshold = float(threshold)

    def _fill(self, p):
        p.param[0] = self.threshold
        p.nparam = 1


class Attachment(_Proc):
    """Attachment(threshold) (slow-electron.jl:78-80, 129-131): the electron is
    removed."""
    kind = _lib.PROC_ATTACHMENT

    def __init__(self, threshold: float = 0.0):
        self.threshold = float(threshold)

    def _fill(self, p):
        p.param[0] = self.threshold
        p.nparam = 1


class NullCollision(_Proc):
    """NullCollision (collisions.jl:3, 58) as an explicit table entry."""
    kind = _lib.PROC_NULL_COLLISION


def totalcs(proc: _Proc, energy) -> np.ndarray:
    """Total cross section per target (m^2) at kinetic energies (J)."""
    E = np.ascontiguousarray(np.atleast_1d(np.asarray(energy, dtype=np.float64)))
    out = np.zeros_like(E)
    p = proc.to_c(1.0)
    _lib.check(_lib.lib().pcl_totalcs(C.byref(p), E.size, _lib.dptr(E), _lib.dptr(out)), None, "pcl_totalcs")
    return out if np.ndim(energy) else out[0]
