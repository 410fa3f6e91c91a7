"""Oracle-only set-up of the avalanche workload (test infrastructure only).

The CPU reference arm of the benchmark and the tests that want an
independent set-up build the oracle from here: the collision tables, the
Seltzer-Berger inverse-CDF tables and the continuum-loss fits come from the
numpy restatement of the reference's init path (``tables_ref``:
collision_table.jl:115-167, seltzer.jl:23-64,163-211, continuum.jl:36-43,
63-139), never from the library's C++ builders, and nothing here loads the
GPU library.  The package is imported only for its pure-Python parts: the
process descriptors (their fields), the dataclasses the oracle harness reads,
the data-file reader and the workload recipes.  PARITY UNPINNED: the
restatement is checked against the reference by reading only.
"""
from __future__ import annotations

import math

import numpy as np

from . import tables_ref as ref
from .harness import OracleWorld


def _pkg():
    import particulator_gb300 as pcl
    return pcl


def library_loaded() -> bool:
    """True when the GPU library has been loaded into this process."""
    try:
        with open("/proc/self/maps") as f:
            return "libparticulator_gb300" in f.read()
    except OSError:
        return _pkg()._lib._lib is not None


_SB = {}


def seltzer_berger(Z: int, ncum: int = 1000):
    """A SeltzerBerger process descriptor whose inverse-CDF table and cross
    section come from ``tables_ref.sb_build`` (its constructor, which calls
    the library's builder, is not run)."""
    if Z not in _SB:
        pcl = _pkg()
        _, x, y, value = pcl.data.read_g4_2dvector(pcl.data.sb_path(Z))
        le, tcs, data = ref.sb_build(Z, x, y, value, ncum=ncum)
        proc = object.__new__(pcl.SeltzerBerger)
        proc.Z = Z
        proc.ncum = ncum
        proc.pcum = np.linspace(0.0, 1.0, ncum)
        proc.log_energy = np.ascontiguousarray(le)
        proc.totalcs = np.ascontiguousarray(tcs)
        proc.data = np.ascontiguousarray(data.T).ravel()    # [ne][ncum], pcum fastest, as the device reads it
        _SB[Z] = proc
    return _SB[Z]


def electron_processes(comp, tcut: float = 1e4 * ref.eV):
    pcl = _pkg()
    return [(2 * comp["N2"], pcl.RelativisticCoulomb(7)), (2 * comp["O2"], pcl.RelativisticCoulomb(8)),
            (2 * comp["N2"], seltzer_berger(7)), (2 * comp["O2"], seltzer_berger(8)),
            (2 * comp["N2"], pcl.Moller(7, tcut)), (2 * comp["O2"], pcl.Moller(8, tcut))]


def positron_processes(comp, tcut: float = 1e4 * ref.eV):
    pcl = _pkg()
    return [(2 * comp["N2"], pcl.RelativisticCoulomb(7)), (2 * comp["O2"], pcl.RelativisticCoulomb(8)),
            (2 * comp["N2"], pcl.Bhaba(7, tcut)), (2 * comp["O2"], pcl.Bhaba(8, tcut)),
            (2 * comp["N2"], pcl.PositronAnihilation(7)), (2 * comp["O2"], pcl.PositronAnihilation(8))]


def photon_processes(comp):
    pcl = _pkg()
    return [(2 * comp["N2"], pcl.PhotoElectric(7)), (2 * comp["O2"], pcl.PhotoElectric(8)),
            (2 * comp["N2"], pcl.BetheHeitler(7)), (2 * comp["O2"], pcl.BetheHeitler(8)),
            (2 * comp["N2"], pcl.Compton(7)), (2 * comp["O2"], pcl.Compton(8))]


def collision_table(processes, particle: int, Fdt: float, safety: float = 1.15, nintervals: int = 32,
                    order: int = 3, max_energy: float = 1e3 * ref.eV * 2 ** 18):
    """collision_table_from_processes (collision_table.jl:115-149) from the
    numpy restatement, in the table layout the oracle reads."""
    pcl = _pkg()
    a, rb, perm = ref.collision_table(processes, particle == pcl.Photon, particle != pcl.Photon, Fdt,
                                      safety=safety, nintervals=nintervals, order=order, max_energy=max_energy)
    asort = a[:, perm, :]
    return pcl.ChebyshevCollisionTable(proc=tuple(processes[p][1] for p in perm),
                                       coef=np.array([processes[p][0] for p in perm], dtype=np.float64),
                                       b=pcl.BinaryIntervals(nintervals, float(max_energy)), order=order,
                                       rate=np.ascontiguousarray(asort.transpose(2, 1, 0)).ravel(),
                                       ratebound=np.ascontiguousarray(rb.T).ravel(),
                                       perm=np.asarray(perm, np.int32), particle=particle)


def continuum_loss(comp, I: float = 85.7 * ref.eV, Tcut: float = 1e4 * ref.eV,
                   Tmax: float = 1e3 * ref.eV * 2 ** 18, n: int = 3):
    """ChebContinuumLoss(ContinuumLoss(nel, I, Tcut), Tmax, n) (continuum.jl:36-43)."""
    pcl = _pkg()
    nel = 14 * comp["N2"] + 16 * comp["O2"]
    k = int(math.ceil(math.log2(Tmax / Tcut)))
    xmax = 2.0 ** k * Tcut
    ec = ref.chebfit(lambda E: ref.energy_loss(nel, I, Tcut, False, E), k, xmax, n)
    pc = ref.chebfit(lambda E: ref.energy_loss(nel, I, Tcut, True, E), k, xmax, n)
    return pcl.ChebContinuumLoss(pcl.BinaryIntervals(k, xmax), np.ascontiguousarray(ec.T).ravel(),
                                 np.ascontiguousarray(pc.T).ravel(), n)


def avalanche_world(seed: int, efield: float = 5e5, dt: float = 1e-12, safety: float = 1.15):
    """The oracle configured for the mixed avalanche in air (1 atm, 293 K, E
    along -z, cuts 10 keV e+- and 5 keV photons) with independently built
    tables; returns (world, tables dict, cuts dict, pusher)."""
    pcl = _pkg()
    comp = pcl.workloads.air_composition()
    Fdt = pcl.co.elementary_charge * efield * dt
    tabs = {pcl.Electron: collision_table(electron_processes(comp), pcl.Electron, Fdt, safety),
            pcl.Photon: collision_table(photon_processes(comp), pcl.Photon, 0.0, safety),
            pcl.Positron: collision_table(positron_processes(comp), pcl.Positron, Fdt, safety)}
    cl = continuum_loss(comp)
    pusher = pcl.workloads.pusher((0.0, 0.0, -efield), cl=cl)
    cuts = {pcl.Electron: 1e4 * ref.eV, pcl.Photon: 5e3 * ref.eV, pcl.Positron: 1e4 * ref.eV}
    return OracleWorld(seed, tabs, cuts, pusher), tabs, cuts, pusher
