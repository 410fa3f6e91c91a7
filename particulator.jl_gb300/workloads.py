"""Air, its process lists and the benchmark workloads.

The process lists follow the reference's beam script (scripts/beam.jl:94-129)
with Moller ionisation in place of the RBEB orbitals for electrons; the
coefficient of every atomic process is the atom density 2 n_X2.
"""
from __future__ import annotations

import json
import os
from dataclasses import dataclass

import numpy as np

from . import constants as co
from .forcing import CombinedForcing, ElectromagneticField, HomogeneousField, RK2Pusher
from .population import MultiPopulation, ParticleArrays, Population
from .processes import (BetheHeitler, Bhaba, Compton, Elastic, Excitation, Moller, ORBITALS, PhotoElectric,
                        PositronAnihilation, RelativisticCoulomb, SeltzerBerger)
from .tables import (ChebContinuumLoss, ContinuumLoss, Electron, Photon, Positron,
                     collision_table_from_processes, lxcat_table, momentum_norm_from_kin)

KEV = 1e3 * co.eV
MEV = 1e6 * co.eV


def air_composition(T: float = 293.0, p: float = co.atm, f_n2: float = 0.79, f_o2: float = 0.21):
    """Molecule densities (1/m^3) of N2/O2 air at pressure p and temperature T."""
    n = p / (co.Boltzmann * T)
    return {"N2": f_n2 * n, "O2": f_o2 * n}


_SB_CACHE = {}


def seltzer_berger(Z: int) -> SeltzerBerger:
    if Z not in _SB_CACHE:
        _SB_CACHE[Z] = SeltzerBerger(Z)
    return _SB_CACHE[Z]


def electron_processes(comp, tcut: float = 10 * KEV, ionization: str = "moller"):
    procs = [(2 * comp["N2"], RelativisticCoulomb(7)), (2 * comp["O2"], RelativisticCoulomb(8)),
             (2 * comp["N2"], seltzer_berger(7)), (2 * comp["O2"], seltzer_berger(8))]
    if ionization == "moller":
        procs += [(2 * comp["N2"], Moller(7, tcut)), (2 * comp["O2"], Moller(8, tcut))]
    elif ionization == "rbeb":
        procs += [(comp["N2"], orb) for orb in ORBITALS["N2"]] + [(comp["O2"], orb) for orb in ORBITALS["O2"]]
    return procs


def positron_processes(comp, tcut: float = 10 * KEV):
    return [(2 * comp["N2"], RelativisticCoulomb(7)), (2 * comp["O2"], RelativisticCoulomb(8)),
            (2 * comp["N2"], Bhaba(7, tcut)), (2 * comp["O2"], Bhaba(8, tcut)),
            (2 * comp["N2"], PositronAnihilation(7)), (2 * comp["O2"], PositronAnihilation(8))]


def photon_processes(comp):
    return [(2 * comp["N2"], PhotoElectric(7)), (2 * comp["O2"], PhotoElectric(8)),
            (2 * comp["N2"], BetheHeitler(7)), (2 * comp["O2"], BetheHeitler(8)),
            (2 * comp["N2"], Compton(7)), (2 * comp["O2"], Compton(8))]


def air_continuum_loss(comp, I: float = 85.7 * co.eV, Tcut: float = 10 * KEV, Tmax: float = 1e3 * co.eV * 2 ** 18,
                       n: int = 3) -> ChebContinuumLoss:
    """ChebContinuumLoss(ContinuumLoss(nel, I, Tcut), Tmax, n) of air; nel counts
    14 electrons per N2 and 16 per O2."""
    nel = 14 * comp["N2"] + 16 * comp["O2"]
    return ChebContinuumLoss.build(ContinuumLoss(nel, I, Tcut), Tmax, n)


def pusher(efield, bfield=(0.0, 0.0, 0.0), cl: ChebContinuumLoss | None = None) -> RK2Pusher:
    em = ElectromagneticField(HomogeneousField(efield), HomogeneousField(bfield))
    return RK2Pusher(CombinedForcing(em, cl) if cl is not None else CombinedForcing(em))


def isotropic(n: int, kin: float, rng: np.random.Generator, particle: int = Electron) -> np.ndarray:
    """n momenta of kinetic energy `kin` with isotropic directions (SI)."""
    u = 2 * rng.random(n) - 1
    phi = 2 * np.pi * rng.random(n)
    s = np.sqrt(1 - u * u)
    d = np.stack([s * np.cos(phi), s * np.sin(phi), u], axis=1)
    return d * float(momentum_norm_from_kin(particle, kin))


@dataclass
class Workload:
    mpopl: MultiPopulation
    pusher: RK2Pusher
    dt: float
    tfinal: float
    name: str


def beam_tables(comp, efield: float, dt: float, safety: float = 1.15, cut_e: float = 10 * KEV,
                cut_p: float = 10 * KEV, ionization: str = "moller"):
    Fdt = co.elementary_charge * abs(efield) * dt
    et = collision_table_from_processes(electron_processes(comp, cut_e, ionization), Electron, Fdt, safety=safety)
    pt = collision_table_from_processes(positron_processes(comp, cut_p), Positron, Fdt, safety=safety)
    gt = collision_table_from_processes(photon_processes(comp), Photon, 0.0, safety=safety)
    return et, gt, pt


def plain_electrons(n: int = 1000, kin: float = 1 * MEV, efield: float = 1e6, dt: float = 1e-12,
                    tfinal: float = 50e-9, cut: float = 10 * KEV, seed: int = 1, capacity: int | None = None,
                    **cfg) -> Workload:
    """Electrons only in air, E along -z, n e- at the origin with momentum along
    +z (a 1e-6 y component avoids the pole of `turn`, as scripts/beam.jl:56
    does); Moller, Seltzer-Berger, screened Coulomb, continuum loss below the
    cut; bremsstrahlung photons tallied, not tracked."""
    comp = air_composition()
    Fdt = co.elementary_charge * efield * dt
    et = collision_table_from_processes(electron_processes(comp, cut), Electron, Fdt, safety=1.15)
    pn = float(momentum_norm_from_kin(Electron, kin))
    x = np.zeros((n, 3))
    p = np.tile([0.0, 1e-6 * pn, pn], (n, 1))
    arr = ParticleArrays(x, p, np.ones(n), np.zeros(n))
    cap = capacity or max(4 * n, 4096)
    electrons = Population(cap, arr, et, cut, particle=Electron)
    photons = Population(0, ParticleArrays.empty(), None, 0.0, particle=Photon, tally_only=True)
    mp = MultiPopulation(("electron", electrons), ("photon", photons), seed=seed, **cfg)
    cl = air_continuum_loss(comp, Tcut=cut)
    return Workload(mp, pusher((0.0, 0.0, -efield), cl=cl), dt, tfinal, "electrons-air-1MVm")


def avalanche(n: int = 10000, kin: float = 1 * MEV, efield: float = 5e5, dt: float = 1e-12,
              cut_e: float = 10 * KEV, cut_g: float = 5 * KEV, cut_p: float = 10 * KEV, seed: int = 0,
              capacity: int = 1 << 22, capacity_p: int | None = None, **cfg) -> Workload:
    """Mixed e-/gamma/e+ relativistic runaway avalanche in air: n e- at the
    origin, isotropic, E along -z; photons tracked through Compton,
    photoelectric and Bethe-Heitler; positrons through Bhabha, annihilation
    and Coulomb."""
    comp = air_composition()
    et, gt, pt = beam_tables(comp, efield, dt, cut_e=cut_e, cut_p=cut_p)
    rng = np.random.Generator(np.random.Philox(seed))
    p = isotropic(n, kin, rng)
    arr = ParticleArrays(np.zeros((n, 3)), p, np.ones(n), np.zeros(n))
    capp = capacity_p or max(capacity // 8, 4096)
    electrons = Population(capacity, arr, et, cut_e, particle=Electron)
    photons = Population(capacity, ParticleArrays.empty(), gt, cut_g, particle=Photon)
    positrons = Population(capp, ParticleArrays.empty(), pt, cut_p, particle=Positron)
    mp = MultiPopulation(("electron", electrons), ("photon", photons), ("positron", positrons), seed=seed, **cfg)
    cl = air_continuum_loss(comp, Tcut=cut_e)
    return Workload(mp, pusher((0.0, 0.0, -efield), cl=cl), dt, 1.0, "rrea-air-0.5MVm")


RREA_STATE_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "rrea_mixed_0.5MVm.json")
_RECIPES = {}


def rrea_recipe(path: str | None = None) -> dict:
    """The recipe of the grown mixed avalanche at 0.5 MV/m (written by
    data/grow_rrea.py): per-species fractions and (log10 E, cos theta_z)
    histograms of the state reached from 10^4 seed electrons."""
    path = path or RREA_STATE_PATH
    if path not in _RECIPES:
        with open(path) as f:
            _RECIPES[path] = json.load(f)
    return _RECIPES[path]


def rrea_species_counts(n_total: int, path: str | None = None):
    """Particles per species (electron, photon, positron) for a sample of
    n_total: each species' share of the grown state, rounded down, the
    remainder to the electrons."""
    rec = rrea_recipe(path)
    fr = [rec["species"][k]["fraction"] for k in ("electron", "photon", "positron")]
    counts = [0, int(n_total * fr[1]), int(n_total * fr[2])]
    counts[0] = int(n_total) - counts[1] - counts[2]
    return counts


def rrea_mixed_state(n_total: int, seed: int = 0, path: str | None = None) -> dict:
    """n_total particles drawn from the grown avalanche's recipe (Philox
    seed): species in the recorded fractions, each particle's cell of the
    (log10 E, cos theta_z) histogram drawn by its count, E and cos theta
    uniform within the cell, azimuth uniform, positions normal with the
    recorded mean and spread, weight 1, t = 0; no energy below the species'
    cut.  Returns {species: ParticleArrays}."""
    rec = rrea_recipe(path)
    rng = np.random.Generator(np.random.Philox(seed))
    le = np.asarray(rec["log10_energy_eV_edges"])
    ce = np.asarray(rec["cos_theta_z_edges"])
    out = {}
    for sp, name, m in zip((Electron, Photon, Positron), ("electron", "photon", "positron"),
                           rrea_species_counts(n_total, path)):
        d = rec["species"][name]
        cells = np.asarray(d["cells"], dtype=np.int64).reshape(-1, 3)
        if m == 0 or len(cells) == 0:
            out[sp] = ParticleArrays.empty()
            continue
        w = cells[:, 2].astype(np.float64)
        cdf = np.cumsum(w)
        idx = np.minimum(np.searchsorted(cdf, rng.random(m) * cdf[-1], side="right"), len(cells) - 1)
        iE, ic = cells[idx, 0], cells[idx, 1]
        # within a cell, energies start at the species' cut (the state has none below it)
        lo = np.maximum(le[iE], np.log10(rec["growth"]["cuts_eV"][name]))
        lg = lo + rng.random(m) * (le[iE + 1] - lo)
        cz = ce[ic] + rng.random(m) * (ce[ic + 1] - ce[ic])
        phi = 2 * np.pi * rng.random(m)
        pn = momentum_norm_from_kin(sp, 10.0 ** lg * co.eV)
        st = np.sqrt(np.maximum(0.0, 1 - cz * cz))
        p = np.stack([st * np.cos(phi), st * np.sin(phi), cz], axis=1) * pn[:, None]
        x = np.asarray(d["x_mean_m"]) + rng.standard_normal((m, 3)) * np.asarray(d["x_std_m"])
        out[sp] = ParticleArrays(x, p, np.ones(m), np.zeros(m))
    return out


def rrea_mixed(n_total: int = 1 << 24, seed: int = 0, dt: float = 1e-12, efield: float = 5e5,
               path: str | None = None, tables=None, **cfg) -> Workload:
    """The mixed avalanche at 0.5 MV/m started from n_total particles drawn
    from the grown state's recipe (rrea_mixed_state): the 2^24-particle point
    of the avalanche with its grown e- / gamma / e+ mix and spectra.
    Capacities leave room for the growth of a few hundred steps."""
    comp = air_composition()
    et, gt, pt = tables if tables is not None else beam_tables(comp, efield, dt)
    st = rrea_mixed_state(n_total, seed, path)
    ne, ng, npos = (len(st[s]) for s in (Electron, Photon, Positron))
    mp = MultiPopulation(
        ("electron", Population(int(ne * 1.25) + (1 << 16), st[Electron], et, 10 * KEV, particle=Electron)),
        ("photon", Population(int(ng * 1.25) + (1 << 20), st[Photon], gt, 5 * KEV, particle=Photon)),
        ("positron", Population(int(npos * 1.5) + (1 << 16), st[Positron], pt, 10 * KEV, particle=Positron)),
        seed=seed, **cfg)
    cl = air_continuum_loss(comp)
    return Workload(mp, pusher((0.0, 0.0, -efield), cl=cl), dt, 1.0, "rrea-air-0.5MVm-mixed")


def reid_table(density: float, emax: float = 8.0 * co.eV, n: int = 4001, mass_ratio: float = 4e-3):
    """Reid's ramp model gas: elastic sigma = 6e-20 m^2 (constant), inelastic
    sigma = 10e-20 (eps - 0.2 eV)/eV m^2 above a 0.2 eV threshold, on a linear
    grid [0, emax] with the constant majorant of load_lxcat."""
    thr = 0.2 * co.eV
    el = (Elastic(mass_ratio), density, lambda E: np.full_like(E, 6e-20))
    ex = (Excitation(thr), density, lambda E: np.where(E > thr, 10e-20 * (E - thr) / co.eV, 0.0))
    return lxcat_table([el, ex], (0.0, emax, n))


def reid_ramp(n: int = 1 << 20, EN_Td: float = 12.0, density: float = 2.504e25, dt: float = 1e-12, seed: int = 2,
              mean_energy: float = 1.0 * co.eV, emax: float = 8.0 * co.eV, **cfg) -> Workload:
    """Low-energy swarm in Reid's ramp model gas: n electrons with a Maxwellian of
    the given mean energy, field E = (E/N) N along -z, no energy cut."""
    tab = reid_table(density, emax)
    rng = np.random.Generator(np.random.Philox(seed))
    kT = 2.0 / 3.0 * mean_energy
    p = rng.normal(scale=np.sqrt(co.electron_mass * kT), size=(n, 3))
    arr = ParticleArrays(np.zeros((n, 3)), p, np.ones(n), np.zeros(n))
    electrons = Population(n + n // 8, arr, tab, 0.0, particle=Electron)
    mp = MultiPopulation(("electron", electrons), seed=seed, **cfg)
    E = EN_Td * co.Td * density
    return Workload(mp, pusher((0.0, 0.0, -E)), dt, 1.0, f"reid-ramp-{EN_Td:g}Td")


@dataclass
class SwarmBatch:
    mpopl: MultiPopulation
    pusher: RK2Pusher
    dt: float
    E: np.ndarray          # [nswarm] field magnitudes (V/m, along -z)
    n0: np.ndarray         # [nswarm] initial electrons
    tables: tuple          # (electron, photon, positron) tables of the batch
    arrays: list           # per-swarm initial ParticleArrays (electrons)


def swarm_initial(nswarm: int = 256, e_range=(3e5, 3e6), n_range=(1e2, 1e5), seed: int = 3, kin: float = 1 * MEV):
    """Fields log-spaced over e_range, initial sizes log-uniform over n_range
    (Philox seed), electrons at `kin` with isotropic directions at the origin;
    stream ids carry the swarm in their top 8 bits."""
    rng = np.random.Generator(np.random.Philox(seed))
    E = np.geomspace(e_range[0], e_range[1], nswarm)
    n0 = np.exp(rng.uniform(np.log(n_range[0]), np.log(n_range[1]), nswarm)).astype(int)
    arrays = []
    for s in range(nswarm):
        p = isotropic(int(n0[s]), kin, rng)
        sid = (np.uint64(s) << np.uint64(56)) | np.arange(n0[s], dtype=np.uint64)
        arrays.append(ParticleArrays(np.zeros((n0[s], 3)), p, np.ones(n0[s]), np.zeros(n0[s]), sid=sid))
    return E, n0, arrays


def swarm_batch(nswarm: int = 256, e_range=(3e5, 3e6), n_range=(1e2, 1e5), seed: int = 3, dt: float = 1e-12,
                swarms=None, growth: float = 1.5, tables=None, initial=None, **cfg) -> SwarmBatch:
    """`nswarm` independent avalanche swarms in one context (swarm mode): each
    has its own field and rate bound; photons and positrons are tracked as in
    the mixed avalanche.  ``swarms`` restricts the batch to a subset (e.g. one
    swarm run alone); ``tables`` and ``initial`` reuse what an earlier call
    built (the rates do not depend on the field, only the rate bound does, and
    swarm mode replaces that per swarm)."""
    comp = air_composition()
    E, n0, arrays = initial if initial is not None else swarm_initial(nswarm, e_range, n_range, seed)
    sel = list(range(nswarm)) if swarms is None else list(swarms)
    Fdt = co.elementary_charge * E * dt
    et, gt, pt = tables if tables is not None else beam_tables(comp, float(E[sel[0]]), dt)
    x = np.concatenate([arrays[s].x for s in sel]); p = np.concatenate([arrays[s].p for s in sel])
    sid = np.concatenate([arrays[s].sid for s in sel])
    n = len(sid)
    arr = ParticleArrays(x, p, np.ones(n), np.zeros(n), sid=sid)
    cap = int(growth * n) + (1 << 14)
    mp = MultiPopulation(("electron", Population(cap, arr, et, 10 * KEV, particle=Electron)),
                         ("photon", Population(max(cap // 2, 1 << 14), ParticleArrays.empty(), gt, 5 * KEV,
                                               particle=Photon)),
                         ("positron", Population(max(cap // 16, 1 << 12), ParticleArrays.empty(), pt, 10 * KEV,
                                                 particle=Positron)),
                         seed=seed, **cfg)
    Evec = np.zeros((nswarm, 3))
    Evec[:, 2] = -E
    # a subset keeps its swarm ids: all swarms are described, the subset populated
    mp.set_swarms(Evec, Fdt, safety=1.15)
    cl = air_continuum_loss(comp)
    return SwarmBatch(mp, pusher((0.0, 0.0, -float(E[sel[0]])), cl=cl), dt, E, n0, (et, gt, pt), arrays)
