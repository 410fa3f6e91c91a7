"""Collision tables and continuum losses: thin wrappers over the library's
FP64 host builders, with the reference's names and keyword defaults."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Sequence

import numpy as np

from . import _lib
from . import constants as co

Electron, Photon, Positron = _lib.ELECTRON, _lib.PHOTON, _lib.POSITRON
PARTICLE_NAMES = {Electron: "electron", Photon: "photon", Positron: "positron"}


def speed(particle: int, eng):
    """speed(::Type{P}, eng) (electron.jl:47, positron.jl:34, photon.jl:46)."""
    if particle == Photon:
        return co.c * np.ones_like(np.asarray(eng, dtype=float))
    return co.c * np.sqrt(1 - (co.electron_mc2 / (co.electron_mc2 + np.asarray(eng))) ** 2)


def momentum_norm_from_kin(particle: int, kin):
    """momentum_norm_from_kin (electron.jl:51, photon.jl:47)."""
    kin = np.asarray(kin, dtype=float)
    if particle == Photon:
        return kin / co.c
    return np.sqrt((kin + co.electron_mc2) ** 2 - co.electron_mc2 ** 2) / co.c


@dataclass
class BinaryIntervals:
    """BinaryIntervals(k, xmax) (cheby.jl:15-21)."""
    k: int
    xmax: float

    def interval(self, i: int):
        if i == 0:
            l, _ = self.interval(1)
            return 0.0, l
        l = 2.0 ** (i - self.k - 1)
        return l * self.xmax, 2 * l * self.xmax


def precheb(x, b: BinaryIntervals, n: int):
    """precheb (cheby.jl:127-143) for scalar x: (interval, (T_0..T_{n-1}))."""
    x1 = x / b.xmax
    s, l = np.frexp(x1)
    i = 0 if x1 == 0 else int(l) + b.k
    if i > 0:
        xi = 4 * s - 3
    else:
        xi = 2.0 ** (b.k + 1) * x1 - 1
        i = 0
    t = [1.0, xi][:n]
    while len(t) < n:
        t.append(2 * xi * t[-1] - t[-2])
    return i, tuple(t)


@dataclass
class ChebyshevCollisionTable:
    """ChebyshevCollisionTable (collision_table.jl:63-106): processes in table
    order, binary intervals, rate a[k, j, i] and ratebound[k, i] (SI, 1/s)."""
    proc: tuple
    coef: np.ndarray
    b: BinaryIntervals
    order: int
    rate: np.ndarray          # flat, a[k + order*(j + nproc*i)]
    ratebound: np.ndarray     # flat, rb[k + order*i]
    perm: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    particle: int = Electron

    def __len__(self):
        return len(self.proc)

    @property
    def nproc(self):
        return len(self.proc)

    def rate_array(self) -> np.ndarray:
        """a as an array indexed [k, j, i]."""
        return self.rate.reshape(self.b.k + 1, self.nproc, self.order).transpose(2, 1, 0)

    def rate_at(self, j: int, eng: float) -> float:
        i, t = precheb(eng, self.b, self.order)
        a = self.rate_array()
        return float(sum(a[q, j, i] * t[q] for q in range(self.order)))

    def ratebound_at(self, eng: float) -> float:
        i, t = precheb(eng, self.b, self.order)
        rb = self.ratebound.reshape(self.b.k + 1, self.order)
        return float(sum(rb[i, q] * t[q] for q in range(self.order)))

    def c_procs(self):
        arr = (_lib.Process * max(1, self.nproc))()
        for j, (cf, p) in enumerate(zip(self.coef, self.proc)):
            arr[j] = p.to_c(float(cf))
        return arr


def collision_table_from_processes(processes, particle: int, Fdt: float, *, safety: float = 1.1,
                                   nintervals: int = 32, order: int = 3,
                                   max_energy: float = 1e3 * co.eV * 2 ** 18) -> ChebyshevCollisionTable:
    """collision_table_from_processes(processes, particle, Fdt; safety,
    nintervals, order, max_energy) (collision_table.jl:115-149).
    ``processes`` is a list of ``(coef, process)``."""
    n = len(processes)
    procs = (_lib.Process * max(1, n))()
    for j, (cf, p) in enumerate(processes):
        procs[j] = p.to_c(float(cf))
    rate = np.zeros(order * max(1, n) * (nintervals + 1))
    rb = np.zeros(order * (nintervals + 1))
    perm = np.zeros(max(1, n), dtype=np.int32)
    rc = _lib.lib().pcl_build_collision_table(int(particle), n, procs, float(Fdt), float(safety), int(nintervals),
                                              int(order), float(max_energy), _lib.dptr(rate), _lib.dptr(rb),
                                              _lib.i32ptr(perm))
    _lib.check(rc, None, "pcl_build_collision_table")
    perm = perm[:n]
    return ChebyshevCollisionTable(proc=tuple(processes[p][1] for p in perm),
                                   coef=np.array([processes[p][0] for p in perm], dtype=np.float64),
                                   b=BinaryIntervals(nintervals, float(max_energy)), order=order,
                                   rate=rate[:order * n * (nintervals + 1)] if n else np.zeros(0), ratebound=rb,
                                   perm=perm, particle=particle)


@dataclass
class ContinuumLoss:
    """ContinuumLoss(nel, I, Tcut) (continuum.jl:6-15)."""
    nel: float
    I: float
    Tcut: float


@dataclass
class ChebContinuumLoss:
    """ChebContinuumLoss(cl, Tmax, n) (continuum.jl:25-43): Chebyshev fits of the
    restricted stopping power of electrons (ec) and positrons (pc), [n][k+1]."""
    bints: BinaryIntervals
    ec: np.ndarray
    pc: np.ndarray
    n: int

    @classmethod
    def build(cls, cl: ContinuumLoss, Tmax: float, n: int) -> "ChebContinuumLoss":
        cap = n * 64
        ec = np.zeros(cap)
        pc = np.zeros(cap)
        k = C.c_int(0)
        xmax = C.c_double(0)
        rc = _lib.lib().pcl_build_continuum_loss(float(cl.nel), float(cl.I), float(cl.Tcut), float(Tmax), int(n),
                                                 C.byref(k), C.byref(xmax), _lib.dptr(ec), _lib.dptr(pc), cap)
        _lib.check(rc, None, "pcl_build_continuum_loss")
        m = n * (k.value + 1)
        return cls(BinaryIntervals(k.value, xmax.value), ec[:m].copy(), pc[:m].copy(), n)

    def force_magnitude(self, particle: int, eng: float) -> float:
        a = (self.ec if particle == Electron else self.pc).reshape(self.bints.k + 1, self.n)
        i, t = precheb(eng, self.bints, self.n)
        return float(sum(a[i, q] * t[q] for q in range(self.n)))


@dataclass
class CollisionTable:
    """CollisionTable (collision_table.jl:15-57): rates of processes j on the linear
    energy grid LinRange(e0, e1, n), rate[j, k] (1/s), and a rate bound that is one
    number or one value per grid point."""
    proc: tuple
    energy: tuple            # (e0, e1, n) in J
    rate: np.ndarray         # (nproc, n)
    ratebound: np.ndarray    # (1,) or (n,)
    particle: int = Electron

    def __len__(self):
        return len(self.proc)

    @property
    def nproc(self):
        return len(self.proc)

    def grid(self) -> np.ndarray:
        e0, e1, n = self.energy
        i = np.arange(n)
        return (e0 * (n - 1 - i) + e1 * i) / (n - 1)

    def c_procs(self):
        arr = (_lib.Process * max(1, self.nproc))()
        for j, p in enumerate(self.proc):
            arr[j] = p.to_c(1.0)
        return arr


def lxcat_table(entries: Sequence, energy: tuple, null: bool = True, particle: int = Electron) -> CollisionTable:
    """A linear-grid table built the way load_lxcat builds one (lxcat.jl:17-134):
    nu_j = density_j * v * sigma_j(E) with v = sqrt(2 E / m) on the grid, a
    NullCollision filling up to the maximum total rate, which is the constant
    rate bound, and the processes ordered by their rate summed over the grid
    (descending).  ``entries`` are ``(process, density, sigma)`` with
    ``sigma(E)`` in m^2 for energies in J."""
    e0, e1, n = energy
    i = np.arange(n)
    E = (e0 * (n - 1 - i) + e1 * i) / (n - 1)
    v = np.sqrt(2 * E / co.electron_mass)
    procs = [p for p, _, _ in entries]
    rate = np.array([dens * v * np.asarray(sig(E), dtype=float) for _, dens, sig in entries])
    total = rate.sum(axis=0)
    maxrate = float(total.max())
    if null:
        from .processes import NullCollision
        procs.append(NullCollision())
        rate = np.vstack([rate, maxrate - total])
    perm = sorted(range(len(procs)), key=lambda j: -float(rate[j].sum()))
    return CollisionTable(tuple(procs[j] for j in perm), (float(e0), float(e1), int(n)),
                          np.ascontiguousarray(rate[perm]), np.array([maxrate]), particle)


def ratebound_split(tab: ChebyshevCollisionTable, safety: float = 1.1):
    """(A, B) with compratebound(Fdt) = A + Fdt B (collision_table.jl:152-167),
    each [order][k+1] flat like ``tab.ratebound``."""
    nI = tab.b.k + 1
    A = np.zeros(tab.order * nI)
    B = np.zeros(tab.order * nI)
    rate = np.ascontiguousarray(tab.rate) if tab.nproc else np.zeros(1)
    rc = _lib.lib().pcl_ratebound_split(int(tab.particle), tab.order, tab.nproc, tab.b.k, tab.b.xmax,
                                        _lib.dptr(rate), float(safety), _lib.dptr(A), _lib.dptr(B))
    _lib.check(rc, None, "pcl_ratebound_split")
    return A, B


@dataclass
class LXCatSet:
    """What load_lxcat returns (lxcat.jl:17-134): processes and their rates
    (nproc x len(energy), the null process included, sorted by the rate summed
    over the grid, descending), the maximum total rate (the rate bound) and the
    permutation back to the reading order."""
    proc: tuple
    rate: np.ndarray
    maxrate: float
    origperm: np.ndarray


def load_lxcat(fnames, densities: dict, energy, photon_weight: float = 1.0,
               photon_multiplier: float = 1.0) -> LXCatSet:
    """load_lxcat(fnames, densities, energy; photon_weight, photon_multiplier)
    (lxcat.jl:17-134).  Reads LXCat-style JSON files (a list of items with
    target, kind, data [[E (eV), sigma (m^2)], ...], comment, and optional
    rescale / weight_scale / threshold / mass_ratio), keeps the targets with a
    density, interpolates each cross section linearly in energy (flat outside
    its data) onto `energy` (J), scales by density and speed v = sqrt(2 E / m),
    turns EFFECTIVE into ELASTIC by subtracting the target's excitation and
    ionization rates (ensure_elastic, lxcat.jl:146-156) and adds the null
    process up to the maximum total rate.  Targets are taken in reading order
    (the reference iterates a Dict; the final order only depends on it for
    equal summed rates).  PHOTOEMISSION items need the slow-electron photon
    model, which has no device implementation, and are rejected."""
    import json
    from .processes import Elastic, Excitation, Ionization, Attachment, NullCollision
    if isinstance(fnames, (str, bytes)):
        fnames = [fnames]
    db = []
    for fn in fnames:
        with open(fn) as f:
            db.extend(json.load(f))
    energy = np.asarray(energy, dtype=float)
    v = np.sqrt(2 * energy / co.electron_mass)
    targets: dict = {}
    for item in db:
        dens = float(densities.get(item["target"], 0.0))
        if dens == 0.0:
            continue
        e0 = np.array([q[0] for q in item["data"]], dtype=float) * co.eV
        cs0 = np.array([q[1] for q in item["data"]], dtype=float)
        if "3-body" in item.get("comment", ""):
            cs0 = cs0 * densities[item["target"]] / co.centi ** -3
        if "rescale" in item:
            cs0 = cs0 * item["rescale"]
        if "weight_scale" in item:
            cs0 = cs0 * item["weight_scale"]
        if item["kind"] == "PHOTOEMISSION":
            # the reference draws a photon count for it (slow-electron.jl:141-144)
            # into a MultiplePhotonOutcome that no apply! method takes
            # (collisions.jl:79-130), so a PHOTOEMISSION collision cannot
            # complete there: there is no behaviour to reproduce
            raise NotImplementedError("PHOTOEMISSION: the reference has no apply! for its MultiplePhotonOutcome "
                                      "(collisions.jl:79-130); not reproduced")
        it = dict(item)
        it["nu"] = dens * v * np.interp(energy, e0, cs0)
        targets.setdefault(item["target"], []).append(it)
    kinds = {"ATTACHMENT": lambda itm: Attachment(itm.get("threshold", 0.0) * co.eV),
             "EXCITATION": lambda itm: Excitation(itm["threshold"] * co.eV),
             "IONIZATION": lambda itm: Ionization(itm["threshold"] * co.eV),
             "ELASTIC": lambda itm: Elastic(itm["mass_ratio"])}
    procs, rows = [], []
    for name, ps in targets.items():
        for p in ps:  # ensure_elastic
            if p["kind"] != "EFFECTIVE":
                continue
            for p2 in ps:
                if p2 is not p and p2["kind"] in ("EXCITATION", "IONIZATION"):
                    p["nu"] = p["nu"] - p2["nu"]
            p["kind"] = "ELASTIC"
        for p in ps:
            procs.append(kinds[p["kind"]](p))
            rows.append(p["nu"])
    rate = np.array(rows) if rows else np.zeros((0, len(energy)))
    total = rate.sum(axis=0)
    maxrate = float(total.max()) if len(rows) else 0.0
    procs.append(NullCollision())
    rate = np.vstack([rate, maxrate - total])
    inteng = rate.sum(axis=1)
    perm = sorted(range(len(procs)), key=lambda j: -inteng[j])
    origperm = np.argsort(perm)
    return LXCatSet(tuple(procs[j] for j in perm), np.ascontiguousarray(rate[perm]), maxrate, origperm)


def lxcat_collision_table(fnames, densities: dict, energy, particle: int = Electron, **kw) -> CollisionTable:
    """CollisionTable on the linear grid `energy` (equally spaced, J) from
    load_lxcat, with its maximum total rate as the constant rate bound."""
    energy = np.asarray(energy, dtype=float)
    n = len(energy)
    step = (energy[-1] - energy[0]) / (n - 1)
    if not np.allclose(np.diff(energy), step, rtol=1e-9, atol=0.0):
        raise ValueError("the energy grid must be equally spaced")
    r = load_lxcat(fnames, densities, energy, **kw)
    return CollisionTable(r.proc, (float(energy[0]), float(energy[-1]), n), r.rate, np.array([r.maxrate]), particle)
