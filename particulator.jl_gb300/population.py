"""Populations and the step/run API (population.jl, mixed_population.jl,
run.jl, callback.jl), backed by the device context of the C ABI.

Names follow the reference; Julia's `!` suffix is dropped (``advance`` is
``advance!``, ``run`` is ``run!``, ``init`` is ``init!``).
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from . import _lib
from . import constants as co
from .forcing import RK2Pusher
from .tables import Electron, Photon, Positron, PARTICLE_NAMES, ChebyshevCollisionTable, CollisionTable

SPECIES_BY_NAME = {"electron": Electron, "photon": Photon, "positron": Positron}


@dataclass
class _State:
    x: tuple
    p: tuple
    w: float = 1.0
    t: float = 0.0
    s: float | None = None   # None: s = nextcoll() drawn from the particle's stream


class ElectronState(_State):
    """ElectronState(x, p, w=1, t=0) (electron.jl:13-34)."""
    particle = Electron


class PhotonState(_State):
    """PhotonState(x, p, w=1, t=0) (photon.jl:6-33)."""
    particle = Photon


class PositronState(_State):
    """PositronState(x, p, w=1, t=0) (positron.jl:3-22)."""
    particle = Positron


@dataclass
class ParticleArrays:
    """A structure-of-arrays batch of particle states (SI units)."""
    x: np.ndarray
    p: np.ndarray
    w: np.ndarray
    t: np.ndarray
    s: np.ndarray | None = None
    sid: np.ndarray | None = None
    ctr: np.ndarray | None = None

    def __len__(self):
        return len(self.w)

    @classmethod
    def from_states(cls, states):
        n = len(states)
        x = np.array([st.x for st in states], dtype=np.float64).reshape(n, 3)
        p = np.array([st.p for st in states], dtype=np.float64).reshape(n, 3)
        w = np.array([st.w for st in states], dtype=np.float64)
        t = np.array([st.t for st in states], dtype=np.float64)
        s = None
        if n and all(st.s is not None for st in states):
            s = np.array([st.s for st in states], dtype=np.float64)
        return cls(x, p, w, t, s)

    @classmethod
    def empty(cls):
        return cls(np.zeros((0, 3)), np.zeros((0, 3)), np.zeros(0), np.zeros(0))


def kinenergy(particle: int, p) -> np.ndarray:
    """kinenergy for an (n, 3) array of SI momenta (electron.jl:53, photon.jl:50)."""
    p = np.asarray(p, dtype=np.float64)
    p2 = np.sum(p * p, axis=-1)
    if particle == Photon:
        return np.sqrt(p2) * co.c
    q = p2 / co.electron_mc ** 2
    return co.electron_mc2 * q / (np.sqrt(1 + q) + 1)


class Population:
    """Population(max_particles, inparticles, collisions, energy_cut)
    (population.jl:7-44).  ``inparticles`` is a list of states or a
    ``ParticleArrays``.  ``tally_only=True`` makes a population whose
    secondaries are counted and binned but not stored."""

    def __init__(self, max_particles: int, inparticles, collisions: ChebyshevCollisionTable | None,
                 energy_cut: float = 0.0, *, particle: int | None = None, tally_only: bool = False,
                 sid_base: int | None = None):
        if isinstance(inparticles, ParticleArrays):
            arr = inparticles
        else:
            inparticles = list(inparticles)
            arr = ParticleArrays.from_states(inparticles) if inparticles else ParticleArrays.empty()
            if particle is None and inparticles:
                particle = inparticles[0].particle
        if particle is None:
            particle = collisions.particle if collisions is not None else Electron
        if len(arr) > max_particles:
            raise ValueError("more initial particles than max_particles")
        self.particle = particle
        self.max_particles = int(max_particles)
        self.collisions = collisions
        self.energy_cut = float(energy_cut)
        self.tally_only = tally_only
        self.sid_base = sid_base
        self._init = arr
        self._mp: MultiPopulation | None = None

    @property
    def ctx(self):
        if self._mp is None:
            raise RuntimeError("population is not part of a MultiPopulation")
        return self._mp.ctx

    def moments(self) -> np.ndarray:
        out = np.zeros(10)
        _lib.check(_lib.lib().pcl_moments(self.ctx, self.particle, _lib.dptr(out)), self.ctx, "pcl_moments")
        return out

    def energy_histogram(self, edges, swarm: int = -1):
        """Device histogram of the live particles' kinetic energies (J) over
        `edges` (pcl_energy_histogram): (counts, summed weights) per bin
        edges[i] <= E < edges[i+1], as StatsBase.fit(Histogram, ...) in the
        reference's scripts.  swarm >= 0 keeps one swarm of a batch."""
        e = np.ascontiguousarray(np.asarray(edges, dtype=float))
        nb = len(e) - 1
        counts = np.zeros(max(nb, 0), dtype=np.int64)
        w = np.zeros(max(nb, 0))
        _lib.check(_lib.lib().pcl_energy_histogram(self.ctx, self.particle, int(swarm), len(e), _lib.dptr(e),
                                                   _lib.i64ptr(counts), _lib.dptr(w)), self.ctx,
                   "pcl_energy_histogram")
        return counts, w

    def particles(self) -> ParticleArrays:
        """Download the live particles (SI)."""
        L = _lib.lib()
        n = C.c_int64(self.max_particles)
        x = np.zeros((self.max_particles, 3)); p = np.zeros((self.max_particles, 3))
        w = np.zeros(self.max_particles); t = np.zeros(self.max_particles); s = np.zeros(self.max_particles)
        sid = np.zeros(self.max_particles, np.uint64); ctr = np.zeros(self.max_particles, np.uint32)
        if self.max_particles and not self.tally_only:
            _lib.check(L.pcl_download(self.ctx, self.particle, C.byref(n), _lib.dptr(x), _lib.dptr(p), _lib.dptr(w),
                                      _lib.dptr(t), _lib.dptr(s), _lib.u64ptr(sid), _lib.u32ptr(ctr)),
                       self.ctx, "pcl_download")
        else:
            n.value = 0
        m = n.value
        return ParticleArrays(x[:m], p[:m], w[:m], t[:m], s[:m], sid[:m], ctr[:m])


class PinnedBlock:
    """numpy arrays in one page-locked block allocated by CUDA
    (pcl_host_alloc), freed when the last array viewing it is collected."""

    def __init__(self, shapes_dtypes):
        sizes = [int(np.prod(sh)) * np.dtype(dt).itemsize for sh, dt in shapes_dtypes]
        offs = np.cumsum([0] + [(z + 4095) // 4096 * 4096 for z in sizes])
        self.ptr = C.c_void_p()
        rc = _lib.lib().pcl_host_alloc(C.byref(self.ptr), C.c_size_t(max(int(offs[-1]), 1)))
        if rc != 0:
            raise RuntimeError(f"pcl_host_alloc failed ({rc})")
        raw = (C.c_uint8 * int(offs[-1])).from_address(self.ptr.value)
        raw._owner = self   # every view keeps the block (and so the memory) alive
        base = np.frombuffer(raw, dtype=np.uint8)
        self.arrays = tuple(base[o:o + z].view(dt).reshape(sh)
                            for o, z, (sh, dt) in zip(offs[:-1], sizes, shapes_dtypes))
        for a in self.arrays:
            a[...] = 0

    def __del__(self):
        try:
            if self.ptr:
                _lib.lib().pcl_host_free(self.ptr)
                self.ptr = C.c_void_p()
        except Exception:
            pass


class PinnedHost:
    """Page-locks numpy arrays for asynchronous copies (pcl_host_register) and
    releases them when collected."""

    def __init__(self, arrays):
        self.ptrs = []
        self.arrays = arrays
        for a in arrays:
            if a.nbytes:
                rc = _lib.lib().pcl_host_register(C.c_void_p(a.ctypes.data), C.c_size_t(a.nbytes))
                if rc != 0:
                    self.release()
                    raise RuntimeError(f"pcl_host_register failed ({rc})")
                self.ptrs.append(a.ctypes.data)

    def release(self):
        for p in self.ptrs:
            _lib.lib().pcl_host_unregister(C.c_void_p(p))
        self.ptrs = []

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


# Nodes at which roulette!/split! functions of the kinetic energy are
# tabulated for the device: 4096 log-spaced energies from 1 meV to 10 GeV
# (0.73 % apart; f is linear between them, constant beyond).
ENERGY_TABLE_NODES = np.geomspace(1e-3, 1e10, 4096) * co.eV


def energy_table(f):
    """(energies in J, values) of a roulette!/split! function of the kinetic
    energy for pcl_roulette_fn / pcl_split_fn: a pair of arrays as given, or a
    callable evaluated at ENERGY_TABLE_NODES (on the array if it takes one,
    else node by node)."""
    if not callable(f):
        E, v = (np.ascontiguousarray(np.asarray(a, dtype=float)) for a in f)
        if E.ndim != 1 or E.shape != v.shape:
            raise ValueError("a table is two 1-D arrays of the same length")
        return E, v
    E = ENERGY_TABLE_NODES.copy()
    try:
        v = np.asarray(f(E), dtype=float)
        if v.shape != E.shape:
            raise ValueError
    except Exception:
        v = np.array([float(f(e)) for e in E])
    return E, np.ascontiguousarray(v)


class MultiPopulation:
    """MultiPopulation(:electron => ..., :photon => ..., :positron => ...)
    (mixed_population.jl:4-12).  Owns one device context; configuration
    keywords select the device, the Philox seed and the launch shape."""

    def __init__(self, *pairs, seed: int = 0, device: int = 0, steps_per_launch: int = 1,
                 compaction_period: int = 0, block_size: int = 0, grid_blocks: int = 0, blocks_per_sm: int = 0,
                 use_graph: bool = False, classic_step: bool = False, stash_entries: int = 0, **named):
        index = {}
        for name, pop in list(pairs) + list(named.items()):
            key = SPECIES_BY_NAME[name] if isinstance(name, str) else int(name)
            index[key] = pop
        self.index = index
        cfg = _lib.Config()
        cfg.seed = seed
        cfg.device = device
        cfg.steps_per_launch = steps_per_launch
        cfg.compaction_period = compaction_period
        cfg.block_size = block_size
        cfg.grid_blocks = grid_blocks
        cfg.blocks_per_sm = blocks_per_sm
        cfg.use_graph = 1 if use_graph else 0
        cfg.classic_step = 1 if classic_step else 0
        cfg.stash_entries = stash_entries
        self.config = cfg
        h = C.c_void_p()
        rc = _lib.lib().pcl_create(C.byref(cfg), C.byref(h))
        if rc != _lib.PCL_OK:
            raise _lib.PCLError(rc, "pcl_create failed (is a CUDA device available?)")
        self.ctx = h
        self._pusher_key = None
        self._keep = []
        sid_base = 0
        for key in sorted(index):
            pop = index[key]
            pop._mp = self
            self._configure(key, pop, sid_base)
            sid_base += pop.max_particles
        self.t = 0.0

    def _configure(self, key, pop: Population, sid_base: int):
        L = _lib.lib()
        flags = _lib.SPECIES_TALLY_ONLY if pop.tally_only else _lib.SPECIES_TRACKED
        _lib.check(L.pcl_set_species(self.ctx, key, pop.energy_cut, pop.max_particles, flags), self.ctx,
                   "pcl_set_species")
        tab = pop.collisions
        if isinstance(tab, CollisionTable):
            procs = tab.c_procs()
            self._keep.append((procs, tab))
            rate = np.ascontiguousarray(tab.rate.T)   # rate[j + nproc * k]
            rb = np.ascontiguousarray(tab.ratebound, dtype=float)
            e0, e1, n = tab.energy
            _lib.check(L.pcl_set_linear_table(self.ctx, key, tab.nproc, n, e0, e1, _lib.dptr(rate), _lib.dptr(rb),
                                              len(rb), procs), self.ctx, "pcl_set_linear_table")
        elif tab is not None:
            procs = tab.c_procs()
            self._keep.append((procs, tab))
            rate = np.ascontiguousarray(tab.rate) if tab.nproc else np.zeros(1)
            rb = np.ascontiguousarray(tab.ratebound)
            _lib.check(L.pcl_set_collision_table(self.ctx, key, tab.order, tab.nproc, tab.b.k, tab.b.xmax,
                                                 _lib.dptr(rate), _lib.dptr(rb), procs), self.ctx,
                       "pcl_set_collision_table")
        arr = pop._init
        if not pop.tally_only and len(arr):
            base = pop.sid_base if pop.sid_base is not None else sid_base
            x = np.ascontiguousarray(arr.x, dtype=np.float64).reshape(-1)
            p = np.ascontiguousarray(arr.p, dtype=np.float64).reshape(-1)
            w = np.ascontiguousarray(arr.w, dtype=np.float64)
            t = np.ascontiguousarray(arr.t, dtype=np.float64)
            s = None if arr.s is None else np.ascontiguousarray(arr.s, dtype=np.float64)
            sid = None if arr.sid is None else np.ascontiguousarray(arr.sid, dtype=np.uint64)
            _lib.check(L.pcl_upload(self.ctx, key, len(arr), _lib.dptr(x), _lib.dptr(p), _lib.dptr(w), _lib.dptr(t),
                                    _lib.dptr(s), _lib.u64ptr(sid), int(base)), self.ctx, "pcl_upload")

    def get(self, particle):
        key = SPECIES_BY_NAME[particle] if isinstance(particle, str) else int(particle)
        return self.index[key]

    def __getitem__(self, particle):
        return self.get(particle)

    def pairs(self):
        return [(PARTICLE_NAMES[k], v) for k, v in sorted(self.index.items())]

    def set_pusher(self, pusher):
        """RK2Pusher, RestrictedPusher or NullPusher (pusher.jl:37-76)."""
        E, B, cl = pusher.device_forcing()
        kind, fparams = pusher.device_efield()
        bkind, bparams = pusher.device_bfield()
        masks = tuple(int(m) for m in pusher.device_masks())
        key = (tuple(E), tuple(B), id(cl), kind, tuple(fparams), bkind, tuple(bparams), masks)
        if key == self._pusher_key:
            return
        L = _lib.lib()
        E = np.ascontiguousarray(E); B = np.ascontiguousarray(B)
        if cl is None:
            rc = L.pcl_set_forcing(self.ctx, _lib.dptr(E), _lib.dptr(B), 0, 0, 0.0, None, None)
        else:
            self._keep.append(cl)
            rc = L.pcl_set_forcing(self.ctx, _lib.dptr(E), _lib.dptr(B), cl.n, cl.bints.k, cl.bints.xmax,
                                   _lib.dptr(cl.ec), _lib.dptr(cl.pc))
        _lib.check(rc, self.ctx, "pcl_set_forcing")
        fp = np.ascontiguousarray(np.asarray(fparams, dtype=float)) if fparams else None
        _lib.check(L.pcl_set_field(self.ctx, int(kind), _lib.dptr(fp), len(fparams)), self.ctx, "pcl_set_field")
        bp = np.ascontiguousarray(np.asarray(bparams, dtype=float)) if bparams else None
        _lib.check(L.pcl_set_bfield(self.ctx, int(bkind), _lib.dptr(bp), len(bparams)), self.ctx, "pcl_set_bfield")
        _lib.check(L.pcl_set_push_mask(self.ctx, *masks), self.ctx, "pcl_set_push_mask")
        self._pusher_key = key

    def set_swarms(self, E, Fdt, safety: float = 1.15):
        """Swarm mode (pcl_set_swarms): swarm s (top 8 bits of a particle's
        stream id) feels field E[s] (V/m) and uses the rate bound for Fdt[s]."""
        E = np.ascontiguousarray(np.asarray(E, dtype=float).reshape(-1, 3))
        Fdt = np.ascontiguousarray(np.asarray(Fdt, dtype=float).reshape(-1))
        self._keep.append((E, Fdt))
        _lib.check(_lib.lib().pcl_set_swarms(self.ctx, len(Fdt), _lib.dptr(E), _lib.dptr(Fdt), float(safety)),
                   self.ctx, "pcl_set_swarms")
        self.nswarm = len(Fdt)

    def swarm_moments(self, particle, nswarm: int | None = None) -> np.ndarray:
        """Per-swarm FP64 moments [nswarm, 6]: live, sum w, sum w E (J), sum w z,
        sum w z^2, sum w (x^2 + y^2)."""
        key = SPECIES_BY_NAME[particle] if isinstance(particle, str) else int(particle)
        ns = nswarm or getattr(self, "nswarm", 1)
        out = np.zeros(6 * ns)
        _lib.check(_lib.lib().pcl_swarm_moments(self.ctx, key, ns, _lib.dptr(out)), self.ctx, "pcl_swarm_moments")
        return out.reshape(ns, 6)

    def roulette(self, particle, pkeep):
        """roulette!(pkeep, popl) (population.jl:291-311) on the device.
        pkeep: a number; a function of the kinetic energy (J), as roulette!(f,
        popl) takes it, tabulated by `energy_table`; or such a table
        (energies, keep probabilities), linear between nodes."""
        key = SPECIES_BY_NAME[particle] if isinstance(particle, str) else int(particle)
        if np.ndim(pkeep) == 0 and not callable(pkeep):
            _lib.check(_lib.lib().pcl_roulette(self.ctx, key, float(pkeep)), self.ctx, "pcl_roulette")
            return
        E, v = energy_table(pkeep)
        _lib.check(_lib.lib().pcl_roulette_fn(self.ctx, key, len(E), _lib.dptr(E), _lib.dptr(v)), self.ctx,
                   "pcl_roulette_fn")

    def roulette_swarms(self, particle, pkeep):
        """Per-swarm roulette! (pcl_roulette_swarms): keep probability pkeep[s]
        for swarm s; entries >= 1 leave a swarm untouched."""
        key = SPECIES_BY_NAME[particle] if isinstance(particle, str) else int(particle)
        q = np.ascontiguousarray(np.asarray(pkeep, dtype=float))
        _lib.check(_lib.lib().pcl_roulette_swarms(self.ctx, key, len(q), _lib.dptr(q)), self.ctx,
                   "pcl_roulette_swarms")

    def swarm_counts(self, particle, nswarm: int | None = None) -> np.ndarray:
        """Live particles of each swarm (pcl_swarm_counts); with one swarm,
        the whole population."""
        key = SPECIES_BY_NAME[particle] if isinstance(particle, str) else int(particle)
        ns = nswarm or max(1, getattr(self, "nswarm", 1))
        out = np.zeros(ns, dtype=np.int64)
        _lib.check(_lib.lib().pcl_swarm_counts(self.ctx, key, ns, _lib.i64ptr(out)), self.ctx, "pcl_swarm_counts")
        return out

    def set_swarm_cap(self, cap: int, particles=(Electron,)):
        """Device RouletteCallback per swarm (pcl_set_swarm_cap): after every
        launch group of run!, each swarm of the given species with n > cap
        live particles gets roulette!(cap / n).  cap = 0 turns it off."""
        for sp in particles:
            key = SPECIES_BY_NAME[sp] if isinstance(sp, str) else int(sp)
            _lib.check(_lib.lib().pcl_set_swarm_cap(self.ctx, key, int(cap)), self.ctx, "pcl_set_swarm_cap")

    def cap_swarms(self, cap: int, particles=(Electron, Photon, Positron)):
        """Hold every swarm of a batched context at `cap` live particles per
        species now: swarms above it get roulette!(cap / n), weights
        compensating, then the population is repacked.  Returns the per-swarm
        live counts before the cap."""
        out = {}
        cut = False
        for sp in particles:
            pop = self.index.get(sp)
            if pop is None or pop.tally_only or pop.max_particles == 0:
                continue
            n = self.swarm_counts(sp, self.nswarm).astype(float)
            out[sp] = n.copy()
            q = np.where(n > cap, cap / np.maximum(n, 1), 1.0)
            if np.any(q < 1.0):
                self.roulette_swarms(sp, q)
                cut = True
        if cut:
            _lib.check(_lib.lib().pcl_compact(self.ctx), self.ctx, "pcl_compact")
        return out

    def split(self, particle, p):
        """split!(p, popl) (population.jl:316-335) on the device.  p: a
        number; a function of the kinetic energy (J) giving the mean number of
        copies, tabulated by `energy_table` (the reference's docstring says f
        receives the energy, its code passes the particle state,
        population.jl:320: the device form covers f of the energy); or such a
        table (energies, means in [0, 64])."""
        key = SPECIES_BY_NAME[particle] if isinstance(particle, str) else int(particle)
        if np.ndim(p) == 0 and not callable(p):
            _lib.check(_lib.lib().pcl_split(self.ctx, key, float(p)), self.ctx, "pcl_split")
            return
        E, v = energy_table(p)
        _lib.check(_lib.lib().pcl_split_fn(self.ctx, key, len(E), _lib.dptr(E), _lib.dptr(v)), self.ctx,
                   "pcl_split_fn")

    def packed_buffers(self, pinned: bool = False):
        """Host buffers in the packed device layout for every species, sized to
        its capacity: [(xw float32 [cap, 4], ps float32 [cap, 4], meta uint32
        [cap, 4], owner)]; pinned=True places them in page-locked memory
        (pcl_host_alloc), freed when `owner` is collected."""
        bufs = []
        for s in (Electron, Photon, Positron):
            pop = self.index.get(s)
            cap = 0 if (pop is None or pop.tally_only) else pop.max_particles
            if pinned and cap:
                blk = PinnedBlock([((cap, 4), np.float32), ((cap, 4), np.float32), ((cap, 4), np.uint32)])
                bufs.append(blk.arrays + (blk,))
            else:
                bufs.append((np.zeros((cap, 4), np.float32), np.zeros((cap, 4), np.float32),
                             np.zeros((cap, 4), np.uint32), None))
        return bufs

    @staticmethod
    def _packed(b):
        return _lib.Packed(b[0].ctypes.data_as(C.POINTER(C.c_float)), b[1].ctypes.data_as(C.POINTER(C.c_float)),
                           b[2].ctypes.data_as(C.POINTER(C.c_uint32)))

    def download_packed(self, bufs):
        """pcl_download_packed of every species into `bufs`; returns the slot counts."""
        ns = []
        for s in (Electron, Photon, Positron):
            n = C.c_int64(len(bufs[s][0]))
            if len(bufs[s][0]):
                _lib.check(_lib.lib().pcl_download_packed(self.ctx, s, C.byref(n), C.byref(self._packed(bufs[s]))),
                           self.ctx, "pcl_download_packed")
            else:
                n.value = 0
            ns.append(int(n.value))
        return ns

    def upload_packed(self, bufs, ns):
        for s in (Electron, Photon, Positron):
            if len(bufs[s][0]):
                _lib.check(_lib.lib().pcl_upload_packed(self.ctx, s, int(ns[s]), C.byref(self._packed(bufs[s]))),
                           self.ctx, "pcl_upload_packed")

    def advance_host(self, tfinal: float, bufs, ns, out=None, nchunks: int = 8, compact: bool = False):
        """advance! of host-resident populations (pcl_advance_host): bufs[s]
        hold ns[s] slots of species s in the packed layout; the stepped
        populations are written to `out` (default: in place).  Returns the
        slot counts after the step."""
        out = bufs if out is None else out
        inp = (_lib.Packed * 3)(*[self._packed(b) for b in bufs])
        outp = (_lib.Packed * 3)(*[self._packed(b) for b in out])
        n_in = (C.c_int64 * 3)(*[int(x) for x in ns])
        n_out = (C.c_int64 * 3)()
        caps = (C.c_int64 * 3)(*[len(b[0]) for b in out])
        _lib.check(_lib.lib().pcl_advance_host(self.ctx, float(tfinal), n_in, inp, n_out, outp, caps, int(nchunks),
                                               int(bool(compact))), self.ctx, "pcl_advance_host")
        self.t = float(tfinal)
        return [int(n_out[s]) for s in range(3)]

    def set_host_io(self, mode: int):
        """How advance_host moves the population over the CPU-GPU link
        (pcl_set_host_io): 0 the library's default (the copy pipeline), 1
        copy pipeline, 2 direct (the step kernel reads and writes the
        page-locked host arrays)."""
        _lib.check(_lib.lib().pcl_set_host_io(self.ctx, int(mode)), self.ctx, "pcl_set_host_io")

    def set_learned(self, particle, proc_index: int, kind: int, net=None):
        """Attach (net) or detach (None) a learned sampler for one table
        position (pcl_set_learned)."""
        key = SPECIES_BY_NAME[particle] if isinstance(particle, str) else int(particle)
        h = net.h if net is not None else None
        if net is not None:
            self._keep.append(net)
        _lib.check(_lib.lib().pcl_set_learned(self.ctx, key, int(proc_index), int(kind), h), self.ctx,
                   "pcl_set_learned")

    def autotune(self, pusher: RK2Pusher, dt: float, steps: int = 480) -> dict:
        """Choose the launch shape (blocks per SM, steps per launch, compaction
        period, graph replay) by timing real steps of dt (pcl_autotune); the
        population advances by the steps the search uses."""
        self.set_pusher(pusher)
        r = _lib.TuneResult()
        _lib.check(_lib.lib().pcl_autotune(self.ctx, float(dt), int(steps), C.byref(r)), self.ctx, "pcl_autotune")
        t = _lib.Tallies()
        _lib.check(_lib.lib().pcl_get_tallies(self.ctx, C.byref(t)), self.ctx, "pcl_get_tallies")
        self.t = t.t
        for f in ("blocks_per_sm", "steps_per_launch", "compaction_period", "use_graph"):
            setattr(self.config, f, getattr(r, f))
        self.config.classic_step = 0 if r.blocks_per_sm == 0 else 1
        return {"blocks_per_sm": r.blocks_per_sm, "steps_per_launch": r.steps_per_launch,
                "compaction_period": r.compaction_period, "use_graph": r.use_graph, "rate": r.rate,
                "trials": r.trials, "steps": r.steps}

    def set_launch(self, blocks_per_sm: int, steps_per_launch: int, compaction_period: int, use_graph: bool):
        """Set the launch shape (pcl_set_launch); blocks_per_sm 0 selects the
        event step kernel, 2-4 the classic one."""
        _lib.check(_lib.lib().pcl_set_launch(self.ctx, int(blocks_per_sm), int(steps_per_launch),
                                             int(compaction_period), 1 if use_graph else 0), self.ctx, "pcl_set_launch")
        self.config.blocks_per_sm = blocks_per_sm
        self.config.classic_step = 0 if blocks_per_sm == 0 else 1
        self.config.steps_per_launch = steps_per_launch
        self.config.compaction_period = compaction_period
        self.config.use_graph = 1 if use_graph else 0

    def learn_stats(self):
        """(collisions answered by a network, learned rounds) so far."""
        a, b = C.c_int64(), C.c_int64()
        _lib.check(_lib.lib().pcl_learn_stats(self.ctx, C.byref(a), C.byref(b)), self.ctx, "pcl_learn_stats")
        return a.value, b.value

    def tallies(self) -> _lib.Tallies:
        t = _lib.Tallies()
        _lib.check(_lib.lib().pcl_get_tallies(self.ctx, C.byref(t)), self.ctx, "pcl_get_tallies")
        return t

    def close(self):
        if getattr(self, "ctx", None):
            _lib.lib().pcl_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------ callbacks --
class AbstractCallback:
    """Hook protocol (callback.jl:15-35).  Device-side callbacks only: the
    built-ins below; arbitrary Python hooks run on the host between steps."""

    def onstep(self, mpopl, t):
        return True

    def onoutput(self, mpopl, t, i):
        return None


class VoidCallback(AbstractCallback):
    pass


class CombinedCallback(AbstractCallback):
    """CombinedCallback((a, b, ...)) (callback.jl:41-108)."""

    def __init__(self, tpl):
        self.tpl = tuple(tpl)

    def onstep(self, mpopl, t):
        ok = True
        for c in self.tpl:
            ok = c.onstep(mpopl, t) and ok
        return ok

    def onoutput(self, mpopl, t, i):
        for c in self.tpl:
            c.onoutput(mpopl, t, i)


class CollisionCounter(AbstractCallback):
    """CollisionCounter (callback.jl:118-141): per-process collision counts,
    tallied on the device; ``counts(mpopl)`` maps (species, process) -> count."""

    def counts(self, mpopl):
        t = mpopl.tallies()
        out = {}
        for key, pop in mpopl.index.items():
            if pop.collisions is None:
                continue
            for j, proc in enumerate(pop.collisions.proc):
                out[(PARTICLE_NAMES[key], j, type(proc).__name__)] = t.collisions[key][j]
            out[(PARTICLE_NAMES[key], -1, "NullCollision")] = t.nulls[key]
        return out


class PopulationTargetCallback(AbstractCallback):
    """PopulationTargetCallback{S}(n, ismax) (callback.jl:253-267)."""

    def __init__(self, particle, n: int, ismax: bool = True):
        self.particle = SPECIES_BY_NAME[particle] if isinstance(particle, str) else int(particle)
        self.n = int(n)
        self.ismax = ismax

    def onstep(self, mpopl, t):
        live = mpopl.tallies().live[self.particle]
        return live < self.n if self.ismax else live > self.n


class RouletteCallback(AbstractCallback):
    """RouletteCallback(m) (callback.jl:210-227): after every step, each
    population with more than m active particles gets roulette!(m / n), then
    every population is repacked."""

    def __init__(self, m: int):
        self.m = int(m)

    def onstep(self, mpopl, t):
        for key, pop in mpopl.index.items():
            if pop.tally_only or pop.max_particles == 0:
                continue
            n = nactives(pop)
            if n > self.m:
                mpopl.roulette(key, self.m / n)
        _lib.check(_lib.lib().pcl_compact(mpopl.ctx), mpopl.ctx, "pcl_compact")
        return True


class SplitCallback(AbstractCallback):
    """SplitCallback{S}(m, min_frac) (callback.jl:230-247): after every step,
    if population S has fewer than m * min_frac active particles it gets
    split!(m / n - 1), then is repacked."""

    def __init__(self, particle, m: int, min_frac: float):
        self.particle = SPECIES_BY_NAME[particle] if isinstance(particle, str) else int(particle)
        self.m = int(m)
        self.min_frac = float(min_frac)

    def onstep(self, mpopl, t):
        n = nactives(mpopl.get(self.particle))
        if 0 < n < self.m * self.min_frac:
            mpopl.split(self.particle, self.m / n - 1)
        _lib.check(_lib.lib().pcl_compact(mpopl.ctx), mpopl.ctx, "pcl_compact")
        return True


class WallCallback(AbstractCallback):
    """WallCallback{P}(coord, v, drop=true) (callback.jl:146-184): particles
    of `particle` crossing the plane x[coord] = v (coord 1-3 as in Julia) in
    the +axis direction are recorded, interpolated to the wall, and dropped if
    `drop`.  Crossings are detected on the device during the step; `accum`
    collects them (ParticleArrays with stream ids) after every device run."""

    def __init__(self, particle, coord: int, v: float, drop: bool = True, capacity: int = 1 << 20):
        self.particle = SPECIES_BY_NAME[particle] if isinstance(particle, str) else int(particle)
        if coord not in (1, 2, 3):
            raise ValueError("coord is 1, 2 or 3")
        self.coord, self.v, self.drop, self.capacity = int(coord), float(v), bool(drop), int(capacity)
        self.accum = []
        self.t = []

    def attach(self, mpopl):
        _lib.check(_lib.lib().pcl_set_wall(mpopl.ctx, self.particle, self.coord - 1, self.v, 1 if self.drop else 0,
                                           self.capacity), mpopl.ctx, "pcl_set_wall")

    def collect(self, mpopl):
        L = _lib.lib()
        n = C.c_int64(0)
        _lib.check(L.pcl_get_wall(mpopl.ctx, C.byref(n), None, None, None, None, None, None), mpopl.ctx,
                   "pcl_get_wall")
        m = n.value
        if m == 0:
            return
        sp = np.zeros(m, np.int32); sid = np.zeros(m, np.uint64)
        x = np.zeros((m, 3)); p = np.zeros((m, 3)); w = np.zeros(m); t = np.zeros(m)
        _lib.check(L.pcl_get_wall(mpopl.ctx, C.byref(n), _lib.i32ptr(sp), _lib.u64ptr(sid), _lib.dptr(x),
                                  _lib.dptr(p), _lib.dptr(w), _lib.dptr(t)), mpopl.ctx, "pcl_get_wall")
        sel = sp == self.particle
        self.accum.append(ParticleArrays(x[sel], p[sel], w[sel], t[sel], None, sid[sel]))

    def states(self) -> ParticleArrays:
        if not self.accum:
            return ParticleArrays.empty()
        return ParticleArrays(*[np.concatenate([getattr(a, f) for a in self.accum]) for f in ("x", "p", "w", "t")],
                              None, np.concatenate([a.sid for a in self.accum]))


class ParticleCountCallback(AbstractCallback):
    """ParticleCountCallback(particles) (callback.jl:190-204): total weight of
    each listed species at every output time."""

    def __init__(self, particles):
        self.p = [SPECIES_BY_NAME[s] if isinstance(s, str) else int(s) for s in particles]
        self.counts = []

    def onoutput(self, mpopl, t, i):
        self.counts.append([t] + [weight(mpopl.get(s)) for s in self.p])


# ---------------------------------------------------------------- stepping --
def init(mpopl: MultiPopulation):
    """init! (mixed_population.jl:20-35): the rate bounds are set on the
    device at the start of every step, so there is nothing to do here."""
    return None


def advance(mpopl: MultiPopulation, pusher: RK2Pusher, tfinal: float, callback=None):
    """advance!(mpopl, pusher, tfinal, callback) followed by droplow! on every
    population (mixed_population.jl:38-47, run.jl:7): one device step."""
    mpopl.set_pusher(pusher)
    _lib.check(_lib.lib().pcl_advance(mpopl.ctx, float(tfinal)), mpopl.ctx, "pcl_advance")
    mpopl.t = float(tfinal)


def run(mpopl: MultiPopulation, pusher: RK2Pusher, tfinal: float, dt: float, callback=None, *,
        output_dt: float | None = None, verbosity: int = 0):
    """run!(mpopl, pusher, tfinal, dt, callback; output_dt, verbosity)
    (run.jl:1-29).  Steps run on the device in launches of
    ``steps_per_launch``; host callbacks are evaluated after each launch."""
    callback = callback or VoidCallback()
    mpopl.set_pusher(pusher)
    L = _lib.lib()
    opts = _lib.RunOpts()
    opts.target_species = -1
    cbs = callback.tpl if isinstance(callback, CombinedCallback) else (callback,)
    host_step = [c for c in cbs if type(c).onstep is not AbstractCallback.onstep
                 and not isinstance(c, PopulationTargetCallback)]
    for c in cbs:
        if isinstance(c, PopulationTargetCallback):
            opts.target_species = c.particle
            opts.target_ismax = 1 if c.ismax else 0
            opts.target_n = c.n
    walls = [c for c in cbs if isinstance(c, WallCallback)]
    for w in walls:
        w.attach(mpopl)
    t = mpopl.t
    nxt = t
    isave = 0
    tallies = _lib.Tallies()
    while t < tfinal * (1 - 1e-15):
        chunk_end = tfinal
        if output_dt is not None:
            chunk_end = min(tfinal, max(nxt, t + dt))
        if host_step:
            chunk_end = min(chunk_end, t + dt)
        _lib.check(L.pcl_run(mpopl.ctx, float(chunk_end), float(dt), C.byref(opts), C.byref(tallies)), mpopl.ctx,
                   "pcl_run")
        t = tallies.t
        mpopl.t = t
        for w in walls:
            w.collect(mpopl)
        cont = all(c.onstep(mpopl, t) for c in host_step) if host_step else True
        if opts.target_species >= 0:
            live = tallies.live[opts.target_species]
            hit = live >= opts.target_n if opts.target_ismax else live <= opts.target_n
            cont = cont and not hit
        if output_dt is not None and t >= nxt * (1 - 1e-12):
            nxt += output_dt
            isave += 1
            if verbosity > 0:
                print(f"{100 * t / tfinal:.2f}% complete, time = {t / 1e-9:.3f} ns, "
                      + ", ".join(f"{n} => {tallies.live[k]}" for k, n in PARTICLE_NAMES.items()))
            callback.onoutput(mpopl, t, isave)
        if not cont:
            if verbosity > 0:
                print("Early stop due to onstep() callback")
            break
    return tallies


# -------------------------------------------------------------- statistics --
def nparticles(pop: Population) -> int:
    """nparticles (population.jl:78): slots in use, live or not."""
    return int(mpop_tallies(pop).n[pop.particle])


def mpop_tallies(pop: Population):
    return pop._mp.tallies()


def nactives(pop: Population) -> int:
    """nactives (population.jl:89-97)."""
    return int(pop.moments()[9])


def weight(pop: Population) -> float:
    """weight (population.jl:130-140)."""
    return float(pop.moments()[0])


def meanenergy(pop: Population) -> float:
    """meanenergy (population.jl:152-166)."""
    m = pop.moments()
    return float(m[1] / m[0]) if m[0] else math.nan


def spectrum(pop: Population, edges, n: float = 1.0, weighted: bool = True, swarm: int = -1) -> np.ndarray:
    """Energy spectrum per unit energy as plotspec builds it (scripts/beam.jl:137-147
    unweighted, scripts/swarm.jl:149-158 weighted): the histogram over `edges`
    (J) normalised as StatsBase.normalize(mode=:density), i.e. divided by the
    bin widths, then divided by n (e.g. the number of primaries)."""
    counts, w = pop.energy_histogram(edges, swarm)
    h = w if weighted else counts.astype(float)
    return h / np.diff(np.asarray(edges, dtype=float)) / n


def maxenergy(pop: Population) -> float:
    """maxenergy (population.jl:172-174)."""
    return float(pop.moments()[8])


def spread(pop: Population):
    """spread (population.jl:180-198): centroid and rms distance from it."""
    m = pop.moments()
    tot = m[0]
    xm = m[2:5] / tot
    x2 = (m[5] + m[6] + m[7]) / tot
    return xm, math.sqrt(abs(x2 - float(np.dot(xm, xm))))


def posvar(pop: Population) -> np.ndarray:
    """posvar (population.jl:204-223)."""
    m = pop.moments()
    tot = m[0]
    return m[5:8] / tot - (m[2:5] / tot) ** 2


def repack(pop: Population):
    """repack! (population.jl:229-259): compact dead slots (all species)."""
    _lib.check(_lib.lib().pcl_compact(pop.ctx), pop.ctx, "pcl_compact")


def roulette(f, pop: Population):
    """roulette!(f, popl) (population.jl:291-309): f a keep probability, a
    function of the kinetic energy (J) or a table of it (MultiPopulation.
    roulette); on the device, over the population's species."""
    if pop._mp is None:
        raise RuntimeError("population is not attached to a MultiPopulation")
    pop._mp.roulette(pop.particle, f)


def split(f, pop: Population):
    """split!(f, popl) (population.jl:316-335): f a mean number of copies, a
    function of the kinetic energy (J) or a table of it (MultiPopulation.
    split); on the device, over the population's species."""
    if pop._mp is None:
        raise RuntimeError("population is not attached to a MultiPopulation")
    pop._mp.split(pop.particle, f)


def droplow(pop: Population):
    """droplow! (population.jl:273-284): the device step already drops
    particles below the cut; this compacts the population."""
    repack(pop)
