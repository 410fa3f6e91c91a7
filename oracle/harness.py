"""Python side of the CPU oracle (test infrastructure only).

Loads ``oracle/_build/liboracle.so`` (built by ``oracle/build.py``), feeds it
the same tables, forcing and particles as the GPU library, and compares the
two populations stream id by stream id.  Imported only by tests/, by
``__graft_entry__.smoke()`` and by bench.py's CPU-baseline leg.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

_P = C.POINTER
_d = C.c_double
_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            from . import build as b  # noqa
            b.build_oracle()
        L = C.CDLL(LIB_PATH)
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.c_uint64, _d]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_set_species.argtypes = [C.c_void_p, C.c_int, _d, C.c_int]
        L.orc_set_table.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, _d, _P(_d), _P(_d),
                                    _P(C.c_int32), _P(C.c_int32), _P(_d), _P(C.c_int32)]
        L.orc_set_sb.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, _P(_d), _P(_d)]
        L.orc_set_swarms.argtypes = [C.c_void_p, C.c_int, _P(_d), _P(_d), _P(_d)]
        L.orc_set_field.argtypes = [C.c_void_p, C.c_int, _P(_d), C.c_int]
        L.orc_set_push_mask.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int]
        L.orc_set_bfield.argtypes = [C.c_void_p, C.c_int, _P(_d), C.c_int]
        L.orc_set_wall.argtypes = [C.c_void_p, C.c_int, C.c_int, _d, C.c_int]
        L.orc_roulette.argtypes = [C.c_void_p, C.c_int, _d]
        L.orc_split.argtypes = [C.c_void_p, C.c_int, _d]
        L.orc_roulette_fn.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(_d), C.POINTER(_d)]
        L.orc_split_fn.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(_d), C.POINTER(_d)]
        L.orc_poisson_inv.argtypes = [_d, _d]
        L.orc_poisson_inv.restype = C.c_int
        L.orc_get_wall.argtypes = [C.c_void_p, _P(C.c_int32), _P(C.c_uint64), _P(_d), _P(_d), _P(_d), _P(_d)]
        L.orc_get_wall.restype = C.c_int64
        L.orc_set_linear_table.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, _d, _d, _P(_d), _P(_d),
                                           _P(C.c_int32), _P(_d)]
        L.orc_set_forcing.argtypes = [C.c_void_p, _P(_d), _P(_d), C.c_int, C.c_int, _d, _P(_d), _P(_d)]
        L.orc_upload.argtypes = [C.c_void_p, C.c_int, C.c_int64, _P(_d), _P(_d), _P(_d), _P(_d), _P(_d),
                                 _P(C.c_uint64), _P(C.c_uint32)]
        L.orc_advance.argtypes = [C.c_void_p, _d, C.c_int]
        L.orc_count.restype = C.c_int64
        L.orc_count.argtypes = [C.c_void_p, C.c_int]
        L.orc_download.argtypes = [C.c_void_p, C.c_int, _P(_d), _P(_d), _P(_d), _P(_d), _P(_d), _P(C.c_uint64),
                                   _P(C.c_uint32), _P(C.c_uint8)]
        L.orc_counters.argtypes = [C.c_void_p, _P(C.c_int64), _P(C.c_int64), _P(C.c_int64), _P(C.c_int64),
                                   _P(_d), _P(_d), _P(C.c_int64), _P(C.c_int64)]
        L.orc_reset_counters.argtypes = [C.c_void_p]
        L.orc_sample.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int64, _P(_d), _P(C.c_uint64), _P(_d), _P(_d),
                                 _P(C.c_int32), _P(C.c_uint32), _P(C.c_uint8)]
        L.orc_philox.argtypes = [_P(C.c_uint32), _P(C.c_uint32), _P(C.c_uint32)]
        _lib = L
    return _lib


def _p(a, t=_d):
    return None if a is None else a.ctypes.data_as(_P(t))


class Arrays:
    """Particle batch (SI) with stream ids, counters and tie flags."""

    def __init__(self, x, p, w, t, s, sid, ctr, tie=None):
        self.x, self.p, self.w, self.t, self.s = x, p, w, t, s
        self.sid, self.ctr = sid, ctr
        self.tie = tie if tie is not None else np.zeros(len(w), np.uint8)

    def __len__(self):
        return len(self.w)


class OracleWorld:
    """One oracle instance configured like a GPU MultiPopulation.

    tabs: {species: ChebyshevCollisionTable or None}; cuts: {species: J};
    pusher: the RK2Pusher given to the GPU; tally_only: species tallied only.
    """

    def __init__(self, seed, tabs, cuts, pusher, tally_only=(), tie_tol=2e-5):
        L = lib()
        self.h = L.orc_create(int(seed), float(tie_tol))
        self._keep = []
        for sp, cut in cuts.items():
            L.orc_set_species(self.h, int(sp), float(cut), 1 if sp in tally_only else 0)
        for sp, tab in tabs.items():
            if tab is None:
                continue
            if hasattr(tab, "energy"):  # linear-grid CollisionTable
                n = tab.nproc
                kinds = np.array([p.kind for p in tab.proc], np.int32)
                params = np.zeros((max(1, n), 8))
                for j, proc in enumerate(tab.proc):
                    params[j] = list(proc.to_c(1.0).param)
                e0, e1, ng = tab.energy
                rate = np.ascontiguousarray(tab.rate.T)
                rb = np.ascontiguousarray(np.broadcast_to(tab.ratebound, (ng,)) if len(tab.ratebound) == 1
                                          else tab.ratebound, dtype=float)
                self._keep += [kinds, params, rate, rb]
                L.orc_set_linear_table(self.h, int(sp), n, ng, e0, e1, _p(rate), _p(rb), _p(kinds, C.c_int32),
                                       _p(params))
                continue
            n = tab.nproc
            kinds = np.array([p.kind for p in tab.proc] or [0], np.int32)
            Z = np.zeros(max(1, n), np.int32)
            params = np.zeros((max(1, n), 8))
            nparam = np.zeros(max(1, n), np.int32)
            for j, (cf, proc) in enumerate(zip(tab.coef, tab.proc)):
                cp = proc.to_c(cf)
                Z[j] = cp.Z if cp.Z else int(round(cp.param[0]))
                params[j] = list(cp.param)
                nparam[j] = cp.nparam
            rate = np.ascontiguousarray(tab.rate) if n else np.zeros(1)
            rb = np.ascontiguousarray(tab.ratebound)
            self._keep += [kinds, Z, params, nparam, rate, rb]
            L.orc_set_table(self.h, int(sp), tab.order, n, tab.b.k, tab.b.xmax, _p(rate), _p(rb),
                            _p(kinds, C.c_int32), _p(Z, C.c_int32), _p(params), _p(nparam, C.c_int32))
            for j, proc in enumerate(tab.proc):
                if hasattr(proc, "log_energy"):
                    L.orc_set_sb(self.h, int(sp), j, len(proc.log_energy), proc.ncum, _p(proc.log_energy),
                                 _p(proc.data))
        E, B, cl = pusher.device_forcing()
        E = np.ascontiguousarray(E, dtype=float)
        B = np.ascontiguousarray(B, dtype=float)
        if cl is None:
            L.orc_set_forcing(self.h, _p(E), _p(B), 0, 0, 0.0, None, None)
        else:
            self._keep += [cl.ec, cl.pc]
            L.orc_set_forcing(self.h, _p(E), _p(B), cl.n, cl.bints.k, cl.bints.xmax, _p(cl.ec), _p(cl.pc))
        kind, fparams = pusher.device_efield()
        fp = np.ascontiguousarray(np.asarray(fparams, dtype=float)) if fparams else np.zeros(1)
        self._keep.append(fp)
        L.orc_set_field(self.h, int(kind), _p(fp), len(fparams))
        L.orc_set_push_mask(self.h, *(int(m) for m in pusher.device_masks()))
        bkind, bparams = pusher.device_bfield()
        bp = np.ascontiguousarray(np.asarray(bparams, dtype=float)) if bparams else np.zeros(1)
        self._keep.append(bp)
        L.orc_set_bfield(self.h, int(bkind), _p(bp), len(bparams))

    def set_swarms(self, tabs, E, Fdt, safety=1.15):
        """Swarm mode: per-swarm field E [n,3] (V/m) and the rate bound of the
        lepton tables for each swarm's Fdt, A + Fdt B from ratebound_split."""
        import particulator_gb300 as pcl
        E = np.ascontiguousarray(np.asarray(E, dtype=float).reshape(-1, 3))
        Fdt = np.asarray(Fdt, dtype=float)
        rbs = {}
        for sp in (0, 2):
            tab = tabs.get(sp)
            if tab is None or not hasattr(tab, "b") or tab.nproc == 0:
                rbs[sp] = None
                continue
            A, B = pcl.ratebound_split(tab, safety)
            rbs[sp] = np.ascontiguousarray(np.concatenate([A + f * B for f in Fdt]))
        self._keep += [E, rbs[0], rbs[2]]
        lib().orc_set_swarms(self.h, len(Fdt), _p(E), _p(rbs[0]), _p(rbs[2]))

    def roulette(self, sp, pkeep):
        """pkeep: a number, or a table (energies in J, keep probabilities)."""
        if np.ndim(pkeep) == 0:
            lib().orc_roulette(self.h, int(sp), float(pkeep))
        else:
            E, v = (np.ascontiguousarray(np.asarray(a, dtype=float)) for a in pkeep)
            lib().orc_roulette_fn(self.h, int(sp), len(E), _p(E), _p(v))

    def split(self, sp, p):
        """p: a number, or a table (energies in J, mean numbers of copies)."""
        if np.ndim(p) == 0:
            lib().orc_split(self.h, int(sp), float(p))
        else:
            E, v = (np.ascontiguousarray(np.asarray(a, dtype=float)) for a in p)
            lib().orc_split_fn(self.h, int(sp), len(E), _p(E), _p(v))

    def set_wall(self, sp, coord0, v, drop=True):
        lib().orc_set_wall(self.h, int(sp), int(coord0), float(v), 1 if drop else 0)

    def get_wall(self):
        """(species, sid, x, p, w, t) of every crossing recorded so far."""
        L = lib()
        n = L.orc_get_wall(self.h, None, None, None, None, None, None)
        sp = np.zeros(n, np.int32); sid = np.zeros(n, np.uint64)
        x = np.zeros((n, 3)); p = np.zeros((n, 3)); w = np.zeros(n); t = np.zeros(n)
        if n:
            L.orc_get_wall(self.h, _p(sp, C.c_int32), _p(sid, C.c_uint64), _p(x), _p(p), _p(w), _p(t))
        return sp, sid, x, p, w, t

    def upload(self, sp, a):
        n = len(a.w)
        x = np.ascontiguousarray(a.x, dtype=float).reshape(-1)
        p = np.ascontiguousarray(a.p, dtype=float).reshape(-1)
        w = np.ascontiguousarray(a.w, dtype=float)
        t = np.ascontiguousarray(a.t, dtype=float)
        s = np.ascontiguousarray(a.s, dtype=float)
        sid = np.ascontiguousarray(a.sid, dtype=np.uint64)
        ctr = np.ascontiguousarray(a.ctr, dtype=np.uint32)
        lib().orc_upload(self.h, int(sp), n, _p(x), _p(p), _p(w), _p(t), _p(s), _p(sid, C.c_uint64),
                         _p(ctr, C.c_uint32))

    def advance(self, tfinal, nthreads=1):
        lib().orc_advance(self.h, float(tfinal), int(nthreads))

    def download(self, sp):
        L = lib()
        n = L.orc_count(self.h, int(sp))
        x = np.zeros((n, 3)); p = np.zeros((n, 3)); w = np.zeros(n); t = np.zeros(n); s = np.zeros(n)
        sid = np.zeros(n, np.uint64); ctr = np.zeros(n, np.uint32); tie = np.zeros(n, np.uint8)
        if n:
            L.orc_download(self.h, int(sp), _p(x), _p(p), _p(w), _p(t), _p(s), _p(sid, C.c_uint64),
                           _p(ctr, C.c_uint32), _p(tie, C.c_uint8))
        return Arrays(x, p, w, t, s, sid, ctr, tie)

    def counters(self):
        coll = np.zeros(48, np.int64); nulls = np.zeros(3, np.int64); spawned = np.zeros(3, np.int64)
        tc = np.zeros(3, np.int64); tw = np.zeros(3); twe = np.zeros(3); err = np.zeros(8, np.int64)
        ties = np.zeros(1, np.int64)
        lib().orc_counters(self.h, _p(coll, C.c_int64), _p(nulls, C.c_int64), _p(spawned, C.c_int64),
                           _p(tc, C.c_int64), _p(tw), _p(twe), _p(err, C.c_int64), _p(ties, C.c_int64))
        return dict(coll=coll.reshape(3, 16), nulls=nulls, spawned=spawned, tally_count=tc, tally_w=tw,
                    tally_wE=twe, err=err, ties=int(ties[0]))

    def reset_counters(self):
        lib().orc_reset_counters(self.h)

    def sample(self, sp, j, p, sid):
        n = len(sid)
        p = np.ascontiguousarray(p, dtype=float).reshape(-1)
        sid = np.ascontiguousarray(sid, dtype=np.uint64)
        op = np.zeros(9 * n); os_ = np.zeros(3 * n); ok = np.zeros(3 * n, np.int32)
        oc = np.zeros(n, np.uint32); ot = np.zeros(n, np.uint8)
        lib().orc_sample(self.h, int(sp), int(j), n, _p(p), _p(sid, C.c_uint64), _p(op), _p(os_),
                         _p(ok, C.c_int32), _p(oc, C.c_uint32), _p(ot, C.c_uint8))
        return op.reshape(n, 3, 3), os_.reshape(n, 3), ok.reshape(n, 3), oc, ot

    def __del__(self):
        try:
            lib().orc_destroy(self.h)
        except Exception:
            pass


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().orc_philox(c, k, o)
    return list(o)


def compare_populations(gpu, orc, species, rtol=1e-5, xtol=None, max_unmatched_frac=0.01, stol=None, max_bad=0):
    """Match GPU and oracle particles by stream id.  Oracle particles not in a
    tie lineage must exist on the GPU with the same draw counter (up to
    `max_bad` exceptions), and momenta / s / positions within tolerance.
    Returns a report dict."""
    rep = {"species": int(species), "n_gpu": len(gpu.w), "n_orc": len(orc.w), "ties": int(orc.tie.sum())}
    og = {int(s): i for i, s in enumerate(np.asarray(gpu.sid, dtype=np.uint64))}
    clean = np.nonzero(orc.tie == 0)[0]
    rep["clean"] = len(clean)
    missing = 0
    bad_ctr = 0
    idx_g = []
    idx_o = []
    for i in clean:
        j = og.get(int(orc.sid[i]))
        if j is None:
            missing += 1
            continue
        if int(gpu.ctr[j]) != int(orc.ctr[i]):
            bad_ctr += 1
            continue
        idx_g.append(j)
        idx_o.append(i)
    rep["missing"] = missing
    rep["bad_ctr"] = bad_ctr
    ig = np.array(idx_g, dtype=int)
    io = np.array(idx_o, dtype=int)
    if len(ig):
        pn = np.linalg.norm(orc.p[io], axis=1)
        dp = np.linalg.norm(gpu.p[ig] - orc.p[io], axis=1) / np.maximum(pn, 1e-300)
        rep["max_dp_rel"] = float(dp.max())
        ds = np.abs(gpu.s[ig] - orc.s[io]) / np.maximum(1.0, np.abs(orc.s[io]))
        rep["max_ds"] = float(ds.max())
        dx = np.linalg.norm(gpu.x[ig] - orc.x[io], axis=1)
        scale = xtol if xtol is not None else max(1e-6, float(np.linalg.norm(orc.x[io], axis=1).max()))
        rep["max_dx_rel"] = float(dx.max() / scale)
        # weights are 1 unless roulette / split rescaled them (FP32 on the device)
        rep["w_equal"] = bool(np.allclose(gpu.w[ig], orc.w[io], rtol=1e-6, atol=0.0))
    else:
        rep.update(max_dp_rel=0.0, max_ds=0.0, max_dx_rel=0.0, w_equal=True)
    extra = len(gpu.w) - len(ig)
    rep["gpu_unmatched"] = int(extra)
    tie_budget = int(orc.tie.sum()) + max(2, int(max_unmatched_frac * max(1, len(orc.w))))
    stol = 2 * rtol if stol is None else stol
    rep["ok"] = (missing <= max_bad and bad_ctr + missing <= max_bad and rep["max_dp_rel"] <= rtol
                 and rep["max_ds"] <= stol
                 and rep["max_dx_rel"] <= 10 * rtol and rep["w_equal"] and extra <= tie_budget)
    return rep
