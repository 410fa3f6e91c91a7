"""Generate the golden fixtures in tests/golden/ from the CPU oracle and the
library's host table builders.

    python tests/golden/make_golden.py

The reference (Julia) cannot run here and ships no vectors of its own, so these
fixtures pin the oracle and the builders against regressions, and the device
against them; they are not reference outputs.
Files:
  tables_air.npz   collision tables of air at 0.5 MV/m, dt = 1 ps (rate, ratebound, perm)
  samplers.npz     every air process sampled for 32 fixed primaries (outcomes, draws)
  step.npz         a mixed population before and after 3 steps of 5 ps
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def setup():
    import __graft_entry__ as g
    g.build()
    pcl = g.load_package()
    comp = pcl.workloads.air_composition()
    et, gt, pt = pcl.workloads.beam_tables(comp, 5e5, 1e-12)
    cl = pcl.workloads.air_continuum_loss(comp)
    tabs = {pcl.Electron: et, pcl.Photon: gt, pcl.Positron: pt}
    cuts = {pcl.Electron: 1e4 * pcl.co.eV, pcl.Photon: 5e3 * pcl.co.eV, pcl.Positron: 1e4 * pcl.co.eV}
    pusher = pcl.workloads.pusher((0.0, 0.0, -5e5), cl=cl)
    return pcl, tabs, cuts, pusher


WINDOWS = {"RelativisticCoulomb": (1e4, 1e8), "Moller": (2.1e4, 1e8), "SeltzerBerger": (1.1e4, 1e8),
           "Compton": (5e3, 1e8), "PhotoElectric": (5e3, 1e6), "BetheHeitler": (1.1e6, 1e8),
           "Bhaba": (2.1e4, 1e8), "PositronAnihilation": (1e4, 1e8)}


def sampler_inputs(pcl, tabs, n=32, seed=2025):
    rng = np.random.default_rng(seed)
    rows = []
    for sp, tab in tabs.items():
        for j, proc in enumerate(tab.proc):
            lo, hi = WINDOWS[type(proc).__name__]
            E = np.exp(rng.uniform(np.log(lo), np.log(hi), n)) * pcl.co.eV
            d = pcl.workloads.isotropic(n, 1.0, rng, sp)
            p = d * (pcl.momentum_norm_from_kin(sp, E) / np.linalg.norm(d, axis=1))[:, None]
            p = (p / pcl.co.electron_mc).astype(np.float32).astype(np.float64) * pcl.co.electron_mc
            sid = rng.integers(0, 2 ** 62, n, dtype=np.uint64)
            rows.append((sp, j, p, sid))
    return rows


def step_inputs(pcl, seed=77):
    rng = np.random.default_rng(seed)
    out = {}
    for sp, n, lo, hi in ((0, 64, 1e4, 3e7), (1, 32, 5e3, 3e7), (2, 16, 1e4, 3e7)):
        E = np.exp(rng.uniform(np.log(lo), np.log(hi), n)) * pcl.co.eV
        d = pcl.workloads.isotropic(n, 1.0, rng, sp)
        p = d * (pcl.momentum_norm_from_kin(sp, E) / np.linalg.norm(d, axis=1))[:, None]
        p = (p / pcl.co.electron_mc).astype(np.float32).astype(np.float64) * pcl.co.electron_mc
        s = (-np.log(rng.random(n))).astype(np.float32).astype(np.float64)
        out[sp] = dict(x=np.zeros((n, 3)), p=p, w=np.ones(n), t=np.zeros(n), s=s,
                       sid=np.arange(n, dtype=np.uint64) + (np.uint64(sp) << np.uint64(40)),
                       ctr=np.ones(n, np.uint32))
    return out


def main():
    from oracle.harness import Arrays, OracleWorld
    pcl, tabs, cuts, pusher = setup()
    np.savez_compressed(os.path.join(HERE, "tables_air.npz"),
                        **{f"rate{k}": t.rate for k, t in tabs.items()},
                        **{f"rb{k}": t.ratebound for k, t in tabs.items()},
                        **{f"perm{k}": t.perm for k, t in tabs.items()})
    W = OracleWorld(4242, tabs, cuts, pusher)
    d = {}
    for q, (sp, j, p, sid) in enumerate(sampler_inputs(pcl, tabs)):
        op, os_, ok, oc, ot = W.sample(sp, j, p, sid)
        d.update({f"p{q}": p, f"sid{q}": sid, f"sp{q}": sp, f"j{q}": j, f"op{q}": op, f"os{q}": os_,
                  f"ok{q}": ok, f"oc{q}": oc, f"ot{q}": ot})
    d["n"] = q + 1
    np.savez_compressed(os.path.join(HERE, "samplers.npz"), **d)
    inp = step_inputs(pcl)
    W = OracleWorld(4242, tabs, cuts, pusher)
    for sp, a in inp.items():
        W.upload(sp, Arrays(a["x"], a["p"], a["w"], a["t"], a["s"], a["sid"], a["ctr"]))
    for k in range(3):
        W.advance((k + 1) * 5e-12, 1)
    d = {}
    for sp in (0, 1, 2):
        o = W.download(sp)
        for f in ("x", "p", "w", "t", "s", "sid", "ctr"):
            d[f"in_{f}{sp}"] = inp[sp][f]
        for f in ("x", "p", "w", "t", "s", "sid", "ctr", "tie"):
            d[f"out_{f}{sp}"] = getattr(o, f)
    np.savez_compressed(os.path.join(HERE, "step.npz"), **d)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
