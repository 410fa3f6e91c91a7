"""Grow the mixed e-/gamma/e+ relativistic runaway avalanche and write its
state as a sampling recipe (``rrea_mixed_0.5MVm.json`` beside this file).

The avalanche: air (N2/O2 0.79/0.21, 1 atm, 293 K) at E = 0.5 MV/m along -z,
10^4 electrons at 1 MeV with isotropic directions (Philox seed 0), electrons
through Coulomb / Seltzer-Berger / Moller, photons through photoelectric /
Bethe-Heitler / Compton, positrons through Coulomb / Bhabha / annihilation,
continuum losses below 10 keV, cuts 10 keV (e+-) and 5 keV (photons),
dt = 1 ps, no roulette and no splitting (every weight stays 1).  The run
stops through PopulationTargetCallback on the electrons (callback.jl:253-267,
tested after every step by pcl_run) and records every species' count and mean
energy along the way, so that the recipe shows whether the species mix had
settled.

The recipe holds, per species, its share of the particles, the joint
histogram of (log10 kinetic energy in eV, cos of the angle between the
momentum and +z, the direction the field accelerates electrons) as non-zero
cells, and the mean and spread of the positions.  ``workloads.rrea_mixed_state``
samples any number of particles from it (uniform within a cell, azimuth
uniform), which keeps the species fractions, the spectra and the angular
distributions to the histogram's resolution.

Needs a GPU:  python particulator.jl_gb300/data/grow_rrea.py [--target N] [--out PATH]
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
DEFAULT_OUT = os.path.join(HERE, "rrea_mixed_0.5MVm.json")

LOG_E_EDGES = np.round(np.linspace(3.5, 9.0, 111), 6)   # log10(E / eV), 0.05 per bin
COS_EDGES = np.round(np.linspace(-1.0, 1.0, 21), 6)


def _histogram(pcl, sp, arr):
    E = pcl.kinenergy(sp, arr.p) / pcl.co.eV
    pn = np.linalg.norm(arr.p, axis=1)
    cz = np.clip(arr.p[:, 2] / np.where(pn > 0, pn, 1.0), -1.0, 1.0)
    h, _, _ = np.histogram2d(np.log10(np.maximum(E, 1e-30)), cz, bins=[LOG_E_EDGES, COS_EDGES])
    outside = len(E) - int(h.sum())
    iE, ic = np.nonzero(h)
    cells = [[int(a), int(b), int(h[a, b])] for a, b in zip(iE, ic)]
    return {"count": int(len(E)), "outside_histogram": outside, "cells": cells,
            "mean_energy_eV": float(E.mean()) if len(E) else 0.0,
            "x_mean_m": arr.x.mean(axis=0).tolist() if len(E) else [0.0] * 3,
            "x_std_m": arr.x.std(axis=0).tolist() if len(E) else [0.0] * 3}


def grow(target: int, out: str, tmax: float = 2.5e-6, output_dt: float = 20e-9, steps_per_launch: int = 16):
    sys.path.insert(0, ROOT)
    import __graft_entry__ as graft
    graft.build()
    pcl = graft.load_package()
    co = pcl.co
    dt, efield, n0 = 1e-12, 5e5, 10_000
    comp = pcl.workloads.air_composition()
    et, gt, pt = pcl.workloads.beam_tables(comp, efield, dt)
    cl = pcl.workloads.air_continuum_loss(comp)
    pusher = pcl.workloads.pusher((0.0, 0.0, -efield), cl=cl)
    rng = np.random.Generator(np.random.Philox(0))
    p = pcl.workloads.isotropic(n0, 1e6 * co.eV, rng)
    arr = pcl.ParticleArrays(np.zeros((n0, 3)), p, np.ones(n0), np.zeros(n0))
    cuts = {pcl.Electron: 1e4 * co.eV, pcl.Photon: 5e3 * co.eV, pcl.Positron: 1e4 * co.eV}
    mp = pcl.MultiPopulation(
        ("electron", pcl.Population(int(target * 1.3) + (1 << 16), arr, et, cuts[pcl.Electron], particle=pcl.Electron)),
        ("photon", pcl.Population(1 << 25, [], gt, cuts[pcl.Photon], particle=pcl.Photon)),
        ("positron", pcl.Population(1 << 21, [], pt, cuts[pcl.Positron], particle=pcl.Positron)),
        seed=0, steps_per_launch=steps_per_launch)

    class History(pcl.AbstractCallback):
        """onoutput hook: time, live counts and mean kinetic energies (no
        onstep of its own, so the steps stay in multi-step launches)."""

        def __init__(self):
            self.rows = []

        def onoutput(self, mpopl, t, i):
            tal = mpopl.tallies()
            means = []
            for sp in (pcl.Electron, pcl.Photon, pcl.Positron):
                m = mpopl.get(sp).moments()
                means.append(float(m[1] / m[0] / co.eV) if m[0] else 0.0)
            self.rows.append([t / 1e-9] + [int(v) for v in tal.live] + means)
            print(f"t = {t / 1e-9:8.2f} ns  live e/g/e+ = {list(tal.live)}  mean E (eV) = "
                  f"{[round(v) for v in means]}", flush=True)

    hist = History()
    cb = pcl.CombinedCallback((pcl.PopulationTargetCallback(pcl.Electron, target), hist))
    t0 = time.time()
    tal = pcl.run(mp, pusher, tmax, dt, cb, output_dt=output_dt)
    wall = time.time() - t0
    hist.onoutput(mp, mp.t, -1)
    live = [int(v) for v in tal.live]
    errors = {pcl._lib.ERROR_NAMES[q]: int(tal.errors[q]) for q in range(8) if tal.errors[q]}
    species = {}
    for sp, name in ((pcl.Electron, "electron"), (pcl.Photon, "photon"), (pcl.Positron, "positron")):
        species[name] = _histogram(pcl, sp, mp.get(sp).particles())
    total = sum(v["count"] for v in species.values())
    for v in species.values():
        v["fraction"] = v["count"] / total
    rows = np.array(hist.rows)
    tail = rows[-4:]
    ratio = tail[:, 2] / np.maximum(tail[:, 1], 1)
    settled = {"photon_per_electron_last_4_outputs": ratio.tolist(),
               "positron_per_electron_last_4_outputs": (tail[:, 3] / np.maximum(tail[:, 1], 1)).tolist(),
               "mean_energy_eV_last_4_outputs": tail[:, 4:7].tolist()}
    recipe = {
        "what": "state of the mixed e-/gamma/e+ avalanche in air at 0.5 MV/m, grown from 10^4 electrons "
                "until the electron population reached the target; a sampling recipe (histograms), not particles",
        "growth": {"seed_electrons": n0, "seed_energy_eV": 1e6, "directions": "isotropic", "philox_seed": 0,
                   "field_V_m": [0.0, 0.0, -efield], "dt_s": dt, "air": "N2/O2 0.79/0.21, 1 atm, 293 K",
                   "cuts_eV": {"electron": 1e4, "photon": 5e3, "positron": 1e4}, "roulette": None,
                   "split": None, "steps_per_launch": steps_per_launch,
                   "stop": {"callback": "PopulationTargetCallback", "species": "electron", "n": target},
                   "steps": int(tal.steps), "t_s": float(mp.t), "live_at_stop": live, "errors": errors,
                   "wall_s": wall, "particle_steps": int(tal.particle_steps)},
        "history_columns": ["t_ns", "live_e", "live_gamma", "live_e+", "mean_eV_e", "mean_eV_gamma", "mean_eV_e+"],
        "history": hist.rows,
        "settling": settled,
        "log10_energy_eV_edges": LOG_E_EDGES.tolist(),
        "cos_theta_z_edges": COS_EDGES.tolist(),
        "species": species,
    }
    with open(out, "w") as f:
        json.dump(recipe, f, separators=(",", ":"))
    print(json.dumps({"live_at_stop": live, "steps": int(tal.steps), "t_ns": mp.t / 1e-9, "wall_s": wall,
                      "fractions": {k: v["fraction"] for k, v in species.items()}, "errors": errors,
                      "settling": settled}))
    mp.close()
    return recipe


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--target", type=int, default=1 << 22, help="electron count that stops the growth")
    ap.add_argument("--out", default=DEFAULT_OUT)
    ap.add_argument("--tmax", type=float, default=2.5e-6, help="simulated-time limit (s)")
    ap.add_argument("--steps-per-launch", type=int, default=16)
    a = ap.parse_args()
    grow(a.target, a.out, tmax=a.tmax, steps_per_launch=a.steps_per_launch)


if __name__ == "__main__":
    main()
