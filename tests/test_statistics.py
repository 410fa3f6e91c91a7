"""Stochastic observables of the avalanche, device against an independent
oracle run (different seeds, so the two are statistically independent
samples of the same process): secondary production (growth), mean energy and
drift of the electrons, and the electron and photon spectra agree within
3 sigma (KS at the 3-sigma critical value)."""
import numpy as np
import pytest

from conftest import random_population

pytestmark = pytest.mark.gpu

C3 = np.sqrt(-0.5 * np.log(0.0027 / 2))   # KS critical coefficient at 3 sigma (two-sided 0.27 %)


def _ks(a, b):
    a = np.sort(a); b = np.sort(b)
    z = np.concatenate([a, b])
    return float(np.max(np.abs(np.searchsorted(a, z, side="right") / len(a) -
                               np.searchsorted(b, z, side="right") / len(b))))


def _ks_ok(a, b):
    n, m = len(a), len(b)
    return _ks(a, b) <= C3 * np.sqrt((n + m) / (n * m)), (_ks(a, b), C3 * np.sqrt((n + m) / (n * m)))


def _within3(a, sa, b, sb):
    return abs(a - b) <= 3 * np.hypot(sa, sb), (a, b, np.hypot(sa, sb))


def test_avalanche_observables_vs_oracle(pcl, oracle, gpu, air):
    n, steps, dt, E = 32768, 40, 25e-12, 2e6
    pusher = pcl.workloads.pusher((0.0, 0.0, -E), cl=air["cl"])
    res = {}
    for side, seed in (("gpu", 101), ("cpu", 202)):
        rng = np.random.default_rng(seed)
        arr = random_population(pcl, pcl.Electron, n, 1e5, 3e6, rng)
        if side == "gpu":
            mp = pcl.MultiPopulation(*[(k, pcl.Population(1 << 17, arr if k == 0 else pcl.ParticleArrays.empty(),
                                                          air["tabs"][k], air["cuts"][k], particle=k))
                                       for k in (0, 1, 2)], seed=seed)
            for k in range(steps):
                pcl.advance(mp, pusher, (k + 1) * dt)
            t = mp.tallies()
            e, g = mp.get(0).particles(), mp.get(1).particles()
            res[side] = dict(spawn_e=int(t.spawned[0]), spawn_g=int(t.spawned[1]), e=e, g=g)
            mp.close()
        else:
            W = oracle.OracleWorld(seed, air["tabs"], air["cuts"], pusher)
            sid = np.arange(n, dtype=np.uint64)
            rs = np.random.default_rng(seed + 1)
            W.upload(pcl.Electron, oracle.Arrays(arr.x, arr.p, arr.w, arr.t, -np.log(rs.random(n)), sid,
                                                 np.zeros(n, np.uint32)))
            for k in range(steps):
                W.advance((k + 1) * dt, 16)
            c = W.counters()
            res[side] = dict(spawn_e=int(c["spawned"][0]), spawn_g=int(c["spawned"][1]),
                             e=W.download(pcl.Electron), g=W.download(pcl.Photon))
    a, b = res["gpu"], res["cpu"]
    # secondary production (Poisson)
    for key in ("spawn_e", "spawn_g"):
        ok, info = _within3(a[key], np.sqrt(a[key]), b[key], np.sqrt(b[key]))
        assert ok, (key, info)
    Ea, Eb = pcl.kinenergy(0, a["e"].p), pcl.kinenergy(0, b["e"].p)
    ok, info = _within3(Ea.mean(), Ea.std() / np.sqrt(len(Ea)), Eb.mean(), Eb.std() / np.sqrt(len(Eb)))
    assert ok, ("mean energy", info)
    za, zb = a["e"].x[:, 2], b["e"].x[:, 2]
    ok, info = _within3(za.mean(), za.std() / np.sqrt(len(za)), zb.mean(), zb.std() / np.sqrt(len(zb)))
    assert ok, ("drift", info)
    ok, info = _ks_ok(np.log(Ea), np.log(Eb))
    assert ok, ("electron spectrum", info)
    ka, kb = pcl.kinenergy(1, a["g"].p), pcl.kinenergy(1, b["g"].p)
    assert len(ka) > 50 and len(kb) > 50   # the KS critical value accounts for the sample sizes
    ok, info = _ks_ok(np.log(ka), np.log(kb))
    assert ok, ("photon spectrum", info)
