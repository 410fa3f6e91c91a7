"""GPU parity: the device step against the CPU oracle on identical inputs.

Both sides consume the same per-particle Philox streams, so for every particle
whose decisions are not within FP32 rounding of a threshold (the oracle's
tie flag) the draw counters, surviving stream ids and collision choices must
be identical, and momenta, s and positions must agree within 1e-5 relative
(FP32 device vs Float64 oracle).
"""
import numpy as np
import pytest

from conftest import random_population

pytestmark = pytest.mark.gpu

RTOL = 1e-5   # relative tolerance on momenta (FP32 device vs Float64 oracle)


def _mixed(pcl, air, n=(4096, 2048, 1024), seed=3, **cfg):
    rng = np.random.default_rng(seed)
    pops = {pcl.Electron: random_population(pcl, pcl.Electron, n[0], 1e4, 3e7, rng),
            pcl.Photon: random_population(pcl, pcl.Photon, n[1], 5e3, 3e7, rng),
            pcl.Positron: random_population(pcl, pcl.Positron, n[2], 1e4, 3e7, rng)}
    cap = 1 << 16
    mp = pcl.MultiPopulation(*[(k, pcl.Population(cap, pops[k], air["tabs"][k], air["cuts"][k], particle=k))
                               for k in pops], seed=seed, **cfg)
    return mp


def _oracle_from(oracle, pcl, mp, air, pusher, tally_only=()):
    W = oracle.OracleWorld(int(mp.config.seed), air["tabs"], air["cuts"], pusher, tally_only=tally_only)
    for k in mp.index:
        if not mp.get(k).tally_only:
            W.upload(k, mp.get(k).particles())
    return W


def _check(pcl, oracle, mp, W, species=(0, 1, 2), rtol=RTOL, stol=None):
    reports = []
    for k in species:
        rep = oracle.compare_populations(mp.get(k).particles(), W.download(k), k, rtol=rtol, stol=stol)
        reports.append(rep)
        assert rep["ok"], str(rep)
    return reports


def _pusher(pcl, air, E=5e5):
    return pcl.workloads.pusher((0.0, 0.0, -E), cl=air["cl"])


@pytest.mark.parametrize("dt", [1e-12, 25e-12])
def test_one_step_mixed(pcl, oracle, gpu, air, dt):
    mp = _mixed(pcl, air, seed=3 if dt < 1e-11 else 4)
    pusher = _pusher(pcl, air)
    W = _oracle_from(oracle, pcl, mp, air, pusher)
    pcl.advance(mp, pusher, dt)
    W.advance(dt, 4)
    # s after a step carries the FP32 rate-bound error (~1e-6 relative) once per
    # collision: ~r dt collisions per step, ~75 at 25 ps
    _check(pcl, oracle, mp, W, stol=2 * RTOL * max(1.0, dt / 1e-12 / 3))
    t = mp.tallies()
    c = W.counters()
    # per-process collision counts agree up to tie-affected lineages
    diff = np.abs(np.array([list(t.collisions[s]) for s in range(3)]) - c["coll"]).sum()
    assert diff <= 4 * (c["ties"] + 1), (diff, c["ties"])
    assert sum(t.errors[q] for q in (2, 3, 5)) == 0, list(t.errors)
    mp.close()


def test_several_steps_then_compare(pcl, oracle, gpu, air):
    """Ten plain steps of 1 ps: state, secondaries and removals all carry over."""
    mp = _mixed(pcl, air, n=(2048, 1024, 512), seed=5)
    pusher = _pusher(pcl, air)
    W = _oracle_from(oracle, pcl, mp, air, pusher)
    for k in range(10):
        pcl.advance(mp, pusher, (k + 1) * 1e-12)
        W.advance((k + 1) * 1e-12, 4)
    _check(pcl, oracle, mp, W, rtol=3 * RTOL)
    mp.close()


def test_multistep_launch_matches_plain(pcl, oracle, gpu, air):
    """Eight steps fused into one launch equal eight oracle steps."""
    mp = _mixed(pcl, air, n=(2048, 1024, 512), seed=6, steps_per_launch=8)
    pusher = _pusher(pcl, air)
    W = _oracle_from(oracle, pcl, mp, air, pusher)
    opts_dt = 1e-12
    pcl.run(mp, pusher, 8 * opts_dt, opts_dt)
    for k in range(8):
        W.advance((k + 1) * opts_dt, 4)
    assert mp.tallies().steps == 8
    _check(pcl, oracle, mp, W, rtol=3 * RTOL)
    mp.close()


def test_graph_matches_plain(pcl, gpu, air):
    """Launch groups replayed from CUDA graphs (prologue, step, device-gated
    spill passes, compaction inside the graph) give bit-identical particles and
    tallies to plain launches."""
    pusher = _pusher(pcl, air, E=2e6)
    runs = []
    for graph in (False, True):
        mp = _mixed(pcl, air, n=(4096, 2048, 1024), seed=12, steps_per_launch=2, compaction_period=4,
                    use_graph=graph)
        pcl.run(mp, pusher, 12 * 25e-12, 25e-12)
        runs.append(mp)
    a, b = runs
    ta, tb = a.tallies(), b.tallies()
    assert ta.steps == tb.steps == 12
    for s in range(3):
        assert list(ta.collisions[s]) == list(tb.collisions[s])
        assert ta.spawned[s] == tb.spawned[s] and ta.live[s] == tb.live[s]
    assert list(ta.errors) == list(tb.errors)
    for k in a.index:
        pa, pb = a.get(k).particles(), b.get(k).particles()
        oa, ob = np.argsort(pa.sid), np.argsort(pb.sid)
        for f in ("sid", "ctr", "p", "x", "s", "w"):
            np.testing.assert_array_equal(getattr(pa, f)[oa], getattr(pb, f)[ob])
    a.close(); b.close()


def test_autotune_keeps_physics(pcl, gpu, air):
    """The autotuner advances real steps and keeps a valid launch shape; the
    population it leaves equals a plain run of the same number of steps
    (launch shapes do not change the physics; a multi-step launch keeps the
    sub-eps remainder of a step as a double-float where separate launches
    round it to FP32, so a rare particle may differ in its last bits)."""
    pusher = _pusher(pcl, air, E=2e6)
    a = _mixed(pcl, air, n=(2048, 1024, 512), seed=21)
    r = a.autotune(pusher, 1e-12, steps=480)
    assert r["blocks_per_sm"] in (2, 3, 4) and r["steps_per_launch"] in (1, 2, 4, 8, 16)
    assert r["compaction_period"] in (2, 4, 8, 16, 32) and r["use_graph"] in (0, 1)
    assert r["trials"] == 15 and r["steps"] == 480 and r["rate"] > 0
    ta = a.tallies()
    assert ta.steps == 480
    b = _mixed(pcl, air, n=(2048, 1024, 512), seed=21)
    pcl.run(b, pusher, 480e-12, 1e-12)
    tb = b.tallies()
    for s in range(3):
        assert abs(ta.live[s] - tb.live[s]) <= 2 + ta.live[s] // 1000
    for k in a.index:
        pa, pb = a.get(k).particles(), b.get(k).particles()
        common, ia, ib = np.intersect1d(pa.sid, pb.sid, return_indices=True)
        assert len(common) >= 0.999 * max(len(pa.sid), len(pb.sid)) - 2
        dp = np.linalg.norm(pa.p[ia] - pb.p[ib], axis=1) / np.maximum(np.linalg.norm(pb.p[ib], axis=1), 1e-300)
        assert np.mean(dp > 1e-5) <= 1e-3, np.sort(dp)[-5:]
    a.close(); b.close()


def test_electrons_tally_photons(pcl, oracle, gpu):
    """Electrons-only workload with bremsstrahlung photons tallied."""
    wl = pcl.workloads.plain_electrons(n=1000, tfinal=20e-12, seed=1)
    mp, pusher = wl.mpopl, wl.pusher
    e = mp.get(pcl.Electron)
    tabs = {pcl.Electron: e.collisions}
    cuts = {pcl.Electron: e.energy_cut, pcl.Photon: 0.0}
    W = oracle.OracleWorld(1, tabs, cuts, pusher, tally_only=(pcl.Photon,))
    W.upload(pcl.Electron, e.particles())
    for k in range(20):
        pcl.advance(mp, pusher, (k + 1) * wl.dt)
        W.advance((k + 1) * wl.dt, 4)
    rep = oracle.compare_populations(e.particles(), W.download(pcl.Electron), pcl.Electron, rtol=3 * RTOL)
    assert rep["ok"], str(rep)
    t = mp.tallies()
    c = W.counters()
    assert abs(t.tally_count[1] - c["tally_count"][1]) <= c["ties"] + 1
    mp.close()


def test_compaction_preserves_particles(pcl, gpu, air):
    mp = _mixed(pcl, air, n=(2048, 1024, 512), seed=8, compaction_period=1000)
    pusher = _pusher(pcl, air)
    for k in range(5):
        pcl.advance(mp, pusher, (k + 1) * 5e-12)
    before = {k: mp.get(k).particles() for k in mp.index}
    t = mp.tallies()
    assert t.n[0] >= t.live[0]
    pcl.repack(mp.get(0))
    t2 = mp.tallies()
    for k in mp.index:
        after = mp.get(k).particles()
        assert t2.n[k] == len(after.w) == len(before[k].w)
        assert np.array_equal(np.sort(after.sid), np.sort(before[k].sid))
        # order preserving
        assert np.array_equal(after.sid, before[k].sid)
    mp.close()


def test_moments_match_download(pcl, gpu, air):
    mp = _mixed(pcl, air, n=(2048, 1024, 512), seed=9)
    pusher = _pusher(pcl, air)
    pcl.advance(mp, pusher, 3e-12)
    for k in mp.index:
        pop = mp.get(k)
        a = pop.particles()
        m = pop.moments()
        E = pcl.kinenergy(k, a.p)
        assert m[9] == len(a.w)
        np.testing.assert_allclose(m[0], a.w.sum(), rtol=1e-12)
        np.testing.assert_allclose(m[1], (a.w * E).sum(), rtol=1e-5)
        np.testing.assert_allclose(m[2:5], (a.w[:, None] * a.x).sum(0), rtol=1e-5, atol=1e-12)
        assert abs(pcl.meanenergy(pop) - (a.w * E).sum() / a.w.sum()) <= 1e-5 * pcl.meanenergy(pop)
    mp.close()
