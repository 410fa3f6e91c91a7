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


def _check(pcl, oracle, mp, W, species=(0, 1, 2), rtol=RTOL, stol=None, max_bad=0):
    reports = []
    for k in species:
        rep = oracle.compare_populations(mp.get(k).particles(), W.download(k), k, rtol=rtol, stol=stol,
                                         max_bad=max_bad)
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


@pytest.mark.parametrize("spl", [4, 16])
def test_photons_fly_through_launch(pcl, oracle, gpu, air, spl):
    """Photons whose clock runs past the end of a multi-step launch fly through
    its remaining steps in one push.  Their per-step live counts (the
    particle-steps, built from them) equal those of one-step launches, the
    photons equal those launches' photons to FP32 rounding, and the population
    matches the oracle."""
    pusher = _pusher(pcl, air)
    runs = []
    for k in (1, spl):
        mp = _mixed(pcl, air, n=(512, 16384, 128), seed=31, steps_per_launch=k)
        pcl.run(mp, pusher, 32e-12, 1e-12)
        runs.append(mp)
    a, b = runs
    ta, tb = a.tallies(), b.tallies()
    assert ta.steps == tb.steps == 32
    assert abs(ta.particle_steps - tb.particle_steps) <= 2, (ta.particle_steps, tb.particle_steps)
    assert ta.particle_steps > 30 * 16000
    for q in range(3):
        assert abs(ta.live[q] - tb.live[q]) <= 1, (list(ta.live), list(tb.live))
    pa, pb = a.get(pcl.Photon).particles(), b.get(pcl.Photon).particles()
    common, ia, ib = np.intersect1d(pa.sid, pb.sid, return_indices=True)
    assert len(common) >= len(pa.sid) - 2
    np.testing.assert_allclose(pb.x[ib], pa.x[ia], rtol=1e-5, atol=1e-9)
    np.testing.assert_allclose(pb.s[ib], pa.s[ia], rtol=1e-4, atol=1e-6)
    assert np.array_equal(pb.p[ib], pa.p[ia]) or np.mean(np.any(pb.p[ib] != pa.p[ia], axis=1)) < 1e-3
    a.close()
    # the same run against the oracle, step by step
    mp = _mixed(pcl, air, n=(512, 16384, 128), seed=31, steps_per_launch=spl)
    W = _oracle_from(oracle, pcl, mp, air, pusher)
    pcl.run(mp, pusher, 8e-12, 1e-12)
    for k in range(8):
        W.advance((k + 1) * 1e-12, 4)
    _check(pcl, oracle, mp, W, rtol=3 * RTOL)
    mp.close(); b.close()


@pytest.mark.parametrize("spl", [1, 8])
def test_full_stash_same_results(pcl, gpu, air, spl):
    """A collision that finds its warp's stash full stays in its lane and
    collides at the start of the next iteration.  With 8 or 40 of the stash's
    entries in use that happens all the time (the full stash of 72 rarely
    fills on these populations), and the particles and tallies are bit for bit
    those of the full stash: where a particle collides changes the order of a
    warp's work, not any particle's operations."""
    pusher = _pusher(pcl, air, E=2e6)
    runs = [_mixed(pcl, air, n=(8192, 2048, 1024), seed=14, steps_per_launch=spl, stash_entries=st)
            for st in (0, 8, 40)]
    for mp in runs:
        pcl.run(mp, pusher, 8 * 25e-12, 25e-12)
    ta = runs[0].tallies()
    for b in runs[1:]:
        tb = b.tallies()
        assert tb.steps == ta.steps == 8
        assert list(tb.live) == list(ta.live) and tb.particle_steps == ta.particle_steps
        assert list(tb.spawned) == list(ta.spawned)
        for q in range(3):
            assert list(tb.collisions[q]) == list(ta.collisions[q])
        for k in runs[0].index:
            pa, pb = runs[0].get(k).particles(), b.get(k).particles()
            oa, ob = np.argsort(pa.sid), np.argsort(pb.sid)
            for f in ("sid", "ctr", "p", "x", "s", "w"):
                np.testing.assert_array_equal(getattr(pb, f)[ob], getattr(pa, f)[oa])
    for mp in runs:
        mp.close()
    with pytest.raises(pcl.PCLError):
        _mixed(pcl, air, n=(64, 64, 64), seed=14, stash_entries=73)


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


@pytest.mark.parametrize("dt", [1e-12, 25e-12])
def test_classic_kernel_vs_oracle(pcl, oracle, gpu, air, dt):
    """The classic step kernel (each lane collides in place) against the
    oracle; every other parity test runs the default event kernel."""
    mp = _mixed(pcl, air, seed=3 if dt < 1e-11 else 4, classic_step=True)
    pusher = _pusher(pcl, air)
    W = _oracle_from(oracle, pcl, mp, air, pusher)
    pcl.advance(mp, pusher, dt)
    W.advance(dt, 4)
    _check(pcl, oracle, mp, W, stol=2 * RTOL * max(1.0, dt / 1e-12 / 3))
    t = mp.tallies()
    c = W.counters()
    diff = np.abs(np.array([list(t.collisions[s]) for s in range(3)]) - c["coll"]).sum()
    assert diff <= 4 * (c["ties"] + 1), (diff, c["ties"])
    mp.close()


@pytest.mark.parametrize("spl", [1, 4])
def test_event_kernel_matches_plain(pcl, gpu, air, spl):
    """Event and plain step kernels over 12 steps of 25 ps: the same draw
    counts for all but rounding-separated particles, momenta equal to FP32
    rounding, collision counts equal to 1e-4."""
    pusher = _pusher(pcl, air, E=2e6)
    runs = []
    for ev in (False, True):
        mp = _mixed(pcl, air, n=(8192, 2048, 1024), seed=14, steps_per_launch=spl, classic_step=not ev)
        pcl.run(mp, pusher, 12 * 25e-12, 25e-12)
        runs.append(mp)
    a, b = runs
    ta, tb = a.tallies(), b.tallies()
    ca = np.array([list(ta.collisions[s]) for s in range(3)]); cb = np.array([list(tb.collisions[s]) for s in range(3)])
    assert np.abs(ca - cb).sum() <= 1e-4 * ca.sum() + 2
    for k in a.index:
        pa, pb = a.get(k).particles(), b.get(k).particles()
        common, ia, ib = np.intersect1d(pa.sid, pb.sid, return_indices=True)
        assert len(common) >= 0.995 * max(len(pa.sid), len(pb.sid))
        same = pa.ctr[ia] == pb.ctr[ib]
        assert same.mean() >= 0.995
        dp = np.linalg.norm(pa.p[ia] - pb.p[ib], axis=1)[same] / np.linalg.norm(pb.p[ib], axis=1)[same]
        assert np.quantile(dp, 0.99) < 1e-4, np.quantile(dp, [0.5, 0.99])
    a.close(); b.close()


def test_autotune_keeps_physics(pcl, gpu, air):
    """The autotuner advances real steps and keeps a valid launch shape; the
    population it leaves equals a plain run of the same number of steps up to
    FP32 rounding (launch shapes do not change the physics, but the event and
    classic kernels may round their inlined arithmetic differently, and a
    multi-step launch keeps the sub-eps remainder of a step as a double-float
    where separate launches round it to FP32)."""
    pusher = _pusher(pcl, air, E=2e6)
    a = _mixed(pcl, air, n=(2048, 1024, 512), seed=21)
    # a budget of 512 steps: 8 trials of 64 (the step kernels, then 1-8 steps
    # per launch) before the budget ends the search
    r = a.autotune(pusher, 1e-12, steps=512)
    assert r["blocks_per_sm"] in (0, 2, 3, 4) and r["steps_per_launch"] in (1, 2, 4, 8)
    assert r["compaction_period"] in (2, 4, 8, 16, 32) and r["use_graph"] in (0, 1)
    assert r["trials"] == 8 and r["steps"] == 512 and r["rate"] > 0
    ta = a.tallies()
    assert ta.steps == 512
    b = _mixed(pcl, air, n=(2048, 1024, 512), seed=21)
    pcl.run(b, pusher, 512e-12, 1e-12)
    tb = b.tallies()
    for s in range(3):
        assert abs(ta.live[s] - tb.live[s]) <= 2 + ta.live[s] // 1000
    for k in a.index:
        pa, pb = a.get(k).particles(), b.get(k).particles()
        common, ia, ib = np.intersect1d(pa.sid, pb.sid, return_indices=True)
        assert len(common) >= 0.999 * max(len(pa.sid), len(pb.sid)) - 2
        dp = np.linalg.norm(pa.p[ia] - pb.p[ib], axis=1) / np.maximum(np.linalg.norm(pb.p[ib], axis=1), 1e-300)
        assert np.mean(dp > 1e-4) <= 2e-3, np.sort(dp)[-5:]
    a.close(); b.close()


@pytest.mark.parametrize("kind", ["double_layer", "step", "confined"])
def test_position_dependent_fields(pcl, oracle, gpu, air, kind):
    """DoubleLayerField, StepField, ConfinedDoubleLayerField (field.jl:10-52),
    evaluated at both RK2 stage positions, against the oracle."""
    F = {"double_layer": pcl.DoubleLayerField(-0.004, 0.004, (0.0, 0.0, -1.5e6)),
         "step": pcl.StepField(0.0, (0.0, 0.0, -1.5e6), (2e5, 0.0, 3e5)),
         "confined": pcl.ConfinedDoubleLayerField(0.01, 0.008, 0.004, -1.5e6)}[kind]
    pusher = pcl.RK2Pusher(pcl.CombinedForcing(pcl.ElectromagneticField(F, pcl.HomogeneousField((0.0, 0.0, 0.0))),
                                               air["cl"]))
    rng = np.random.default_rng(40)
    pops = {pcl.Electron: random_population(pcl, pcl.Electron, 4096, 1e4, 3e7, rng, spread_x=0.004),
            pcl.Positron: random_population(pcl, pcl.Positron, 1024, 1e4, 3e7, rng, spread_x=0.004)}
    mp = pcl.MultiPopulation(*[(k, pcl.Population(1 << 15, pops[k], air["tabs"][k], air["cuts"][k], particle=k))
                               for k in pops], (pcl.Photon, pcl.Population(1 << 15, [], air["tabs"][1],
                                                                            air["cuts"][1], particle=pcl.Photon)),
                             seed=40)
    W = _oracle_from(oracle, pcl, mp, air, pusher)
    for k in range(8):
        pcl.advance(mp, pusher, (k + 1) * 5e-12)
        W.advance((k + 1) * 5e-12, 4)
    # 40 ps: s carries the FP32 rate-bound error once per collision (as the 25-ps
    # test).  A field that jumps at a plane (double layer, step) can separate a
    # trajectory whose earlier sub-step the tie tracking did not see as close
    # (observed: 1 of ~4000 electrons in 8 steps): up to 2 draw-count mismatches
    _check(pcl, oracle, mp, W, rtol=3 * RTOL, stol=4e-4, max_bad=0 if kind == "confined" else 2)
    mp.close()


@pytest.mark.parametrize("wall_species", ["electron", "photon"])
def test_general_kernel_multistep(pcl, gpu, air, wall_species):
    """The general kernel (position-dependent field, wall records) with four
    and eight steps per launch (its multi-step instance: collide batches with
    the lanes' particles held, photon flights over collision-free whole steps
    unless the photons have the wall) equals one step per launch bit for bit:
    the particles and the wall crossings (matched by stream id; their times,
    kept in FP32 from the launch's start, to that rounding)."""
    F = pcl.DoubleLayerField(-0.004, 0.004, (0.0, 0.0, -1.5e6))
    pusher = pcl.RK2Pusher(pcl.CombinedForcing(pcl.ElectromagneticField(F, pcl.HomogeneousField((0.0, 0.0, 0.0))),
                                               air["cl"]))
    wsp = {"electron": pcl.Electron, "photon": pcl.Photon}[wall_species]
    out = []
    for K in (1, 4, 8):
        rng = np.random.default_rng(41)
        arr = random_population(pcl, pcl.Electron, 4096, 1e4, 3e7, rng, spread_x=0.004)
        ph = random_population(pcl, pcl.Photon, 4096, 1e4, 3e7, rng, spread_x=0.004)
        mp = pcl.MultiPopulation((pcl.Electron, pcl.Population(1 << 15, arr, air["tabs"][0], air["cuts"][0],
                                                              particle=pcl.Electron)),
                                 (pcl.Photon, pcl.Population(1 << 15, ph, air["tabs"][1], air["cuts"][1],
                                                             particle=pcl.Photon)), seed=41, steps_per_launch=K)
        wall = pcl.WallCallback(wsp, 3, 0.002, drop=False)
        pcl.run(mp, pusher, 8 * 5e-12, 5e-12, wall)
        out.append(([mp.get(q).particles() for q in (0, 1)], wall.states()))
        mp.close()
    pa, wa = out[0]
    assert len(wa.w) > 50
    oa = np.lexsort((wa.t, wa.sid))
    for pb, wb in out[1:]:
        for a, b in zip(pa, pb):
            ia, ib = np.argsort(a.sid), np.argsort(b.sid)
            for f in ("sid", "ctr", "p", "x", "s", "w"):
                np.testing.assert_array_equal(getattr(b, f)[ib], getattr(a, f)[ia])
        assert len(wa.w) == len(wb.w)
        ob = np.lexsort((wb.t, wb.sid))
        for f in ("sid", "x", "p", "w"):
            np.testing.assert_array_equal(getattr(wb, f)[ob], getattr(wa, f)[oa])
        np.testing.assert_allclose(wb.t[ob], wa.t[oa], rtol=0, atol=1e-17)


@pytest.mark.parametrize("drop", [True, False])
def test_wall_callback(pcl, oracle, gpu, air, drop):
    """WallCallback (callback.jl:146-184): the same crossings as the oracle
    (stream ids, interpolated positions on the wall, momenta, times), the
    crossing's extra draw, and the dropped particles."""
    pusher = _pusher(pcl, air, E=1e6)
    rng = np.random.default_rng(50)
    n = 4096
    arr = random_population(pcl, pcl.Electron, n, 3e4, 3e7, rng, spread_x=0.002)
    mp = pcl.MultiPopulation((pcl.Electron, pcl.Population(1 << 15, arr, air["tabs"][0], air["cuts"][0],
                                                          particle=pcl.Electron)),
                             (pcl.Photon, pcl.Population(1 << 15, [], air["tabs"][1], air["cuts"][1],
                                                         particle=pcl.Photon)), seed=50)
    wall = pcl.WallCallback(pcl.Electron, 3, 0.003, drop=drop)
    W = _oracle_from(oracle, pcl, mp, {**air, "tabs": {0: air["tabs"][0], 1: air["tabs"][1]},
                                       "cuts": {0: air["cuts"][0], 1: air["cuts"][1]}}, pusher)
    W.set_wall(pcl.Electron, 2, 0.003, drop)
    pcl.run(mp, pusher, 10 * 5e-12, 5e-12, wall)
    for k in range(10):
        W.advance((k + 1) * 5e-12, 4)
    g = wall.states()
    osp, osid, ox, op, ow, ot = W.get_wall()
    assert len(g.w) > 100
    og = dict(zip(g.sid.tolist(), range(len(g.w))))
    ties = W.download(pcl.Electron).tie
    matched = 0
    for i in range(len(ow)):
        j = og.get(int(osid[i]))
        if j is None:
            continue
        matched += 1
        assert abs(g.x[j, 2] - 0.003) < 1e-7
        np.testing.assert_allclose(g.p[j], op[i], rtol=1e-4, atol=1e-4 * np.linalg.norm(op[i]))
        assert abs(g.t[j] - ot[i]) < 1e-4 * 50e-12
    assert matched >= 0.99 * len(ow) - 2 and abs(len(g.w) - len(ow)) <= max(2, 0.01 * len(ow)), \
        (matched, len(g.w), len(ow))
    rep = oracle.compare_populations(mp.get(0).particles(), W.download(pcl.Electron), pcl.Electron, rtol=3 * RTOL,
                                     stol=2e-4)
    assert rep["ok"], str(rep)
    mp.close()


def test_roulette_split_parity(pcl, oracle, gpu, air):
    """roulette! and split! (population.jl:291-335) on the device against the
    oracle: the same survivors and copies (stream ids), weights, and the same
    evolution of the copies afterwards."""
    mp = _mixed(pcl, air, n=(4096, 1024, 512), seed=60)
    pusher = _pusher(pcl, air, E=1e6)
    W = _oracle_from(oracle, pcl, mp, air, pusher)
    pcl.advance(mp, pusher, 5e-12)
    W.advance(5e-12, 4)
    mp.roulette(pcl.Electron, 0.375)
    W.roulette(pcl.Electron, 0.375)
    pcl.repack(mp.get(pcl.Electron))
    g, o = mp.get(0).particles(), W.download(0)
    assert 0.3 * 4096 < len(g.w) < 0.45 * 4096
    rep = oracle.compare_populations(g, o, pcl.Electron, rtol=3 * RTOL, max_unmatched_frac=0.002)
    assert rep["ok"], str(rep)
    mp.split(pcl.Positron, 0.75)
    W.split(pcl.Positron, 0.75)
    g, o = mp.get(2).particles(), W.download(2)
    assert len(g.w) > 1.5 * 400
    rep = oracle.compare_populations(g, o, pcl.Positron, rtol=3 * RTOL, max_unmatched_frac=0.002)
    assert rep["ok"], str(rep)
    for k in range(3):
        pcl.advance(mp, pusher, (k + 2) * 5e-12)
        W.advance((k + 2) * 5e-12, 4)
    _check(pcl, oracle, mp, W, rtol=3 * RTOL, stol=2e-4)
    mp.close()


def test_roulette_split_tables(pcl, oracle, gpu, air):
    """roulette!(f, popl) and split!(f, popl) with f of the kinetic energy
    (population.jl:291-305, 316-331) on the device (pcl_roulette_fn,
    pcl_split_fn): a constant table gives the constant roulette's particles
    bit for bit; energy-dependent tables match the oracle (survivors, copies,
    weights, and the copies' evolution afterwards); a callable gives the same
    particles as its own tabulation."""
    eV = pcl.co.eV
    out = []
    for f in (0.375, (np.array([1.0, 1e8]) * eV, np.array([0.375, 0.375]))):
        mp = _mixed(pcl, air, n=(4096, 1024, 512), seed=62)
        mp.roulette(pcl.Electron, f)
        pcl.repack(mp.get(pcl.Electron))
        out.append(mp.get(0).particles())
        mp.close()
    a, b = out
    assert 0.3 * 4096 < len(a.w) < 0.45 * 4096
    oa, ob = np.argsort(a.sid), np.argsort(b.sid)
    for fld in ("sid", "ctr", "p", "x", "w"):
        np.testing.assert_array_equal(getattr(b, fld)[ob], getattr(a, fld)[oa])
    keep = (np.array([1e4, 3e7]) * eV, np.array([0.1, 0.9]))
    copies = (np.array([1e4, 3e7]) * eV, np.array([0.0, 2.0]))
    mp = _mixed(pcl, air, n=(4096, 1024, 1024), seed=63)
    pusher = _pusher(pcl, air, E=1e6)
    W = _oracle_from(oracle, pcl, mp, air, pusher)
    mp.roulette(pcl.Electron, keep)
    W.roulette(pcl.Electron, keep)
    mp.split(pcl.Positron, copies)
    W.split(pcl.Positron, copies)
    pcl.repack(mp.get(pcl.Electron))
    # log-uniform energies over 10 keV - 30 MeV: a value linear in E averages
    # 1/8 of the way along its range (keep ~0.2, ~0.25 copies)
    for k, lo, hi in ((pcl.Electron, 0.15 * 4096, 0.3 * 4096), (pcl.Positron, 1.15 * 1024, 1.4 * 1024)):
        g, o = mp.get(k).particles(), W.download(k)
        assert lo < len(g.w) < hi, (k, len(g.w))
        rep = oracle.compare_populations(g, o, k, rtol=3 * RTOL, max_unmatched_frac=0.002)
        assert rep["ok"], str(rep)
    for k in range(3):
        pcl.advance(mp, pusher, (k + 1) * 5e-12)
        W.advance((k + 1) * 5e-12, 4)
    _check(pcl, oracle, mp, W, rtol=3 * RTOL, stol=2e-4)
    mp.close()
    out = []
    for f in (lambda E: np.clip(0.1 + 0.8 * np.log(E / (1e4 * eV)) / np.log(3e3), 0.1, 0.9),
              pcl.energy_table(lambda E: np.clip(0.1 + 0.8 * np.log(E / (1e4 * eV)) / np.log(3e3), 0.1, 0.9))):
        mp = _mixed(pcl, air, n=(4096, 1024, 512), seed=64)
        pcl.roulette(f, mp.get(pcl.Electron))
        pcl.split(f, mp.get(pcl.Photon))
        out.append([mp.get(q).particles() for q in (0, 1)])
        mp.close()
    for a, b in zip(*out):
        oa, ob = np.argsort(a.sid), np.argsort(b.sid)
        for fld in ("sid", "ctr", "p", "w"):
            np.testing.assert_array_equal(getattr(b, fld)[ob], getattr(a, fld)[oa])


@pytest.mark.parametrize("spl", [1, 8])
def test_restricted_pushers(pcl, oracle, gpu, air, spl):
    """RestrictedForcing{T}, RestrictedPusher{T} and NullPusher (pusher.jl:
    28-34, 67-76) on the device against the oracle (pcl_set_push_mask; a
    species that is not pushed runs on the general kernel, the others on the
    homogeneous one), with one and eight steps per launch; and the restricted
    forcing's starting electrons (field, no loss) equal those of a run with the
    field alone bit for bit (the same kernel: a forcing restricted away from a
    species is a zero charge or no loss table in its header)."""
    zero = pcl.HomogeneousField((0.0, 0.0, 0.0))
    em = pcl.ElectromagneticField(pcl.HomogeneousField((0.0, 0.0, -2e6)), zero)
    full = pcl.RK2Pusher(pcl.CombinedForcing(em, air["cl"]))
    pushers = {"restricted_forcing": pcl.RK2Pusher(pcl.CombinedForcing(pcl.RestrictedForcing("electron", em),
                                                                      pcl.RestrictedForcing("positron", air["cl"]))),
               "restricted_pusher": pcl.RestrictedPusher("electron", full),
               "null": pcl.NullPusher()}
    finals = {}
    for name, pusher in pushers.items():
        mp = _mixed(pcl, air, n=(2048, 1024, 1024), seed=70, steps_per_launch=spl)
        W = _oracle_from(oracle, pcl, mp, air, pusher)
        x0 = {k: mp.get(k).particles() for k in (0, 1, 2)}
        pcl.run(mp, pusher, 8e-12, 1e-12)
        for k in range(8):
            W.advance((k + 1) * 1e-12, 4)
        _check(pcl, oracle, mp, W, rtol=3 * RTOL, stol=2e-4)
        if name == "null":
            start = np.concatenate([x0[k].x for k in x0]).astype(np.float32)
            for k in (0, 1, 2):
                x = mp.get(k).particles().x.astype(np.float32)
                assert np.all((x[:, None, :] == start[None, :, :]).all(axis=2).any(axis=1)), k
        finals[name] = mp.get(pcl.Electron).particles()
        mp.close()
    # the restricted forcing's electrons feel the field and no loss
    mp = _mixed(pcl, air, n=(2048, 1024, 1024), seed=70, steps_per_launch=spl)
    sids = mp.get(pcl.Electron).particles().sid
    pcl.run(mp, pcl.RK2Pusher(pcl.CombinedForcing(em)), 8e-12, 1e-12)
    ref = mp.get(pcl.Electron).particles()
    mp.close()
    a, b = ref, finals["restricted_forcing"]
    ia, ib = np.isin(a.sid, sids), np.isin(b.sid, sids)
    assert ia.sum() == ib.sum() > 1000
    oa, ob = np.argsort(a.sid[ia]), np.argsort(b.sid[ib])
    for fld in ("sid", "ctr", "p", "x", "s", "w"):
        np.testing.assert_array_equal(getattr(b, fld)[ib][ob], getattr(a, fld)[ia][oa])


@pytest.mark.parametrize("spl", [1, 8])
def test_position_dependent_b(pcl, oracle, gpu, air, spl):
    """A position-dependent B (ElectromagneticField(e, b) with b a field
    functor, field.jl:54-70; pcl_set_bfield): a 0.1 T slab across the middle
    of the population, with the field and the continuum loss, on the general
    kernel with one and eight steps per launch, against the oracle."""
    B = pcl.DoubleLayerField(-0.001, 0.001, (0.1, 0.0, 0.05))
    pusher = pcl.RK2Pusher(pcl.CombinedForcing(
        pcl.ElectromagneticField(pcl.HomogeneousField((0.0, 0.0, -2e6)), B), air["cl"]))
    rng = np.random.default_rng(71)
    pops = {pcl.Electron: random_population(pcl, pcl.Electron, 4096, 1e4, 3e7, rng, spread_x=0.003),
            pcl.Photon: random_population(pcl, pcl.Photon, 1024, 5e3, 3e7, rng, spread_x=0.003),
            pcl.Positron: random_population(pcl, pcl.Positron, 1024, 1e4, 3e7, rng, spread_x=0.003)}
    mp = pcl.MultiPopulation(*[(k, pcl.Population(1 << 16, pops[k], air["tabs"][k], air["cuts"][k], particle=k))
                               for k in pops], seed=71, steps_per_launch=spl)
    W = _oracle_from(oracle, pcl, mp, air, pusher)
    pcl.run(mp, pusher, 8 * 5e-12, 5e-12)
    for k in range(8):
        W.advance((k + 1) * 5e-12, 4)
    # s carries the FP32 rate-bound error once per collision: 5-ps steps, the
    # bound of the E-field shapes' test
    _check(pcl, oracle, mp, W, rtol=3 * RTOL, stol=4e-4)
    mp.close()


def test_new_entry_points_refuse_bad_arguments(pcl, gpu, air):
    """pcl_roulette_fn / pcl_split_fn / pcl_set_push_mask / pcl_set_bfield
    refuse malformed input with PCL_ERR_INVALID and a message, and leave the
    context usable: tables that are empty, too long, not increasing, or with a
    split mean outside [0, 64]; masks beyond 3 bits; unknown field kinds or a
    confined layer without widths."""
    eV = pcl.co.eV
    mp = _mixed(pcl, air, n=(512, 256, 128), seed=72)
    bad_tables = [(np.array([]), np.array([])),
                  (np.geomspace(1.0, 1e9, 4097) * eV, np.full(4097, 0.5)),
                  (np.array([2.0, 1.0]) * eV, np.array([0.5, 0.5])),
                  (np.array([1.0, 1.0]) * eV, np.array([0.5, 0.5])),
                  (np.array([1.0, np.nan]) * eV, np.array([0.5, 0.5]))]
    for E, v in bad_tables:
        with pytest.raises(pcl.PCLError):
            mp.roulette(pcl.Electron, (E, v))
        with pytest.raises(pcl.PCLError):
            mp.split(pcl.Electron, (E, v))
    with pytest.raises(pcl.PCLError):
        mp.split(pcl.Electron, (np.array([1.0, 2.0]) * eV, np.array([0.5, 65.0])))
    L = pcl.lib()
    for masks in ((8, 7, 7), (7, -1, 7), (7, 7, 9)):
        with pytest.raises(pcl.PCLError):
            pcl._lib.check(L.pcl_set_push_mask(mp.ctx, *masks), mp.ctx, "pcl_set_push_mask")
    for kind, params in ((4, [0.0] * 8), (1, [0.0, 1.0]), (3, [0.0, 1.0, 1.0, 1.0])):
        p = np.ascontiguousarray(np.asarray(params, dtype=float))
        with pytest.raises(pcl.PCLError):
            pcl._lib.check(L.pcl_set_bfield(mp.ctx, kind, pcl._lib.dptr(p), len(params)), mp.ctx, "pcl_set_bfield")
    n0 = len(mp.get(pcl.Electron).particles().w)
    mp.roulette(pcl.Electron, (np.array([1.0, 1e9]) * eV, np.array([1.0, 1.0])))
    pcl.advance(mp, _pusher(pcl, air), 1e-12)
    assert len(mp.get(pcl.Electron).particles().w) > 0.9 * n0
    mp.close()


def test_roulette_callback_keeps_weight(pcl, gpu, air):
    """RouletteCallback(m): populations stay near m while the total weight is
    kept in expectation."""
    pusher = _pusher(pcl, air, E=1e6)
    a = _mixed(pcl, air, n=(8192, 2048, 512), seed=61)
    b = _mixed(pcl, air, n=(8192, 2048, 512), seed=61)
    pcl.run(a, pusher, 3e-12, 1e-12, pcl.RouletteCallback(2000))
    pcl.run(b, pusher, 3e-12, 1e-12)
    n = pcl.nactives(a.get(0))
    wa, wb = pcl.weight(a.get(0)), pcl.weight(b.get(0))
    # roulette at keep probability q adds variance n (1/q - 1) per application
    sigma = np.sqrt(3 * 8192 * (8192 / 2000 - 1))
    assert 1500 < n < 2600 and abs(wa - wb) < 6 * sigma, (n, wa, wb, sigma)
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


@pytest.mark.gpu
def test_energy_histogram(pcl, gpu, air):
    """pcl_energy_histogram against numpy on the downloaded particles: counts
    and summed weights per bin edges[i] <= E < edges[i+1] (StatsBase.fit
    semantics), equal except for particles within 1e-9 of an edge."""
    rng = np.random.default_rng(21)
    n = 200_000
    E0 = 10 ** rng.uniform(3.5, 7.5, n) * pcl.co.eV
    p = pcl.workloads.isotropic(n, 1e6 * pcl.co.eV, rng)
    p *= (pcl.momentum_norm_from_kin(pcl.Electron, E0) / np.linalg.norm(p, axis=1))[:, None]
    w = rng.uniform(0.5, 2.0, n)
    arr = pcl.ParticleArrays(np.zeros((n, 3)), p, w, np.zeros(n))
    mp = pcl.MultiPopulation(
        ("electron", pcl.Population(n, arr, air["tabs"][0], air["cuts"][0], particle=pcl.Electron)), seed=3)
    pop = mp.get(pcl.Electron)
    g = pop.particles()
    E = pcl.kinenergy(pcl.Electron, g.p)
    for edges in (10 ** np.linspace(4, 7, 201) * pcl.co.eV, np.array([0.0, 1e5 * pcl.co.eV]),
                  np.sort(rng.uniform(1e4, 1e7, 4097)) * pcl.co.eV):
        counts, wsum = pop.energy_histogram(edges)
        b = np.searchsorted(edges, E, side="right") - 1
        ok = (b >= 0) & (b < len(edges) - 1)
        ref_c = np.bincount(b[ok], minlength=len(edges) - 1)
        ref_w = np.bincount(b[ok], weights=g.w[ok], minlength=len(edges) - 1)
        k = np.searchsorted(edges, E)
        lo, hi = edges[np.clip(k - 1, 0, len(edges) - 1)], edges[np.clip(k, 0, len(edges) - 1)]
        near = (np.abs(E - lo) <= 1e-9 * E) | (np.abs(E - hi) <= 1e-9 * E)
        slack = int(near.sum())
        assert np.abs(counts - ref_c).sum() <= 2 * slack, (np.abs(counts - ref_c).sum(), slack)
        np.testing.assert_allclose(wsum, ref_w, rtol=1e-9, atol=2.0 * slack + 1e-9)
    dens = pcl.spectrum(pop, edges, n=10.0)
    np.testing.assert_allclose(dens * np.diff(edges) * 10.0, wsum, rtol=1e-12)
    with pytest.raises(Exception):
        pop.energy_histogram(np.array([1.0, 0.5]))
    mp.close()


def _live_sorted(b, n):
    xw, ps, meta = b[0][:n], b[1][:n], b[2][:n]
    live = meta[:, 2] != np.uint32(0xFFFFFFFF)
    sid = meta[live, 0].astype(np.uint64) | (meta[live, 1].astype(np.uint64) << np.uint64(32))
    o = np.argsort(sid, kind="stable")
    return sid[o], xw[live][o], ps[live][o], meta[live][o], int((~live).sum())


@pytest.mark.gpu
@pytest.mark.parametrize("nchunks,mode", [(1, "auto"), (3, "auto"), (8, "auto"), (8, "direct"), (3, "direct")])
def test_advance_host_equals_upload_advance_download(pcl, gpu, nchunks, mode):
    """pcl_advance_host gives the particles of pcl_upload_packed + pcl_advance
    + pcl_download_packed, bit for bit (matched by stream id; dead slots in the
    same number), with and without the device repack, in both of its modes:
    the copy pipeline (chunked uploads, range launches and downloads on three
    streams; the default) and host-direct (the step kernel reads and writes
    the page-locked arrays over the link; refused for pageable arrays)."""
    a = pcl.workloads.avalanche(n=60_000, seed=4, capacity=1 << 18)
    b = pcl.workloads.avalanche(n=60_000, seed=4, capacity=1 << 18)
    ba, bb = a.mpopl.packed_buffers(pinned=(nchunks == 8)), b.mpopl.packed_buffers()
    if nchunks == 3:   # existing arrays page-locked in place (pcl_host_register)
        pins = [pcl.population.PinnedHost(x[:3]) for x in ba]
    a.mpopl.set_host_io({"auto": 0, "copy": 1, "direct": 2}[mode])
    if nchunks == 1:   # pageable arrays: host-direct mode is refused
        b.mpopl.set_host_io(2)
        nb0 = b.mpopl.download_packed(bb)
        with pytest.raises(Exception):
            b.mpopl.advance_host(b.dt, bb, nb0)
        b.mpopl.set_host_io(0)
    na, nb = a.mpopl.download_packed(ba), b.mpopl.download_packed(bb)
    small = [(x[0][:10], x[1][:10], x[2][:10], None) for x in ba]
    with pytest.raises(Exception):      # output arrays smaller than the input: refused before any work
        a.mpopl.advance_host(a.dt, ba, na, out=small, nchunks=nchunks)
    for k in range(3):
        t = (k + 1) * a.dt
        compact = k == 1
        if k == 0:
            a.mpopl.set_pusher(a.pusher)
        na = a.mpopl.advance_host(t, ba, na, nchunks=nchunks, compact=compact)
        b.mpopl.upload_packed(bb, nb)
        pcl.advance(b.mpopl, b.pusher, t)
        if compact:
            pcl.lib().pcl_compact(b.mpopl.ctx)
        nb = b.mpopl.download_packed(bb)
        assert na == nb, (k, na, nb)
        for s in (0, 1, 2):
            x, y = _live_sorted(ba[s], na[s]), _live_sorted(bb[s], nb[s])
            assert x[4] == y[4]
            for u, v in zip(x[:4], y[:4]):
                np.testing.assert_array_equal(u, v)
    ta, tb = a.mpopl.tallies(), b.mpopl.tallies()
    assert ta.particle_steps == tb.particle_steps
    if nchunks == 3:
        for q in pins:
            q.release()
    assert [list(r) for r in ta.collisions] == [list(r) for r in tb.collisions]
    a.mpopl.close()
    b.mpopl.close()


@pytest.mark.gpu
def test_device_cap_equals_roulette_callback(pcl, gpu):
    """pcl_set_swarm_cap on a context without swarms is RouletteCallback(m)
    (callback.jl:210-227) on the device: after the same steps it keeps and
    reweights exactly the particles the host-driven callback keeps."""
    a = pcl.workloads.avalanche(n=40_000, seed=6, capacity=1 << 18)
    b = pcl.workloads.avalanche(n=40_000, seed=6, capacity=1 << 18)
    m = 30_000
    cb = pcl.RouletteCallback(m)
    b.mpopl.set_swarm_cap(m, particles=(pcl.Electron, pcl.Photon, pcl.Positron))
    for k in range(2):
        t = (k + 1) * a.dt
        pcl.run(a.mpopl, a.pusher, t, a.dt)
        cb.onstep(a.mpopl, t)
        pcl.run(b.mpopl, b.pusher, t, b.dt)
    pcl.lib().pcl_compact(b.mpopl.ctx)
    ne = pcl.nactives(b.mpopl.get(pcl.Electron))
    assert abs(ne - m) < 5 * np.sqrt(m) + 1
    for sp in (pcl.Electron, pcl.Photon, pcl.Positron):
        ga, gb = a.mpopl.get(sp).particles(), b.mpopl.get(sp).particles()
        oa, ob = np.argsort(ga.sid), np.argsort(gb.sid)
        np.testing.assert_array_equal(ga.sid[oa], gb.sid[ob])
        np.testing.assert_array_equal(ga.w[oa], gb.w[ob])
        np.testing.assert_array_equal(ga.p[oa], gb.p[ob])
    a.mpopl.close()
    b.mpopl.close()


def _subset(a, m):
    return type(a)(**{f: getattr(a, f)[m] for f in ("x", "p", "w", "t", "s", "sid", "ctr")})


def test_full_size_subset_parity(pcl, oracle, gpu, air):
    """The bench workload at full size: 2^24 particles drawn from the grown
    mixed e-/gamma/e+ state, stepped twice on the device; a random 4096 of
    them, across the three species (2800 electrons, 512 positrons, photons
    for the rest), stepped by the oracle from the same state.  A particle's
    step depends only on its own state and stream, so the subset and all its
    secondaries must match the oracle as in the small cases (draw counts,
    stream ids, momenta to 1e-5)."""
    n = 1 << 24
    wl = pcl.workloads.rrea_mixed(n, seed=0, tables=(air["tabs"][0], air["tabs"][1], air["tabs"][2]))
    mp, pusher = wl.mpopl, _pusher(pcl, air)
    g0 = {sp: mp.get(sp).particles() for sp in (0, 1, 2)}
    assert sum(len(g0[sp].w) for sp in g0) == n
    assert min(len(g0[sp].w) for sp in g0) > 1000
    rng = np.random.Generator(np.random.Philox(1))
    npos = len(g0[2].w)
    share = {0: 2800, 1: 4096 - 2800 - min(npos, 512), 2: min(npos, 512)}
    W = oracle.OracleWorld(0, air["tabs"], air["cuts"], pusher)
    for sp in (0, 1, 2):
        sel = np.sort(rng.choice(len(g0[sp].w), share[sp], replace=False))
        W.upload(sp, _subset(g0[sp], sel))
    del g0
    dt = 1e-12
    for k in range(2):
        pcl.advance(mp, pusher, (k + 1) * dt)
        W.advance((k + 1) * dt, 8)
    t = mp.tallies()
    assert sum(t.live) > n * 0.99 and not any(t.errors), (list(t.live), list(t.errors))
    for sp in (pcl.Electron, pcl.Photon, pcl.Positron):
        o = W.download(sp)
        assert len(o.w) > 0.9 * share[sp]
        g = mp.get(sp).particles()
        gs = _subset(g, np.isin(g.sid, o.sid))
        rep = oracle.compare_populations(gs, o, sp, rtol=RTOL, stol=2 * RTOL)
        assert rep["ok"], str(rep)
    mp.close()


def test_bounded_wait_times_out_and_context_survives(pcl, gpu, air):
    """Failure detection without a fault: a device wait that nothing completes
    gives up at its poll limit, the call returns PCL_ERR_TIMEOUT, and the same
    context then steps as usual."""
    mp = _mixed(pcl, air, n=(1024, 256, 128), seed=12)
    L = pcl.lib()
    assert L.pcl_test_timeout(mp.ctx, 0) == pcl._lib.PCL_ERR_INVALID
    assert L.pcl_test_timeout(mp.ctx, 2000) == pcl._lib.PCL_ERR_TIMEOUT
    assert b"bounded wait" in L.pcl_last_error(mp.ctx)
    pcl.advance(mp, _pusher(pcl, air), 1e-12)
    t = mp.tallies()
    assert t.steps == 1 and t.particle_steps > 0
    mp.close()


@pytest.mark.parametrize("kind", ["grow", "decay"])
def test_population_target_stop(pcl, oracle, gpu, air, kind):
    """PopulationTargetCallback{S}(n, ismax) (callback.jl:253-267) through
    pcl_run: run! (run.jl:1-29) stops after the first step on which the
    species reaches the target.  A run without a target gives the per-step
    counts and the target; the run with it must stop on the first step that
    reaches it, with one step per launch and with eight (the launches shrink
    near the target), leave the same particles in both, bit for bit, and match
    the oracle stepped as many steps."""
    dt, nsteps = 5e-12, 40
    rising = kind == "grow"
    seed = 70 if rising else 71
    sp = pcl.Electron if rising else pcl.Photon
    rng = np.random.default_rng(seed)
    # grow: MeV electrons (Moller secondaries are born faster than electrons
    # stop); decay: soft photons (photoelectric absorption)
    pops = {pcl.Electron: random_population(pcl, pcl.Electron, 2048, 3e6 if rising else 1e5, 3e7, rng),
            pcl.Photon: random_population(pcl, pcl.Photon, 2048 if not rising else 256, 6e3,
                                          2e4 if not rising else 1e6, rng),
            pcl.Positron: random_population(pcl, pcl.Positron, 128, 1e5, 1e7, rng)}

    def make(K):
        return pcl.MultiPopulation(*[(k, pcl.Population(1 << 16, pops[k], air["tabs"][k], air["cuts"][k],
                                                        particle=k)) for k in pops], seed=seed, steps_per_launch=K)
    pusher = _pusher(pcl, air, E=2e6)
    free = make(1)
    W = _oracle_from(oracle, pcl, free, air, pusher)
    counts = []
    for k in range(nsteps):
        pcl.advance(free, pusher, (k + 1) * dt)
        counts.append(int(free.tallies().live[sp]))
    free.close()
    c = np.asarray(counts)
    assert (c[-1] > c[0]) if rising else (c[-1] < c[0]), counts
    target = int(c[nsteps // 2])
    k_stop = int(np.argmax(c >= target)) if rising else int(np.argmax(c <= target))
    for k in range(k_stop + 1):
        W.advance((k + 1) * dt, 4)
    states = {}
    for K in (1, 8):
        mp = make(K)
        tal = pcl.run(mp, pusher, nsteps * dt, dt, pcl.PopulationTargetCallback(sp, target, ismax=rising))
        assert tal.steps == k_stop + 1, (K, tal.steps, k_stop + 1, counts, target)
        assert tal.live[sp] == counts[k_stop]
        # s carries the FP32 rate-bound rounding once per collision, ~3 per ps
        # (the scaling of the other multi-step comparisons)
        stol = 2 * RTOL * (k_stop + 1) * dt / 3e-12
        for q in (0, 1, 2):
            rep = oracle.compare_populations(mp.get(q).particles(), W.download(q), q, rtol=3 * RTOL, stol=stol)
            assert rep["ok"], (K, q, str(rep))
        states[K] = [mp.get(q).particles() for q in (0, 1, 2)]
        mp.close()
    # the launch shape does not change the physics: the same particles, bit
    # for bit (every collision goes through one call site of the samplers, and
    # photon flights replay each step's arithmetic)
    for a, b in zip(states[1], states[8]):
        oa, ob = np.argsort(a.sid), np.argsort(b.sid)
        np.testing.assert_array_equal(a.sid[oa], b.sid[ob])
        np.testing.assert_array_equal(a.p[oa], b.p[ob])
