"""The learned inverse-CDF sampler: training data from the table samplers,
networks trained on the GPU by the tensor-core kernels, their accuracy against
the table samplers (KS distance and chi^2 on the physical variable), the time
and uniforms a draw costs with and without the network, and the step with the
networks attached against the plain step."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KS_MAX = 0.01   # 1 % KS distance against the table sampler


@pytest.fixture(scope="module")
def setup(pcl, air, gpu):
    mp = pcl.MultiPopulation(*[(k, pcl.Population(1024, [], air["tabs"][k], air["cuts"][k], particle=k))
                               for k in air["tabs"]], seed=77)
    mp.set_pusher(pcl.workloads.pusher((0.0, 0.0, -5e5), cl=air["cl"]))
    et = air["tabs"][pcl.Electron]
    sb = pcl.learned.table_positions(et, pcl.learned.LEARN_SB)
    mo = pcl.learned.table_positions(et, pcl.learned.LEARN_MOLLER)
    nets = {}
    for j in (sb[0], mo[0]):
        kind = pcl.learned.LEARN_SB if j in sb else pcl.learned.LEARN_MOLLER
        net, loss = pcl.learned.train_sampler(mp, pcl.Electron, j, kind, samples=2e7, nT=256, Q=256, steps=6000,
                                              batch=8192, lr=2e-3, seed=j)
        nets[j] = (net, kind, loss)
    yield mp, et, sb, mo, nets
    for net, _, _ in nets.values():
        net.close()
    mp.close()


def _table_samples(pcl, mp, j, T, n, seed):
    """n draws of the table sampler at kinetic energies T (J, scalar or per
    draw), primary along z: the photon energy fraction k/T or the Moller
    fraction eps."""
    L = pcl.lib()
    T = np.broadcast_to(np.asarray(T, dtype=float), (n,))
    p = np.zeros((n, 3)); p[:, 2] = pcl.momentum_norm_from_kin(pcl.Electron, T)
    # the device works in FP32: use the energy its momentum represents
    p = (p / pcl.co.electron_mc).astype(np.float32).astype(np.float64) * pcl.co.electron_mc
    T = pcl.kinenergy(pcl.Electron, p)
    sid = (np.uint64(seed) << np.uint64(40)) + np.arange(n, dtype=np.uint64)
    gp = np.zeros(9 * n); gs = np.zeros(3 * n); gk = np.zeros(3 * n, np.int32); gc = np.zeros(n, np.uint32)
    rc = L.pcl_test_sampler(mp.ctx, pcl.Electron, j, n, pcl._lib.dptr(p.reshape(-1)), pcl._lib.u64ptr(sid),
                            pcl._lib.dptr(gp), pcl._lib.dptr(gs), pcl._lib.i32ptr(gk), pcl._lib.u32ptr(gc))
    assert rc == 0
    child = gp.reshape(n, 3, 3)[:, 1]
    kind = gk.reshape(n, 3)[:, 1]
    if kind[0] == pcl.Photon:
        return np.linalg.norm(child, axis=1) * pcl.co.c / T, gc
    return pcl.kinenergy(pcl.Electron, child) / T, gc


def _learned_samples(pcl, net, kind, T, n, seed, tcut=None, sb=None):
    u = np.random.default_rng(seed).random(n)
    T = np.broadcast_to(np.asarray(T, dtype=float), (n,))
    y = net.forward(pcl.learned.features(T, u)).astype(np.float64)
    if kind == pcl.learned.LEARN_SB:
        h = np.clip(y, 0.0, 1.0)
        return np.exp(np.minimum((1.0 - h) * pcl.learned.sb_ymin(sb, T), -1e-6))
    e0 = tcut / T
    v = np.clip(y, 0.0, 1.0)
    return e0 / (1.0 - v * (1.0 - 2.0 * e0))


def _ks(a, b):
    a = np.sort(a); b = np.sort(b)
    z = np.concatenate([a, b])
    return float(np.max(np.abs(np.searchsorted(a, z, side="right") / len(a) -
                               np.searchsorted(b, z, side="right") / len(b))))


def test_training_data_are_quantiles(pcl, setup):
    mp, et, sb, mo, nets = setup
    x, t = pcl.learned.learn_data(mp, pcl.Electron, sb[0], pcl.learned.LEARN_SB, samples=2e6, nT=16, Q=64)
    assert x.shape == (16 * 64, 2)
    a = x[:, 0].reshape(16, 64)
    assert np.allclose(a[:, 0], -1 + 2 * np.arange(16) / 15, atol=1e-6)
    tt = t.reshape(16, 64)
    assert np.all(np.diff(tt, axis=1) >= 0) and np.all((tt >= 0) & (tt <= 1))
    # the Moller set has no rows where tcut / T >= 0.45
    x2, t2 = pcl.learned.learn_data(mp, pcl.Electron, mo[0], pcl.learned.LEARN_MOLLER, samples=2e6, nT=16, Q=64)
    T = 10 ** (6 + 2 * x2[:, 0]) * pcl.co.eV
    assert np.all(1e4 * pcl.co.eV / T < 0.45) and len(x2) < len(x)
    assert np.all((t2 >= 0) & (t2 <= 1))


@pytest.mark.parametrize("which", ["sb", "moller"])
def test_learned_matches_table(pcl, setup, which):
    """KS distance < 1 % against the table sampler for primaries log-uniform in
    each decade of the trained range, and chi^2 per bin near 1.

    Single energies are reported, not held to 1 %: with the reference's
    swapped-corner interpolation weights (seltzer.jl:114-118, reproduced) the
    bremsstrahlung table sampler's distribution is piecewise constant in T
    (the pcum fraction picks the energy row), with steps at the 57 grid
    energies that a smooth network averages over."""
    mp, et, sb, mo, nets = setup
    j = sb[0] if which == "sb" else mo[0]
    net, kind, loss = nets[j]
    tcut = et.proc[j].tcut if which == "moller" else None
    n = 200_000
    rng = np.random.default_rng(17)
    decades = []
    for i, (lo, hi) in enumerate(((2.5e4, 1e5), (1e5, 1e6), (1e6, 1e7), (1e7, 1e8))):
        T = np.exp(rng.uniform(np.log(lo), np.log(hi), n)) * pcl.co.eV
        ref, _ = _table_samples(pcl, mp, j, T, n, seed=100 + i)
        got = _learned_samples(pcl, net, kind, T, n, seed=200 + i, tcut=tcut, sb=et.proc[j])
        ks = _ks(np.log(ref), np.log(got))
        edges = np.quantile(np.log(ref), np.linspace(0, 1, 41))
        edges[0], edges[-1] = -np.inf, np.inf
        h1, _ = np.histogram(np.log(ref), edges)
        h2, _ = np.histogram(np.log(got), edges)
        chi2 = float(np.sum((h1 - h2) ** 2 / np.maximum(h1 + h2, 1)) / 40)
        decades.append((lo, hi, ks, chi2))
    single = []
    for i, Tev in enumerate((3e4, 1e6, 5e7)):
        ref, _ = _table_samples(pcl, mp, j, Tev * pcl.co.eV, n, seed=300 + i)
        got = _learned_samples(pcl, net, kind, Tev * pcl.co.eV, n, seed=400 + i, tcut=tcut, sb=et.proc[j])
        single.append((Tev, _ks(np.log(ref), np.log(got))))
    print(which, "loss", loss, "decades", decades, "single", single)
    assert max(d[2] for d in decades) < KS_MAX, (loss, decades, single)


def test_gain_over_table_sampler_timed(pcl, setup):
    """What the trained network gains over the sampler it replaces, measured on
    the GPU (pcl_time_energy_draw, CUDA events, fastest of 5): the time per
    secondary-energy draw of 2^22 primaries spread over 1e4-1e8 eV, table
    sampler (one kernel) against network (inputs, tensor-core inference,
    output map), and the uniforms each draw consumes.  Both paths must give the
    same distribution (KS < 1 %); the times and draws are reported, whichever
    way they fall."""
    import ctypes as C
    mp, et, sb, mo, nets = setup
    L = pcl.lib()
    n = 1 << 22
    Tev = 10.0 ** (4.0 + 4.0 * (np.arange(n) + 0.5) / n)
    report = {}
    for which, j in (("sb", sb[0]), ("moller", mo[0])):
        net, kind, _ = nets[j]
        ms_t, ms_n = C.c_double(), C.c_double()
        ot = np.zeros(n, np.float32); on = np.zeros(n, np.float32); dr = np.zeros(n, np.uint32)
        rc = L.pcl_time_energy_draw(mp.ctx, pcl.Electron, j, kind, net.h, n, 5, C.byref(ms_t), C.byref(ms_n),
                                    ot.ctypes.data_as(C.POINTER(C.c_float)), on.ctypes.data_as(C.POINTER(C.c_float)),
                                    dr.ctypes.data_as(C.POINTER(C.c_uint32)))
        assert rc == 0, L.pcl_last_error(mp.ctx)
        ok = np.ones(n, bool) if which == "sb" else (et.proc[j].tcut / (Tev * pcl.co.eV) < 0.45)
        ks = _ks(np.log(ot[ok]), np.log(on[ok]))
        assert ks < KS_MAX, (which, ks)
        assert np.all(dr >= 1) and (which == "sb" or dr.mean() > 2.0)
        report[which] = {"ns_per_draw_table": 1e6 * ms_t.value / n, "ns_per_draw_network": 1e6 * ms_n.value / n,
                         "network_over_table_time": ms_n.value / ms_t.value,
                         "uniforms_per_draw_table": float(dr.mean()), "uniforms_per_draw_network": 1.0, "ks": ks}
        assert np.isfinite(ms_t.value) and np.isfinite(ms_n.value) and ms_t.value > 0 and ms_n.value > 0
    print("energy-draw cost", report)


def test_step_with_learned_samplers(pcl, air, setup):
    """The avalanche step with the networks attached: collisions are handed to
    the networks, and spawn counts, live counts and the photon spectrum agree
    with the plain step (same initial state) within statistics."""
    mp0, et, sb, mo, nets = setup
    runs = []
    for learned in (False, True):
        rng = np.random.default_rng(31)
        n = 1 << 18
        p = pcl.workloads.isotropic(n, 1e6 * pcl.co.eV, rng)
        arr = pcl.ParticleArrays(np.zeros((n, 3)), p, np.ones(n), np.zeros(n))
        mp = pcl.MultiPopulation(
            ("electron", pcl.Population(n * 2, arr, air["tabs"][0], air["cuts"][0], particle=pcl.Electron)),
            ("photon", pcl.Population(n, [], air["tabs"][1], air["cuts"][1], particle=pcl.Photon)),
            ("positron", pcl.Population(1 << 14, [], air["tabs"][2], air["cuts"][2], particle=pcl.Positron)),
            seed=5)
        if learned:
            for j in sb:
                mp.set_learned(pcl.Electron, j, pcl.learned.LEARN_SB, nets[sb[0]][0])
            for j in mo:
                mp.set_learned(pcl.Electron, j, pcl.learned.LEARN_MOLLER, nets[mo[0]][0])
        pusher = pcl.workloads.pusher((0.0, 0.0, -5e5), cl=air["cl"])
        for k in range(4):
            pcl.advance(mp, pusher, (k + 1) * 25e-12)
        t = mp.tallies()
        g = mp.get(pcl.Photon).particles()
        runs.append((t, pcl.kinenergy(pcl.Photon, g.p), mp.learn_stats(), list(t.errors)))
        mp.close()
    (t0, k0, s0, e0), (t1, k1, s1, e1) = runs
    assert s0 == (0, 0) and s1[0] > 1000 and s1[1] >= 1, s1
    # 3 sigma: Poisson counts, and the two-sample KS critical value at a
    # two-sided 0.27 % (the runs share the initial state and most draws, which
    # only makes them closer than independent samples)
    for sp in (pcl.Electron, pcl.Photon):
        a, b = t0.spawned[sp], t1.spawned[sp]
        assert abs(a - b) <= 3 * np.sqrt(a + b), (sp, a, b)
    n0, n1 = len(k0), len(k1)
    c3 = np.sqrt(-0.5 * np.log(0.0027 / 2))
    assert _ks(np.log(k0), np.log(k1)) <= c3 * np.sqrt((n0 + n1) / (n0 * n1))
    assert e1[5] == 0 and e1[6] == 0, e1   # no capacity or kinematics errors


def test_learned_multistep_launches(pcl, air, setup):
    """The learned round with several steps per launch: a collision suspended
    at any step of a launch is finished after the launch by the resume pass,
    which carries the particle through the launch's remaining steps.  Eight
    25-ps steps at 8 steps per launch leave the particles of one step per
    launch (the same operations per particle; the launch shape only changes
    the rounding of a step's sub-eps remainder, kept as a double-float within
    a launch and rounded to FP32 when a particle is stored between launches,
    which every resumed collision is at one step per launch: a few particles
    in a thousand drift apart over the eight steps)."""
    mp0, et, sb, mo, nets = setup
    states, stats = [], []
    for K in (1, 8):
        rng = np.random.default_rng(43)
        n = 1 << 16
        p = pcl.workloads.isotropic(n, 1e6 * pcl.co.eV, rng)
        arr = pcl.ParticleArrays(np.zeros((n, 3)), p, np.ones(n), np.zeros(n))
        mp = pcl.MultiPopulation(
            ("electron", pcl.Population(n * 2, arr, air["tabs"][0], air["cuts"][0], particle=pcl.Electron)),
            ("photon", pcl.Population(n, [], air["tabs"][1], air["cuts"][1], particle=pcl.Photon)),
            ("positron", pcl.Population(1 << 14, [], air["tabs"][2], air["cuts"][2], particle=pcl.Positron)),
            seed=9, steps_per_launch=K)
        for j in sb:
            mp.set_learned(pcl.Electron, j, pcl.learned.LEARN_SB, nets[sb[0]][0])
        for j in mo:
            mp.set_learned(pcl.Electron, j, pcl.learned.LEARN_MOLLER, nets[mo[0]][0])
        pusher = pcl.workloads.pusher((0.0, 0.0, -5e5), cl=air["cl"])
        pcl.run(mp, pusher, 8 * 25e-12, 25e-12)
        t = mp.tallies()
        assert not any(t.errors[q] for q in (2, 3, 5, 6)), list(t.errors)
        stats.append((mp.learn_stats(), list(t.live), [t.spawned[q] for q in range(3)]))
        states.append([mp.get(q).particles() for q in (0, 1, 2)])
        mp.close()
    (s1, live1, sp1), (s8, live8, sp8) = stats
    assert s1[0] > 100 and s8[0] > 100, (s1, s8)
    assert s8[1] < s1[1]                       # one learned round per launch
    for q in range(3):
        assert abs(live1[q] - live8[q]) <= 2 + live1[q] // 1000, (live1, live8)
        a, b = states[0][q], states[1][q]
        common, ia, ib = np.intersect1d(a.sid, b.sid, return_indices=True)
        assert len(common) >= 0.999 * max(len(a.sid), len(b.sid)) - 2
        dp = np.linalg.norm(a.p[ia] - b.p[ib], axis=1) / np.maximum(np.linalg.norm(b.p[ib], axis=1), 1e-300)
        # drifted particles: a few per thousand, and at most two in a small species
        assert np.count_nonzero(dp > 1e-4) <= 2 + 5e-3 * len(dp), np.sort(dp)[-5:]
        assert len(dp) == 0 or np.median(dp) == 0.0
