"""Low-energy swarm (Reid's ramp model gas) on the linear-grid table:
sampler invariants in the oracle (CPU), device parity against the oracle, and
the FP32-device versus Float64-oracle comparison of swarm observables."""
import numpy as np
import pytest

EV = 1.6021766208e-19


@pytest.fixture(scope="module")
def reid(pcl):
    N = 2.504e25
    tab = pcl.workloads.reid_table(N)
    return N, tab


def _pusher(pcl, N, EN):
    return pcl.workloads.pusher((0.0, 0.0, -EN * pcl.co.Td * N))


def _maxwell(pcl, n, mean_ev, seed):
    rng = np.random.default_rng(seed)
    kT = 2.0 / 3.0 * mean_ev * EV
    p = rng.normal(scale=np.sqrt(pcl.co.electron_mass * kT), size=(n, 3))
    return p


def test_lxcat_table_layout(pcl, reid):
    N, tab = reid
    names = [type(p).__name__ for p in tab.proc]
    assert names == ["NullCollision", "Excitation", "Elastic"]
    E = tab.grid()
    tot = tab.rate.sum(axis=0)
    np.testing.assert_allclose(tot, tab.ratebound[0], rtol=1e-12)  # null fills up to the majorant
    v = np.sqrt(2 * E / pcl.co.electron_mass)
    el = tab.rate[names.index("Elastic")]
    np.testing.assert_allclose(el, N * v * 6e-20, rtol=1e-12)


def test_swarm_samplers_oracle(pcl, oracle, reid):
    N, tab = reid
    W = oracle.OracleWorld(3, {pcl.Electron: tab}, {pcl.Electron: 0.0}, _pusher(pcl, N, 12.0))
    p = _maxwell(pcl, 2000, 2.0, 1)
    sid = np.arange(2000, dtype=np.uint64)
    E = pcl.kinenergy(pcl.Electron, p)
    names = [type(q).__name__ for q in tab.proc]
    # Elastic: |p - p_cm| is kept, p_cm = m/(1+m) p
    j = names.index("Elastic")
    op, os_, ok, oc, ot = W.sample(pcl.Electron, j, p, sid)
    mr = tab.proc[j].mass_ratio
    cm = mr / (1 + mr) * p
    np.testing.assert_allclose(np.linalg.norm(op[:, 0] - cm, axis=1), np.linalg.norm(p - cm, axis=1), rtol=1e-12)
    assert np.all(oc == 3)  # randsphere (2) + s
    # Excitation: loses the threshold (or stops)
    j = names.index("Excitation")
    op, os_, ok, oc, ot = W.sample(pcl.Electron, j, p, sid)
    E1 = pcl.kinenergy(pcl.Electron, op[:, 0])
    # momentum_norm_from_kin cancels near E1 = 0 (electron.jl:51): 1e-7 relative there
    np.testing.assert_allclose(E1, np.maximum(0, E - 0.2 * EV), rtol=1e-7, atol=1e-30)


def _swarm(pcl, reid, n, EN, seed, **cfg):
    N, tab = reid
    p = _maxwell(pcl, n, 1.0, seed)
    arr = pcl.ParticleArrays(np.zeros((n, 3)), p, np.ones(n), np.zeros(n))
    mp = pcl.MultiPopulation(("electron", pcl.Population(n + 64, arr, tab, 0.0, particle=pcl.Electron)),
                             seed=seed, **cfg)
    return mp


@pytest.mark.gpu
def test_swarm_parity(pcl, oracle, gpu, reid):
    """A few steps of 1 ps (~35 sub-steps each, mostly null collisions): draws
    bit-exact and momenta within 1e-5 against the oracle."""
    N, tab = reid
    pusher = _pusher(pcl, N, 24.0)
    mp = _swarm(pcl, reid, 4096, 24.0, 7)
    W = oracle.OracleWorld(7, {pcl.Electron: tab}, {pcl.Electron: 0.0}, pusher)
    W.upload(pcl.Electron, mp.get(pcl.Electron).particles())
    for k in range(3):
        pcl.advance(mp, pusher, (k + 1) * 1e-12)
        W.advance((k + 1) * 1e-12, 4)
    rep = oracle.compare_populations(mp.get(pcl.Electron).particles(), W.download(pcl.Electron), pcl.Electron,
                                     rtol=1e-5, stol=2e-4)
    assert rep["ok"], str(rep)
    t = mp.tallies()
    c = W.counters()
    assert abs(int(np.sum(t.collisions[0])) - int(c["coll"][0].sum())) <= 4 * (c["ties"] + 1)
    mp.close()


@pytest.mark.gpu
def test_swarm_observables_fp32_vs_fp64(pcl, oracle, gpu, reid):
    """Drift velocity, mean energy and longitudinal diffusion of the FP32 device
    against the Float64 oracle from the same initial swarm and streams, after
    the swarm relaxes: within 3 sigma of the combined statistical error of
    two independent swarms of this size (the shared streams only make the two
    closer)."""
    N, tab = reid
    EN = 12.0
    pusher = _pusher(pcl, N, EN)
    n, steps, dt = 8192, 120, 2e-12
    mp = _swarm(pcl, reid, n, EN, 11)
    W = oracle.OracleWorld(11, {pcl.Electron: tab}, {pcl.Electron: 0.0}, pusher)
    W.upload(pcl.Electron, mp.get(pcl.Electron).particles())
    zg, zo, tt = [], [], []
    for k in range(steps):
        t = (k + 1) * dt
        pcl.advance(mp, pusher, t)
        W.advance(t, 8)
        if k >= steps // 2:
            m = mp.get(pcl.Electron).moments()
            zg.append(m[4] / m[0])
            zo.append(np.mean(W.download(pcl.Electron).x[:, 2]))
            tt.append(t)
    g = mp.get(pcl.Electron).particles()
    o = W.download(pcl.Electron)
    Eg, Eo = pcl.kinenergy(0, g.p), pcl.kinenergy(0, o.p)
    se = np.hypot(Eg.std() / np.sqrt(len(Eg)), Eo.std() / np.sqrt(len(Eo)))
    assert abs(Eg.mean() - Eo.mean()) <= 3 * se, (Eg.mean() / EV, Eo.mean() / EV, se / EV)
    Wg = np.polyfit(tt, zg, 1)[0]
    Wo = np.polyfit(tt, zo, 1)[0]
    assert Wg > 0 and Wo > 0
    # drift: the mean velocity's standard error
    vz_sd = np.hypot(np.std(g.p[:, 2]), np.std(o.p[:, 2])) / pcl.co.electron_mass / np.sqrt(n)
    assert abs(Wg - Wo) <= 3 * vz_sd, (Wg, Wo, vz_sd)

    # spread along z: the sample variance's standard error, sqrt((m4 - var^2) / n)
    def var_se(z):
        d = z - z.mean()
        return np.var(z), np.sqrt(max(np.mean(d ** 4) - np.var(z) ** 2, 0.0) / len(z))
    (Dg, sg), (Do, so) = var_se(g.x[:, 2]), var_se(o.x[:, 2])
    assert abs(Dg - Do) <= 3 * np.hypot(sg, so), (Dg, Do, sg, so)
    mp.close()


# ------------------------------------------------- batched swarms (swarm mode) --
def test_ratebound_split_is_linear_in_fdt(pcl, air):
    """A + Fdt B reproduces compratebound (collision_table.jl:152-167) for any Fdt."""
    comp = pcl.workloads.air_composition()
    for particle, procs in ((pcl.Electron, pcl.workloads.electron_processes(comp)),
                            (pcl.Positron, pcl.workloads.positron_processes(comp))):
        base = pcl.collision_table_from_processes(procs, particle, 0.0, safety=1.15)
        A, B = pcl.ratebound_split(base, 1.15)
        for Fdt in (0.0, 1e-25, 3e-24):
            tab = pcl.collision_table_from_processes(procs, particle, Fdt, safety=1.15)
            np.testing.assert_allclose(A + Fdt * B, tab.ratebound, rtol=1e-9,
                                       atol=1e-12 * np.abs(tab.ratebound).max())


def _batch(pcl, swarms=None, **cfg):
    return pcl.workloads.swarm_batch(8, e_range=(4e5, 3e6), n_range=(40, 400), seed=5, swarms=swarms, **cfg)


def _by_sid(a):
    o = np.argsort(a.sid)
    return a.sid[o], a.p[o], a.x[o], a.s[o], a.ctr[o]


@pytest.mark.gpu
def test_batched_equals_alone(pcl, gpu):
    """Swarm mode processes each swarm independently: a swarm run inside the
    batch and run alone give bit-identical particles (matched by stream id)."""
    b = _batch(pcl)
    for k in range(6):
        pcl.advance(b.mpopl, b.pusher, (k + 1) * b.dt)
    for s in (1, 6):
        a = _batch(pcl, swarms=[s])
        for k in range(6):
            pcl.advance(a.mpopl, a.pusher, (k + 1) * a.dt)
        for sp in (pcl.Electron, pcl.Photon, pcl.Positron):
            g = b.mpopl.get(sp).particles()
            m = (g.sid >> np.uint64(56)) == s
            ga = a.mpopl.get(sp).particles()
            assert np.all((ga.sid >> np.uint64(56)) == s)
            x, y = _by_sid(type(g)(**{f: getattr(g, f)[m] for f in ("x", "p", "w", "t", "s", "sid", "ctr")})), \
                _by_sid(ga)
            for u, v in zip(x, y):
                np.testing.assert_array_equal(u, v)
        a.mpopl.close()
    b.mpopl.close()


@pytest.mark.gpu
def test_batched_oracle_parity(pcl, oracle, gpu):
    """The batch against the oracle in swarm mode: per-swarm field and rate
    bound, children inheriting the swarm bits."""
    b = _batch(pcl)
    et, gt, pt = b.tables
    tabs = {pcl.Electron: et, pcl.Photon: gt, pcl.Positron: pt}
    W = oracle.OracleWorld(5, tabs, {pcl.Electron: 10e3 * EV, pcl.Photon: 5e3 * EV, pcl.Positron: 10e3 * EV},
                           b.pusher)
    Evec = np.zeros((len(b.E), 3))
    Evec[:, 2] = -b.E
    W.set_swarms(tabs, Evec, pcl.co.elementary_charge * b.E * b.dt, safety=1.15)
    W.upload(pcl.Electron, b.mpopl.get(pcl.Electron).particles())
    for k in range(4):
        pcl.advance(b.mpopl, b.pusher, (k + 1) * b.dt)
        W.advance((k + 1) * b.dt, 4)
    for sp in (pcl.Electron, pcl.Photon, pcl.Positron):
        rep = oracle.compare_populations(b.mpopl.get(sp).particles(), W.download(sp), sp, rtol=3e-5, stol=1e-4)
        assert rep["ok"], (sp, str(rep))
    b.mpopl.close()


@pytest.mark.gpu
def test_batched_multistep_launches(pcl, oracle, gpu):
    """The batch at eight steps per launch (the multi-step kernel in swarm
    mode: per-swarm field and rate bound, full-warp collide batches, photon
    flights) equals eight one-step launches bit for bit and matches the
    oracle."""
    runs = []
    for K in (1, 8):
        b = _batch(pcl, steps_per_launch=K)
        pcl.run(b.mpopl, b.pusher, 8 * b.dt, b.dt)
        runs.append(b)
    a, b = runs
    assert a.mpopl.tallies().steps == b.mpopl.tallies().steps == 8
    for sp in (pcl.Electron, pcl.Photon, pcl.Positron):
        for u, v in zip(_by_sid(a.mpopl.get(sp).particles()), _by_sid(b.mpopl.get(sp).particles())):
            np.testing.assert_array_equal(u, v)
    a.mpopl.close()
    c = _batch(pcl, steps_per_launch=8)
    et, gt, pt = c.tables
    tabs = {pcl.Electron: et, pcl.Photon: gt, pcl.Positron: pt}
    W = oracle.OracleWorld(5, tabs, {pcl.Electron: 10e3 * EV, pcl.Photon: 5e3 * EV, pcl.Positron: 10e3 * EV},
                           c.pusher)
    Evec = np.zeros((len(c.E), 3))
    Evec[:, 2] = -c.E
    W.set_swarms(tabs, Evec, pcl.co.elementary_charge * c.E * c.dt, safety=1.15)
    W.upload(pcl.Electron, c.mpopl.get(pcl.Electron).particles())
    pcl.run(c.mpopl, c.pusher, 4 * c.dt, c.dt)
    for k in range(4):
        W.advance((k + 1) * c.dt, 4)
    for sp in (pcl.Electron, pcl.Photon, pcl.Positron):
        rep = oracle.compare_populations(c.mpopl.get(sp).particles(), W.download(sp), sp, rtol=3e-5, stol=1e-4)
        assert rep["ok"], (sp, str(rep))
    b.mpopl.close(); c.mpopl.close()


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["constant", "table"])
def test_split_keeps_swarm(pcl, oracle, gpu, form):
    """split! in swarm mode, with a constant mean or a table of f(E)
    (pcl_split_fn): every copy stays in its parent's swarm (top 8 bits of the
    stream id), so each swarm's count grows by its own copies; the copies and
    weights equal the oracle's, and the next steps still match."""
    b = _batch(pcl)
    et, gt, pt = b.tables
    tabs = {pcl.Electron: et, pcl.Photon: gt, pcl.Positron: pt}
    W = oracle.OracleWorld(5, tabs, {pcl.Electron: 10e3 * EV, pcl.Photon: 5e3 * EV, pcl.Positron: 10e3 * EV},
                           b.pusher)
    Evec = np.zeros((len(b.E), 3))
    Evec[:, 2] = -b.E
    W.set_swarms(tabs, Evec, pcl.co.elementary_charge * b.E * b.dt, safety=1.15)
    W.upload(pcl.Electron, b.mpopl.get(pcl.Electron).particles())
    for k in range(2):
        pcl.advance(b.mpopl, b.pusher, (k + 1) * b.dt)
        W.advance((k + 1) * b.dt, 4)
    nsw = len(b.E)
    n0 = b.mpopl.swarm_counts(pcl.Electron)
    mu = 0.6
    f = mu if form == "constant" else (np.array([1.0, 1e9]) * EV, np.array([mu, mu]))
    b.mpopl.split(pcl.Electron, f)
    W.split(pcl.Electron, f)
    n1 = b.mpopl.swarm_counts(pcl.Electron)
    g = b.mpopl.get(pcl.Electron).particles()
    assert np.all((g.sid >> np.uint64(56)) < nsw)
    for s in range(nsw):
        assert abs((n1[s] - n0[s]) - mu * n0[s]) < 5 * np.sqrt(mu * n0[s]) + 2, (s, n0[s], n1[s])
    rep = oracle.compare_populations(g, W.download(pcl.Electron), pcl.Electron, rtol=3e-5, stol=1e-4)
    assert rep["ok"], str(rep)
    for k in range(2, 4):
        pcl.advance(b.mpopl, b.pusher, (k + 1) * b.dt)
        W.advance((k + 1) * b.dt, 4)
    for sp in (pcl.Electron, pcl.Photon, pcl.Positron):
        rep = oracle.compare_populations(b.mpopl.get(sp).particles(), W.download(sp), sp, rtol=3e-5, stol=1e-4)
        assert rep["ok"], (sp, str(rep))
    b.mpopl.close()


@pytest.mark.gpu
def test_swarm_moments(pcl, gpu):
    """Per-swarm moments on the device against the downloaded particles."""
    b = _batch(pcl)
    for k in range(3):
        pcl.advance(b.mpopl, b.pusher, (k + 1) * b.dt)
    m = b.mpopl.swarm_moments(pcl.Electron, len(b.E))
    g = b.mpopl.get(pcl.Electron).particles()
    sw = (g.sid >> np.uint64(56)).astype(int)
    E = pcl.kinenergy(pcl.Electron, g.p)
    for s in range(len(b.E)):
        q = sw == s
        ref = [q.sum(), g.w[q].sum(), (g.w * E)[q].sum(), (g.w * g.x[:, 2])[q].sum(),
               (g.w * g.x[:, 2] ** 2)[q].sum(), (g.w * (g.x[:, 0] ** 2 + g.x[:, 1] ** 2))[q].sum()]
        np.testing.assert_allclose(m[s], ref, rtol=1e-5, atol=1e-30)
    b.mpopl.close()


# ------------------------------------------------------------ LXCat loader --
_LXCAT = [
    {"target": "X", "kind": "EFFECTIVE", "mass_ratio": 2e-5, "comment": "made-up test set",
     "data": [[0.0, 5e-20], [10.0, 8e-20], [100.0, 4e-20]]},
    {"target": "X", "kind": "EXCITATION", "threshold": 5.0, "comment": "",
     "data": [[5.0, 0.0], [20.0, 2e-20], [100.0, 1e-20]]},
    {"target": "X", "kind": "IONIZATION", "threshold": 12.0, "comment": "",
     "data": [[12.0, 0.0], [50.0, 3e-20], [100.0, 2e-20]]},
    {"target": "X", "kind": "ATTACHMENT", "threshold": 0.0, "comment": "",
     "data": [[0.0, 1e-22], [2.0, 5e-22], [100.0, 0.0]]},
    {"target": "Y", "kind": "ELASTIC", "mass_ratio": 1e-5, "comment": "no density given: skipped",
     "data": [[0.0, 1e-20], [100.0, 1e-20]]},
]


@pytest.fixture
def lxcat_file(tmp_path):
    import json
    f = tmp_path / "set.json"
    f.write_text(json.dumps(_LXCAT))
    return str(f)


def test_load_lxcat(pcl, lxcat_file):
    """load_lxcat (lxcat.jl:17-156): densities, linear interpolation, the
    EFFECTIVE -> ELASTIC correction, the null process and the ordering."""
    N = 2e25
    E = np.linspace(0.0, 100.0 * EV, 2001)
    r = pcl.load_lxcat([lxcat_file], {"X": N}, E)
    names = [type(p).__name__ for p in r.proc]
    assert sorted(names) == ["Attachment", "Elastic", "Excitation", "Ionization", "NullCollision"]
    inteng = r.rate.sum(axis=1)
    assert np.all(np.diff(inteng) <= 0)
    v = np.sqrt(2 * E / pcl.co.electron_mass)
    sig = {k: np.interp(E / EV, [q[0] for q in it["data"]], [q[1] for q in it["data"]])
           for k, it in zip(("eff", "exc", "ion", "att"), _LXCAT[:4])}
    el = r.rate[names.index("Elastic")]
    np.testing.assert_allclose(el, N * v * (sig["eff"] - sig["exc"] - sig["ion"]), rtol=1e-12, atol=1e-3)
    np.testing.assert_allclose(r.rate[names.index("Ionization")], N * v * sig["ion"], rtol=1e-12)
    tot = r.rate.sum(axis=0)
    np.testing.assert_allclose(tot, r.maxrate, rtol=1e-12)
    assert r.proc[names.index("Ionization")].threshold == pytest.approx(12 * EV)
    # origperm maps the sorted order back to the reading order (EFFECTIVE first)
    assert type(r.proc[r.origperm[0]]).__name__ == "Elastic"
    tab = pcl.lxcat_collision_table([lxcat_file], {"X": N}, E)
    assert tab.nproc == 5 and tab.energy[2] == 2001


@pytest.mark.gpu
def test_lxcat_swarm_parity(pcl, oracle, gpu, lxcat_file):
    """A swarm on the loaded set at 300 Td (ionization and attachment both
    active) against the oracle: secondaries from ionization, removals from
    attachment, momenta within 1e-5."""
    N = 2e25
    E = np.linspace(0.0, 100.0 * EV, 2001)
    tab = pcl.lxcat_collision_table([lxcat_file], {"X": N}, E)
    pusher = pcl.workloads.pusher((0.0, 0.0, -300.0 * pcl.co.Td * N))
    n = 4096
    rng = np.random.default_rng(9)
    p = _maxwell(pcl, n, 8.0, 9)
    arr = pcl.ParticleArrays(np.zeros((n, 3)), p, np.ones(n), np.zeros(n))
    mp = pcl.MultiPopulation(("electron", pcl.Population(8 * n, arr, tab, 0.0, particle=pcl.Electron)), seed=9)
    W = oracle.OracleWorld(9, {pcl.Electron: tab}, {pcl.Electron: 0.0}, pusher)
    W.upload(pcl.Electron, mp.get(pcl.Electron).particles())
    for k in range(4):
        pcl.advance(mp, pusher, (k + 1) * 1e-12)
        W.advance((k + 1) * 1e-12, 4)
    t = mp.tallies()
    names = [type(q).__name__ for q in tab.proc]
    assert t.collisions[0][names.index("Ionization")] > 100 and t.collisions[0][names.index("Attachment")] > 0
    assert t.spawned[0] > 100
    rep = oracle.compare_populations(mp.get(pcl.Electron).particles(), W.download(pcl.Electron), pcl.Electron,
                                     rtol=1e-5, stol=2e-4)
    assert rep["ok"], str(rep)
    mp.close()


@pytest.mark.gpu
def test_swarm_cap(pcl, gpu):
    """cap_swarms: swarms above the cap are rouletted to it (weights scaled by
    1 / pkeep), swarms below are untouched."""
    b = _batch(pcl)
    for k in range(2):
        pcl.advance(b.mpopl, b.pusher, (k + 1) * b.dt)
    m0 = b.mpopl.swarm_moments(pcl.Electron, len(b.E))
    cap = int(np.median(m0[:, 0]))
    before = b.mpopl.cap_swarms(cap, particles=(pcl.Electron,))
    m1 = b.mpopl.swarm_moments(pcl.Electron, len(b.E))
    for s in range(len(b.E)):
        n0, w0 = m0[s, 0], m0[s, 1]
        if n0 <= cap:
            assert m1[s, 0] == n0 and m1[s, 1] == pytest.approx(w0, rel=1e-6)
        else:
            q = cap / n0
            assert abs(m1[s, 0] - cap) < 5 * np.sqrt(n0 * q * (1 - q)) + 1
            assert abs(m1[s, 1] - w0) < 6 * np.sqrt(n0 * (1 - q) / q) + 1
    b.mpopl.close()


@pytest.mark.gpu
def test_device_swarm_cap(pcl, gpu):
    """set_swarm_cap (per-swarm counts and roulette on the device after each
    launch group of run!) removes and reweights exactly the particles that
    the host-driven cap_swarms does after the same steps."""
    a, b = _batch(pcl), _batch(pcl)
    for q in (a, b):
        for k in range(2):
            pcl.advance(q.mpopl, q.pusher, (k + 1) * q.dt)
    n0 = a.mpopl.swarm_counts(pcl.Electron)
    np.testing.assert_array_equal(n0, b.mpopl.swarm_moments(pcl.Electron, len(b.E))[:, 0].astype(np.int64))
    cap = int(np.median(n0))
    pcl.run(a.mpopl, a.pusher, 3 * a.dt, a.dt)
    before = a.mpopl.cap_swarms(cap, particles=(pcl.Electron,))
    b.mpopl.set_swarm_cap(cap)
    pcl.run(b.mpopl, b.pusher, 3 * b.dt, b.dt)
    pcl.lib().pcl_compact(b.mpopl.ctx)
    assert np.any(before[pcl.Electron] > cap)
    na, nb = a.mpopl.swarm_counts(pcl.Electron), b.mpopl.swarm_counts(pcl.Electron)
    np.testing.assert_array_equal(na, nb)
    for sp in (pcl.Electron, pcl.Photon, pcl.Positron):
        ga, gb = a.mpopl.get(sp).particles(), b.mpopl.get(sp).particles()
        for u, v in zip(_by_sid(ga), _by_sid(gb)):
            np.testing.assert_array_equal(u, v)
        np.testing.assert_array_equal(ga.w[np.argsort(ga.sid)], gb.w[np.argsort(gb.sid)])
    a.mpopl.close()
    b.mpopl.close()


@pytest.mark.gpu
def test_swarm_energy_histogram(pcl, gpu):
    """Per-swarm spectra (pcl_energy_histogram with a swarm): each swarm's
    counts and weights are those of its particles, and they sum to the whole."""
    b = _batch(pcl)
    for k in range(3):
        pcl.advance(b.mpopl, b.pusher, (k + 1) * b.dt)
    pop = b.mpopl.get(pcl.Electron)
    g = pop.particles()
    E = pcl.kinenergy(pcl.Electron, g.p)
    sw = (g.sid >> np.uint64(56)).astype(int)
    edges = 10 ** np.linspace(3.5, 7.5, 65) * pcl.co.eV
    call, wall = pop.energy_histogram(edges)
    tot_c, tot_w = np.zeros_like(call), np.zeros_like(wall)
    for s in range(len(b.E)):
        c, w = pop.energy_histogram(edges, swarm=s)
        m = sw == s
        ref = np.histogram(E[m], bins=edges)[0]
        assert np.abs(c - ref).sum() <= 2, (s, c, ref)
        tot_c += c
        tot_w += w
    np.testing.assert_array_equal(tot_c, call)
    np.testing.assert_allclose(tot_w, wall, rtol=1e-12)
    b.mpopl.close()
