"""Golden fixtures (tests/golden/, made by make_golden.py from the oracle and
the host builders): regression pins on CPU, and the device against them."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, HERE)
import make_golden  # noqa: E402


@pytest.fixture(scope="module")
def setup(pcl):
    return make_golden.setup()


def test_tables_golden(setup):
    pcl, tabs, cuts, pusher = setup
    g = np.load(os.path.join(HERE, "tables_air.npz"))
    for k, t in tabs.items():
        np.testing.assert_allclose(t.rate, g[f"rate{k}"], rtol=1e-12, atol=0)
        np.testing.assert_allclose(t.ratebound, g[f"rb{k}"], rtol=1e-12, atol=0)
        assert np.array_equal(t.perm, g[f"perm{k}"])


def test_samplers_golden_oracle(setup, oracle):
    pcl, tabs, cuts, pusher = setup
    g = np.load(os.path.join(HERE, "samplers.npz"))
    W = oracle.OracleWorld(4242, tabs, cuts, pusher)
    for q in range(int(g["n"])):
        op, os_, ok, oc, ot = W.sample(int(g[f"sp{q}"]), int(g[f"j{q}"]), g[f"p{q}"], g[f"sid{q}"])
        assert np.array_equal(oc, g[f"oc{q}"]) and np.array_equal(ok, g[f"ok{q}"])
        np.testing.assert_allclose(op, g[f"op{q}"], rtol=1e-13, atol=1e-40)
        np.testing.assert_allclose(os_, g[f"os{q}"], rtol=1e-13)


def test_step_golden_oracle(setup, oracle):
    pcl, tabs, cuts, pusher = setup
    g = np.load(os.path.join(HERE, "step.npz"))
    W = oracle.OracleWorld(4242, tabs, cuts, pusher)
    for sp in (0, 1, 2):
        W.upload(sp, oracle.Arrays(*(g[f"in_{f}{sp}"] for f in ("x", "p", "w", "t", "s", "sid", "ctr"))))
    for k in range(3):
        W.advance((k + 1) * 5e-12, 2)
    for sp in (0, 1, 2):
        o = W.download(sp)
        assert np.array_equal(o.sid, g[f"out_sid{sp}"]) and np.array_equal(o.ctr, g[f"out_ctr{sp}"])
        np.testing.assert_allclose(o.p, g[f"out_p{sp}"], rtol=1e-13, atol=1e-40)


@pytest.mark.gpu
def test_samplers_golden_device(setup, gpu):
    """The device samplers reproduce the committed outcomes: identical draw
    counts and outcome kinds, momenta within 1e-5 of the incoming momentum."""
    pcl, tabs, cuts, pusher = setup
    g = np.load(os.path.join(HERE, "samplers.npz"))
    mp = pcl.MultiPopulation(*[(k, pcl.Population(64, [], tabs[k], cuts[k], particle=k)) for k in tabs], seed=4242)
    L = pcl.lib()
    for q in range(int(g["n"])):
        sp, j, p, sid = int(g[f"sp{q}"]), int(g[f"j{q}"]), np.ascontiguousarray(g[f"p{q}"]), g[f"sid{q}"]
        n = len(sid)
        gp = np.zeros(9 * n); gs = np.zeros(3 * n); gk = np.zeros(3 * n, np.int32); gc = np.zeros(n, np.uint32)
        assert L.pcl_test_sampler(mp.ctx, sp, j, n, pcl._lib.dptr(p.reshape(-1)), pcl._lib.u64ptr(sid),
                                  pcl._lib.dptr(gp), pcl._lib.dptr(gs), pcl._lib.i32ptr(gk), pcl._lib.u32ptr(gc)) == 0
        clean = g[f"ot{q}"] == 0
        assert np.array_equal(gc[clean], g[f"oc{q}"][clean]), q
        assert np.array_equal(gk.reshape(n, 3)[clean], g[f"ok{q}"][clean]), q
        pn = np.linalg.norm(p, axis=1)[clean][:, None]
        dp = np.abs(gp.reshape(n, 3, 3)[clean] - g[f"op{q}"][clean]).max(axis=2) / pn
        assert dp.max() <= 1e-5, (q, dp.max())
    mp.close()
