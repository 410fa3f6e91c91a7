"""The oracle-only set-up used by the CPU reference arm of the benchmark:
its tables (numpy restatement of the reference's init path) agree with the
library's C++ builders, laid out as the oracle reads them, and a process that
builds and steps it never loads the GPU library."""
import os
import subprocess
import sys

import numpy as np

from oracle import reference_world as rw

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_tables_match_library(pcl, air):
    comp = air["comp"]
    Fdt = pcl.co.elementary_charge * 5e5 * 1e-12
    got = {pcl.Electron: rw.collision_table(rw.electron_processes(comp), pcl.Electron, Fdt),
           pcl.Photon: rw.collision_table(rw.photon_processes(comp), pcl.Photon, 0.0),
           pcl.Positron: rw.collision_table(rw.positron_processes(comp), pcl.Positron, Fdt)}
    for sp, want in air["tabs"].items():
        g = got[sp]
        assert [type(p).__name__ for p in g.proc] == [type(p).__name__ for p in want.proc]
        assert [p.Z for p in g.proc] == [p.Z for p in want.proc]
        np.testing.assert_allclose(g.coef, want.coef, rtol=1e-15)
        np.testing.assert_allclose(g.rate, want.rate, rtol=1e-9, atol=1e-6 * np.abs(want.rate).max())
        np.testing.assert_allclose(g.ratebound, want.ratebound, rtol=1e-9, atol=1e-6 * np.abs(want.ratebound).max())
    for Z in (7, 8):
        a, b = rw.seltzer_berger(Z), pcl.workloads.seltzer_berger(Z)
        np.testing.assert_allclose(a.log_energy, b.log_energy, rtol=1e-15)
        np.testing.assert_allclose(a.totalcs, b.totalcs, rtol=1e-12)
        np.testing.assert_allclose(a.data, b.data, rtol=1e-9, atol=1e-9)
    cl = rw.continuum_loss(comp)
    assert cl.bints.k == air["cl"].bints.k and cl.bints.xmax == air["cl"].bints.xmax
    np.testing.assert_allclose(cl.ec, air["cl"].ec, rtol=1e-10)
    np.testing.assert_allclose(cl.pc, air["cl"].pc, rtol=1e-10)


def test_reference_world_never_loads_the_library(pcl, oracle):
    """Build the oracle avalanche from the independent tables, step a few
    hundred electrons, and check the process maps: no libparticulator_gb300."""
    code = (
        "import sys; sys.path.insert(0, %r)\n"
        "import numpy as np\n"
        "import __graft_entry__ as g\n"
        "pcl = g.load_package()\n"
        "from oracle import reference_world as rw\n"
        "from oracle.harness import Arrays\n"
        "W, tabs, cuts, pusher = rw.avalanche_world(0)\n"
        "rng = np.random.default_rng(0)\n"
        "n = 256\n"
        "p = pcl.workloads.isotropic(n, 1e6 * pcl.co.eV, rng)\n"
        "W.upload(0, Arrays(np.zeros((n, 3)), p, np.ones(n), np.zeros(n), -np.log(rng.random(n)),\n"
        "                   np.arange(n, dtype=np.uint64), np.zeros(n, np.uint32)))\n"
        "W.advance(1e-12, 2); W.advance(2e-12, 2)\n"
        "assert len(W.download(0).w) > 200\n"
        "print('LOADED' if rw.library_loaded() else 'CLEAN')\n" % ROOT)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip().endswith("CLEAN"), r.stdout
