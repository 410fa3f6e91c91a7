import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import __graft_entry__ as graft  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _has_gpu():
    try:
        pcl = graft.load_package()
        return pcl.lib().pcl_device_count() > 0
    except Exception:
        return False


@pytest.fixture(scope="session")
def pcl():
    graft.build()
    return graft.load_package()


@pytest.fixture(scope="session")
def oracle(pcl):
    from oracle import harness
    harness.lib()
    return harness


@pytest.fixture(scope="session")
def gpu(pcl):
    if pcl.lib().pcl_device_count() == 0:
        pytest.fail("a CUDA device is required for -m gpu tests")
    return True


@pytest.fixture(scope="session")
def air(pcl):
    """Air at 293 K / 1 atm with the beam-script tables at 0.5 MV/m, dt = 1 ps."""
    comp = pcl.workloads.air_composition()
    et, gt, pt = pcl.workloads.beam_tables(comp, 5e5, 1e-12)
    cl = pcl.workloads.air_continuum_loss(comp)
    return dict(comp=comp, tabs={pcl.Electron: et, pcl.Photon: gt, pcl.Positron: pt}, cl=cl,
                cuts={pcl.Electron: 1e4 * pcl.co.eV, pcl.Photon: 5e3 * pcl.co.eV, pcl.Positron: 1e4 * pcl.co.eV})


def random_population(pcl, sp, n, lo_ev, hi_ev, rng, spread_x=0.0):
    """n particles with log-uniform energies in [lo, hi] eV, isotropic, SI."""
    E = np.exp(rng.uniform(np.log(lo_ev), np.log(hi_ev), n)) * pcl.co.eV
    p = pcl.workloads.isotropic(n, 1.0, rng, sp)
    p *= (pcl.momentum_norm_from_kin(sp, E) / np.linalg.norm(p, axis=1))[:, None]
    x = rng.normal(scale=spread_x, size=(n, 3)) if spread_x else np.zeros((n, 3))
    return pcl.ParticleArrays(x, p, np.ones(n), np.zeros(n))
