"""The C-ABI library: it loads, exports every entry point the header declares,
its host-only builders work without a GPU, and device entry points fail
with a status (never a crash) when no device is usable."""
import ctypes as C
import os
import re

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    with open(os.path.join(ROOT, "include", "particulator_gb300.h")) as f:
        src = f.read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(pcl_[a-z_0-9]+)\s*\(", src)))


def test_every_declared_symbol_is_exported(pcl):
    L = pcl.lib()
    names = _declared()
    assert len(names) >= 29
    for n in names:
        assert hasattr(L, n), n
    # and the ctypes binding covers them all
    assert sorted(pcl._lib.exported_symbols()) == names


def test_no_device_means_status_not_crash(pcl):
    L = pcl.lib()
    if L.pcl_device_count() > 0:
        return
    h = C.c_void_p()
    cfg = pcl._lib.Config()
    assert L.pcl_create(C.byref(cfg), C.byref(h)) == pcl._lib.PCL_ERR_CUDA
    assert L.pcl_advance(None, 1.0) == pcl._lib.PCL_ERR_INVALID
    # page-locked host memory needs the runtime too: a status, never a crash
    p = C.c_void_p()
    assert L.pcl_host_alloc(C.byref(p), 4096) == pcl._lib.PCL_ERR_CUDA and not p.value
    assert L.pcl_host_alloc(None, 4096) == pcl._lib.PCL_ERR_INVALID
    buf = (C.c_uint8 * 4096)()
    assert L.pcl_host_register(buf, 4096) == pcl._lib.PCL_ERR_CUDA
    assert L.pcl_host_register(None, 4096) == pcl._lib.PCL_ERR_INVALID


def test_builder_argument_checks(pcl):
    L = pcl.lib()
    rate = np.zeros(3 * 33)
    rb = np.zeros(3 * 33)
    perm = np.zeros(1, np.int32)
    # bad species / order / interval counts
    assert L.pcl_build_collision_table(7, 0, None, 0.0, 1.1, 32, 3, 1.0, None, pcl._lib.dptr(rb), None) == -1
    assert L.pcl_build_collision_table(0, 0, None, 0.0, 1.1, 32, 9, 1.0, None, pcl._lib.dptr(rb), None) == -1
    assert L.pcl_build_collision_table(0, 0, None, 0.0, 1.1, 0, 3, 1.0, None, pcl._lib.dptr(rb), None) == -1
    # an empty table is valid (photons tracked with no processes: rate bound 0)
    assert L.pcl_build_collision_table(1, 0, None, 0.0, 1.1, 32, 3, 1.0, pcl._lib.dptr(rate), pcl._lib.dptr(rb),
                                       pcl._lib.i32ptr(perm)) == 0
    assert np.all(rb == 0)
    # a process on the wrong species is rejected (no device sampler for it)
    comp = pcl.workloads.air_composition()
    procs = (pcl._lib.Process * 1)()
    procs[0] = pcl.Compton(7).to_c(1.0)
    assert L.pcl_build_collision_table(0, 1, procs, 0.0, 1.1, 32, 3, 1.0, pcl._lib.dptr(rate), pcl._lib.dptr(rb),
                                       pcl._lib.i32ptr(perm)) == pcl._lib.PCL_ERR_UNSUPPORTED


def test_version_string(pcl):
    assert b"sm_103a" in pcl.lib().pcl_version()
