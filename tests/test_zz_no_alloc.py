"""pcl_compact_noalloc: compaction of caller-owned device buffers with no
device allocation, for callers that cannot call cudaMalloc (a host memory
pool that owns the device, a stream under capture, a loop that must not
allocate).  Its output must equal pcl_compact's, bit for bit, on two calls in
a row; sizes above the static scratch limit are refused before any launch.
This file sorts last so that a run stopping at the first failure has run
every other test first."""
import ctypes as C

import numpy as np
import pytest

from conftest import random_population

pytestmark = pytest.mark.gpu


def _packed_host(pcl, mp, sp):
    L = pcl.lib()
    cap = mp.get(sp).max_particles
    xw = np.zeros((cap, 4), np.float32)
    ps = np.zeros((cap, 4), np.float32)
    meta = np.zeros((cap, 4), np.uint32)
    pk = pcl._lib.Packed(xw.ctypes.data_as(C.POINTER(C.c_float)), ps.ctypes.data_as(C.POINTER(C.c_float)),
                         meta.ctypes.data_as(C.POINTER(C.c_uint32)))
    n = C.c_int64(cap)
    assert L.pcl_download_packed(mp.ctx, sp, C.byref(n), C.byref(pk)) == 0
    return xw[:n.value].copy(), ps[:n.value].copy(), meta[:n.value].copy()


def test_compact_noalloc_matches_compact(pcl, gpu, air):
    import torch
    L = pcl.lib()
    rng = np.random.default_rng(21)
    pops = {pcl.Electron: random_population(pcl, pcl.Electron, 3000, 1e4, 3e6, rng),
            pcl.Photon: random_population(pcl, pcl.Photon, 3000, 5e3, 2e5, rng)}
    mp = pcl.MultiPopulation(*[(k, pcl.Population(1 << 14, pops[k], air["tabs"][k], air["cuts"][k], particle=k))
                               for k in pops], seed=21, compaction_period=1000)
    pusher = pcl.workloads.pusher((0.0, 0.0, -5e5), cl=air["cl"])
    for k in range(4):
        pcl.advance(mp, pusher, (k + 1) * 25e-12)
    dev = torch.device("cuda", 0)
    results = {}
    for sp in (pcl.Electron, pcl.Photon):        # two calls in a row
        xw, ps, meta = _packed_host(pcl, mp, sp)
        n = len(xw)
        assert (meta[:, 2] == 0xFFFFFFFF).sum() > 0, "want dead slots to squeeze out"
        t_in = [torch.from_numpy(a.view(np.int32)).to(dev) for a in (xw, ps, meta)]
        t_out = [torch.zeros((n, 4), dtype=torch.int32, device=dev) for _ in range(3)]
        n_out = torch.zeros(1, dtype=torch.int64, device=dev)
        rc = L.pcl_compact_noalloc(n, *[t.data_ptr() for t in t_in], *[t.data_ptr() for t in t_out],
                                   n_out.data_ptr(), None)
        assert rc == 0, L.pcl_last_error(None)
        torch.cuda.synchronize()
        m = int(n_out.item())
        results[sp] = (m, [t[:m].cpu().numpy() for t in t_out])
        assert m == int((meta[:, 2] != 0xFFFFFFFF).sum())
    # the entry point that allocates: compact in place through the context
    pcl.repack(mp.get(pcl.Electron))
    for sp in (pcl.Electron, pcl.Photon):
        xw, ps, meta = _packed_host(pcl, mp, sp)
        m, (oxw, ops, ometa) = results[sp]
        assert len(xw) == m
        assert np.array_equal(oxw.view(np.float32), xw)
        assert np.array_equal(ops.view(np.float32), ps)
        assert np.array_equal(ometa.view(np.uint32), meta)
    # beyond the static scratch: refused with a clear error, nothing launched
    dummy = torch.zeros(4, dtype=torch.int32, device=dev).data_ptr()
    rc = L.pcl_compact_noalloc(pcl._lib.NOALLOC_MAX_SLOTS + 1, dummy, dummy, dummy, dummy, dummy, dummy, dummy, None)
    assert rc == pcl._lib.PCL_ERR_CAPACITY
    assert b"PCL_NOALLOC_MAX_SLOTS" in L.pcl_last_error(None)
    mp.close()


def test_compact_noalloc_many_scan_chunks(pcl, gpu, air):
    """More than 1024 tiles of 2048 slots, so the tile-offset scan runs over
    several chunks of its block: 3,000,000 slots of synthetic records, about a
    third of them dead, compacted by the allocation-free entry point (twice in
    a row) and by pcl_compact through a context; the two must agree bit for
    bit.  Overlapping input and output buffers are refused."""
    import torch
    L = pcl.lib()
    n = 3_000_000
    assert (n + 2047) // 2048 > 1024
    rng = np.random.default_rng(5)
    xw = rng.standard_normal((n, 4)).astype(np.float32)
    ps = rng.standard_normal((n, 4)).astype(np.float32)
    meta = rng.integers(0, 1 << 32, size=(n, 4), dtype=np.uint64).astype(np.uint32)
    meta[:, 2] = rng.integers(0, 1000, size=n, dtype=np.uint32)
    dead = rng.random(n) < 0.35
    meta[dead, 2] = 0xFFFFFFFF
    live = int((~dead).sum())
    dev = torch.device("cuda", 0)
    t_in = [torch.from_numpy(a.view(np.int32)).to(dev) for a in (xw, ps, meta)]
    outs = []
    for _ in range(2):                           # two calls in a row
        t_out = [torch.full((n, 4), -7, dtype=torch.int32, device=dev) for _ in range(3)]
        n_out = torch.zeros(1, dtype=torch.int64, device=dev)
        rc = L.pcl_compact_noalloc(n, *[t.data_ptr() for t in t_in], *[t.data_ptr() for t in t_out],
                                   n_out.data_ptr(), None)
        assert rc == 0, L.pcl_last_error(None)
        torch.cuda.synchronize()
        assert int(n_out.item()) == live
        outs.append([t[:live].cpu().numpy() for t in t_out])
    # the allocating entry point on the same records
    mp = pcl.MultiPopulation(("electron", pcl.Population(n, [], air["tabs"][pcl.Electron], air["cuts"][pcl.Electron],
                                                         particle=pcl.Electron)), seed=5, compaction_period=1000)
    bufs = [(xw, ps, meta, None), (np.zeros((0, 4), np.float32),) * 3 + (None,),
            (np.zeros((0, 4), np.float32),) * 3 + (None,)]
    mp.upload_packed(bufs, [n, 0, 0])
    pcl.repack(mp.get(pcl.Electron))
    back = [(np.zeros((n, 4), np.float32), np.zeros((n, 4), np.float32), np.zeros((n, 4), np.uint32), None),
            bufs[1], bufs[2]]
    ns = mp.download_packed(back)
    assert ns[0] == live
    for oxw, ops, ometa in outs:
        assert np.array_equal(oxw.view(np.float32), back[0][0][:live])
        assert np.array_equal(ops.view(np.float32), back[0][1][:live])
        assert np.array_equal(ometa.view(np.uint32), back[0][2][:live])
    # in place (or any overlap of an output with an input) is refused before any launch
    n_out = torch.zeros(1, dtype=torch.int64, device=dev)
    ptrs = [t.data_ptr() for t in t_in]
    rc = L.pcl_compact_noalloc(n, *ptrs, *ptrs, n_out.data_ptr(), None)
    assert rc == pcl._lib.PCL_ERR_INVALID
    assert b"overlap" in L.pcl_last_error(None)
    mp.close()
