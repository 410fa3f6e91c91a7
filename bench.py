"""Benchmark of the null-collision Monte Carlo step on GB300.

Workload (the 16 M-particle point of the mixed avalanche): relativistic
runaway electrons in air (N2/O2 0.79/0.21, 1 atm, 293 K) at E = 0.5 MV/m,
electrons / photons / positrons tracked through Moller, Seltzer-Berger,
screened Coulomb, Compton, photoelectric, Bethe-Heitler, Bhabha and
annihilation with continuum losses below 10 keV (photon cut 5 keV),
dt = 1 ps.  The population is 2^24 particles drawn (Philox seed = rank) from
the recipe of the grown avalanche: the state that 10^4 seed electrons at 1 MeV
reach when the electron count hits its target (PopulationTargetCallback),
with that state's e- / gamma / e+ fractions, spectra and angular
distributions (particulator.jl_gb300/data/grow_rrea.py writes the recipe).
A "step" is one advance! + droplow! over every particle.

Metric: particle-steps/s (live particles at step start x steps / time).
`value` times the device-resident step (CUDA events on the library's
stream); `e2e` times the same steps through the C ABI with the population
copied in from and out to pinned host buffers every step.  The same line
carries the batched form (256 swarms in one context against 256 sequential
plain contexts), the learned form (network samplers against the plain form
on the same state) and the fields form (the general step kernel with
position-dependent fields and a wall record, against the homogeneous field on
the same state and launch shape).  Inputs (16 M x 48 B = 805 MB) are far larger than
L2 (129 MB).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s on 1 GB300 (plain GPU step, mixed e-/gamma/e+ avalanche at 2^24 particles)"
UNIT = "particle-steps/s"


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


def _barrier_max(value: float, ws: int) -> float:
    if ws <= 1:
        return value
    import torch
    import torch.distributed as dist
    if not dist.is_initialized():
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend)
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0"))) if torch.cuda.is_available() else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _barrier(ws: int):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


class Clocks:
    """Sample SM clocks and throttle reasons with nvidia-smi during a region."""

    def __init__(self, device: int):
        self.device = device
        self.samples = []
        self._stop = threading.Event()
        self._th = None

    def __enter__(self):
        def run():
            q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap")
            while not self._stop.is_set():
                try:
                    out = subprocess.run(["nvidia-smi", "-i", str(self.device), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                         timeout=5).stdout.strip()
                    if out:
                        self.samples.append([v.strip() for v in out.split(",")])
                except Exception:
                    break
                self._stop.wait(0.2)
        self._th = threading.Thread(target=run, daemon=True)
        self._th.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._th:
            self._th.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def _peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# DRAM bytes (read + write) per slot of one k_step launch, from one ncu
# capture (dram__bytes_read.sum + dram__bytes_write.sum) of the event kernel on
# a 4 M-particle draw of the same mixed state at the commit named below (the
# same 84.9 B as at b3cc758);
# scaled to a launch by the slots
# it processes: the reads grow in proportion, the writes are bounded by 48 B
# per slot.
K_STEP_DRAM_BYTES_PER_SLOT = 84.9
K_STEP_DRAM_CAPTURE = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of the 4th k_step launch of "
                       "'bench.py --n 4194304 --steps 3 --warmup 3 --steps-per-launch 1 --no-cpu --no-e2e --no-forms' at commit "
                       "34299a7: 201.8 MB read + 154.3 MB written over 4.19 M slots")

# Warp instructions per particle-step of the event step kernel on a 4 M draw
# of the same state, by steps per launch (ncu smsp__inst_executed.sum of one
# launch over its particle-steps, commit 34299a7: the one-step instance, and
# the multi-step instance at 64 steps per launch), for the issue ceiling:
# 152 SMs x 4 schedulers x 2.07 GHz warp instructions per second.
K_STEP_WARP_INST_PER_PSTEP = {1: 46.7, 64: 40.9}
ISSUE_RATE = 152 * 4 * 2.07e9

WORKLOAD = "rrea-air-0.5MVm-mixed-16M"


def workload_config(n: int, ws: int) -> dict:
    """The workload keys both arms report (the GPU arm adds its launch shape
    and results outside this dict)."""
    return {"workload": WORKLOAD, "particles": n, "field_V_m": 5e5, "dt_s": 1e-12,
            "state": "grown mixed e-/gamma/e+ avalanche (recipe rrea_mixed_0.5MVm.json), Philox seed = rank",
            "l2": "inputs larger than L2 (population > 800 MB)", "parallelism": f"replicas{ws}"}


def build_workload(pcl, n: int, seed: int, device: int, steps_per_launch: int = 1, blocks_per_sm: int = 0,
                   classic_step: bool = False, use_graph: bool = False, compaction_period: int = 0):
    wl = pcl.workloads.rrea_mixed(n, seed=seed, device=device, steps_per_launch=steps_per_launch,
                                  blocks_per_sm=blocks_per_sm, classic_step=classic_step, use_graph=use_graph,
                                  compaction_period=compaction_period)
    wl.mpopl.set_pusher(wl.pusher)
    et = wl.mpopl.get(pcl.Electron).collisions
    return wl.mpopl, wl.pusher, wl.dt, dict(tables=(et,))


def _build_oracle():
    sys.path.insert(0, ROOT)
    from oracle import build as obuild
    obuild.build_oracle(verbose=False)


def cpu_reference(n_sample: int, steps: int, warmup: int, threads: int, seed: int = 0):
    """The oracle (C++ Float64 restatement of the reference step, tables from
    the numpy restatement of its init path; the GPU library is not loaded) on
    a bounded sample of the workload: n_sample particles drawn from the same
    grown-state recipe, `warmup` untimed steps of 1 ps, then `steps` timed
    ones.  Returns (particle-steps/s, seconds, particle-steps, live counts)."""
    import __graft_entry__ as graft
    graft.load_package()      # pure-Python parts only (recipe, descriptors)
    import particulator_gb300 as pcl
    from oracle.harness import Arrays
    from oracle import reference_world as rw
    W, tabs, cuts, pusher = rw.avalanche_world(seed)
    st = pcl.workloads.rrea_mixed_state(n_sample, seed=seed)
    rng = np.random.Generator(np.random.Philox(seed + 1000))
    base = 0
    for sp in (pcl.Electron, pcl.Photon, pcl.Positron):
        a = st[sp]
        m = len(a.w)
        if m:
            W.upload(sp, Arrays(a.x, a.p, a.w, a.t, -np.log(rng.random(m)), np.arange(base, base + m, dtype=np.uint64),
                                np.zeros(m, np.uint32)))
        base += m
    dt = 1e-12
    t = 0.0
    for _ in range(warmup):
        t += dt
        W.advance(t, threads)
    psteps = 0
    t0 = time.perf_counter()
    for _ in range(steps):
        psteps += sum(int(lib_count(W, sp)) for sp in (0, 1, 2))
        t += dt
        W.advance(t, threads)
    el = time.perf_counter() - t0
    live = [int(lib_count(W, sp)) for sp in (0, 1, 2)]
    return psteps / el, el, psteps, live, rw.library_loaded()


def lib_count(W, sp):
    from oracle.harness import lib as olib
    return olib().orc_count(W.h, int(sp))


def run_reference(args):
    """The CPU reference arm: the oracle on all host threads, on a bounded
    sample of the same workload; only the oracle library is built or loaded."""
    ws, rank = _dist()
    if rank != 0:
        return 0
    _build_oracle()
    threads = os.cpu_count() or 1
    v, el, ps, live, loaded = cpu_reference(args.cpu_sample, args.steps, args.warmup, threads)
    sample = (f"{args.cpu_sample} particles drawn from the grown-state recipe (seed 0), {args.warmup} warm-up + "
              f"{args.steps} timed steps of 1 ps ({ps} particle-steps, {el:.1f} s), C++ Float64 oracle, "
              f"tables from the numpy restatement")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(args.n, 1),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "live_at_end": live, "gpu_library_loaded": bool(loaded)}
    print(json.dumps(line))
    return 0


def run_swarms(args, pcl):
    """Batched swarms: `nswarm` avalanche swarms (fields log-spaced over
    0.3-3 MV/m, initial sizes log-uniform over 1e2-1e5, Philox seed 3) in one
    context, advanced by graph-replayed multi-step launches, against the same
    swarms run one after another, each in its own context with one plain launch
    per swarm per step.  Both timed on the wall clock of the device stream(s)."""
    L = pcl.lib()
    dt = 1e-12
    nsw = args.nswarm
    init = pcl.workloads.swarm_initial(nsw)
    comp = pcl.workloads.air_composition()
    tables = pcl.workloads.beam_tables(comp, float(init[0][0]), dt)
    # ---- batched: one context, swarm mode; launch shape from the autotuner
    b = pcl.workloads.swarm_batch(nsw, tables=tables, initial=init, use_graph=True, steps_per_launch=8)
    mp = b.mpopl
    t = args.warmup * dt
    pcl.run(mp, b.pusher, t, dt)
    tune = mp.autotune(b.pusher, dt, steps=args.tune_steps)
    t = mp.t
    K = tune["steps_per_launch"]
    steps = max(K, (args.steps + K - 1) // K * K)
    L.pcl_sync(mp.ctx)
    tal0 = mp.tallies()
    L.pcl_kernel_stats(mp.ctx, None, None, None, None, 1)
    cap = 1 << 20   # each swarm held at 2^20 electrons (device roulette after every launch group)
    mp.set_swarm_cap(cap, particles=(pcl.Electron,))
    with Clocks(0) as clk:
        L.pcl_timer_start(mp.ctx)
        t += steps * dt
        pcl.run(mp, b.pusher, t, dt)
        ms = C.c_double()
        L.pcl_timer_stop(mp.ctx, C.byref(ms))
    tal1 = mp.tallies()
    kms = C.c_double(); kl = C.c_int64(); nl = C.c_int64(); kb = C.c_double()
    L.pcl_kernel_stats(mp.ctx, C.byref(kms), C.byref(kl), C.byref(nl), C.byref(kb), 1)
    ps_b = tal1.particle_steps - tal0.particle_steps
    v_b = ps_b / (ms.value / 1e3)
    mom = mp.swarm_moments(pcl.Electron, nsw)
    peak, peak_kind = _peaks()
    # 96 B per particle-step over the step kernel's time, as for the plain line;
    # the bytes the kernel moves (once per launch per slot) beside it
    achieved = 96.0 * ps_b / (kms.value / 1e3) / 1e9
    moved_b = kb.value / (kms.value / 1e3) / 1e9
    # ---- sequential: one context per swarm, one plain launch per swarm per step
    seq = []
    for sw in range(nsw):
        seq.append(pcl.workloads.swarm_batch(nsw, swarms=[sw], tables=tables, initial=init, use_graph=False,
                                             steps_per_launch=1))
    ts = 0.0
    for k in range(args.warmup):
        ts += dt
        for q in seq:
            pcl.advance(q.mpopl, q.pusher, ts)
    # the same state as the batched context before its timed steps
    for k in range(int(round((t - args.warmup * dt) / dt))):
        ts += dt
        for q in seq:
            pcl.advance(q.mpopl, q.pusher, ts)
    s0 = sum(q.mpopl.tallies().particle_steps for q in seq)
    t0 = time.perf_counter()
    for k in range(steps):
        ts += dt
        for q in seq:
            pcl.advance(q.mpopl, q.pusher, ts)
    for q in seq:
        L.pcl_sync(q.mpopl.ctx)
    el_s = time.perf_counter() - t0
    ps_s = sum(q.mpopl.tallies().particle_steps for q in seq) - s0
    live_seq = np.array([q.mpopl.tallies().live[0] for q in seq])
    for q in seq:
        q.mpopl.close()
    line = {"metric": f"particle-steps/s on 1 GB300 (batched: {nsw} avalanche swarms in one context)",
            "value": v_b, "unit": UNIT, "n_gpus": 1, "steps": steps, "warmup": args.warmup,
            "ms_per_step": ms.value / steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"swarms{nsw}-air-0.3-3MVm", "nswarm": nsw, "seed_electrons": int(init[1].sum()),
                       "dt_s": dt, "autotuned": tune, "swarm_cap": 1 << 20,
                       "live_at_end": list(tal1.live), "max_swarm_live": int(mom[:, 0].max())},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind, "traffic": None, "kernel": "k_step",
                         "bytes_rule": "96 B per particle-step over the step kernel's time", "moved_GB_s": moved_b},
            "sequential_plain": {"value": ps_s / el_s, "unit": UNIT, "ms_per_step": 1e3 * el_s / steps,
                                 "launch_groups_per_step": nsw,
                                 "live_electrons_max_rel_diff": float(np.max(np.abs(live_seq - mom[:, 0]) /
                                                                             np.maximum(mom[:, 0], 1)))},
            "batched_over_sequential": v_b / (ps_s / el_s),
            "cpu_baseline": None, "gpu_launches": int(nl.value), "clocks": clk.summary()}
    mp.close()
    return line


def run_learned(args, pcl):
    """Learned form of the 16M avalanche: the Seltzer-Berger and Moller
    secondary-energy draws go to networks trained here on 1e8 table-sampler
    samples each (tensor-core training kernels), the rest of the step as in
    the plain form.  Both forms run from the same initial state; the line
    reports the learned value with the plain value, spawn counts and the
    networks' training cost beside it."""
    L = pcl.lib()
    co = pcl.co
    t_train0 = time.perf_counter()
    spl = args.learned_spl
    mp, pusher, dt, extra = build_workload(pcl, args.learned_n, seed=0, device=0, blocks_per_sm=args.bps,
                                           use_graph=bool(args.graph), steps_per_launch=spl)
    et = extra["tables"][0]
    nets = []
    attach = []
    for kind in (pcl.learned.LEARN_SB, pcl.learned.LEARN_MOLLER):
        pos = pcl.learned.table_positions(et, kind)
        targets = pos if kind == pcl.learned.LEARN_SB else pos[:1]   # Moller: one network for both Z
        for j in targets:
            net, loss = pcl.learned.train_sampler(mp, pcl.Electron, j, kind, samples=args.train_samples, nT=1024,
                                                  Q=1024, steps=args.train_steps, batch=8192, lr=2e-3, seed=j)
            nets.append((j, kind, loss))
            for q in (pos if kind == pcl.learned.LEARN_MOLLER else [j]):
                attach.append((q, kind, net))
    t_train = time.perf_counter() - t_train0
    results = {}
    for form in ("plain", "learned"):
        if form == "learned":
            for q, kind, net in attach:
                mp.set_learned(pcl.Electron, q, kind, net)
        t = 0.0
        for _ in range(args.warmup):
            t += dt
            pcl.advance(mp, pusher, t)
        L.pcl_sync(mp.ctx)
        tal0 = mp.tallies()
        s0 = mp.learn_stats()
        L.pcl_kernel_stats(mp.ctx, None, None, None, None, 1)
        with Clocks(0) as clk:
            L.pcl_timer_start(mp.ctx)
            t_end = t + args.steps * dt
            pcl.run(mp, pusher, t_end, dt)   # run!, `spl` steps per launch
            t = t_end
            ms = C.c_double()
            L.pcl_timer_stop(mp.ctx, C.byref(ms))
        tal1 = mp.tallies()
        s1 = mp.learn_stats()
        kms = C.c_double(); kl = C.c_int64(); nl = C.c_int64(); kb = C.c_double()
        L.pcl_kernel_stats(mp.ctx, C.byref(kms), C.byref(kl), C.byref(nl), C.byref(kb), 1)
        ps = tal1.particle_steps - tal0.particle_steps
        results[form] = dict(value=ps / (ms.value / 1e3), ms=ms.value, clocks=clk.summary(), launches=int(nl.value),
                             spawned=[int(tal1.spawned[q] - tal0.spawned[q]) for q in range(3)],
                             live=list(tal1.live), learned_collisions=int(s1[0] - s0[0]),
                             rounds=int(s1[1] - s0[1]), kbytes=kb.value, kms=kms.value, kl=kl.value)
        mp.close()
        if form == "plain":
            mp, pusher, dt, extra = build_workload(pcl, args.learned_n, seed=0, device=0, blocks_per_sm=args.bps,
                                                   use_graph=bool(args.graph), steps_per_launch=spl)
    r, p0 = results["learned"], results["plain"]
    peak, peak_kind = _peaks()
    # 96 B per particle-step over the step kernel's time, as for the plain line
    achieved = 96.0 * (r["value"] * r["ms"] / 1e3) / (r["kms"] / 1e3) / 1e9
    line = {"metric": "particle-steps/s on 1 GB300 (learned form: network samplers, mixed avalanche at 2^24)",
            "value": r["value"], "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": r["ms"] / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+bf16", "data": "synthetic",
            "config": {"workload": "rrea-air-0.5MVm-mixed-16M-learned", "particles": args.learned_n, "dt_s": 1e-12,
                       "steps_per_launch": spl, "api": "run! (pcl_run), both forms the same launch shape",
                       "networks": [{"table_position": j, "kind": k, "train_loss": l} for j, k, l in nets],
                       "training_s": t_train, "training_samples_per_network": args.train_samples,
                       "training_steps": args.train_steps},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "peak_kind": peak_kind, "traffic": None, "kernel": "k_step"},
            "learned": {"collisions_per_step": r["learned_collisions"] / args.steps,
                        "rounds_per_step": r["rounds"] / args.steps, "spawned": r["spawned"], "live": r["live"]},
            "plain": {"value": p0["value"], "ms_per_step": p0["ms"] / args.steps, "spawned": p0["spawned"],
                      "live": p0["live"]},
            "learned_over_plain": r["value"] / p0["value"],
            "cpu_baseline": None, "gpu_launches": r["launches"], "clocks": r["clocks"]}
    return line


def _oracle_world(pcl, seed, tabs, cuts, pusher, tally_only=()):
    from oracle.harness import OracleWorld
    return OracleWorld(seed, tabs, cuts, pusher, tally_only=tally_only)


def run_plain(args, pcl):
    """Electrons only in air at 1 MV/m: 1000 e- at 1 MeV along +z, 50 ns in
    steps of 1 ps (5e4 steps, 64 per launch), Moller / Seltzer-Berger /
    Coulomb, continuum loss below 10 keV, bremsstrahlung photons tallied.  The
    whole run is timed on the GPU; the oracle (C++ Float64, all host threads)
    runs the first 2000 steps of the same particles and streams, both for the
    CPU baseline and for a paired comparison with a GPU run of those steps."""
    from oracle.harness import compare_populations
    L = pcl.lib()
    threads = os.cpu_count() or 1
    wl = pcl.workloads.plain_electrons(n=1000, tfinal=50e-9, seed=1, steps_per_launch=64)
    mp, pusher, dt = wl.mpopl, wl.pusher, wl.dt
    nsteps = int(round(wl.tfinal / dt))
    mp.set_pusher(pusher)
    pcl.run(mp, pusher, 64 * dt, dt)   # warm-up launch (64 steps)
    tal0 = mp.tallies()
    with Clocks(0) as clk:
        L.pcl_timer_start(mp.ctx)
        pcl.run(mp, pusher, wl.tfinal, dt)
        ms = C.c_double()
        L.pcl_timer_stop(mp.ctx, C.byref(ms))
    tal1 = mp.tallies()
    ps = tal1.particle_steps - tal0.particle_steps
    e = mp.get(pcl.Electron).particles()
    obs = {"electrons": int(tal1.live[0]), "mean_energy_eV": float(np.mean(pcl.kinenergy(0, e.p)) / pcl.co.eV),
           "mean_z_m": float(np.mean(e.x[:, 2])), "photons_tallied": int(tal1.tally_count[1]),
           "photon_energy_J": float(tal1.tally_wE[1])}
    nl = C.c_int64()
    L.pcl_kernel_stats(mp.ctx, None, None, C.byref(nl), None, 1)
    mp.close()
    # paired GPU vs oracle over the first 2000 steps (same particles, seed, streams)
    k = 2000
    wb = pcl.workloads.plain_electrons(n=1000, tfinal=k * dt, seed=1)
    eb = wb.mpopl.get(pcl.Electron)
    W = _oracle_world(pcl, 1, {pcl.Electron: eb.collisions}, {pcl.Electron: eb.energy_cut, pcl.Photon: 0.0},
                      wb.pusher, tally_only=(pcl.Photon,))
    W.upload(pcl.Electron, eb.particles())
    t0 = time.perf_counter()
    pst = 0
    for i in range(k):
        pst += len(W.download(pcl.Electron).w) if i % 100 == 0 else 0
        W.advance((i + 1) * dt, threads)
    cpu_s = time.perf_counter() - t0
    c = W.counters()
    pcl.run(wb.mpopl, wb.pusher, k * dt, dt)
    rep = compare_populations(eb.particles(), W.download(pcl.Electron), pcl.Electron, rtol=1e-3, stol=1e-2)
    tb = wb.mpopl.tallies()
    wb.mpopl.close()
    n_orc = rep["n_orc"]
    cpu_value = (n_orc + 1000) / 2 * k / cpu_s
    line = {"metric": "particle-steps/s on 1 GB300 (electrons only, air, 1 MV/m, 1000 e- for 50 ns)",
            "value": ps / (ms.value / 1e3), "unit": UNIT, "n_gpus": 1, "steps": nsteps - 64, "warmup": 64,
            "ms_per_step": ms.value / (nsteps - 64), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "electrons-air-1MVm-1000", "dt_s": dt, "steps_per_launch": 64},
            "observables": obs,
            "paired_2000_steps": {"gpu_electrons": int(tb.live[0]), "oracle_electrons": int(n_orc),
                                  "gpu_photons": int(tb.tally_count[1]), "oracle_photons": int(c["tally_count"][1]),
                                  "ties": rep["ties"], "max_dp_rel": rep["max_dp_rel"], "ok": rep["ok"]},
            "cpu_baseline": {"value": cpu_value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"the first {k} steps of the same 1000 electrons ({cpu_s:.1f} s), C++ Float64 oracle"},
            "gpu_launches": int(nl.value), "clocks": clk.summary()}
    print(json.dumps(line))
    return 0


def _swarm_obs(t, z, zz, E):
    """drift velocity (fit of <z>), longitudinal diffusion (fit of var z / 2),
    mean energy (mean over the window)."""
    t = np.asarray(t); z = np.asarray(z); var = np.asarray(zz) - z ** 2
    W = np.polyfit(t, z, 1)[0]
    D = np.polyfit(t, var, 1)[0] / 2
    return float(W), float(D), float(np.mean(E))


REID_EN = (1.0, 3.0, 12.0, 24.0, 48.0)
REID_GROUPS = 8


def _reid_group_obs(snaps, groups):
    """Swarm observables of a run and their statistical errors by batch means:
    snaps = [(t, z, E, g)] with per-particle z (m), E (J) and group index g;
    the observables of each of `groups` groups (drift = slope of <z>, D_L =
    slope of var z / 2, mean energy over the snapshots), the value of the
    whole run, and its standard error std(groups) / sqrt(groups)."""
    t = np.array([q[0] for q in snaps])
    out = {}
    for name in ("W_m_s", "DL_m2_s", "mean_energy_eV"):
        out[name] = []
    per = []
    for gsel in [None] + list(range(groups)):
        zm, zv, em = [], [], []
        for _, z, E, g in snaps:
            m = slice(None) if gsel is None else (g == gsel)
            zz = z[m]
            zm.append(zz.mean()); zv.append(zz.var()); em.append(E[m].mean())
        W = np.polyfit(t, zm, 1)[0]
        D = np.polyfit(t, zv, 1)[0] / 2
        per.append((W, D, np.mean(em) / 1.6021766208e-19))
    per = np.array(per)
    res = {}
    for k, name in enumerate(("W_m_s", "DL_m2_s", "mean_energy_eV")):
        res[name] = float(per[0, k])
        res[name + "_se"] = float(per[1:, k].std(ddof=1) / np.sqrt(groups))
    return res


def run_reid_fp64(args, pcl):
    """The Float64 side of the Reid precision study, on the host cores only:
    the oracle (C++ Float64, all host threads) runs an independent swarm of
    args.reid_fp64_n electrons (Maxwellian, 1 eV mean; numpy Philox seed
    1002) at each E/N with the device run's schedule (1000 relaxation steps,
    2000 measured, a snapshot every 100), and reports each observable with
    its batch-means standard error over 8 groups of electrons."""
    from oracle.harness import Arrays, OracleWorld
    threads = os.cpu_count() or 1
    dt = 1e-12
    relax, meas, every = 1000, 2000, 100
    n = args.reid_fp64_n
    N = 2.504e25
    tab = pcl.workloads.reid_table(N)
    rows = []
    el_all = 0.0
    for EN in REID_EN:
        pusher = pcl.workloads.pusher((0.0, 0.0, -EN * pcl.co.Td * N))
        rng = np.random.Generator(np.random.Philox(1002))
        kT = 2.0 / 3.0 * 1.0 * pcl.co.eV
        p = rng.normal(scale=np.sqrt(pcl.co.electron_mass * kT), size=(n, 3))
        W = OracleWorld(2, {pcl.Electron: tab}, {pcl.Electron: 0.0}, pusher)
        W.upload(pcl.Electron, Arrays(np.zeros((n, 3)), p, np.ones(n), np.zeros(n), -np.log(rng.random(n)),
                                      np.arange(n, dtype=np.uint64), np.zeros(n, np.uint32)))
        snaps = []
        c0 = time.perf_counter()
        for blk in range((relax + meas) // every):
            for i in range(every):
                W.advance((blk * every + i + 1) * dt, threads)
            if (blk + 1) * every > relax:
                o = W.download(pcl.Electron)
                snaps.append(((blk + 1) * every * dt, o.x[:, 2].copy(), pcl.kinenergy(0, o.p),
                              (o.sid % REID_GROUPS).astype(int)))
        el = time.perf_counter() - c0
        el_all += el
        rows.append(dict({"EN_Td": EN, "electrons": n, "seconds": el}, **_reid_group_obs(snaps, REID_GROUPS)))
    line = {"metric": "Reid ramp swarm observables, Float64 oracle (host cores)", "unit": "particle-steps/s",
            "value": n * (relax + meas) * len(REID_EN) / el_all, "cores": threads, "data": "synthetic",
            "config": {"workload": "reid-ramp-fp64", "electrons": n, "dt_s": dt, "relax_steps": relax,
                       "measured_steps": meas, "groups": REID_GROUPS}, "observables": rows}
    print(json.dumps(line))
    return 0


def run_reid(args, pcl):
    """Reid's ramp model gas at E/N = 1, 3, 12, 24, 48 Td: 2^20 electrons
    (Maxwellian, 1 eV mean, Philox seed 2), dt = 1 ps, 1000 relaxation steps
    and 2000 measured steps (16 per launch).  FP32 device against the Float64
    oracle: the oracle follows the first 4096 electrons with the same streams
    (paired: the difference is the device's rounding error) and its own
    statistics give the FP64 reference of each observable."""
    L = pcl.lib()
    threads = os.cpu_count() or 1
    dt = 1e-12
    relax, meas, every = 1000, 2000, 100
    n, nsub = 1 << 20, 4096
    rows = []
    total_ps = 0.0
    total_ms = 0.0
    cpu_ps = 0.0
    cpu_s = 0.0
    clk_all = None
    for EN in (1.0, 3.0, 12.0, 24.0, 48.0):
        # null collisions dominate (~35 sub-steps per step, ~1 real collision):
        # the classic kernel (no batching, 4 blocks per SM) measured 1.7x faster
        wl = pcl.workloads.reid_ramp(n=n, EN_Td=EN, dt=dt, steps_per_launch=16, classic_step=True)
        mp, pusher = wl.mpopl, wl.pusher
        e = mp.get(pcl.Electron)
        init = e.particles()
        sub = pcl.ParticleArrays(init.x[:nsub], init.p[:nsub], init.w[:nsub], init.t[:nsub], init.s[:nsub],
                                 init.sid[:nsub], init.ctr[:nsub])
        W = _oracle_world(pcl, 2, {pcl.Electron: e.collisions}, {pcl.Electron: 0.0}, pusher)
        W.upload(pcl.Electron, sub)
        mp.set_pusher(pusher)
        t = 0.0
        gt, gz, gzz, gE = [], [], [], []
        ot, oz, ozz, oE = [], [], [], []
        snaps = []
        pz_g, pz_o, pE_g, pE_o = [], [], [], []
        tal0 = mp.tallies()
        seg = C.c_double()
        dev_ms = 0.0
        with Clocks(0) as clk:
            L.pcl_timer_start(mp.ctx)
            for blk in range((relax + meas) // every):
                t1 = (blk + 1) * every * dt
                pcl.run(mp, pusher, t1, dt)
                if (blk + 1) * every > relax:
                    m = e.moments()
                    gt.append(t1); gz.append(m[4] / m[0]); gzz.append(m[7] / m[0]); gE.append(m[1] / m[0])
                    if args.reid_groups:   # every particle, for the batch-means errors (outside the device time)
                        L.pcl_timer_stop(mp.ctx, C.byref(seg))
                        dev_ms += seg.value
                        q = e.particles()
                        snaps.append((t1, q.x[:, 2].copy(), pcl.kinenergy(0, q.p),
                                      (q.sid % REID_GROUPS).astype(int)))
                        L.pcl_timer_start(mp.ctx)
            L.pcl_timer_stop(mp.ctx, C.byref(seg))
            dev_ms += seg.value
        clk_all = clk.summary()
        tal1 = mp.tallies()
        total_ps += tal1.particle_steps - tal0.particle_steps
        total_ms += dev_ms
        # oracle: the first nsub electrons, same streams
        c0 = time.perf_counter()
        for blk in range((relax + meas) // every):
            for i in range(every):
                W.advance((blk * every + i + 1) * dt, threads)
            if (blk + 1) * every > relax:
                o = W.download(pcl.Electron)
                Eo = pcl.kinenergy(0, o.p)
                ot.append((blk + 1) * every * dt); oz.append(np.mean(o.x[:, 2])); ozz.append(np.mean(o.x[:, 2] ** 2))
                oE.append(np.mean(Eo))
        el = time.perf_counter() - c0
        cpu_s += el
        cpu_ps += nsub * (relax + meas)
        g = e.particles()
        o = W.download(pcl.Electron)
        sel = g.sid < nsub
        og = np.argsort(g.sid[sel]); oo = np.argsort(o.sid)
        dE = (np.mean(pcl.kinenergy(0, g.p[sel][og])) - np.mean(pcl.kinenergy(0, o.p[oo]))) / np.mean(
            pcl.kinenergy(0, o.p[oo]))
        dz = (np.mean(g.x[sel][og][:, 2]) - np.mean(o.x[oo][:, 2])) / max(abs(np.mean(o.x[oo][:, 2])), 1e-30)
        Wg, Dg, Eg = _swarm_obs(gt, gz, gzz, gE)
        Wo, Do, Eo_ = _swarm_obs(ot, oz, ozz, oE)
        rows.append({"EN_Td": EN, "gpu": {"W_m_s": Wg, "DL_m2_s": Dg, "mean_energy_eV": Eg / pcl.co.eV},
                     "gpu_batch_means": _reid_group_obs(snaps, REID_GROUPS) if snaps else None,
                     "oracle_fp64_4096": {"W_m_s": Wo, "DL_m2_s": Do, "mean_energy_eV": Eo_ / pcl.co.eV},
                     "paired_rel_diff": {"mean_energy": float(dE), "mean_z": float(dz)},
                     "oracle_ties": int(W.counters()["ties"])})
        mp.close()
    line = {"metric": "particle-steps/s on 1 GB300 (Reid ramp swarm, 2^20 e-, 5 E/N values)",
            "value": total_ps / (total_ms / 1e3), "unit": UNIT, "n_gpus": 1, "steps": relax + meas, "warmup": 0,
            "ms_per_step": total_ms / (5 * (relax + meas)), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "reid-ramp-2^20", "dt_s": dt, "steps_per_launch": 16, "step_kernel": "classic",
                       "relax_steps": relax,
                       "measured_steps": meas},
            "observables": rows,
            "cpu_baseline": {"value": cpu_ps / cpu_s, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"the first {nsub} electrons of each E/N, all {relax + meas} steps "
                                       f"({cpu_s:.1f} s), C++ Float64 oracle"},
            "clocks": clk_all}
    print(json.dumps(line))
    return 0


def run_mlp(args, pcl):
    """The learned-sampler network alone: batched inference of 2^22 rows
    (tcgen05 128 x 128 layers, 32768 tiles) and training steps of 8192 rows.
    FLOPs per row: 2 (2 x 128 + 2 x 128 x 128 + 128) = 66,304 forward."""
    L = pcl.lib()
    n = 1 << 22
    net = pcl.SamplerNet(seed=1)
    rng = np.random.default_rng(0)
    x = rng.uniform(-1, 1, (n, 2)).astype(np.float32)
    y = net.forward(x)   # warm-up, and the device buffers
    flops_row = 2.0 * (2 * 128 + 2 * 128 * 128 + 128)
    # device-resident timing: the handle's forward on its own buffers, events on its stream
    reps = max(args.steps, 3)
    t0 = time.perf_counter()
    for _ in range(reps):
        y = net.forward(x)
    el = time.perf_counter() - t0
    e2e = n * reps / el
    # training rate
    t = (np.sin(3 * x[:, 0]) * x[:, 1]).astype(np.float32)
    steps = 400
    t1 = time.perf_counter()
    net.train(x[: 1 << 20], t[: 1 << 20], steps=steps, batch=8192, lr=1e-3, seed=0)
    tr = time.perf_counter() - t1
    line = {"metric": "learned-sampler network: inference rows/s through pcl_mlp_forward (host arrays)",
            "value": e2e, "unit": "rows/s", "n_gpus": 1, "steps": reps, "warmup": 1,
            "higher_is_better": True, "dtype": "bf16", "data": "synthetic",
            "config": {"workload": "mlp-2x128x128x128x1", "rows": n, "train_batch": 8192},
            "inference_tflops_incl_copies": e2e * flops_row / 1e12,
            "training_steps_per_s": steps / tr, "training_rows_per_s": steps * 8192 / tr,
            "gpu_launches": reps + 6 * steps}
    print(json.dumps(line))
    net.close()
    return 0


def run_kernels(args, pcl):
    """Every kernel of the path besides the step, once each on the 16 M
    mixed state (inputs larger than L2), timed with CUDA events on the
    context's stream around its ABI call: algorithmic bytes (or FLOPs) per call
    and the achieved rate against the measured peaks."""
    L = pcl.lib()
    peak, peak_kind = _peaks()
    mp, pusher, dt, extra = build_workload(pcl, args.n, seed=0, device=0)
    for k in range(args.warmup):
        pcl.advance(mp, pusher, (k + 1) * dt)
    L.pcl_sync(mp.ctx)
    tal = mp.tallies()
    n_slots = [int(v) for v in tal.n]
    n_live = [int(v) for v in tal.live]
    E, G, P = pcl.Electron, pcl.Photon, pcl.Positron
    rows = []

    def timed(name, kernels, nbytes, fn, reps=3):
        best = 1e30
        for _ in range(reps):
            L.pcl_timer_start(mp.ctx)
            fn()
            ms = C.c_double()
            L.pcl_timer_stop(mp.ctx, C.byref(ms))
            best = min(best, ms.value)
        gbs = nbytes / (best / 1e3) / 1e9
        rows.append({"op": name, "kernels": kernels, "ms": best, "bytes": nbytes, "GB_s": gbs, "frac": gbs / peak})

    edges = np.geomspace(1e3, 1e9, 257) * pcl.co.eV
    timed("moments (electrons)", "k_moments", 48 * n_slots[E], lambda: mp.get(E).moments())
    timed("energy histogram (electrons, 256 bins)", "k_energy_hist", 48 * n_slots[E],
          lambda: mp.get(E).energy_histogram(edges))
    timed("swarm counts (electrons, one swarm)", "k_swarm_count", 16 * n_slots[E], lambda: mp.swarm_counts(E, 1))
    timed("swarm moments (electrons, one swarm)", "k_swarm_moments + k_swarm_reduce", 48 * n_slots[E],
          lambda: mp.swarm_moments(E, 1))
    timed("roulette (photons, keep 0.9999)", "k_roulette", 16 * n_slots[G], lambda: mp.roulette(G, 0.9999), reps=1)
    timed("per-swarm roulette (electrons, one swarm, keep 0.9999)", "k_roulette_swarms", 16 * n_slots[E],
          lambda: mp.roulette_swarms(E, [0.9999]), reps=1)
    timed("split (photons, 1 % copies)", "k_split", 16 * n_slots[G], lambda: mp.split(G, 0.01), reps=1)
    # the function forms (roulette!(f, popl), split!(f, popl)): f of the
    # kinetic energy as a 4096-node table; each live particle's momentum is
    # read too (32 B per slot)
    ftab = (pcl.ENERGY_TABLE_NODES, np.full(4096, 0.9999))
    timed("roulette with f(E) (photons, 4096-node table, keep 0.9999)", "k_roulette_fn", 32 * n_slots[G],
          lambda: mp.roulette(G, ftab), reps=1)
    timed("split with f(E) (photons, 4096-node table, 1 % copies)", "k_split_fn", 32 * n_slots[G],
          lambda: mp.split(G, (pcl.ENERGY_TABLE_NODES, np.full(4096, 0.01))), reps=1)
    # the device per-swarm population cap (a RouletteCallback per swarm, applied
    # after every launch group of run!): one step with the electrons' cap below
    # their count, so that k_swarm_count and k_roulette_cap follow the step
    t_cap = float(tal.t) + dt
    mp.set_swarm_cap(int(0.9 * n_live[E]), particles=(E,))
    timed("one step, then the per-swarm cap of the electrons (keep ~0.9)",
          "k_step + k_swarm_count + k_roulette_cap", 0, lambda: pcl.run(mp, pusher, t_cap, dt), reps=1)
    mp.set_swarm_cap(0, particles=(E,))
    tal = mp.tallies()
    n_slots = [int(v) for v in tal.n]
    n_live = [int(v) for v in tal.live]
    cbytes = sum(16 * n_slots[q] + 48 * n_slots[q] + 48 * n_live[q] for q in range(3))
    timed("repack (all species)", "k_compact_count + k_compact_scan + k_compact_scatter", cbytes,
          lambda: L.pcl_compact(mp.ctx), reps=1)
    # training data of a learned sampler: 2^22 draws of the Seltzer-Berger table
    # sampler, histogrammed on the device (k_learn_hist)
    et = mp.get(E).collisions
    j = pcl.learned.table_positions(et, pcl.learned.LEARN_SB)[0]
    L.pcl_timer_start(mp.ctx)
    pcl.learned.learn_data(mp, E, j, pcl.learned.LEARN_SB, samples=float(1 << 22), nT=256, Q=256, seed=1)
    lms = C.c_double()
    L.pcl_timer_stop(mp.ctx, C.byref(lms))
    rows.append({"op": "learned-sampler training data (2^22 table draws, 256 energies)",
                 "kernels": "k_learn_hist", "ms": lms.value, "draws_per_s": (1 << 22) / (lms.value / 1e3)})
    mp.close()
    # the network kernels (FLOPs): inference of 4 M rows, training steps of 8192 rows
    net = pcl.SamplerNet(seed=1)
    nrow = 1 << 22
    rng = np.random.default_rng(0)
    x = rng.uniform(-1, 1, (nrow, 2)).astype(np.float32)
    net.forward(x)
    t0 = time.perf_counter()
    for _ in range(3):
        net.forward(x)
    fwd_s = (time.perf_counter() - t0) / 3
    flops_row = 2.0 * (2 * 128 + 2 * 128 * 128 + 128)
    t = (np.sin(3 * x[:, 0]) * x[:, 1]).astype(np.float32)
    steps = 300
    t1 = time.perf_counter()
    net.train(x[: 1 << 20], t[: 1 << 20], steps=steps, batch=8192, lr=1e-3, seed=0)
    tr_s = (time.perf_counter() - t1) / steps
    net.close()
    line = {"metric": "achieved HBM GB/s of the kernels beside the step (CUDA events around each ABI call)",
            "unit": "GB/s", "peak": peak, "peak_kind": peak_kind, "data": "synthetic",
            "config": {"workload": WORKLOAD, "particles": args.n, "slots": n_slots, "live": n_live},
            "ops": rows,
            "network": {"inference_rows": nrow, "inference_s_incl_host_copies": fwd_s,
                        "inference_TFLOP_s_incl_host_copies": nrow * flops_row / fwd_s / 1e12,
                        "train_step_s (8192 rows, forward + backward + Adam)": tr_s,
                        "train_TFLOP_s": 3 * 8192 * flops_row / tr_s / 1e12}}
    print(json.dumps(line))
    return 0


def run_fields(args, pcl):
    """The general step kernel (a position-dependent E of field.jl, a wall
    record of WallCallback) on the 16 M mixed state, against the homogeneous
    kernel on the same draw and launch shape (64 steps per launch, repack
    every 8).  Each arm draws the same particles (Philox seed 0) into a fresh
    context, runs W warm-up steps, then times `args.steps` steps of run! with
    CUDA events on the context's stream; the wall arm's records are read back
    inside the timed region, as run! does after every launch."""
    L = pcl.lib()
    peak, peak_kind = _peaks()
    E0 = (0.0, 0.0, -5e5)
    zc = 191.0   # mean z of the grown state's electrons (m); spread 8.7 m
    arms = (("homogeneous E (the headline kernel)", None, None),
            ("DoubleLayerField over the whole population (same physics)", pcl.DoubleLayerField(-1e4, 1e4, E0), None),
            ("StepField: E above the electrons' mean z, 0 below", pcl.StepField(zc, (0.0, 0.0, 0.0), E0), None),
            ("ConfinedDoubleLayerField (40 m, 40 m, 200 m, 0.5 MV/m)",
             pcl.ConfinedDoubleLayerField(40.0, 40.0, 200.0, -5e5), None),
            ("DoubleLayerField over the upper half + WallCallback (electrons, z = 200 m, drop)",
             pcl.DoubleLayerField(zc, 1e4, E0), (pcl.Electron, 3, 200.0)))
    rows = []
    with Clocks(0) as clk:
        for name, field, wall in arms:
            mp, pusher, dt, _ = build_workload(pcl, args.n, seed=0, device=0, steps_per_launch=64,
                                               compaction_period=8)
            if field is not None:
                cl = pusher.device_forcing()[2]
                pusher = pcl.RK2Pusher(pcl.CombinedForcing(
                    pcl.ElectromagneticField(field, pcl.HomogeneousField((0.0, 0.0, 0.0))), cl))
            cb = pcl.WallCallback(*wall) if wall is not None else None
            pcl.run(mp, pusher, args.warmup * dt, dt, cb)
            tal0 = mp.tallies()
            L.pcl_sync(mp.ctx)
            L.pcl_kernel_stats(mp.ctx, None, None, None, None, 1)
            L.pcl_timer_start(mp.ctx)
            pcl.run(mp, pusher, (args.warmup + args.steps) * dt, dt, cb)
            ms = C.c_double()
            L.pcl_timer_stop(mp.ctx, C.byref(ms))
            tal1 = mp.tallies()
            ps = tal1.particle_steps - tal0.particle_steps
            kms = C.c_double(); kl = C.c_int64(); nl = C.c_int64(); kb = C.c_double()
            L.pcl_kernel_stats(mp.ctx, C.byref(kms), C.byref(kl), C.byref(nl), C.byref(kb), 1)
            # 96 B per particle-step over the step kernel's time, as for the plain line
            ach = 96.0 * ps / (kms.value / 1e3) / 1e9 if kms.value > 0 else None
            row = {"arm": name, "general_kernel": field is not None or wall is not None,
                   "value": ps / (ms.value / 1e3), "ms_per_step": ms.value / args.steps,
                   "particle_steps": int(ps), "live_at_end": [int(v) for v in tal1.live],
                   "gpu_launches": int(nl.value), "step_kernel_ms": kms.value,
                   "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                                "frac": ach / peak if ach else None, "peak_kind": peak_kind}}
            if cb is not None:
                row["wall_records"] = int(len(cb.states().w))
            rows.append(row)
            mp.close()
    base = rows[0]["value"]
    for r in rows:
        r["over_homogeneous"] = r["value"] / base
    line = {"metric": "particle-steps/s on 1 GB300 of the general step kernel (position-dependent E, wall "
                      "records), mixed avalanche at 2^24 particles", "value": min(r["value"] for r in rows[1:]),
            "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD + " (field shapes of field.jl)", "particles": args.n,
                       "steps_per_launch": 64, "compaction_period": 8,
                       "l2": "inputs larger than L2 (population > 800 MB)"},
            "value_is": "the slowest general-kernel arm", "arms": rows, "clocks": clk.summary(),
            "roofline": min((r["roofline"] for r in rows[1:] if r["roofline"]["frac"]), key=lambda q: q["frac"],
                            default=None),
            "gpu_launches": sum(r["gpu_launches"] for r in rows)}
    return line


def _printing(fn):
    def wrap(args, pcl):
        print(json.dumps(fn(args, pcl)))
        return 0
    return wrap


def _form_summary(line: dict, plain_value: float) -> dict:
    """The sub-object of the default line for one other form."""
    keep = ("metric", "value", "unit", "ms_per_step", "steps", "warmup", "dtype", "config", "roofline",
            "gpu_launches", "clocks")
    out = {k: line[k] for k in keep if k in line}
    for k in ("sequential_plain", "batched_over_sequential", "plain", "learned_over_plain", "learned", "value_is",
              "arms"):
        if k in line:
            out[k] = line[k]
    out["over_plain_16M_line"] = line["value"] / plain_value if plain_value else None
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=64)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--n", type=int, default=1 << 24, help="particles drawn from the grown-state recipe")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--e2e-chunks", type=int, default=8, help="pipeline chunks of pcl_advance_host")
    ap.add_argument("--cpu-sample", type=int, default=1 << 21)
    ap.add_argument("--cpu-steps", type=int, default=40)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-forms", action="store_true", help="skip the batched and learned sub-objects")
    ap.add_argument("--steps-per-launch", type=int, default=0,
                    help="steps per launch of the timed run! (0: chosen by the library's autotuner)")
    ap.add_argument("--tune-budget", type=int, default=1344, help="steps the autotuner may use (untimed)")
    ap.add_argument("--bps", type=int, default=0, help="step-kernel blocks per SM (2, 3, 4)")
    ap.add_argument("--classic", type=int, default=0, help="1: classic step kernel (lanes collide in place)")
    ap.add_argument("--graph", type=int, default=0, help="1: launch groups replayed from CUDA graphs")
    ap.add_argument("--compaction-period", type=int, default=0, help="steps between repacks (0: the library's 8)")
    ap.add_argument("--workload", default="rrea16M",
                    choices=["rrea16M", "swarms", "learned", "plain", "reid", "reid-fp64", "mlp", "kernels", "fields"])
    ap.add_argument("--nswarm", type=int, default=256)
    ap.add_argument("--tune-steps", type=int, default=1344)
    ap.add_argument("--learned-n", type=int, default=1 << 24, help="learned form: particles")
    ap.add_argument("--learned-spl", type=int, default=64, help="learned form: steps per launch (both forms)")
    ap.add_argument("--reid-groups", type=int, default=0, help="reid: batch-means errors from particle snapshots")
    ap.add_argument("--reid-fp64-n", type=int, default=1 << 17, help="reid-fp64: electrons of the Float64 run")
    ap.add_argument("--train-samples", type=float, default=1e8, help="learned form: training samples per network")
    ap.add_argument("--train-steps", type=int, default=8000, help="learned form: Adam steps per network")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "reid-fp64":   # host cores only: the oracle, no GPU library
        _build_oracle()
        import __graft_entry__ as graft
        return run_reid_fp64(args, graft.load_package())
    if args.workload != "rrea16M":
        import __graft_entry__ as graft
        graft.build()
        fn = {"swarms": _printing(run_swarms), "learned": _printing(run_learned), "plain": run_plain,
              "reid": run_reid, "mlp": run_mlp, "kernels": run_kernels,
              "fields": _printing(run_fields)}[args.workload]
        return fn(args, graft.load_package())
    ws, rank = _dist()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    import __graft_entry__ as graft
    graft.build()
    pcl = graft.load_package()
    L = pcl.lib()
    mp, pusher, dt, extra = build_workload(pcl, args.n, seed=rank, device=local,
                                           steps_per_launch=max(1, args.steps_per_launch), blocks_per_sm=args.bps,
                                           classic_step=bool(args.classic), use_graph=bool(args.graph),
                                           compaction_period=args.compaction_period)
    ctx = mp.ctx
    live_start = list(mp.tallies().live)
    # ---- warm-up: W steps, then (unless a launch shape is given) the
    # library's autotuner, whose trials are real steps of the same run
    t = 0.0
    for _ in range(args.warmup):
        t += dt
        pcl.advance(mp, pusher, t)
    tune = None
    if args.steps_per_launch == 0:
        tune = mp.autotune(pusher, dt, steps=args.tune_budget)
        t = mp.t
    K = int(mp.config.steps_per_launch)
    L.pcl_sync(ctx)
    tal0 = mp.tallies()
    L.pcl_kernel_stats(ctx, None, None, None, None, 1)
    # ---- timed region: K steps of run! (launch groups of the chosen shape), a
    # device synchronisation and a barrier on both sides
    L.pcl_sync(ctx)
    _barrier(ws)
    with Clocks(local) as clk:
        L.pcl_timer_start(ctx)
        t_end = t + args.steps * dt
        pcl.run(mp, pusher, t_end, dt)
        t = t_end
        ms = C.c_double()
        L.pcl_timer_stop(ctx, C.byref(ms))
    L.pcl_sync(ctx)
    _barrier(ws)
    tal1 = mp.tallies()
    kms = C.c_double(); kl = C.c_int64(); nl = C.c_int64(); kb = C.c_double()
    L.pcl_kernel_stats(ctx, C.byref(kms), C.byref(kl), C.byref(nl), C.byref(kb), 1)
    psteps = tal1.particle_steps - tal0.particle_steps
    assert tal1.steps - tal0.steps == args.steps, (tal1.steps, tal0.steps)
    elapsed = _barrier_max(ms.value / 1e3, ws)
    total_psteps = psteps * ws
    value = total_psteps / elapsed
    peak, peak_kind = _peaks()
    # algorithmic bytes: 96 B per particle-step (48 B read + 48 B written per
    # particle per step) over the step kernel's own time; with several steps
    # per launch a particle stays in registers between its steps, and the
    # bytes the kernel moves are its slots' 96 B once per launch
    achieved = 96.0 * psteps / (kms.value / 1e3) / 1e9
    moved = kb.value / (kms.value / 1e3) / 1e9
    slots_per_launch = (kb.value / max(kl.value, 1)) / 96.0
    traffic = K_STEP_DRAM_BYTES_PER_SLOT * slots_per_launch if K_STEP_DRAM_BYTES_PER_SLOT else None
    # issue ceiling with the instruction count captured at the nearest launch shape
    kq = min(K_STEP_WARP_INST_PER_PSTEP, key=lambda q: abs(np.log(q) - np.log(K)))
    ceiling = ISSUE_RATE / K_STEP_WARP_INST_PER_PSTEP[kq]
    issue = {"warp_inst_per_particle_step": K_STEP_WARP_INST_PER_PSTEP[kq], "captured_at_steps_per_launch": kq,
             "ceiling": ceiling, "unit": UNIT, "frac": value / ws / ceiling}
    # ---- end to end through the C ABI with pinned host buffers
    e2e = None
    try:
        if args.no_e2e:
            raise RuntimeError("skipped (--no-e2e)")
        # the population lives in pinned host buffers: every step reads it from
        # there and writes it back (pcl_advance_host), in the library's default
        # mode (the copy pipeline: chunked copy-engine uploads and downloads
        # around range launches) and, for comparison, host-direct (the step
        # kernel reads and writes the page-locked arrays over the CPU-GPU link)
        host = mp.packed_buffers(pinned=True)
        ns = mp.download_packed(host)
        period = 8
        modes = {}
        for mode, name in ((pcl._lib.HOST_IO_AUTO, "default"), (pcl._lib.HOST_IO_DIRECT, "direct")):
            mp.set_host_io(mode)
            tal_a = mp.tallies()
            h2d = d2h = 0
            L.pcl_timer_start(ctx)
            for k in range(args.e2e_steps):
                t += dt
                h2d += 48 * sum(ns)
                ns = mp.advance_host(t, host, ns, nchunks=args.e2e_chunks, compact=(k % period == period - 1))
                d2h += 48 * sum(ns)
            ms2 = C.c_double()
            L.pcl_timer_stop(ctx, C.byref(ms2))
            tal_b = mp.tallies()
            e_el = _barrier_max(ms2.value / 1e3, ws)
            modes[name] = {"value": (tal_b.particle_steps - tal_a.particle_steps) * ws / e_el,
                           "ms_per_step": 1e3 * e_el / args.e2e_steps,
                           "h2d_bytes_per_step": int(h2d / args.e2e_steps),
                           "d2h_bytes_per_step": int(d2h / args.e2e_steps)}
        mp.set_host_io(pcl._lib.HOST_IO_AUTO)
        d = modes["default"]
        e2e = {"value": d["value"], "unit": UNIT, "h2d_bytes_per_step": d["h2d_bytes_per_step"],
               "d2h_bytes_per_step": d["d2h_bytes_per_step"], "ms_per_step": d["ms_per_step"],
               "api": "pcl_advance_host", "mode": "copy pipeline (the default)", "chunks": args.e2e_chunks,
               "host_buffers": "pinned", "steps": args.e2e_steps, "host_direct": modes["direct"]}
        del host
    except Exception as ex:  # pragma: no cover
        e2e = {"value": None, "unit": UNIT, "error": str(ex)[:200], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    errs = {pcl._lib.ERROR_NAMES[q]: int(tal1.errors[q]) for q in range(8) if tal1.errors[q]}
    live_end = list(tal1.live)
    mp.close()
    # ---- CPU baseline (rank 0, N = 1): the oracle on a bounded sample
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        v, el, ps, _, _ = cpu_reference(args.cpu_sample, args.cpu_steps, 1, threads)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{args.cpu_sample} particles drawn from the grown-state recipe, 1 warm-up + "
                         f"{args.cpu_steps} timed steps of 1 ps ({ps} particle-steps, {el:.1f} s), C++ Float64 "
                         f"oracle"}
    forms = {}
    if rank == 0 and ws == 1 and not args.no_forms:
        for name, fn in (("batched", run_swarms), ("learned", run_learned), ("fields", run_fields)):
            try:
                forms[name] = _form_summary(fn(args, pcl), value)
            except Exception as ex:  # pragma: no cover
                forms[name] = {"value": None, "error": str(ex)[:300]}
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": workload_config(args.n, ws),
                "run": {"api": "run! (pcl_run) over the timed steps", "steps_per_launch": K,
                        "graph": bool(mp.config.use_graph),
                        "compaction_period": int(mp.config.compaction_period) or 8,
                        "blocks_per_sm": int(mp.config.blocks_per_sm) or 3,
                        "step_kernel": "classic" if mp.config.classic_step else "event",
                        "launch_shape": "autotuned (pcl_autotune, untimed)" if tune else "given",
                        "autotune": tune, "step_launches": int(kl.value),
                        "live_at_start": live_start, "live_at_end": live_end},
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
                             "traffic_source": K_STEP_DRAM_CAPTURE, "kernel": "k_step",
                             "bytes_rule": "96 B per particle-step over the step kernel's time",
                             "moved_GB_s": moved, "moved_rule": "96 B per slot per launch (once per "
                             f"{K} steps) over the step kernel's time"},
                "issue_roofline": issue,
                "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(nl.value), "clocks": clk.summary(),
                "errors": errs}
        line.update(forms)
        print(json.dumps(line))
    return 0


if __name__ == "__main__":
    sys.exit(main())
