#!/usr/bin/env python3
"""Benchmark of the GB300 force hot path (one JSON line on rank 0).

A step is one pass of the reference's step loop (Simulation.cpp:256-341) over
the whole workload with every particle active: kick + drift, octree build, SPH
density, Barnes-Hut walk with in-walk SPH force, Ueuler for gas, kick.  The
default workload is the 4,194,304-particle galaxy merger (two 2,097,152-particle
disk galaxies with dark halo, stellar disk and gas) at theta = 0.5, eps = 0.02,
dt = 1e-3, computed with the FP32-offset walk.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME]
  python bench.py --impl reference ...   # the reference's CPU algorithm on host cores

value     particle-steps/s, state resident in HBM, CUDA events on the stream
e2e       the same metric through the public C-ABI with host (pinned) buffers:
          every step uploads the particle state and reads it back
roofline  the walk kernel (FP32 FMA / MUFU bound) against this GPU's measured
          FP32 FMA throughput
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "astrogenesis2.0_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))

import ics  # noqa: E402

METRIC = "particle-steps/s, FP32+batched vs plain, at <=1e-4 force error; p99 latency"
UNIT = "particle-steps/s"
FLOP_GRAV = 23  # per gravity interaction (P2P or accepted node)
FLOP_SPH = 60   # per SPH pair

WORKLOADS = {
    "merger4m": dict(desc="galaxy merger, 2 x 2,097,152 particles (3/4 dark halo, 3/16 stars, 1/16 gas), "
                          "parabolic orbit r_peri=5 at separation 40, disks inclined 30/60 deg",
                     make=lambda: ics.merger(2097152, seed=3), e0=0.02, theta=0.5, dt=1e-3),
    "disk1m": dict(desc="isolated disk galaxy, 786,432 DM + 196,608 stars + 65,536 gas",
                   make=lambda: ics.disk_galaxy(seed=2), e0=0.02, theta=0.5, dt=1e-3),
    "ensemble512": dict(desc="512 independent Plummer spheres (M=1, a=1), N log-uniform in [1024, 65536], "
                             "gravity only, one tree build and one walk launch per step over all instances",
                        make=lambda: ics.ensemble(512), e0=0.01, theta=0.5, dt=1e-3),
    "serving": dict(desc="request stream, Poisson arrivals at 10, 50 and 200 requests/s; disk galaxies with N "
                         "log-uniform in [4096, 262144], 30% with gas at gas fraction 0.1, steps uniform in [50, 500]; "
                         "continuous batching under a 150 GB budget", make=None, e0=0.02, theta=0.5, dt=1e-3),
    "plummer16k": dict(desc="Plummer sphere N=16,384, M=1, a=1", make=lambda: ics.plummer(16384, seed=1), e0=0.01,
                       theta=0.5, dt=1e-3),
}


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
CLOCK_Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
           "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
           "clocks_event_reasons.sw_power_cap")


class ClockSampler:
    """nvidia-smi sampling every 50 ms, started before the warm-up so that its
    start-up never overlaps the timed window; only samples taken inside the
    window [mark_start, mark_stop] are reported."""

    def __init__(self, gpu: int):
        import threading

        self.lines = []
        self.t0 = self.t1 = None
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(gpu), f"--query-gpu={CLOCK_Q}",
                                       "--format=csv,noheader,nounits", "-lms", "50"], stdout=subprocess.PIPE,
                                      stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None
            return
        self.th = threading.Thread(target=self._read, daemon=True)
        self.th.start()

    def _read(self):
        for line in self.p.stdout:
            self.lines.append((time.time(), line))

    def mark_start(self):
        self.t0 = time.time()

    def mark_stop(self):
        self.t1 = time.time()

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.3)
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        inside = [l for t, l in self.lines if self.t0 is not None and self.t0 - 0.05 <= t <= (self.t1 or t) + 0.05]
        for line in inside:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                smax.append(float(f[1]))
            except ValueError:
                continue
            for name, v in zip(names, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU legs (the oracle restatement: test infrastructure, used here only as the
# timed CPU baseline / reference arm)
# ---------------------------------------------------------------------------
def cpu_step_time(d: dict, wl: dict, walk_fraction: int, threads: int, world=None) -> tuple[float, object, str]:
    """One step of the reference's algorithm on the host: kick+drift, build,
    gas density, walk for 1/walk_fraction of the particles (time scaled), Ueuler,
    kick.  Returns (seconds per full step, world, sample description)."""
    import numpy as np

    import oracle

    n = len(d["mass"])
    if world is None:
        world = oracle.World(d["pos"], d["mass"], d["type"], d["vel"], d["U"], kind="port")
    dt = wl["dt"]
    idx = np.arange(0, n, walk_fraction, dtype=np.int32)
    t0 = time.perf_counter()
    world.kick(dt)
    world.drift(dt)
    t1 = time.perf_counter()
    world.build(threads)
    if (d["type"] == 2).any():
        world.gas_density(d.get("massInH", 0.0))
    t2 = time.perf_counter()
    if walk_fraction == 1:
        world.forces(wl["e0"], wl["theta"], threads)
    else:
        world.forces_subset(wl["e0"], wl["theta"], idx, threads)
    t3 = time.perf_counter()
    world.ueuler(dt)
    world.kick(dt)
    t4 = time.perf_counter()
    scaled = (t1 - t0) + (t2 - t1) + (t3 - t2) * (n / idx.size) + (t4 - t3)
    if walk_fraction == 1:
        sample = (f"a full step over all {n} particles, timed in full: kick+drift, build, SPH density, walk, "
                  f"Ueuler, kick")
    else:
        sample = (f"full build + SPH density + kick/drift over all {n} particles, walk for every "
                  f"{walk_fraction}th particle ({idx.size}) scaled by {n / idx.size:.1f}")
    return scaled, world, sample


def cpu_step_time_instances(d: dict, wl: dict, every: int, threads: int, worlds=None):
    """One step of every `every`-th independent simulation on the host (each its
    own tree and walk over all its particles), scaled to all particles."""
    import oracle

    first = d["first"]
    ks = list(range(0, len(first) - 1, every))
    if worlds is None:
        worlds = [oracle.World(d["pos"][first[k]:first[k + 1]], d["mass"][first[k]:first[k + 1]],
                               d["type"][first[k]:first[k + 1]], d["vel"][first[k]:first[k + 1]],
                               d["U"][first[k]:first[k + 1]], kind="port") for k in ks]
    dt = wl["dt"]
    m = 0
    t0 = time.perf_counter()
    for w in worlds:
        w.kick(dt)
        w.drift(dt)
        w.build(threads)
        w.forces(wl["e0"], wl["theta"], threads)
        w.kick(dt)
        m += w.n
    t = time.perf_counter() - t0
    n = int(first[-1])
    sample = (f"{len(ks)} of {len(first) - 1} simulations (every {every}th, {m} particles), a full step each, "
              f"scaled by {n / m:.1f}")
    return t * n / m, worlds, sample


def reference_arm(args, wl, d):
    from dist import finalize, init

    D = init(backend="gloo")
    if D.rank != 0:
        finalize(D)
        return
    threads = os.cpu_count() or 1
    n = len(d["mass"])
    world = None
    times = []
    for k in range(args.warmup + args.steps):
        if "first" in d:
            t, world, sample = cpu_step_time_instances(d, wl, args.ref_walk_fraction, threads, world)
        else:
            t, world, sample = cpu_step_time(d, wl, args.ref_walk_fraction, threads, world)
        if k >= args.warmup:
            times.append(t)
    per = sum(times) / len(times)
    value = n / per
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": per * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_block(args, wl, d),
        "method": reference_method(threads),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)
    finalize(D)


L2_BYTES = 129 * 2 ** 20


def _hbm_peak() -> float:
    try:
        return float(json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json")))["hbm_gbs"])
    except (OSError, ValueError, KeyError):
        return 6800.0  # fallback: one earlier copy-bandwidth measurement on a GB300


HBM_PEAK_GBS = _hbm_peak()
BYTES_PER_PARTICLE = 1400  # particle state (~200 B) + ~3.9 nodes of ~300 B


def needs_flush(n: int) -> bool:
    return n * BYTES_PER_PARTICLE < 4 * L2_BYTES


def config_block(args, wl, d):
    """The workload (the same block in both arms: the reference arm runs the
    same particles, parameters and step)."""
    import numpy as np

    n = int(len(d["mass"]))
    l2 = (f"per-step working set ~{n * BYTES_PER_PARTICLE / 2**30:.1f} GiB, far above the 129 MB L2 (no flush)"
          if not needs_flush(n) else "L2 flushed (512 MiB write) between timed steps")
    extra = {"instances": int(len(d["first"]) - 1)} if "first" in d else {}
    return {"workload": f"{args.workload}: {wl['desc']}", "particles": n, **extra,
            "gas_particles": int(np.sum(d["type"] == 2)), "theta": wl["theta"], "eps": wl["e0"], "dt": wl["dt"],
            "G": 1.0, "step": "kick+drift, octree build, SPH density, walk with SPH force, Ueuler, kick; "
                              "every particle active", "parallelism": "replicas", "l2": l2}


TOPOLOGY_NOTE = ("Node::insert switches to serial insertion below threads*100 particles (Node.cpp:420). The octree "
                 "does not depend on that threshold: node count, per-node membership and depth are the same at 100 "
                 "and at 1600 (checked on the restatement at 1, 8 and 16 threads against the reference's own "
                 "fixtures). Only the childParticles duplicates at the nodes where the build turns serial move, "
                 "which changes rho of the gas whose density node is such a node.")


def our_method(args):
    return {"walk": "FP32-offset warp walk with compensated sums" if args.precision == "fp32" else "FP64 warp walk",
            "split_threshold": 100, "threshold_rule": "the reference's deterministic one-thread setting (100)"}


def reference_method(threads):
    return {"walk": "FP64 recursive walk (Node::calculateGravityForce restated), one host thread per particle group",
            "split_threshold": 100 * threads,
            "threshold_rule": f"the reference's own rule on {threads} host threads (threads*100)",
            "topology_note": TOPOLOGY_NOTE}


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
# bytes a snapshot encode moves per particle in HBM: the fields the record
# holds (read) plus the record (written) plus the inverse permutation (read the
# tree-order ids, write and read the inverse)
IO_READ_BYTES = {"age": 24 + 24 + 5 * 8 + 1 + 1 + 4, "ag": 24 + 4 * 8 + 1 + 1 + 4, "agc": 24 + 3 * 8 + 1 + 1}
IO_REC_BYTES = {"age": 94, "ag": 62, "agc": 26}


def io_leg(ctx, d, reps, fmt="age"):
    """Snapshot writer and initial-condition loader (DataManager::saveData /
    loadICs) on the bench's particles: device encode and decode times (phase
    events on the context's stream), end-to-end rates through the C-ABI with a
    pinned host buffer and a file, and the numpy restatement timed on one core
    as the CPU baseline."""
    import tempfile

    import numpy as np
    import torch

    import snapio

    n = ctx.n
    size = ctx.snapshot_size(fmt)
    buf = torch.empty(size, dtype=torch.uint8).pin_memory().numpy()
    ctx.phase_timing(True)
    enc, cpy, wall = [], [], []
    for k in range(reps + 1):
        t0 = time.perf_counter()
        ln = ctx.snapshot_bytes(fmt, None, 1.0, 2.0, 3.0, out=buf)
        t1 = time.perf_counter()
        ph = dict(ctx.phase_times())
        if k:
            enc.append(ph["snapshot encode"])
            cpy.append(ph["snapshot copy"])
            wall.append(t1 - t0)
    assert ln == size
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "snap." + fmt)
        t0 = time.perf_counter()
        ctx.snapshot_write(path, fmt, None, 1.0, 2.0, 3.0, wait=False)
        t_queue = time.perf_counter() - t0
        ctx.snapshot_wait()
        t_write = time.perf_counter() - t0
        ic_copy, ic_dec, ic_wall = [], [], []
        for k in range(reps + 1):
            t0 = time.perf_counter()
            ctx.load_ics(path, fmt)
            t1 = time.perf_counter()
            ph = dict(ctx.phase_times())
            if k:
                ic_copy.append(ph["ic copy"])
                ic_dec.append(ph["ic decode"])
                ic_wall.append(t1 - t0)
    ctx.phase_timing(False)
    # the numpy restatement on a sample, one core
    ns = min(n, 1 << 20)
    p = {"pos": np.asarray(d["pos"][:ns]).reshape(-1, 3), "vel": np.asarray(d["vel"][:ns]).reshape(-1, 3),
         "mass": d["mass"][:ns], "T": np.zeros(ns), "P": np.zeros(ns), "vdens": np.zeros(ns), "U": d["U"][:ns],
         "sfr": np.zeros(ns), "type": d["type"][:ns].astype(np.uint8), "gp": np.ones(ns, np.uint8),
         "id": np.arange(ns, dtype=np.uint32)}
    t0 = time.perf_counter()
    img = snapio.encode(snapio.NAMES[fmt], p, ns, 1.0, 2.0, 3.0)
    t_cpu_enc = time.perf_counter() - t0
    t0 = time.perf_counter()
    snapio.decode(snapio.NAMES[fmt], img)
    t_cpu_dec = time.perf_counter() - t0
    med = lambda v: float(np.median(v))  # noqa: E731
    hbm = n * (IO_READ_BYTES[fmt] + IO_REC_BYTES[fmt] + 12) / (med(enc) * 1e-3) / 1e9
    return {
        "format": fmt, "particles": n, "file_bytes": size,
        "snapshot": {"encode_ms": med(enc), "copy_ms": med(cpy), "e2e_ms": med(wall) * 1e3,
                     "e2e_gbs": size / med(wall) / 1e9, "d2h_gbs": size / (med(cpy) * 1e-3) / 1e9,
                     "file_async_return_ms": t_queue * 1e3, "file_write_ms": t_write * 1e3,
                     "roofline": {"bound": "hbm", "achieved": hbm, "peak": HBM_PEAK_GBS, "unit": "GB/s",
                                  "frac": hbm / HBM_PEAK_GBS,
                                  "bytes_per_particle": IO_READ_BYTES[fmt] + IO_REC_BYTES[fmt] + 12,
                                  "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)"}},
        "load": {"h2d_ms": med(ic_copy), "decode_ms": med(ic_dec), "e2e_ms": med(ic_wall) * 1e3,
                 "e2e_gbs": size / med(ic_wall) / 1e9, "h2d_gbs": size / (med(ic_copy) * 1e-3) / 1e9},
        "cpu_baseline": {"unit": "GB/s", "encode": len(img) / t_cpu_enc / 1e9, "decode": len(img) / t_cpu_dec / 1e9,
                         "cores": 1, "kind": "port",
                         "sample": f"numpy restatement (oracle/snapio.py) on the first {ns} particles"},
    }


def our_arm(args, wl, d):
    import numpy as np
    import torch

    import ag2
    from dist import barrier, finalize, init, max_over_ranks

    D = init()
    torch.cuda.set_device(D.local_rank)
    n = len(d["mass"])
    mih = d.get("massInH", 0.0)
    ctx = ag2.Context(n, e0=wl["e0"], theta=wl["theta"], massInH=mih, precision=args.precision)
    # a stream of our own: the context's work, the L2 flush and the timing
    # events all go on it (a NULL handle would leave the context on its private
    # stream, which events on torch's default stream do not order against)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    ctx.upload(d["pos"], d["mass"], d["type"], vel=d["vel"], U=d["U"])
    if "first" in d:
        ctx.set_instances(d["first"])
    dt = wl["dt"]
    # initial forces as Simulation::init does (Simulation.cpp:120-139)
    ctx.build_tree()
    ctx.sph_density()
    ctx.forces()
    tuning = ctx.autotune_walk() if args.precision == "fp32" else None
    vis = os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",")[0]
    clk = ClockSampler(int(vis) if vis.isdigit() else D.local_rank)

    walk_ev = []

    def step(ev=None):
        ctx.kick_drift(dt)
        if ev is not None:
            ev[2].record(stream)
        ctx.build_tree()
        if ev is not None:
            ev[3].record(stream)
        ctx.sph_density()
        if ev is not None:
            ev[0].record(stream)
        ctx.forces()
        if ev is not None:
            ev[1].record(stream)
        ctx.ueuler(dt)
        ctx.kick(dt)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    barrier(D)
    clk.mark_start()
    with torch.cuda.stream(stream):
        flush = torch.empty(512 * 2 ** 20 // 4, dtype=torch.float32, device="cuda") if needs_flush(n) else None
    l0 = ctx.launches()
    inter_g = inter_s = 0
    step_ev = []
    torch.cuda.nvtx.range_push("timed")  # lets a profiler select the timed steps (--nvtx-include timed/)
    for _ in range(args.steps):
        if flush is not None:
            with torch.cuda.stream(stream):
                flush.fill_(1.0)
        se = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
        ev = tuple(torch.cuda.Event(enable_timing=True) for _ in range(4))  # walk start/end, build start/end
        se[0].record(stream)
        step(ev)
        se[1].record(stream)
        walk_ev.append(ev)
        step_ev.append(se)
        g, s = ctx.interactions()
        inter_g += g
        inter_s += s
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    clk.mark_stop()
    barrier(D)
    clocks = clk.stop()
    launches = ctx.launches() - l0
    t = sum(a.elapsed_time(b) for a, b in step_ev) / 1e3
    tmax = max_over_ranks(t, D)
    value = n * args.steps * D.world / tmax
    walk_ms = [e[0].elapsed_time(e[1]) for e in walk_ev]
    build_ms = [e[2].elapsed_time(e[3]) for e in walk_ev]
    _, n_internal, _ = ctx.node_count()
    # algorithmic build bytes per step, with the records this build writes:
    # N (32 read pos+mass + 12 write key+index) + N 24 (one sort pass) + N 2 x 153 (the particle state
    # read and written in tree order) + occupied nodes x (80 + 64 + 64 written: NodeSum, NodeMom and
    # WalkRec, + 80 read: the NodeSum its parent adds up); occupied nodes = internal nodes + at most N
    # non-empty leaves
    build_bytes = n * (32 + 12 + 24 + 2 * 153) + (n_internal + n) * (80 + 64 + 64 + 80)
    build_avg_s = sum(build_ms) / len(build_ms) / 1e3
    walk_avg_s = sum(walk_ms) / len(walk_ms) / 1e3
    flop_per_walk = (FLOP_GRAV * inter_g + FLOP_SPH * inter_s) / args.steps
    achieved = flop_per_walk / walk_avg_s / 1e12
    peak = ctx.fp32_peak_gflops() / 1e3

    # the same steps replayed from captured CUDA graphs (ag2_step_graphs)
    graph = None
    if args.graph_steps > 0:
        ctx.step_graphs(True)
        for _ in range(3):  # capture, then warm
            ctx.step(dt)
        torch.cuda.synchronize()
        gl0 = ctx.launches()
        gev = []
        for _ in range(args.graph_steps):
            if flush is not None:
                with torch.cuda.stream(stream):
                    flush.fill_(1.0)
            e = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
            e[0].record(stream)
            ctx.step(dt)
            e[1].record(stream)
            gev.append(e)
        torch.cuda.synchronize()
        tg = sum(a.elapsed_time(b) for a, b in gev) / 1e3
        graph = {"value": n * args.graph_steps * D.world / max_over_ranks(tg, D), "unit": UNIT,
                 "steps": args.graph_steps, "ms_per_step": tg / args.graph_steps * 1e3,
                 "gpu_launches": ctx.launches() - gl0}
        ctx.step_graphs(False)

    # energy drift of the FP32 form over --drift-steps further steps (untimed)
    drift = None
    if args.drift_steps > 0 and 0.0 < wl["e0"] < 0.6:
        e_a = ctx.energy()
        for _ in range(args.drift_steps):
            step()
        e_b = ctx.energy()
        drift = {"steps": args.drift_steps, "dt": dt, "start": e_a, "end": e_b,
                 "relative": (e_b["total"] - e_a["total"]) / abs(e_a["total"]),
                 "potential_from": "FP64 tree walk of the pair force's potential -(G m/e0) atan(e0/r)"}

    # plain FP64 walk on the same workload (the reference's arithmetic on the GPU)
    plain = None
    if args.plain_steps > 0:
        ctx.set(precision="fp64")
        torch.cuda.synchronize()
        p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        for _ in range(args.plain_steps):
            step()
        p1.record(stream)
        torch.cuda.synchronize()
        plain = n * args.plain_steps / (p0.elapsed_time(p1) / 1e3)
        ctx.set(precision=args.precision)

    # force error of both walks against FP64 direct summation on sampled
    # gravity-only particles (gas particles also carry SPH forces)
    force_error = None
    if args.error_samples > 0:
        rng = np.random.default_rng(12345)
        cand = np.nonzero(d["type"] != 2)[0]
        ids = np.sort(rng.choice(cand, size=min(args.error_samples, cand.size), replace=False))
        ctx.build_tree()
        ctx.sph_density()
        ctx.forces()
        a32_all = ctx.download("acc")
        direct = ctx.direct_sum(ids)
        ctx.set(precision="fp64")
        ctx.forces()
        a64_all = ctx.download("acc")
        ctx.set(precision=args.precision)
        a32, a64 = a32_all[ids], a64_all[ids]
        nrm = np.maximum(np.linalg.norm(direct, axis=1), 1e-300)
        err32 = np.linalg.norm(a32 - direct, axis=1) / nrm
        err64 = np.linalg.norm(a64 - direct, axis=1) / nrm
        # precision-form error: FP32-offset walk against the FP64 walk, every particle
        ep = np.linalg.norm(a32_all - a64_all, axis=1) / np.maximum(np.linalg.norm(a64_all, axis=1), 1e-300)
        force_error = {"against": "FP64 direct summation (tree approximation + arithmetic)",
                       "samples": int(ids.size), "median": float(np.median(err32)),
                       "p99": float(np.quantile(err32, 0.99)), "p999": float(np.quantile(err32, 0.999)),
                       "fp64_walk_median": float(np.median(err64)), "fp64_walk_p99": float(np.quantile(err64, 0.99)),
                       "fp32_vs_fp64_walk_median": float(np.median(ep)),
                       "fp32_vs_fp64_walk_p999": float(np.quantile(ep, 0.999))}

    # the opening-angle sweep of the precision form: force errors of both walks
    # at the state above (the same tree and direct sum), then each angle timed
    theta_sweep = None
    thetas = [float(t) for t in args.thetas.split(",") if t] if args.thetas else []
    if thetas and force_error is not None:
        theta_sweep = []
        for th in thetas:
            row = {"theta": th}
            ctx.set(theta=th, precision="fp32")
            ctx.forces()
            s32 = ctx.download("acc")
            g32, sph32 = ctx.interactions()
            ctx.set(precision="fp64")
            ctx.forces()
            s64 = ctx.download("acc")
            nrm = np.maximum(np.linalg.norm(direct, axis=1), 1e-300)
            e32 = np.linalg.norm(s32[ids] - direct, axis=1) / nrm
            e64 = np.linalg.norm(s64[ids] - direct, axis=1) / nrm
            ep = np.linalg.norm(s32 - s64, axis=1) / np.maximum(np.linalg.norm(s64, axis=1), 1e-300)
            row["force_error"] = {"samples": int(ids.size), "median": float(np.median(e32)),
                                  "p99": float(np.quantile(e32, 0.99)), "fp64_walk_median": float(np.median(e64)),
                                  "fp64_walk_p99": float(np.quantile(e64, 0.99)),
                                  "fp32_vs_fp64_walk_median": float(np.median(ep)),
                                  "fp32_vs_fp64_walk_p999": float(np.quantile(ep, 0.999))}
            row["interactions_per_step"] = {"gravity": g32, "sph": sph32}
            theta_sweep.append(row)
        for row in theta_sweep:
            th = row["theta"]
            ctx.set(theta=th, precision=args.precision)
            for _ in range(2):
                step()
            q0, q1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            q0.record(stream)
            for _ in range(args.sweep_steps):
                step()
            q1.record(stream)
            torch.cuda.synchronize()
            t32 = q0.elapsed_time(q1) / 1e3 / args.sweep_steps
            ctx.set(precision="fp64")
            q0.record(stream)
            for _ in range(args.plain_steps):
                step()
            q1.record(stream)
            torch.cuda.synchronize()
            t64 = q0.elapsed_time(q1) / 1e3 / max(1, args.plain_steps)
            row.update({"value": n / t32, "ms_per_step": t32 * 1e3, "steps": args.sweep_steps,
                        "plain_fp64": n / t64, "plain_ms_per_step": t64 * 1e3, "speedup_vs_plain": t64 / t32})
        ctx.set(theta=wl["theta"], precision=args.precision)

    # end to end through the C-ABI with pinned host buffers
    e2e = None
    if args.e2e_steps > 0:
        pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()  # noqa: E731
        hpos, hvel, hmass = pin(ctx.download("pos")), pin(ctx.download("vel")), pin(d["mass"])
        hU, htype, hacc = pin(ctx.download("U")), pin(d["type"]), pin(ctx.download("acc"))
        outs = {"pos": hpos, "vel": hvel, "acc": hacc, "U": hU}
        for _ in range(3):  # warm-up: the first call makes the acceleration staging and the copy stream
            ctx.step_host(dt, hpos, hmass, htype, vel=hvel, U=hU, acc=hacc, out=outs, first=d.get("first"))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):  # one call: upload, step, read-back (positions during the walk)
            ctx.step_host(dt, hpos, hmass, htype, vel=hvel, U=hU, acc=hacc, out=outs, first=d.get("first"))
        te = time.perf_counter() - t0
        te = max_over_ranks(te, D)
        e2e = {"value": n * args.e2e_steps * D.world / te, "unit": UNIT,
               "h2d_bytes_per_step": int(n * (24 + 24 + 8 + 8 + 1 + 24)),
               "d2h_bytes_per_step": int(n * (24 + 24 + 24 + 8))}

    io = io_leg(ctx, d, args.io_reps) if args.io_reps > 0 and D.rank == 0 else None

    # independent simulations: each one stepped on its own (its own context and
    # launches), with the plain FP64 walk and with the FP32 walk
    per_launch = None
    if "first" in d and args.plain_steps > 0:
        ctx.close()
        per_launch = one_sim_per_launch(d, wl, args.plain_steps, stream)

    cpu = None
    if D.rank == 0 and D.world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        if "first" in d:
            tcpu, _, sample = cpu_step_time_instances(d, wl, args.cpu_walk_fraction, threads)
        else:
            tcpu, _, sample = cpu_step_time(d, wl, args.cpu_walk_fraction, threads)
        cpu = {"value": n / tcpu, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample}

    # DRAM bytes of one build (every build kernel of one step), likewise
    btraffic, btraffic_src = None, None
    bpath = os.path.join(REPO, "profiles", "build_traffic.json")
    if os.path.exists(bpath):
        try:
            import hashlib

            bj = json.load(open(bpath))
            btraffic = bj.get(args.workload)
            cur = hashlib.sha256(open(os.path.join(REPO, "astrogenesis2.0_gb300", "csrc", "ag2_build.cu"),
                                      "rb").read()).hexdigest()[:16]
            btraffic_src = {"file": "profiles/build_traffic.json", "build_source_sha": bj.get("build_source_sha"),
                            "current_build_source_sha": cur, "current": bj.get("build_source_sha") == cur}
        except (OSError, ValueError):
            btraffic = None
    # DRAM bytes of one walk launch, from the committed ncu summary; it states
    # the walk source it was measured on, so a changed kernel shows as stale
    traffic, traffic_src = None, None
    tpath = os.path.join(REPO, "profiles", "walk_traffic.json")
    if os.path.exists(tpath):
        try:
            import hashlib

            tj = json.load(open(tpath))
            traffic = tj.get(args.workload, {}).get(args.precision)
            cur = hashlib.sha256(open(os.path.join(REPO, "astrogenesis2.0_gb300", "csrc", "ag2_walk.cu"),
                                      "rb").read()).hexdigest()[:16]
            traffic_src = {"file": "profiles/walk_traffic.json", "walk_source_sha": tj.get("walk_source_sha"),
                           "current_walk_source_sha": cur, "current": tj.get("walk_source_sha") == cur}
        except (OSError, ValueError):
            traffic = None

    if D.rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": D.world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": tmax / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32" if args.precision == "fp32" else "f64",
            "data": "synthetic", "config": config_block(args, wl, d), "method": our_method(args), "e2e": e2e,
            "gpu_launches": launches, "clocks": clocks,
            "walk_tuning": tuning,
            "roofline": {"bound": "fp32", "kernel": "k_walk32" if args.precision == "fp32" else "k_walk64",
                         "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                         "traffic": traffic, "traffic_source": traffic_src,
                         "peak_source": "measured FP32 FMA throughput (ag2_fp32_peak_probe, "
                                                            "this run)", "walk_ms": walk_avg_s * 1e3,
                         "flop_per_launch": flop_per_walk},
            "roofline_build": {"bound": "hbm", "kernel": "octree build (every build kernel, one step)",
                               "achieved": build_bytes / build_avg_s / 1e9, "peak": HBM_PEAK_GBS, "unit": "GB/s",
                               "frac": build_bytes / build_avg_s / 1e9 / HBM_PEAK_GBS, "traffic": btraffic,
                               "traffic_over_algorithmic": btraffic / build_bytes if btraffic else None,
                               "dram_achieved": btraffic / build_avg_s / 1e9 if btraffic else None,
                               "dram_frac": btraffic / build_avg_s / 1e9 / HBM_PEAK_GBS if btraffic else None,
                               "traffic_source": btraffic_src,
                               "bytes_per_build": build_bytes, "build_ms": build_avg_s * 1e3,
                               "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)"},
            "cpu_baseline": cpu,
            "interactions_per_s": (inter_g + inter_s) / args.steps / walk_avg_s,
            "interactions_per_step": {"gravity": inter_g / args.steps, "sph": inter_s / args.steps},
            "plain_fp64": {"value": plain, "unit": UNIT, "steps": args.plain_steps} if plain else None,
            "speedup_vs_plain": value / plain if plain else None,
            "force_error": force_error,
            "accuracy_bar": ACCURACY_NOTE,
            "theta_sweep": theta_sweep,
            "energy_drift": drift,
            "step_graph": graph,
            "io": io,
        }
        if per_launch:
            out["one_sim_per_launch"] = per_launch
            out["speedup_vs_plain_per_launch"] = value / per_launch["fp64"]["value"]
    else:
        out = None
    ctx.close()
    return out, D


ACCURACY_NOTE = ("The <= 1e-4 median force-error bar applies to the FP32-offset walk against the FP64 walk at the same "
                 "opening angle (force_error.fp32_vs_fp64_walk_median). Against FP64 direct summation both walks "
                 "carry the reference's monopole-tree error at that angle (force_error.median / fp64_walk_median; "
                 "per angle in theta_sweep).")

SERVE_BUDGET_BYTES = 150e9
SERVE_BYTES_PER_PARTICLE = 2 * BYTES_PER_PARTICLE  # the step context and the initial-force context


def _serve_trace(specs, arrivals):
    import serving

    return [serving.Request(rid=k, pos=q["pos"], vel=q["vel"], mass=q["mass"], type=q["type"], U=q["U"],
                            steps=q["steps"], massInH=q["massInH"], arrival=float(arrivals[k]))
            for k, q in enumerate(specs)]


def _fcfs(arrivals, service):
    """Completion latencies of one server taking requests in arrival order."""
    t_free, lat, end = 0.0, [], 0.0
    for a, s_ in sorted(zip(arrivals, service)):
        start = max(a, t_free)
        t_free = start + s_
        lat.append(t_free - a)
        end = t_free
    return lat, end


def _serve_rate(eng, specs, rate, seed):
    """One real-time pass of the request trace at `rate` requests/s."""
    import numpy as np

    import serving

    arr = ics.poisson_arrivals(len(specs), rate, seed=seed)
    trace = _serve_trace(specs, arr)
    ps0, st0 = eng.particle_steps, eng.steps_done
    t0 = time.perf_counter()
    res = serving.serve(eng, trace, realtime=True)
    span = time.perf_counter() - t0
    lat = np.array([r.completed - r.arrival for r in res])
    wait = np.array([r.admitted - r.arrival for r in res])
    return {"rate_per_s": rate, "requests": len(res), "p50_latency_s": float(np.quantile(lat, 0.5)),
            "p99_latency_s": float(np.quantile(lat, 0.99)), "max_latency_s": float(lat.max()),
            "p99_admission_wait_s": float(np.quantile(wait, 0.99)), "makespan_s": span,
            "particle_steps_per_s": (eng.particle_steps - ps0) / span, "engine_steps": eng.steps_done - st0}


def serving_leg(args, wl):
    """Continuous batching of a Poisson request stream (config: serving), and
    the same requests served one at a time on the plain FP64 path."""
    import numpy as np
    import torch

    import ag2
    import serving

    specs = ics.serving_requests(args.serve_requests)
    sizes = np.array([len(q["mass"]) for q in specs])
    steps = np.array([q["steps"] for q in specs])
    budget_particles = int(SERVE_BUDGET_BYTES // SERVE_BYTES_PER_PARTICLE)
    cap = int(min(budget_particles, sizes.sum()))
    stream = torch.cuda.Stream()
    eng = serving.Engine(cap, e0=wl["e0"], theta=wl["theta"], dt=wl["dt"], stream=stream)
    warm = _serve_trace(specs[:2], [0.0, 0.0])  # warm-up: two short simulations through the whole loop
    for q in warm:
        q.steps = 3
    serving.serve(eng, warm, realtime=False)
    l0 = eng.ctx.launches() + eng.init_ctx.launches()
    rates = [float(r) for r in args.serve_rates.split(",")]
    per_rate = [_serve_rate(eng, specs, rate, 8 + int(rate)) for rate in rates]
    launches = eng.ctx.launches() + eng.init_ctx.launches() - l0
    eng.close()

    # the same trace at the highest rate under a budget that binds: requests
    # wait for resident ones to finish before they are admitted
    bound = None
    if args.serve_small_budget_gb > 0:
        small = int(max(args.serve_small_budget_gb * 1e9 // SERVE_BYTES_PER_PARTICLE, sizes.max()))
        eng = serving.Engine(small, e0=wl["e0"], theta=wl["theta"], dt=wl["dt"], stream=stream)
        serving.serve(eng, _serve_trace(specs[:1], [0.0]), realtime=False)
        bound = _serve_rate(eng, specs, max(rates), 8 + int(max(rates)))
        bound.update({"budget_gb": args.serve_small_budget_gb, "capacity_particles": small,
                      "offered_particles": int(sizes.sum())})
        eng.close()

    # each request alone on the plain FP64 path, measured request by request:
    # its initial forces (wall clock) and 2 steps after a warm-up step (CUDA
    # events); its service time is the initial forces plus its step count
    # times the measured step
    service, per_step = [], []
    for q in specs:
        c = ag2.Context(len(q["mass"]), e0=wl["e0"], theta=wl["theta"], massInH=q["massInH"], precision="fp64")
        c.set_stream(stream.cuda_stream)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        c.upload(q["pos"], q["mass"], q["type"], vel=q["vel"], U=q["U"])
        c.build_tree()
        c.sph_density()
        c.forces()
        torch.cuda.synchronize()
        t_init = time.perf_counter() - t0
        c.step(wl["dt"])
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(2):
            c.step(wl["dt"])
        e1.record(stream)
        torch.cuda.synchronize()
        per = e0.elapsed_time(e1) / 2 / 1e3
        per_step.append(per)
        service.append(t_init + q["steps"] * per)
        c.close()
    plain = []
    for rate in rates:
        arr = ics.poisson_arrivals(len(specs), rate, seed=8 + int(rate))
        lat, end = _fcfs(arr, service)
        plain.append({"rate_per_s": rate, "p50_latency_s": float(np.quantile(lat, 0.5)),
                      "p99_latency_s": float(np.quantile(lat, 0.99)),
                      "particle_steps_per_s": float((sizes * steps).sum() / end)})
    top = per_rate[-1]
    return {
        "workload": f"serving: {wl['desc']}", "requests": len(specs), "particles": int(sizes.sum()),
        "particle_steps": int((sizes * steps).sum()),
        "gas_requests": int(sum((q["type"] == 2).any() for q in specs)), "theta": wl["theta"], "eps": wl["e0"],
        "dt": wl["dt"], "capacity_particles": cap, "budget_particles": budget_particles,
        "rates": per_rate, "budget_bound": bound, "gpu_launches": launches,
        "plain_alone": {"how": "each request alone in its own context on the FP64 path, one at a time in arrival "
                               "order: initial forces and 2 steps measured per request, service time = initial + "
                               "steps x measured step", "requests_measured": len(specs),
                        "median_step_ms": float(np.median(per_step) * 1e3), "rates": plain},
        "speedup_vs_plain_alone": top["particle_steps_per_s"] / plain[-1]["particle_steps_per_s"],
        "p99_speedup_vs_plain_alone": plain[-1]["p99_latency_s"] / top["p99_latency_s"],
    }


def serving_arm(args, wl):
    """--workload serving: the serving leg as its own line (value = the
    aggregate particle-steps/s at the highest arrival rate)."""
    import torch

    from dist import finalize, init

    D = init()
    torch.cuda.set_device(D.local_rank)
    vis = os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",")[0]
    clk = ClockSampler(int(vis) if vis.isdigit() else D.local_rank)
    time.sleep(0.5)
    clk.mark_start()
    sv = serving_leg(args, wl)
    clk.mark_stop()
    clocks = clk.stop()
    top = sv["rates"][-1]
    specs_bytes = sv["particles"]
    if D.rank == 0:
        out = {
            "metric": METRIC, "value": top["particle_steps_per_s"], "unit": UNIT, "n_gpus": D.world,
            "steps": int(top["engine_steps"]), "warmup": 1,
            "ms_per_step": top["makespan_s"] / top["engine_steps"] * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": sv["workload"], "requests": sv["requests"], "particles": sv["particles"],
                       "theta": wl["theta"], "eps": wl["e0"], "dt": wl["dt"], "parallelism": "replicas",
                       "l2": "resident state far above the 129 MB L2 at the higher rates; no flush"},
            "e2e": {"value": top["particle_steps_per_s"], "unit": UNIT,
                    "h2d_bytes_per_step": specs_bytes * 65 / max(1, top["engine_steps"]),
                    "d2h_bytes_per_step": specs_bytes * 88 / max(1, top["engine_steps"]),
                    "note": "requests arrive as host arrays and results return to the host; latencies are wall clock"},
            "gpu_launches": sv["gpu_launches"], "clocks": clocks, "roofline": None, "serving": sv,
        }
        print(json.dumps(out), flush=True)
    finalize(D)


def ensemble_leg(args):
    """The batched form: 512 independent Plummer spheres in one context (one
    build and one walk launch per step over all of them), against the same
    simulations stepped one per launch with the plain FP64 walk and the FP32
    walk."""
    import numpy as np
    import torch

    import ag2

    wl = WORKLOADS["ensemble512"]
    d = wl["make"]()
    n = len(d["mass"])
    dt = wl["dt"]
    stream = torch.cuda.Stream()
    ctx = ag2.Context(n, e0=wl["e0"], theta=wl["theta"], precision="fp32")
    ctx.set_stream(stream.cuda_stream)
    ctx.upload(d["pos"], d["mass"], d["type"], vel=d["vel"], U=d["U"])
    ctx.set_instances(d["first"])
    ctx.build_tree()
    ctx.forces()
    tune = ctx.autotune_walk()
    for _ in range(3):
        ctx.step(dt)
    torch.cuda.synchronize()
    l0 = ctx.launches()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.ens_steps):
        ctx.step(dt)
    e1.record(stream)
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 1e3 / args.ens_steps
    launches = (ctx.launches() - l0) / args.ens_steps
    ctx.step_graphs(True)
    for _ in range(3):
        ctx.step(dt)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.ens_steps):
        ctx.step(dt)
    e1.record(stream)
    torch.cuda.synchronize()
    tg = e0.elapsed_time(e1) / 1e3 / args.ens_steps
    ctx.step_graphs(False)
    # accuracy of both walks against FP64 direct summation, same state
    rng = np.random.default_rng(4096)
    ids = np.sort(rng.choice(n, size=min(4096, n), replace=False))
    ctx.build_tree()
    ctx.forces()
    a32 = ctx.download("acc")
    direct = ctx.direct_sum(ids)
    ctx.set(precision="fp64")
    ctx.forces()
    a64 = ctx.download("acc")
    ctx.set(precision="fp32")
    nrm = np.maximum(np.linalg.norm(direct, axis=1), 1e-300)
    e32 = np.linalg.norm(a32[ids] - direct, axis=1) / nrm
    e64 = np.linalg.norm(a64[ids] - direct, axis=1) / nrm
    ep = np.linalg.norm(a32 - a64, axis=1) / np.maximum(np.linalg.norm(a64, axis=1), 1e-300)
    # end to end through the C-ABI with pinned host buffers and the instance layout
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()  # noqa: E731
    hpos, hvel, hmass, hU, htype, hacc = (pin(ctx.download("pos")), pin(ctx.download("vel")), pin(d["mass"]),
                                          pin(ctx.download("U")), pin(d["type"]), pin(a32))
    outs = {"pos": hpos, "vel": hvel, "acc": hacc, "U": hU}
    for _ in range(3):  # warm-up
        ctx.step_host(dt, hpos, hmass, htype, vel=hvel, U=hU, acc=hacc, out=outs, first=d["first"])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        ctx.step_host(dt, hpos, hmass, htype, vel=hvel, U=hU, acc=hacc, out=outs, first=d["first"])
    te = (time.perf_counter() - t0) / args.e2e_steps
    ctx.close()
    per_launch = one_sim_per_launch(d, wl, args.plain_steps, stream)
    value = n / t
    return {
        "workload": f"ensemble512: {wl['desc']}", "particles": n, "instances": int(len(d["first"]) - 1),
        "theta": wl["theta"], "eps": wl["e0"], "dt": dt, "value": value, "unit": UNIT, "ms_per_step": t * 1e3,
        "steps": args.ens_steps, "gpu_launches_per_step": launches, "walk_tuning": tune,
        "step_graph": {"value": n / tg, "ms_per_step": tg * 1e3},
        "e2e": {"value": n / te, "unit": UNIT, "h2d_bytes_per_step": int(n * 89), "d2h_bytes_per_step": int(n * 80)},
        "one_sim_per_launch": per_launch,
        "speedup_vs_plain_per_launch": value / per_launch["fp64"]["value"],
        "speedup_vs_fp32_per_launch": value / per_launch["fp32"]["value"],
        "force_error": {"against": "FP64 direct summation within each simulation", "samples": int(ids.size),
                        "median": float(np.median(e32)), "p99": float(np.quantile(e32, 0.99)),
                        "fp64_walk_median": float(np.median(e64)),
                        "fp32_vs_fp64_walk_median": float(np.median(ep)),
                        "fp32_vs_fp64_walk_p999": float(np.quantile(ep, 0.999))},
    }


def serving_reference_arm(args, wl):
    """The reference's CPU algorithm serving the same requests one at a time."""
    import numpy as np

    import oracle
    from dist import finalize, init

    D = init(backend="gloo")
    if D.rank != 0:
        finalize(D)
        return
    specs = ics.serving_requests(args.serve_requests)
    threads = os.cpu_count() or 1
    ks = list(range(0, len(specs), 8))
    per_step = []
    for k in ks:
        q = specs[k]
        w = oracle.World(q["pos"], q["mass"], q["type"], q["vel"], q["U"], kind="port")
        t0 = time.perf_counter()
        w.kick(wl["dt"])
        w.drift(wl["dt"])
        w.build(threads)
        if (q["type"] == 2).any():
            w.gas_density(q["massInH"])
        w.forces(wl["e0"], wl["theta"], threads)
        w.kick(wl["dt"])
        per_step.append(time.perf_counter() - t0)
    sizes = np.array([len(q["mass"]) for q in specs])
    steps = np.array([q["steps"] for q in specs])
    rate_ps = float(sizes[ks].sum() / np.sum(per_step))
    out = {"metric": METRIC, "value": rate_ps, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
           "steps": 1, "warmup": 0, "ms_per_step": float(np.mean(per_step) * 1e3), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": f"serving: {wl['desc']}", "requests": len(specs), "particles": int(sizes.sum()),
                      "total_particle_steps": int((sizes * steps).sum())},
           "cpu_baseline": {"value": rate_ps, "unit": UNIT, "cores": threads, "kind": "port",
                            "sample": f"one step of every 8th request ({len(ks)} requests), each alone"},
           "e2e": {"value": rate_ps, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)
    finalize(D)


def one_sim_per_launch(d, wl, steps, stream):
    """Throughput of the same instances stepped one simulation at a time."""
    import torch

    import ag2

    first = d["first"]
    ctxs = []
    for k in range(len(first) - 1):
        a, b = int(first[k]), int(first[k + 1])
        c = ag2.Context(b - a, e0=wl["e0"], theta=wl["theta"])
        c.set_stream(stream.cuda_stream)
        c.upload(d["pos"][a:b], d["mass"][a:b], d["type"][a:b], vel=d["vel"][a:b], U=d["U"][a:b])
        c.build_tree()
        c.forces()
        ctxs.append(c)
    n = int(first[-1])
    res = {}
    for prec in ("fp64", "fp32"):
        for c in ctxs:
            c.set(precision=prec)
            c.step(wl["dt"])  # warm-up
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            for c in ctxs:
                c.step(wl["dt"])
        e1.record(stream)
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) / 1e3
        res[prec] = {"value": n * steps / t, "unit": UNIT, "steps": steps,
                     "ms_per_step": t / steps * 1e3}
    for c in ctxs:
        c.close()
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="merger4m", choices=sorted(WORKLOADS))
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--plain-steps", type=int, default=2)
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--error-samples", type=int, default=65536)
    ap.add_argument("--cpu-walk-fraction", type=int, default=1)
    ap.add_argument("--ref-walk-fraction", type=int, default=1)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--drift-steps", type=int, default=1000)
    ap.add_argument("--graph-steps", type=int, default=10)
    ap.add_argument("--io-reps", type=int, default=3)
    ap.add_argument("--serve-requests", type=int, default=200)
    ap.add_argument("--serve-rates", default="10,50,200")
    ap.add_argument("--serve-small-budget-gb", type=float, default=8.0,
                    help="budget of the extra serving pass at the highest rate where admission waits (0: skip)")
    ap.add_argument("--thetas", default="0.4,0.5,0.7", help="opening angles of the precision-form sweep")
    ap.add_argument("--sweep-steps", type=int, default=5)
    ap.add_argument("--ens-steps", type=int, default=10)
    ap.add_argument("--no-extra", action="store_true",
                    help="the merger line without the ensemble and serving summaries")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    wl = WORKLOADS[args.workload]
    if args.workload == "serving":
        if args.impl == "reference":
            serving_reference_arm(args, wl)
        else:
            serving_arm(args, wl)
        return
    d = wl["make"]()
    if args.impl == "reference":
        reference_arm(args, wl, d)
        return
    out, D = our_arm(args, wl, d)
    del d
    # the metric's other two parts, on one GPU: the batched ensemble and serving
    if args.workload == "merger4m" and not args.no_extra and D.world == 1:
        out["ensemble512"] = ensemble_leg(args)
        out["serving"] = serving_leg(args, WORKLOADS["serving"])
    if out is not None:
        print(json.dumps(out), flush=True)
    from dist import finalize

    finalize(D)


if __name__ == "__main__":
    main()
