"""Benchmark: particle-steps/s of the Particle Life physics step at 1M, 2D.

Workload (the reference-units restatement of the 1M 2D configuration):
2D periodic unit box, N = 1,000,000 particles, 8 types assigned uniformly,
matrix uniform in [-1,1], positions uniform, velocities zero, rmax = 0.0025
(0.005 in a [-1,1]^2 box, ~19.6 neighbours), beta = 0.3, friction half-life
0.043 s (coefficient 0.7644018106552037), dt = 0.01, force 1.  Seeded
synthetic data (numpy Philox); FP32 state on the GPU.

Our arm (default):
  value  device-resident state; each step timed alone with CUDA events on the
         library's stream; L2 flushed (256 MB write) between steps.
  e2e    the public API with host buffers: per step plg_upload (pinned host
         double/int arrays) + plg_step_download (one step whose force kernel
         writes the snapshot to the host arrays), host wall clock; "unfused"
         beside it: plg_upload + plg_step + plg_download; "host_link": the
         link's DMA ceiling measured live and the calls' fractions of it.
  roofline of the dominant kernel (the force kernel), from per-kernel CUDA
         events over a profiled pass of the same steps.
  cpu_baseline  the oracle (C FP64 restatement of the reference's step, all
         host threads) on a bounded sample of steps of the same workload.
  cfg1_10k  the reference's default 10k world, 1,000 steps on the GPU and
         through the oracle on all host threads.
  blobs_3d  the 4M-particle 3D blob world (uneven cells), device-resident.
  batched  512 uneven 2D worlds through plg_batch_* (autotuned) against the
         same worlds one at a time through single-world contexts.
  serving  the served configuration through plg_server_* (Poisson arrivals
         over a bounded window, see run_serving): completed and unfinished
         requests, completion latency p50/p99, delivered throughput and
         device-busy fraction, against the same requests one at a time.
--impl reference: the same workload through the oracle port on all host
cores (the reference is Java and no JDK exists on either machine).

Multi-GPU: replicas only (one world per rank, no collective on the data path);
value = units of all ranks / max over ranks of the timed region.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO / "particle-life-app_gb300"))
sys.path.insert(0, str(REPO / "oracle"))

METRIC = "particle-steps/s at 1M 2D"
UNIT = "particle-steps/s"
FRICTION = 0.5 ** (1.0 / (60.0 * 0.043))

# Algorithmic work per unit, as include/plg_work.h fixes it (FMA = 2 flops;
# compare and rsqrt = 1; bytes by design, 2D layout).
WORK = {m.group(1): int(m.group(2)) for m in
        re.finditer(r"^#define (PLG_WORK_\w+) (\d+)", (REPO / "include" / "plg_work.h").read_text(), re.M)}
FLOPS_PER_CANDIDATE = {2: WORK["PLG_WORK_FLOPS_CANDIDATE_2D"], 3: WORK["PLG_WORK_FLOPS_CANDIDATE_3D"]}
FLOPS_PER_INTERACTION = {2: WORK["PLG_WORK_FLOPS_INTERACTION_2D"], 3: WORK["PLG_WORK_FLOPS_INTERACTION_3D"]}
BYTES = {"scatter": WORK["PLG_WORK_SCATTER_BYTES"], "gather": WORK["PLG_WORK_GATHER_BYTES_2D"],
         "force": WORK["PLG_WORK_FORCE_BYTES_2D"], "scan_cell": WORK["PLG_WORK_SCAN_BYTES_PER_CELL"]}


class Replicas:
    """The replicas path of a multi-GPU run: one process per GPU, each
    stepping its own world; no collective on the data path.  Reads
    RANK / WORLD_SIZE / LOCAL_RANK from the environment (torchrun); with more
    than one rank it joins a process group (`backend`: nccl on GPUs, gloo for
    the CPU tests).  The timed region's duration is the maximum over ranks and
    a whole-job rate is all ranks' units over that time; only rank 0 prints."""

    def __init__(self, backend: str = "nccl"):
        self.rank = int(os.environ.get("RANK", "0"))
        self.world_size = int(os.environ.get("WORLD_SIZE", "1"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.dist = None
        if self.world_size > 1:
            import torch.distributed as dist

            dist.init_process_group(backend)
            self.dist = dist

    @property
    def leader(self) -> bool:
        return self.rank == 0

    def barrier(self) -> None:
        if self.dist is not None:
            self.dist.barrier()

    def max_over_ranks(self, x: float, device=None) -> float:
        if self.dist is None:
            return float(x)
        import torch

        t = torch.tensor([float(x)], dtype=torch.float64, device=device)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def rate(self, units_per_rank: float, seconds: float, device=None) -> float:
        """Whole-job rate: units of all ranks / the slowest rank's time."""
        return self.world_size * units_per_rank / self.max_over_ranks(seconds, device)

    def close(self) -> None:
        if self.dist is not None:
            self.dist.destroy_process_group()
            self.dist = None


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=1_000_000)
    ap.add_argument("--e2e-steps", type=int, default=30)
    ap.add_argument("--cpu-sample-s", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-flush", action="store_true", help="keep L2 warm between steps (not a headline number)")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-worlds measurement")
    ap.add_argument("--batched-worlds", type=int, default=512)
    ap.add_argument("--batched-steps", type=int, default=500, help="steps of the batched configuration")
    ap.add_argument("--no-cfg1", action="store_true", help="skip the 10k-particle configuration")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving measurement")
    ap.add_argument("--no-3d", action="store_true", help="skip the 3D blob measurement")
    ap.add_argument("--steps-3d", type=int, default=20)
    ap.add_argument("--serve-seconds", type=float, default=60.0, help="arrival window of the serving run")
    ap.add_argument("--serve-drain-s", type=float, default=60.0, help="longest drain after the arrival window")
    ap.add_argument("--serve-rate", type=float, default=200.0)
    ap.add_argument("--serve-alone-s", type=float, default=10.0,
                    help="seconds of one-at-a-time stepping for the serving comparison")
    ap.add_argument("--serve-cap-2d", type=float, default=48e6, help="2D batch capacity (particles)")
    ap.add_argument("--serve-cap-3d", type=float, default=24e6, help="3D batch capacity (particles)")
    ap.add_argument("--serve-cells-2d", type=float, default=24e6)
    ap.add_argument("--serve-cells-3d", type=float, default=24e6)
    return ap.parse_args(argv)


def make_world(n: int, seed: int = 2024):
    rng = np.random.Generator(np.random.Philox(seed))
    pos = np.zeros((n, 3))
    pos[:, :2] = rng.random((n, 2), dtype=np.float32)
    vel = np.zeros((n, 3))
    types = rng.integers(0, 8, n).astype(np.int32)
    m = np.asarray(2 * rng.random((8, 8)) - 1, np.float32).astype(np.float64)
    return pos, vel, types, m


SETTINGS = dict(rmax=0.0025, friction=FRICTION, force=1.0, dt=0.01, beta=0.3, wrap=True)


class Clocks:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        rows = [r.split(",") for r in Path(self.path).read_text().strip().splitlines() if r.strip()]
        os.unlink(self.path)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
            except ValueError:
                continue
            for nm, v in zip(names, r[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_oracle_rate(n, threads, budget_s, steps_cap=None):
    """Times the oracle (C FP64 restatement) on the workload: particle-steps/s."""
    import orc

    orc.build()
    pos, vel, types, m = make_world(n)
    w = orc.World(2, pos, vel, types, np.arange(n, dtype=np.int32), m,
                  orc.settings(SETTINGS["rmax"], SETTINGS["friction"], SETTINGS["force"], SETTINGS["dt"],
                               SETTINGS["beta"], SETTINGS["wrap"]))
    w.run(1, threads)  # warm-up
    t2 = w.run(2, threads) / 2  # estimate
    steps = max(1, int(budget_s / max(t2, 1e-6)))
    if steps_cap:
        steps = min(steps, steps_cap)
    t = w.run(steps, threads)
    return n * steps / t, steps, t


CFG1 = dict(n=10_000, ntypes=6, steps=1000, seed=2023,
            settings=dict(rmax=0.02, friction=FRICTION, force=1.0, dt=0.02, beta=0.3, wrap=True))


def cfg1_world():
    """The reference's own default world (Physics.setParticleCount(10000),
    backend/Physics.java:79): 2D periodic, N = 10,000, 6 types uniform,
    matrix uniform in [-1,1], positions uniform, velocities zero, rmax 0.02
    (0.04 in [-1,1]^2), friction half-life 0.043 s, dt 0.02."""
    rng = np.random.Generator(np.random.Philox(CFG1["seed"]))
    n, t = CFG1["n"], CFG1["ntypes"]
    pos = np.zeros((n, 3))
    pos[:, :2] = rng.random((n, 2), dtype=np.float32)
    types = rng.integers(0, t, n).astype(np.int32)
    m = np.asarray(2 * rng.random((t, t)) - 1, np.float32).astype(np.float64)
    return pos, np.zeros((n, 3)), types, m


def cpu_cfg1(threads: int) -> dict:
    """The 10k configuration's 1,000 steps through the oracle on `threads`
    host threads (C FP64 restatement of Physics.update())."""
    import orc

    orc.build()
    pos, vel, types, m = cfg1_world()
    n = CFG1["n"]
    S = CFG1["settings"]
    w = orc.World(2, pos, vel, types, np.arange(n, dtype=np.int32), m,
                  orc.settings(S["rmax"], S["friction"], S["force"], S["dt"], S["beta"], S["wrap"]))
    w.run(5, threads)
    t = w.run(CFG1["steps"], threads)
    return {"value": n * CFG1["steps"] / t, "unit": UNIT, "ms_per_step": 1e3 * t / CFG1["steps"],
            "steps": CFG1["steps"], "cores": threads, "kind": "port"}


def run_cfg1(args) -> dict:
    """The 10k configuration on the GPU: 1,000 steps enqueued at once
    (plg_step_async), timed with CUDA events on the library's stream."""
    import torch

    from plgpu import _lib
    from plgpu.physics import GpuWorld, check

    pos, vel, types, m = cfg1_world()
    n = CFG1["n"]
    w = GpuWorld(2, n)
    w.set_settings(**CFG1["settings"])
    w.set_matrix(m)
    w.upload(pos, vel, types)
    w.step(args.warmup)
    tile, tile_ms = w.autotune(5)  # untimed; the world is restored
    lib = _lib.load()
    stream = torch.cuda.ExternalStream(w.stream())
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record(stream)
    check(lib.plg_step_async(w.ctx, CFG1["steps"]), w.ctx, "plg_step_async")
    b.record(stream)
    check(lib.plg_sync(w.ctx, 60.0), w.ctx, "plg_sync")
    ms = a.elapsed_time(b)
    w.close()
    return {"metric": "particle-steps/s, 10k 2D (the reference's default world)", "value": n * CFG1["steps"] / (ms * 1e-3),
            "unit": UNIT, "ms_per_step": ms / CFG1["steps"], "steps": CFG1["steps"],
            "autotune": {"chosen_tile_variant": tile, "ms_per_step_by_variant": tile_ms},
            "config": "2D periodic unit box, N=10,000, 6 types, rmax=0.02 (0.04 in [-1,1]^2), friction t1/2=0.043 s, "
                      "dt=0.02, 1,000 steps (one CUDA graph launch per step); seeded Philox"}


def run_batched(args) -> dict:
    """The batched configuration: 512 2D worlds of uneven size advanced by one
    step launch (plg_batch_*), against the same worlds stepped one at a time
    through single-world contexts (plg_step)."""
    import torch

    from plgpu import workloads
    from plgpu.batch import GpuBatch
    from plgpu.physics import GpuWorld

    worlds = workloads.batched_worlds(args.batched_worlds)
    ntot = sum(w.pos.shape[0] for w in worlds)
    ctot = sum(workloads.cells_of(w, 2) for w in worlds)
    b = GpuBatch(2, ntot, len(worlds), ctot)
    b.update(add=worlds)
    stream = torch.cuda.ExternalStream(b.stream())
    b.step(args.warmup)
    choice, tune_ms = b.autotune_worlds(2)  # per world; state restored
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.batched_steps)]
    torch.cuda.synchronize()
    for k in range(args.batched_steps):
        ev[k][0].record(stream)
        b.step_async(1)
        ev[k][1].record(stream)
    b.sync()
    step_ms = np.array([a.elapsed_time(c) for a, c in ev])
    batched = ntot * args.batched_steps / (step_ms.sum() * 1e-3)
    b.close()

    # one at a time: every world in its own context, stepped in turn
    total_s = 0.0
    for w in worlds:
        g = GpuWorld(2, w.pos.shape[0])
        g.set_settings(w.rmax, w.friction, w.force, w.dt, beta=w.beta, wrap=w.wrap)
        g.set_matrix(w.matrix)
        g.upload(w.pos, w.vel, w.types)
        g.step(2)
        t0 = time.perf_counter()
        g.step(args.batched_steps)
        total_s += time.perf_counter() - t0
        g.close()
    single = ntot * args.batched_steps / total_s
    return {"metric": "aggregate particle-steps/s, batched worlds", "value": batched, "unit": UNIT,
            "worlds": len(worlds), "particles": ntot, "cells": ctot, "steps": args.batched_steps,
            "ms_per_step": float(step_ms.mean()), "step_ms_p50": float(np.percentile(step_ms, 50)),
            "step_ms_p99": float(np.percentile(step_ms, 99)),
            "one_at_a_time": {"value": single, "unit": UNIT,
                              "how": "each world in its own context, plg_step(K) in turn, host wall clock"},
            "speedup_vs_one_at_a_time": batched / single,
            "autotune": {"per_world": True,
                         "worlds_by_variant": {str(v): sum(1 for x in choice.values() if x == v)
                                               for v in range(len(tune_ms) - 1)},
                         "ms_per_step": {**{f"variant_{v}": tune_ms[v] for v in range(len(tune_ms) - 1)},
                                         "mixed": tune_ms[-1]}},
            "config": "512 2D periodic worlds, N log-uniform [1e3, 2e5], types 3..12, rmax U[0.005, 0.03] "
                      "(unit box), friction t1/2 U[0.02, 0.1] s, dt 0.02; seeded Philox"}


def run_blobs_3d(args) -> dict:
    """The 3D configuration: 4M particles in 64 Gaussian blobs (uneven cell
    occupancy), 16 types, about 40 neighbours, one world, device-resident."""
    import torch

    from plgpu import _lib, workloads
    from plgpu.physics import GpuWorld

    w = workloads.blob_world_3d()
    n = w.pos.shape[0]
    g = GpuWorld(3, n)
    g.set_settings(w.rmax, w.friction, w.force, w.dt, beta=w.beta, wrap=w.wrap)
    g.set_matrix(w.matrix)
    g.upload(w.pos, None, w.types)
    stream = torch.cuda.ExternalStream(g.stream())
    g.step(args.warmup)
    tile, tile_ms = g.autotune(3)  # untimed; the world is restored
    lib = _lib.load()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps_3d)]
    torch.cuda.synchronize()
    for k in range(args.steps_3d):  # state 2 x 128 MB > L2: no flush needed
        ev[k][0].record(stream)
        plgpu_check(lib.plg_step_async(g.ctx, 1), g.ctx, "plg_step_async")
        ev[k][1].record(stream)
    plgpu_check(lib.plg_sync(g.ctx, 120.0), g.ctx, "plg_sync")
    ms = np.array([a.elapsed_time(b) for a, b in ev])
    lib.plg_profile_enable(g.ctx, 1)
    g.step(5)
    kern = {}
    for k, name in enumerate(_lib.KERNELS):
        t = _lib.C.c_double()
        c = _lib.C.c_int64()
        lib.plg_profile_read(g.ctx, k, _lib.C.byref(t), _lib.C.byref(c))
        kern[name] = {"avg_us": 1e3 * t.value / max(c.value, 1), "launches": c.value}
    lib.plg_profile_enable(g.ctx, 0)
    deferred = g.deferred()
    dbg = g.debug_step()
    g.close()
    cand = dbg["candidates"] / n
    inter = float(dbg["pairs"].mean())
    return {"metric": "particle-steps/s, 3D blobs", "value": n * len(ms) / (ms.sum() * 1e-3), "unit": UNIT,
            "ms_per_step": float(ms.mean()), "kernels": kern, "deferred_targets_last_step": deferred,
            "candidates_per_particle": cand, "interactions_per_particle": inter,
            "autotune": {"chosen_tile_variant": tile, "ms_per_step_by_variant": tile_ms},
            "config": f"3D periodic unit cube, N={n}, 64 Gaussian blobs sigma 0.025 (0.05 in [-1,1]^3), 16 types, "
                      f"rmax {w.rmax} (mean 40 neighbours), dt 0.01; seeded Philox"}


def host_link(dev, nbytes: int = 64 << 20, reps: int = 5) -> dict:
    """The host link's DMA ceiling each way: a page-locked host buffer of
    `nbytes` copied to and from the device, median over `reps` copies timed
    with CUDA events (the ceiling the e2e leg's transfers are held to)."""
    import torch

    h = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    d = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    out = {"bytes": nbytes}
    for key, dst, src in (("h2d_gbs", d, h), ("d2h_gbs", h, d)):
        ts = []
        for k in range(reps + 1):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            dst.copy_(src, non_blocking=True)
            b.record()
            b.synchronize()
            if k:
                ts.append(a.elapsed_time(b))
        out[key] = nbytes / (float(np.median(ts)) * 1e-3) / 1e9
    return out


def plgpu_check(status, ctx, what):
    import plgpu.physics

    plgpu.physics.check(status, ctx, what)


def run_serving(args) -> dict:
    """The served configuration: Poisson arrivals at 200/s for an arrival
    window of --serve-seconds (default 60 s), each request a world spec the
    server generates on the device (2D or 3D 50/50, N log-uniform in
    [1e3, 2e6], types 3..16, matrix uniform in [-1,1], k uniform in [10, 50]
    neighbours, steps uniform in [100, 5000]), admitted under a 150 GB
    device-memory budget and the batch capacities; then a drain of at most
    --serve-drain-s.  The offered load (about 1.3e11 particle-steps/s) is far
    above what one GPU delivers, so most requests are still queued when the
    run ends: the line reports completed and unfinished requests, p50/p99
    completion latency over the completed ones, the delivered rate, the
    device-busy fraction of each batch, and the same requests one at a time
    (each alone in a single-world context) for comparison."""
    import threading

    from plgpu import workloads
    from plgpu.physics import GpuWorld
    from plgpu.serve import Server

    rng = np.random.Generator(np.random.Philox(2025))
    arrivals = []
    t = 0.0
    while True:
        t += float(rng.exponential(1.0 / args.serve_rate))
        if t > args.serve_seconds:
            break
        arrivals.append(t)
    reqs = [workloads.serving_request_generated(rng) for _ in arrivals]
    offered = sum(g.n * st for _, g, st in reqs) / args.serve_seconds
    cap = (int(args.serve_cap_2d), int(args.serve_cap_3d))
    cells = (int(args.serve_cells_2d), int(args.serve_cells_3d))
    srv = Server(memory_budget_bytes=150 << 30, particle_capacity=cap, cell_capacity=cells,
                 max_worlds_per_batch=1024, max_chunk_steps=16, autotune_interval_ms=15000)
    stop = threading.Event()

    def collect():  # hands every finished result back to the host and drops it
        while not stop.is_set():
            rid = srv.wait_any(0.05)
            if rid is not None:
                srv.release(rid)

    collector = threading.Thread(target=collect)
    collector.start()
    t0 = time.perf_counter()
    for (dim, g, steps), ta in zip(reqs, arrivals):
        delay = t0 + ta - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        srv.submit_generated(dim, g, steps)
    end = t0 + args.serve_seconds + args.serve_drain_s
    while time.perf_counter() < end:
        if srv.stats()["completed"] == len(reqs):
            break
        time.sleep(0.05)
    wall = time.perf_counter() - t0
    st = srv.stats()
    stop.set()
    collector.join()
    srv.close()

    # The same requests one at a time, each alone in a single-world context,
    # in arrival order until --serve-alone-s seconds of stepping: a world's
    # time per step does not depend on how many steps it runs, so each is
    # timed over min(steps, 100) steps (after 2 untimed ones) and scaled to
    # its step count.
    alone_ps, alone_s, alone_n, measured = 0.0, 0.0, 0, 0.0
    for dim, g, steps in reqs:
        w = GpuWorld(dim, g.n)
        w.set_settings(g.rmax, g.friction, g.force, g.dt, beta=g.beta, wrap=g.wrap)
        w.set_matrix(g.matrix)
        w.generate(g.n, g.position_setter, g.type_setter, g.seed)
        w.step(2)
        m = min(steps, 100)
        t1 = time.perf_counter()
        w.step(m)
        dt = time.perf_counter() - t1
        w.close()
        measured += dt
        alone_s += dt * steps / m
        alone_ps += g.n * steps
        alone_n += 1
        if measured >= args.serve_alone_s:
            break
    alone = alone_ps / alone_s
    served = st["particle_steps"] / wall
    return {"metric": "served requests: completion latency and aggregate particle-steps/s",
            "requests": len(reqs), "completed": st["completed"],
            "unfinished": {"queued": st["queued"], "resident": st["running"]},
            "latency_p50_ms": st["latency_p50_ms"], "latency_p99_ms": st["latency_p99_ms"],
            "latency_mean_ms": st["latency_mean_ms"],
            "value": served, "unit": UNIT, "offered_particle_steps_per_s": offered,
            "device_busy_fraction": {"2d": st["busy_dim_s"][0] / wall, "3d": st["busy_dim_s"][1] / wall},
            "compactions": st["compactions"], "autotunes": st["autotunes"],
            "one_at_a_time": {"value": alone, "unit": UNIT, "requests": alone_n,
                              "how": "the first requests in arrival order, each generated alone in a single-world "
                                     "context, min(steps, 100) steps timed (host wall clock) and scaled to its step "
                                     "count"},
            "speedup_vs_one_at_a_time": served / alone,
            "wall_s": wall, "peak_resident_bytes": st["peak_resident_bytes"], "budget_bytes": 150 << 30,
            "config": f"Poisson arrivals {args.serve_rate:g}/s for {args.serve_seconds:g} s (then at most "
                      f"{args.serve_drain_s:g} s of drain), 2D/3D 50/50, N log-uniform [1e3, 2e6], types 3..16, "
                      "k U[10, 50], steps U[100, 5000], worlds generated on the device (uniform positions and "
                      f"types, seeded), budget 150 GB, batch capacities {cap[0]:,} (2D) / {cap[1]:,} (3D) "
                      "particles, chunks of <= 16 steps, per-world tile tuning every 15 s; seeded Philox"}


def run_reference(args):
    # The reference is a CPU path: rank 0 alone times it, the other ranks exit.
    if int(os.environ.get("RANK", "0")) != 0:
        return
    threads = os.cpu_count() or 1
    import orc

    orc.build()
    n = args.n
    pos, vel, types, m = make_world(n)
    w = orc.World(2, pos, vel, types, np.arange(n, dtype=np.int32), m,
                  orc.settings(SETTINGS["rmax"], SETTINGS["friction"], SETTINGS["force"], SETTINGS["dt"],
                               SETTINGS["beta"], SETTINGS["wrap"]))
    w.run(args.warmup, threads)
    t = w.run(args.steps, threads)
    v = n * args.steps / t
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Philox: uniform positions, zero velocity)",
        "config": {"workload": f"2D periodic, N={n}, 8 types, rmax=0.0025 (unit box), dt=0.01, C FP64 "
                               f"restatement of Physics.update() on {threads} host threads"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{args.steps} full steps after {args.warmup} warm-up steps (Java/JDK absent: "
                                   "C restatement of the reference's step, same algorithm and threading)"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "cfg1_10k": cpu_cfg1(threads),
    }
    print(json.dumps(line))


def run_ours(args):
    import torch

    import plgpu
    from plgpu import _lib
    from plgpu.physics import GpuWorld

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    reps = Replicas("nccl")
    rank, world_size = reps.rank, reps.world_size
    dev = torch.device("cuda", torch.cuda.current_device())

    import __graft_entry__

    __graft_entry__.build()
    lib = _lib.load()

    n = args.n
    pos, vel, types, m = make_world(n, seed=2024 + rank)
    w = GpuWorld(2, n)
    w.set_settings(**SETTINGS)
    w.set_matrix(m)
    w.upload(pos, vel, types)
    stream = torch.cuda.ExternalStream(w.stream(), device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def flush_l2():
        if not args.no_flush:
            flush.zero_()
        torch.cuda.synchronize()

    def barrier():
        reps.barrier()
        torch.cuda.synchronize()

    check = plgpu.physics.check
    w.step(args.warmup)
    tile, tile_ms = w.autotune(5)  # untimed; the world is restored
    clocks = Clocks(torch.cuda.current_device())
    clocks.start()

    # value: device-resident, each step timed alone, L2 flushed in between
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    barrier()
    for k in range(args.steps):
        flush_l2()
        ev[k][0].record(stream)
        check(lib.plg_step_async(w.ctx, 1), w.ctx, "plg_step_async")
        ev[k][1].record(stream)
        check(lib.plg_sync(w.ctx, 60.0), w.ctx, "plg_sync")
    barrier()
    total_ms = reps.max_over_ranks(sum(a.elapsed_time(b) for a, b in ev), dev)
    ms_per_step = total_ms / args.steps
    value = reps.rate(n * args.steps, total_ms * 1e-3, dev)

    # per-kernel durations over a profiled pass of the same number of steps
    check(lib.plg_profile_enable(w.ctx, 1), w.ctx, "plg_profile_enable")
    for k in range(args.steps):
        flush_l2()
        check(lib.plg_step(w.ctx, 1), w.ctx, "plg_step")
    kern = {}
    for k, name in enumerate(_lib.KERNELS):
        ms = _lib.C.c_double()
        cnt = _lib.C.c_int64()
        lib.plg_profile_read(w.ctx, k, _lib.C.byref(ms), _lib.C.byref(cnt))
        kern[name] = {"avg_us": 1e3 * ms.value / max(cnt.value, 1), "launches": cnt.value}
    check(lib.plg_profile_enable(w.ctx, 0), w.ctx, "plg_profile_enable")

    # e2e through the public API with pinned host buffers
    hp = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
    hv = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
    ht = torch.empty(n, dtype=torch.int32, pin_memory=True).numpy()
    hi = torch.empty(n, dtype=torch.int32, pin_memory=True).numpy()
    P, I = _lib.C.c_double, _lib.C.c_int32
    check(lib.plg_download(w.ctx, _lib.ptr(hp, P), _lib.ptr(hv, P), _lib.ptr(ht, I), _lib.ptr(hi, I)), w.ctx, "dl")
    e2e_s = 0.0
    parts = np.zeros(3)
    barrier()
    for k in range(args.e2e_steps):
        flush_l2()
        t0 = time.perf_counter()
        check(lib.plg_upload(w.ctx, n, _lib.ptr(hp, P), _lib.ptr(hv, P), _lib.ptr(ht, I)), w.ctx, "plg_upload")
        t1 = time.perf_counter()
        check(lib.plg_step(w.ctx, 1), w.ctx, "plg_step")
        t2 = time.perf_counter()
        check(lib.plg_download(w.ctx, _lib.ptr(hp, P), _lib.ptr(hv, P), _lib.ptr(ht, I), _lib.ptr(hi, I)), w.ctx,
              "plg_download")
        t3 = time.perf_counter()
        e2e_s += t3 - t0
        parts += (t1 - t0, t2 - t1, t3 - t2)
    # the same with the download fused into the step (plg_step_download)
    fused_s = 0.0
    fparts = np.zeros(2)
    fuses = _lib.C.c_int32(0)
    check(lib.plg_step_download_fuses(w.ctx, _lib.ptr(hp, P), _lib.ptr(hv, P), _lib.ptr(ht, I), _lib.ptr(hi, I),
                                      _lib.C.byref(fuses)), w.ctx, "plg_step_download_fuses")
    barrier()
    for k in range(args.e2e_steps):
        flush_l2()
        t0 = time.perf_counter()
        check(lib.plg_upload(w.ctx, n, _lib.ptr(hp, P), _lib.ptr(hv, P), _lib.ptr(ht, I)), w.ctx, "plg_upload")
        t1 = time.perf_counter()
        check(lib.plg_step_download(w.ctx, 1, _lib.ptr(hp, P), _lib.ptr(hv, P), _lib.ptr(ht, I), _lib.ptr(hi, I)),
              w.ctx, "plg_step_download")
        t2 = time.perf_counter()
        fused_s += t2 - t0
        fparts += (t1 - t0, t2 - t1)
    barrier()
    clk = clocks.stop()
    e2e_s = reps.max_over_ranks(e2e_s, dev)
    unfused_value = reps.rate(n * args.e2e_steps, e2e_s, dev)
    fused_s = reps.max_over_ranks(fused_s, dev)
    e2e_value = reps.rate(n * args.e2e_steps, fused_s, dev)
    link = host_link(dev)
    up_ms, sd_ms = (1e3 * x / args.e2e_steps for x in fparts)
    h2d, d2h = n * (24 + 24 + 4), n * (24 + 24 + 4 + 4)
    link.update({
        "upload_gbs": h2d / (up_ms * 1e-3) / 1e9, "upload_frac": h2d / (up_ms * 1e-3) / 1e9 / link["h2d_gbs"],
        "stepdownload_gbs": d2h / (sd_ms * 1e-3) / 1e9,
        "stepdownload_frac": d2h / (sd_ms * 1e-3) / 1e9 / link["d2h_gbs"],
        "floor_ms": 1e3 * (h2d / (link["h2d_gbs"] * 1e9) + d2h / (link["d2h_gbs"] * 1e9)),
        "note": "rates are whole-call wall clock (the step-download call includes the sort and the force "
                "arithmetic); floor_ms = the bytes of one step at the DMA ceilings"})

    deferred = w.deferred()
    # pair statistics of the current state (one instrumented step)
    dbg = w.debug_step()
    cand = dbg["candidates"] / n
    inter = float(dbg["pairs"].mean())
    w.close()

    peak = _lib.C.c_double()
    check(lib.plg_probe_fp32_peak(_lib.C.byref(peak)), None, "plg_probe_fp32_peak")
    sfu_peak = _lib.C.c_double()
    check(lib.plg_probe_sfu_peak(_lib.C.byref(sfu_peak)), None, "plg_probe_sfu_peak")
    peaks = {}
    pk = REPO / "MEASURED_PEAKS.json"
    if pk.exists():
        peaks = json.loads(pk.read_text())
    hbm = peaks.get("hbm_gbs")

    force_us = kern["force"]["avg_us"]
    flops = n * (cand * FLOPS_PER_CANDIDATE[2] + inter * FLOPS_PER_INTERACTION[2])
    achieved = flops / (force_us * 1e-6) / 1e12
    traffic = issue_active = None
    tf = REPO / "profiles" / "k_force_tile_2d_1m.md"  # ncu summary of this kernel on this workload
    if tf.exists():
        text = tf.read_text()
        mt = re.search(r"^dram_bytes_per_launch: (\d+)", text, re.M)
        traffic = int(mt.group(1)) if mt else None
        mi = re.search(r"^\| smsp__issue_active \(% of active cycles\) \| ([\d.]+)%", text, re.M)
        issue_active = float(mi.group(1)) / 100 if mi else None
    roofline = {"bound": "fp32", "kernel": "force", "achieved": achieved, "peak": peak.value, "unit": "TFLOP/s",
                "frac": achieved / peak.value, "traffic": traffic,
                "peak_source": "FFMA microbenchmark run live by this bench (MEASURED_PEAKS.json has no FP32 peak)",
                "work": f"{cand:.2f} candidate + {inter:.2f} interacting pairs per particle; "
                        f"{FLOPS_PER_CANDIDATE[2]} / {FLOPS_PER_INTERACTION[2]} flops each",
                # What actually bounds the kernel: instruction issue (compares,
                # selects, shared-memory loads and the rsqrt beside the FMAs),
                # as ncu measured it on this workload.
                "issue_active_ncu": issue_active,
                # The special-function unit: one rsqrt per candidate pair,
                # against an rsqrt.approx microbenchmark run live.
                "sfu": {"achieved": n * cand / (force_us * 1e-6) / 1e9, "peak": sfu_peak.value, "unit": "Gop/s",
                        "frac": n * cand / (force_us * 1e-6) / 1e9 / sfu_peak.value,
                        "work": "one rsqrt.approx per candidate pair"}}
    sort_kernels = {}
    if hbm:
        cells = (int(np.floor(1 / SETTINGS["rmax"]))) ** 2
        for name, b in (("scatter", BYTES["scatter"] * n), ("gather", BYTES["gather"] * n),
                        ("scan", BYTES["scan_cell"] * cells), ("force", BYTES["force"] * n)):
            gbs = b / (kern[name]["avg_us"] * 1e-6) / 1e9
            sort_kernels[name] = {"achieved_gbs": gbs, "frac_of_measured_hbm": gbs / hbm}

    cfg1 = None
    if rank == 0 and not args.no_cfg1:
        cfg1 = run_cfg1(args)
        if not args.no_cpu_baseline:
            cfg1["cpu_baseline"] = cpu_cfg1(os.cpu_count() or 1)
            cfg1["speedup_vs_cpu"] = cfg1["value"] / cfg1["cpu_baseline"]["value"]
    blobs3d = None
    if rank == 0 and not args.no_3d:
        blobs3d = run_blobs_3d(args)
    batched = None
    if rank == 0 and not args.no_batched:
        batched = run_batched(args)
    serving = None
    if rank == 0 and not args.no_serving:
        serving = run_serving(args)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        rate, steps, secs = cpu_oracle_rate(n, threads, args.cpu_sample_s)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{steps} steps of the same 1M workload in {secs:.1f} s (C FP64 restatement of "
                         f"Physics.update(), {threads} threads; no JDK for the Java path)"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world_size, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Philox: uniform positions, zero velocity, uniform types and matrix)",
            "config": {"workload": f"2D periodic unit box, N={n}, 8 types, rmax=0.0025 (0.005 in [-1,1]^2), "
                                   "beta=0.3, friction t1/2=0.043 s, dt=0.01",
                       "parallelism": "replicas" if world_size > 1 else "single GPU",
                       "l2": "warm (not flushed)" if args.no_flush else "flushed (256 MB write) between steps"},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": n * (24 + 24 + 4),
                    "d2h_bytes_per_step": n * (24 + 24 + 4 + 4), "steps": args.e2e_steps,
                    "api": "plg_upload + plg_step_download (the force kernel writes the snapshot), pinned host "
                           "buffers, host wall clock",
                    "snapshot_fused": bool(fuses.value), "host_link": link,
                    "ms_upload_stepdownload": [round(1e3 * x / args.e2e_steps, 4) for x in fparts],
                    "unfused": {"value": unfused_value, "api": "plg_upload + plg_step + plg_download",
                                "ms_upload_step_download": [round(1e3 * x / args.e2e_steps, 4) for x in parts]}},
            "deferred_targets_last_step": deferred,
            "autotune": {"chosen_tile_variant": tile, "ms_per_step_by_variant": tile_ms},
            "gpu_launches": len(_lib.KERNELS) * args.steps,
            "roofline": roofline,
            "kernels": kern,
            "sort_kernels_hbm": sort_kernels,
            "pair_interactions_per_s": value * inter,
            "candidates_per_particle": cand,
            "interactions_per_particle": inter,
            "cpu_baseline": cpu,
            "cfg1_10k": cfg1,
            "blobs_3d": blobs3d,
            "batched": batched,
            "serving": serving,
            "clocks": clk,
        }
        print(json.dumps(line))
    reps.close()


def main():
    args = parse()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
