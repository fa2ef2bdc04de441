#!/usr/bin/env python
"""Benchmark: body-steps/s of the batched AVBD engine on the 4,096-world mix, beside the plain
one-world-per-launch-sequence path and the CPU path.

Workload (default ``world_mix``): 4,096 independent box/sphere piles with log-normal body counts
(median 256, clipped to [16, 8192], ~2.1 M bodies in total), dt 1/60 s, 10 iterations, FP32 state.
One benchmark step advances every world by one solver step (one launch sequence over all worlds).
Inputs (2.1 M bodies, tens of millions of contacts) far exceed the 129 MB L2, so no L2 flush is
needed between steps.

Reported: ``value`` (device-resident, CUDA events on the engine's stream), ``e2e`` (through the
public API with a host-side velocity-command upload and a full pose readback every step),
per-step latency percentiles, the plain path on a sample of the worlds, the dominant kernel's
roofline against the measured HBM copy bandwidth, and the CPU oracle on a bounded sample.

``--impl reference`` times the reference's CPU path (the oracle restatement: the reference is
JavaScript and cannot run here) on a bounded sample of the same workload with all host cores.
"""
from __future__ import annotations

import argparse
import collections
import faulthandler
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path[:0] = [os.path.join(ROOT, "babylon-avbd_gb300"), os.path.join(ROOT, "oracle")]

import numpy as np  # noqa: E402

faulthandler.enable()


def log(msg):
    print(f"[bench {time.strftime('%H:%M:%S')}] {msg}", file=sys.stderr, flush=True)


METRIC = "body-steps/s and p99 tick latency: batched/served vs plain GPU path at 1e-5 tol"
UNIT = "body-steps/s"


def args_parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--workload", choices=["world_mix", "box_pile", "mixed_1m", "cloth_wall", "served"], default="world_mix")
    p.add_argument("--requests", type=int, default=20_000, help="served: requests per stream")
    p.add_argument("--rates", default="2000,10000,50000", help="served: Poisson arrival rates (req/s)")
    p.add_argument("--serve-rate", type=float, default=10_000.0, help="rate of the served stream in the default line")
    p.add_argument("--budget-gb", type=float, default=120.0, help="served: device-memory budget")
    p.add_argument("--serve-depth", type=int, default=2, help="served: ticks in flight on the device at most")
    p.add_argument("--serve-steps", type=int, default=1, help="served: steps per world and tick at most (1: lowest latency; measured 1, 4, 16)")
    p.add_argument("--serve-steps-sweep", default="1,4,16", help="served workload: steps-per-tick values run at --serve-rate")
    p.add_argument("--no-serve", action="store_true")
    p.add_argument("--worlds", type=int, default=4096)
    p.add_argument("--plain-sample", type=int, default=128, help="worlds timed on the plain path")
    p.add_argument("--cpu-sample", type=int, default=256, help="worlds timed on the CPU path")
    p.add_argument("--cpu-seconds", type=float, default=15.0)
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--full-steps", type=int, default=60, help="world_mix: steps of the configuration's whole run")
    p.add_argument("--no-plain", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--spatial-sort", choices=["on", "off", "auto"], default="auto",
                   help="bodies of every world in Morton order (spatialSort, the reference GPU solver's "
                        "default); auto: on for mixed_1m (uniformly seeded bodies), off for the others "
                        "(their bodies are created in lattice or grid order already)")
    p.add_argument("--sleeping", action="store_true",
                   help="world_mix with island sleeping on (a different workload: settled piles sleep)")
    return p.parse_args()


# ------------------------------------------------------------------ distributed plumbing
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as td
            td.init_process_group("gloo")
            self.td = td

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def max(self, v: float) -> float:
        if self.world == 1:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v: float) -> float:
        if self.world == 1:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.SUM)
        return float(t.item())


# ------------------------------------------------------------------ clocks
class Clocks:
    """nvidia-smi samples every 200 ms during the timed region."""

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except ValueError:
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ workloads
def build_worlds(args, rank):
    worlds, cfg = _build_worlds(args, rank)
    mode = getattr(args, "spatial_sort", "off")
    if mode == "on" or (mode == "auto" and args.workload == "mixed_1m"):
        from avbd_gb300.pipeline import spatial_sort
        worlds = [spatial_sort(w) for w in worlds]
        cfg["spatial_sort"] = "Morton order of each world's bodies (spatialSort)"
    return worlds, cfg


def _build_worlds(args, rank):
    from avbd_gb300 import workloads
    if args.workload == "box_pile":
        return [workloads.box_pile_c0()], {"workload": "box_pile_c0", "bodies": 1001, "iterations": 10,
                                           "l2": "one 1,001-body world: L2-resident (launch-bound)"}
    if args.workload == "mixed_1m":
        w = workloads.mixed_pile(1_000_000, seed=workloads.SEED_BASE + 1)
        w.params.broadphase = "hploc"
        w.params.bvh_rebuild = 16
        return [w], {"workload": "mixed_1m", "bodies": int(w.n_bodies), "iterations": 10, "seed": workloads.SEED_BASE + 1,
                     "shapes": "70% boxes (half-extents U[0.25, 1]), 30% spheres (r U[0.25, 0.75])",
                     "volume": "centres uniform in 400 x 200 x 400 m above a 440 x 2 x 440 m static ground",
                     "broadphase": "hploc tree, refit every step, rebuilt every 16",
                     "l2": "inputs larger than L2 (no flush needed)"}
    if args.workload == "cloth_wall":
        w = workloads.cloth_wall()
        return [w], {"workload": "cloth_wall", "bodies": int(w.n_bodies), "joints": int(w.n_cons), "iterations": 15,
                     "cloth": "256x256 boxes of 0.1 m, ball joints, two corners pinned, over a static 5 m sphere",
                     "wall": "100x2x50 bricks of 1x0.5x0.5 m hit by a 2 m sphere at 40 m/s",
                     "l2": "inputs larger than L2 (no flush needed)"}
    seed = workloads.SEED_BASE + 3 + 1000 * rank
    worlds, counts, sigma = workloads.world_mix(args.worlds, target=int(2_100_000 * args.worlds / 4096), seed=seed)
    cfg = {"workload": f"world_mix_{args.worlds}", "worlds": args.worlds, "bodies": int(counts.sum() + len(counts)),
           "count_median": 256, "count_clip": [16, 8192], "lognormal_sigma": round(float(sigma), 4),
           "seed": seed, "iterations": 10, "dt": "1/60", "shapes": "70% boxes, 30% spheres",
           "l2": "inputs larger than L2 (no flush needed)"}
    if getattr(args, "sleeping", False):
        for w in worlds:
            w.params.sleeping = True
        cfg["workload"] += "_sleeping"
        cfg["sleeping"] = {"speedThreshold": 0.08, "timeThreshold": 0.6}
    return worlds, cfg


def sample_worlds(worlds, k):
    idx = np.linspace(0, len(worlds) - 1, min(k, len(worlds))).round().astype(int)
    return [worlds[i] for i in sorted(set(idx.tolist()))]


def cpu_sample(args, worlds):
    """The CPU path's bounded sample of the workload: sampled worlds of a mix; for the 1 M-body
    world one world of the same density and body mix with 1/16 of the bodies (the sequential
    oracle takes about a minute per step on the full world)."""
    if args.workload == "mixed_1m":
        from avbd_gb300 import workloads
        return [workloads.mixed_pile(62_500, seed=workloads.SEED_BASE + 1)], 0
    return sample_worlds(worlds, args.cpu_sample), args.warmup


def cpu_baseline(worlds, warm, steps, seconds, threads=0):
    """The oracle (FP64, reference sequential order) on a bounded sample, OpenMP over worlds."""
    import oracle
    ws = [oracle.OracleWorld(w, fp64=True, app=True, colored=False) for w in worlds]
    if warm:
        oracle.step_parallel(ws, warm, threads)
    bodies = sum(w.n_bodies for w in worlds)
    done, t0 = 0, time.perf_counter()
    used = 1
    while done < steps or time.perf_counter() - t0 < seconds:
        used = oracle.step_parallel(ws, 1, threads)
        done += 1
        if time.perf_counter() - t0 > seconds:
            break
    el = time.perf_counter() - t0
    return {"value": bodies * done / el, "unit": UNIT, "cores": used, "kind": "port",
            "sample": f"{len(worlds)} worlds ({bodies} bodies) x {done} steps after {warm} warm-up steps, "
                      f"FP64 oracle in the reference's sequential order, {el:.1f} s"}


def load_peaks():
    try:
        d = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def load_traffic():
    """DRAM bytes over algorithmic bytes of each kernel class, from the committed ncu summary
    (one step captured; the bench scales it to its own steps by their algorithmic bytes)."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    try:
        return {k: v["dram_over_algorithmic"] for k, v in json.load(open(p))["classes"].items()}
    except Exception:
        return {}


def served_stream(pipe, args, rate, seed, max_steps=None):
    """One Poisson request stream through the world server (the serving configuration: 20,000
    requests, creates of log-normal size and advances by K in {1, 4, 16}, continuous batching,
    budgeted admission with LRU eviction). The loop never waits for the device: each pass admits
    the requests that have arrived and, while fewer than `serve_depth` ticks are on the device,
    queues one multi-step tick (every world with queued steps advances by up to `serve_steps` steps, the
    steps back to back on the device, the poses of each world whose request a step completes
    captured right after it); replies are collected as they arrive.
    Latency of a request = arrival to its reply: a create replies once the world is admitted; an
    advance once its captured poses are on the host."""
    import torch
    from avbd_gb300 import _lib as L
    from avbd_gb300 import workloads
    max_steps = max_steps or args.serve_steps
    r = workloads.request_stream(args.requests, rate, seed)
    creates = np.nonzero(r["create"])[0]
    packed = {int(i): L.PackedScene(workloads.lattice_pile(int(r["count"][i]), int(r["world_seed"][i]))) for i in creates}
    server = pipe.createServer(budgetBytes=int(args.budget_gb * 1e9), initialBodies=1 << 20, initialWorlds=4096)
    stream = torch.cuda.ExternalStream(pipe.stream)
    n = args.requests
    world_of_create = {}  # creation order -> world id
    created = 0
    ticket_info = {}
    lat_create, lat_adv, tick_events = [], [], []
    rejected = 0
    h2d = d2h = 0
    i = 0
    arrival = r["arrival"]
    inflight = collections.deque()  # fences of the ticks still on the device
    pipe.synchronize()
    t0 = time.perf_counter()
    while i < n or ticket_info:
        now = time.perf_counter() - t0
        while i < n and arrival[i] <= now:
            if r["create"][i]:
                pk = packed[i]
                try:
                    wid = server.admit(pk)
                    world_of_create[created] = wid
                    h2d += sum(a.nbytes for a in pk.keep)
                except L.AvbdError:
                    rejected += 1
                    world_of_create[created] = None
                created += 1
                lat_create.append(time.perf_counter() - t0 - arrival[i])
            else:
                wid = world_of_create.get(int(r["target"][i]))
                if wid is not None:
                    ticket_info[server.advance(wid, int(r["steps"][i]))] = arrival[i]
                else:
                    lat_adv.append(time.perf_counter() - t0 - arrival[i])  # refused at once
            i += 1
        while inflight and inflight[0].done:
            inflight.popleft().destroy()
        if len(inflight) < args.serve_depth:
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            if server.tick(maxSteps=max_steps, replies=True):
                e1.record(stream)
                tick_events.append((e0, e1))
                inflight.append(pipe.fence())
        done = server.ready()
        now_s = time.perf_counter() - t0
        for t in done:
            d2h += server.takeReply(t).nbytes
            lat_adv.append(now_s - ticket_info.pop(t))
        if not done and i < n and arrival[i] > time.perf_counter() - t0:
            time.sleep(max(0.0, min(arrival[i] - (time.perf_counter() - t0), 0.0005)))
    pipe.synchronize()
    wall = time.perf_counter() - t0
    for f in inflight:
        f.destroy()
    tick_ms = [a.elapsed_time(b) for a, b in tick_events]
    st = server.stats()
    server.destroy()
    lat = np.array(lat_create + lat_adv) * 1000.0
    la = np.array(lat_adv) * 1000.0
    pct_ = lambda x, q: round(float(np.percentile(x, q)), 3) if len(x) else None  # noqa: E731
    return {"rate_req_s": rate, "requests": n, "creates": int(len(creates)), "wall_s": round(wall, 3),
            "body_steps_per_s": st["body_steps"] / wall, "body_steps": st["body_steps"],
            "latency_ms": {"p50": pct_(lat, 50), "p95": pct_(lat, 95), "p99": pct_(lat, 99)},
            "advance_latency_ms": {"p50": pct_(la, 50), "p95": pct_(la, 95), "p99": pct_(la, 99)},
            "tick_ms": {"p50": pct_(tick_ms, 50), "p95": pct_(tick_ms, 95), "p99": pct_(tick_ms, 99), "ticks": len(tick_ms),
                        "what": f"device time of one serving tick (up to {max_steps} steps of every world with queued steps)"},
            "max_steps_per_tick": max_steps, "ticks_in_flight": args.serve_depth,
            "admitted_worlds": st["admitted"], "rejected_worlds": rejected, "evictions": st["evictions"],
            "restores": st["restores"], "peak_device_gb": round(st["peak_device_bytes"] / 1e9, 2),
            "budget_gb": args.budget_gb, "h2d_bytes": int(h2d), "d2h_bytes": int(d2h),
            "stream": f"seed {seed}, Poisson arrivals, first 256 requests create, then 10% creates; counts log-normal "
                      f"median 256 sigma 1.2078 clipped [16, 65536]; advances K in {{1, 4, 16}} to a uniform earlier world"}


def run_served(args, dist):
    import torch
    from avbd_gb300 import createSolverPipeline, workloads
    dev = dist.local
    torch.cuda.set_device(dev)
    pipe = createSolverPipeline("gb300", device=dev)
    lines = []
    with Clocks(dev) as clk:
        for k, rate in enumerate(float(x) for x in args.rates.split(",")):
            log(f"served stream at {rate:.0f} req/s")
            lines.append(served_stream(pipe, args, rate, workloads.SEED_BASE + 4 + 1000 * dist.rank))
            log(json.dumps(lines[-1]))
        steps_sweep = []
        for m in (int(x) for x in args.serve_steps_sweep.split(",") if x):
            log(f"served stream at {args.serve_rate:.0f} req/s, up to {m} steps per tick")
            steps_sweep.append(served_stream(pipe, args, args.serve_rate, workloads.SEED_BASE + 4 + 1000 * dist.rank, m))
            log(json.dumps(steps_sweep[-1]))
    pipe.destroy()
    if dist.rank != 0:
        return
    best = max(lines, key=lambda x: x["body_steps_per_s"])
    line = {"metric": METRIC, "value": best["body_steps_per_s"], "unit": UNIT, "n_gpus": args.gpus,
            "steps": None, "warmup": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": "served_poisson", "requests": args.requests, "budget_gb": args.budget_gb,
                       "rates": args.rates},
            "served": lines, "steps_per_tick_sweep": steps_sweep, "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ arms
def run_reference(args, dist):
    if dist.rank != 0:
        return
    worlds, cfg = build_worlds(args, 0)
    sample, warm = cpu_sample(args, worlds)
    cb = cpu_baseline(sample, warm, args.steps, args.cpu_seconds)
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": cfg, "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def timed_batch(pipe, stream, worlds, warmup, steps, profile=False, sync_each=False, clocks=None):
    """A fresh batch of `worlds`: `warmup` untimed steps, then `steps` steps queued back to back
    (the engine's step never waits for the device) with a CUDA event on the engine's stream after
    each; returns (per-tick ms, total ms, the batch's profile read, bodies). `profile` turns on
    the engine's per-kernel-class events and algorithmic-byte counting (the instrumented run)."""
    import torch
    batch = pipe.createBatch(worlds)
    for _ in range(warmup):
        batch.step(1)
    pipe.synchronize()
    if profile:
        batch.profile(True)
    p0 = batch.profileRead()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
    pipe.synchronize()
    torch.cuda.synchronize()
    if clocks is not None:
        clocks.__enter__()
    ev[0].record(stream)
    for k in range(steps):
        batch.step(1)
        ev[k + 1].record(stream)
        if sync_each:
            pipe.synchronize()
    pipe.synchronize()
    torch.cuda.synchronize()
    if clocks is not None:
        clocks.__exit__(None, None, None)
    ticks = np.array([ev[k].elapsed_time(ev[k + 1]) for k in range(steps)])
    total = float(ev[0].elapsed_time(ev[-1]))
    p1 = batch.profileRead()
    p1["launches_timed"] = p1["launches"] - p0["launches"]
    p1["graph_replays_timed"] = p1["graph_replays"] - p0["graph_replays"]
    p1["graph_captures_timed"] = p1["graph_captures"] - p0["graph_captures"]
    nb = batch.bodyCount
    batch.destroy()
    return ticks, total, p1, nb


def pct(x, q):
    return round(float(np.percentile(x, q)), 3) if len(x) else None


def parity_c0():
    """One config-0 step from the engine's state after 75 steps against the oracle: float32 in the
    engine's colour order (the parity bar), float64 in the same order and float64 in the
    reference's sequential order (the reported errors)."""
    import parity
    from avbd_gb300 import createSolverPipeline, workloads
    sc = workloads.box_pile_c0()
    pipe = createSolverPipeline("gb300", device=0)
    w = pipe.createSolver(sc)
    rep = parity.compare_step(w, sc, 75)
    pipe.destroy()
    return {"workload": "box_pile_c0 step 76 from the engine's state after 75 steps", "tolerance": parity.TOL,
            "pairs_equal": rep["pairs_equal"], "contact_counts_equal": rep["contact_counts_equal"],
            "colors_equal": rep["colors_equal"], "fp32_same_order_err": rep["max_err_fp32"],
            "fp64_same_order_err": rep["max_err_fp64"], "fp64_sequential_err": rep["max_err_fp64_sequential"],
            "err": "max over positions, quaternions, velocities of |gpu - cpu| / (|cpu| + 1)"}


def run_ours(args, dist):
    import torch
    from avbd_gb300 import createSolverPipeline

    dev = dist.local
    torch.cuda.set_device(dev)
    log("building worlds")
    worlds, cfg = build_worlds(args, dist.rank)
    log(f"{len(worlds)} worlds built; creating pipeline")
    pipe = createSolverPipeline("gb300", device=dev)
    stream = torch.cuda.ExternalStream(pipe.stream, device=dev)
    # ---------------- the autotuner's run (untimed): the first ticks of this workload class each time
    # one candidate schedule (tile queue or colour barriers, chunk width, grid size; the same bits
    # for all) and the fastest is kept for the process
    tb = pipe.createBatch(worlds)
    # the radix width is timed on tree rebuild ticks only (one in bvh_rebuild): tree workloads
    # need that many more ticks for its three candidates' two samples each
    trees = [int(getattr(w.params, "bvh_rebuild", 16) or 16) for w in worlds if getattr(w.params, "broadphase", "auto") != "grid"]
    tb.step(24 + (7 * max(trees) if trees and args.workload in ("mixed_1m", "cloth_wall") else 0))
    pipe.synchronize()
    tp = tb.profileRead()
    tuner = {"tuned": bool(tp["tuned"]), "solve": "tile queue" if tp["solve_queue"] else "colour barriers",
             "chunks_per_block_and_colour": tp["solve_waves"], "persistent_blocks": tp["solve_blocks"] or "all resident",
             "items_per_tile": tp["solve_tile"], "radix_bits": tp["radix_bits"]}
    tb.destroy()
    log(f"tuned: {tuner}")
    # ---------------- timed region: the clean run (no instrumentation; ticks replay their CUDA
    # graph), device-resident, CUDA events on the engine's stream, max over ranks
    log("timed region")
    dist.barrier()
    clk = Clocks(dev)
    ticks, elapsed_ms, pclean, nb = timed_batch(pipe, stream, worlds, args.warmup, args.steps, clocks=clk)
    elapsed_ms = dist.max(elapsed_ms)
    total_bodies = dist.sum(float(nb))
    value = total_bodies * args.steps / (elapsed_ms / 1000.0)
    log(f"timed region done: {elapsed_ms:.1f} ms")
    # ---------------- the same steps instrumented: per-kernel-class events and algorithmic bytes
    iticks, iel, prof, _ = timed_batch(pipe, stream, worlds, args.warmup, args.steps, profile=True)
    peak, peak_kind = load_peaks()
    solve_kernel = "k_solve_queue" if tuner["solve"] == "tile queue" else "k_solve_coop"
    classes = {"solve": (prof["ms_primal"] + prof["ms_dual"], prof["bytes_primal"] + prof["bytes_dual"],
                         f"{solve_kernel} (every iteration's primal with the fused contact and joint duals)"),
               "collide": (prof["ms_collide"], prof["bytes_collide"], "collision kernels")}
    dom = max(classes, key=lambda k: classes[k][0])
    ms, byts, kname = classes[dom]
    nst = max(prof["steps"], 1)
    achieved = byts / (ms / 1000.0) / 1e9 if ms > 0 else 0.0
    ratio = load_traffic().get(dom)
    traffic = round(ratio * byts / nst) if ratio else None
    roof = {"kernel": kname, "bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
            "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_source": peak_kind,
            "traffic": traffic, "algorithmic_bytes_per_step": byts / nst,
            "per": "step (the class's launches of one step: achieved and traffic both per step)",
            "measured": "CUDA events around each launch on the engine's stream over the instrumented run",
            "launches_per_step": (prof["primal_launches"] / nst) if dom == "solve" else None}
    roof["classes"] = {k: {"ms_per_step": round(v[0] / nst, 3), "algorithmic_gb_per_step": round(v[1] / nst / 1e9, 4),
                           "achieved_gbs": round(v[1] / (v[0] / 1000.0) / 1e9, 1) if v[0] > 0 else None}
                       for k, v in classes.items()}
    breakdown = {k: round(v[0] / nst, 3) for k, v in classes.items()}
    breakdown["topology"] = round(prof["ms_topology"] / nst, 3)
    breakdown["other"] = round(prof["ms_other"] / nst, 3)
    instrumented = {"ms_per_step": round(iel / args.steps, 3), "stage_ms_per_step": breakdown,
                    "note": "direct launches with an event pair around each kernel class and a byte-count "
                            "kernel plus a host wait after every tick"}
    # ---------------- the configuration's whole run (60 steps of the world mix), p50/p99 per tick
    full = None
    if args.workload == "world_mix" and args.full_steps > 0:
        fticks, fel, _, _ = timed_batch(pipe, stream, worlds, 0, args.full_steps)
        full = {"steps": args.full_steps, "value": nb * args.full_steps / (fel / 1000.0), "unit": UNIT,
                "tick_ms": {"p50": pct(fticks, 50), "p95": pct(fticks, 95), "p99": pct(fticks, 99),
                            "max": round(float(fticks.max()), 3)},
                "note": "steps 1..N of fresh worlds, queued back to back, CUDA events per tick"}
        log(f"full run done: {fel:.1f} ms")
    # ---------------- the latency-bound operating point: the first half of the worlds in one batch
    # (about half the bodies), whole 60-step run, per-tick p99 against the 5 ms bound
    half = None
    if args.workload == "world_mix" and args.full_steps > 0 and len(worlds) >= 2:
        sub = worlds[: len(worlds) // 2]
        tb = pipe.createBatch(sub)  # the autotuner's ticks for this size class, untimed
        tb.step(24)
        pipe.synchronize()
        tb.destroy()
        hticks, hel, _, hnb = timed_batch(pipe, stream, sub, 0, args.full_steps)
        half = {"worlds": len(sub), "bodies": int(hnb), "steps": args.full_steps,
                "value": hnb * args.full_steps / (hel / 1000.0), "unit": UNIT,
                "tick_ms": {"p50": pct(hticks, 50), "p99": pct(hticks, 99), "max": round(float(hticks.max()), 3)},
                "note": "the first half of the worlds as one batch, steps 1..N, CUDA events per tick"}
        log(f"half batch done: {hel:.1f} ms")
    # ---------------- the whole mix at that operating point: four quarter batches stepped in rotation
    # (each tick steps one quarter of the worlds), every world's steps 1..N, per-tick p99
    rot = None
    if args.workload == "world_mix" and args.full_steps > 0 and len(worlds) >= 4:
        parts = [worlds[k * len(worlds) // 4:(k + 1) * len(worlds) // 4] for k in range(4)]
        for part in parts:  # the autotuner's ticks for each quarter's size class, untimed
            tb = pipe.createBatch(part)
            tb.step(24)
            pipe.synchronize()
            tb.destroy()
        batches = [pipe.createBatch(part) for part in parts]
        pipe.synchronize()
        torch.cuda.synchronize()
        n = 4 * args.full_steps
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(n + 1)]
        ev[0].record(stream)
        for k in range(n):
            batches[k % 4].step(1)
            ev[k + 1].record(stream)
        pipe.synchronize()
        torch.cuda.synchronize()
        rticks = np.array([ev[k].elapsed_time(ev[k + 1]) for k in range(n)])
        rel = float(ev[0].elapsed_time(ev[-1]))
        rnb = sum(b.bodyCount for b in batches)
        for b in batches:
            b.destroy()
        rot = {"batches": 4, "worlds": len(worlds), "bodies": int(rnb), "steps_per_world": args.full_steps, "ticks": n,
               "value": rnb * args.full_steps / (rel / 1000.0), "unit": UNIT,
               "tick_ms": {"p50": pct(rticks, 50), "p99": pct(rticks, 99), "max": round(float(rticks.max()), 3)},
               "note": "all worlds as four quarter batches stepped in rotation (one quarter per tick), "
                       "steps 1..N of every world, CUDA events per tick"}
        log(f"rotation done: {rel:.1f} ms")
    # ---------------- e2e through the public API with host buffers
    e2e = None
    if not args.no_e2e:
        # the same steps of the run as the device-timed region: a fresh batch of the same worlds,
        # the same warm-up (later steps of a pile carry more contacts and take longer)
        batch = pipe.createBatch(worlds)
        for _ in range(args.warmup):
            batch.step(1)
        pipe.synchronize()
        offs = np.cumsum([0] + batch.bodyCounts[:-1])
        # one command per world: set its last body's velocity (world offset + count - 1) upwards
        idx_host = torch.from_numpy((offs + np.array(batch.bodyCounts) - 1).astype(np.int64)).pin_memory()
        vel_host = torch.zeros((len(offs), 3), dtype=torch.float32).pin_memory()
        vel_host[:, 1] = 0.5
        idx_np, vel_np = idx_host.numpy(), vel_host.numpy()
        # every step's poses land in one of two page-locked buffers; the host waits for step k-1's
        # read after queueing step k, so it never stalls the device (the WebGPU backend's reads
        # are asynchronous the same way)
        bufs = [batch.pinnedPoses(), batch.pinnedPoses()]
        dist.barrier()
        pipe.synchronize()
        t0 = time.perf_counter()
        tags = []
        for k in range(args.steps):
            batch.setVelocities(idx_np, linear=vel_np)
            tags.append(batch.stepRead(1, bufs[k % 2]))
            if k >= 1:
                batch.readDone(tags[k - 1], wait=True)
        batch.readDone(tags[-1], wait=True)
        el = time.perf_counter() - t0
        poses_np = bufs[0]
        el = dist.max(el)
        batch.destroy()
        e2e = {"value": total_bodies * args.steps / el, "unit": UNIT,
               "h2d_bytes_per_step": int(idx_np.size * 4 + vel_np.nbytes),
               "d2h_bytes_per_step": int(poses_np.nbytes),
               "how": "Batch.setVelocities (one command per world, pinned) + Batch.stepRead (every pose into a "
                      "page-locked buffer, two in turn) + readDone of the previous step; host clock around the "
                      "loop including the last read"}
    log("e2e done")
    # ---------------- plain path (rank 0): each world in its own launch sequence
    plain = None
    if dist.rank == 0 and not args.no_plain:
        sample = sample_worlds(worlds, args.plain_sample)
        plain_worlds = [pipe.createSolver(w) for w in sample]
        for w in plain_worlds:
            w.step(args.warmup)
        pipe.synchronize()
        psteps = max(2, min(args.steps, 5))
        t0 = time.perf_counter()
        for _ in range(psteps):
            for w in plain_worlds:
                w.step(1)
        pipe.synchronize()
        el = time.perf_counter() - t0
        pb = sum(w.bodyCount for w in plain_worlds)
        plain = {"value": pb * psteps / el, "unit": UNIT,
                 "sample": f"{len(plain_worlds)} of {len(worlds)} worlds ({pb} bodies), each stepped in its own "
                           f"launch sequence (queued without waiting), {psteps} steps after {args.warmup} warm-up steps"}
        for w in plain_worlds:
            w.destroy()
        # config 0 on the plain path: one 1,001-body world, 100 steps queued back to back
        from avbd_gb300 import workloads
        w0 = pipe.createSolver(workloads.box_pile_c0())
        w0.step(max(args.warmup, 16))  # includes the autotuner's ticks for this size
        pipe.synchronize()
        t0 = time.perf_counter()
        w0.step(100)
        pipe.synchronize()
        plain["box_pile_c0_ms_per_step"] = round((time.perf_counter() - t0) * 10.0, 4)
        plain["box_pile_c0_graph_replays"] = w0.profileRead()["graph_replays"]
        w0.destroy()
        log("plain path done")
    cpu = parity = None
    if dist.rank == 0 and not args.no_cpu:
        sample, warm = cpu_sample(args, worlds)
        cpu = cpu_baseline(sample, warm, args.steps, args.cpu_seconds)
        parity = parity_c0()
    log("cpu baseline done")
    served = None
    if not args.no_serve and args.workload == "world_mix":
        from avbd_gb300 import workloads
        served = served_stream(pipe, args, args.serve_rate, workloads.SEED_BASE + 4 + 1000 * dist.rank)
        log("served stream done")
    pipe.destroy()
    if dist.rank != 0:
        return
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": cfg,
            "tick_ms": {"p50": pct(ticks, 50), "p95": pct(ticks, 95), "p99": pct(ticks, 99)},
            "autotuner": tuner,
            "graphs": {"on": bool(pclean["graphs_on"]), "replays_timed": pclean["graph_replays_timed"],
                       "captures_timed": pclean["graph_captures_timed"], "ticks_held": pclean["ticks_held"]},
            "full_run": full, "half_batch": half, "rotation": rot, "instrumented": instrumented, "plain_gpu": plain, "stage_ms_per_step": breakdown,
            "roofline": roof, "cpu_baseline": cpu, "parity": parity, "e2e": e2e,
            "gpu_launches": int(pclean["launches_timed"]), "clocks": clk.summary(), "served": served}
    print(json.dumps(line), flush=True)


def main():
    args = args_parse()
    dist = Dist()
    if args.impl == "reference":
        run_reference(args, dist)
    elif args.workload == "served":
        run_served(args, dist)
    else:
        run_ours(args, dist)


if __name__ == "__main__":
    main()
