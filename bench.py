#!/usr/bin/env python3
"""Benchmark of the GB300 incremental-fluids hot path (one JSON line on stdout).

Default workload (--workload batch): 512 independent ragged scenes of the
batched form (sides log-uniform in [64, 1024], 1-3 inflow rectangles, 0-4
seeded bodies, 4-solid-boundaries, dt = 0.0025), FP32 fields with FP64 PCG
reductions and MIC(0) factor, advanced together through ifl_batch_update
(batched phase launches, one cooperative PCG launch per step, a CUDA graph per
step, autotuned PCG shape).  A step is one update() of every scene.  Metric:
cell-steps/s = sum of w*h over the scenes x steps per second.

* value     device time of K steps (CUDA events inside the step's graph); the
            scene state (about 6 GB) is far larger than L2;
* e2e       a twin batch through the public API, wall clock: per step the body
            tables go up from pinned host memory and every scene's density
            field comes back into a pinned host buffer;
* roofline  the batched PCG kernel (the dominant kernel): algorithmic bytes /
            its device time, against MEASURED_PEAKS.json;
* fp64_dropin  the plain FP64 drop-in (ifl_update, one scene at a time) on a
            size-stratified sample of the same scenes;
* latency   p50/p99 of the step time;
* cpu_baseline  the C oracle (restatement of the reference, FP64) on the host
            cores over a size-stratified sample of the scenes.

--workload single: the single solid-boundary scene at 1024 x 1024 (3 seeded
bodies) instead.  --workload flip: step 8 (FLIP particles) on the reference
main()'s own scene (rotated box, its fixed inflow, rhoAir 0.1, rhoSoot 0.25,
diffusion 0.01, dt 0.0025) at --size (128, the reference's grid), one
handle: FP64 fields and particles, FP32-form solves (--precision fp64: the
FP64 drop-in, which is also timed beside it); its CPU baseline is the
oracle's step-8 restatement.
--workload gs [--gs-variant 1|2]: the Gauss-Seidel steps on their reference
main() scene (128^2 by default), FP64, one handle.  --impl reference times the reference's CPU algorithm (the
oracle port; the reference's own sources are not part of this repository) on
the same workload.  Multi-GPU (torchrun): each rank runs an independent
replica ("replicas only": scenes do not exchange data), barrier + max over
ranks.
"""
from __future__ import annotations

import argparse
import json
import math
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "incremental-fluids_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "cell-steps/s"
# Algorithmic bytes of the PCG solves, per cell, from the fused-schedule word
# counts of the hot-path scope table (a lower bound: every array read or
# written once per pass), with the FP32 form's storage widths: F for the
# matrix, the MIC(0) apply operands, z and s; 8 bytes for r, p, A*s and the
# MIC(0) factor.
#   per iteration   s = z + beta s, A s, z.s   R z s aDiag aX aY, W s As        6F + 8
#                   p, r AXPYs + |r|_inf       R p s r As, W p r               40 + F
#                   forward MIC(0)             R r aX aY precon, W q            5F
#                   backward MIC(0) + z.r      R q aX aY precon r, W z          5F + 8
#                                                                     total   16F + 56
#   per solve       factor                     R aDiag aX aY, W precon          3F + 8
#                   setup                      W p, |r|_inf, first M^-1 r       10F + 24
def pcg_bytes_per_cell(F: int, iterations: int) -> float:
    """Algorithmic bytes per cell of one solve that ran `iterations` iterations."""
    return (3 * F + 8) + (10 * F + 24) + iterations * (16 * F + 56)


# Bytes per cell the kernels of this library actually move for one solve (its
# own layout: 1-byte neighbour bits, the 4-word MIC(0) record, an FP32 copy of
# r; the FP64 form's separate z.r pass, which the FP32 form folds into its
# forward sweep as q.q); reported beside the algorithmic figure.
def pcg_kernel_bytes_per_cell(F: int, iterations: int) -> float:
    copy = F if F == 4 else 0
    factor, setup = 7 * F + 9, 17 + copy
    sweeps = 6 * F + 6 * F + (0 if F == 4 else F + 9)
    per_iter = (6 * F + 9) + (41 + F + copy)
    return factor + setup + sweeps + iterations * per_iter + max(iterations - 1, 0) * sweeps


def max_over_ranks(x: float, world: int, device=None) -> float:
    """Largest value over all ranks (identity for one rank)."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, steps: int, world: int, t_max_ms: float) -> float:
    """Units per second over all ranks: every rank does the same work (replicas)."""
    return world * units_per_rank * steps / (t_max_ms / 1e3)


def sum_over_ranks(x: float, world: int, device=None) -> float:
    """Sum of a per-rank value over all ranks (identity for one rank)."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def scene_work(w: int, h: int) -> float:
    """Relative cost of one update of a w x h scene: cells x PCG iterations, and the
    iterations grow about linearly with the longer side (about 70 at 128^2 and 640
    at 1024^2 in the reference's MIC(0)-PCG)."""
    return float(w) * h * max(w, h)


def shard_scenes(work, rank: int, world: int):
    """Disjoint, balanced share of scene indices for `rank`: scenes by decreasing
    estimated work onto the least-loaded rank (ties to the lower rank and index),
    so every rank computes the same partition without exchanging anything."""
    order = sorted(range(len(work)), key=lambda i: (-work[i], i))
    load = [0.0] * world
    share = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        share[r].append(i)
        load[r] += work[i]
    return sorted(share[rank])


def load_peaks():
    for path in (os.path.join(ROOT, "MEASURED_PEAKS.json"),):
        try:
            with open(path) as f:
                d = json.load(f)
            return float(d["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


# ----------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
        ids = [v.strip() for v in vis.split(",") if v.strip()]
        self.device = ids[device] if device < len(ids) else str(device)
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for k, n in enumerate(names):
                if parts[5 + k].lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------ CPU baseline
def cpu_kind() -> str:
    """'reference' when the reference's own solver was compiled on this host
    (oracle/_ref, built by __graft_entry__.build() from the staged sources),
    else 'port' (the oracle, pinned bit-for-bit to it)."""
    from oracle import oracle as O
    return "reference" if O.ref_available(4) else "port"


def cpu_solver(kind: str):
    from oracle import oracle as O
    return O.RefSolver if kind == "reference" else O.OracleSolver


def cpu_kind_text(kind: str) -> str:
    return ("the reference's own FluidSolver (its Fluid.cpp compiled on this host, -O2 -ffp-contract=off)"
            if kind == "reference" else "the oracle (C restatement of the reference, bit-identical to it)")


def _cpu_worker(args):
    variant, n, steps, warmup, seed, kind = args
    from ifluids import scenes
    sc = scenes.config1(n=n, seed=seed, variant=variant)
    o = cpu_solver(kind)(variant, n, n)
    o.set_bodies(sc.bodies)
    spent, its = 0.0, []
    for k in range(warmup + steps):
        o.add_inflow(*sc.inflows[0])
        t0 = time.perf_counter()
        o.update(sc.dt)
        if k >= warmup:
            spent += time.perf_counter() - t0
            its.append(o.stats()[0][0])
        o.advance_bodies(sc.dt)
    return spent, its


def cpu_baseline(n: int, steps: int, warmup: int, procs: int, seed: int):
    """The CPU solver on `procs` host cores, one independent copy of the scene per
    process, timed at the same step indices as the GPU (after `warmup` updates)."""
    kind = cpu_kind()
    ctx = mp.get_context("spawn")
    with ctx.Pool(procs) as pool:
        res = pool.map(_cpu_worker, [(4, n, steps, warmup, seed, kind)] * procs)
    t = max(r[0] for r in res)
    return {"value": procs * n * n * steps / t, "unit": METRIC, "cores": procs, "kind": kind,
            "sample": f"updates {warmup + 1}..{warmup + steps} (after {warmup} untimed) of the {n}x{n} "
                      f"solid-boundary scene (PCG iterations {res[0][1]}) in each of {procs} processes, "
                      f"{cpu_kind_text(kind)}, FP64",
            "seconds": round(t, 2), "steps": steps, "warmup": warmup}


# ----------------------------------------------------------------- GPU arm
def make_solver(ifl, sc, precision, device, bodies, pcg_cap=0):
    cap = {"max_iter_pressure": pcg_cap} if pcg_cap > 0 else {}
    if sc.variant >= 6:
        return ifl.FluidSolver(sc.w, sc.h, sc.density, sc.density_soot, sc.diffusion, bodies, variant=sc.variant,
                               precision=precision, device=device, **cap)
    return ifl.FluidSolver(sc.w, sc.h, sc.density, bodies, variant=sc.variant, precision=precision,
                           device=device, **cap)


def body_objs(ifl, sc):
    out = []
    for b in sc.bodies:
        out.append(ifl.SolidBox(*b[1:]) if b[0] == 0 else ifl.SolidSphere(b[1], b[2], b[3], *b[5:]))
    return out


def step_host(g, sc, bodies):
    x, y, w, h, d, t, u, v = sc.inflows[0]
    if sc.variant >= 6:
        g.addInflow(x, y, w, h, d, t, u, v)
    else:
        g.addInflow(x, y, w, h, d, u, v)
    g.update(sc.dt)
    for b in bodies:
        b.update(sc.dt)


def run_gpu(args, rank, world, local_rank):
    import torch
    import ifluids as ifl
    from ifluids import scenes

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    prec = ifl.FP32 if args.precision == "fp32" else ifl.FP64
    fbytes = 4 if prec == ifl.FP32 else 8
    sc = scenes.config3(n=args.size) if args.workload == "c3" else scenes.config1(n=args.size, seed=args.seed)
    cells = sc.cells
    # two identical solvers: one for the device-timed pass, one for the end-to-end
    # pass, so that both time the same steps (the PCG iteration count varies with
    # the state of the flow)
    bodies = body_objs(ifl, sc)
    g = make_solver(ifl, sc, prec, local_rank, bodies, args.pcg_cap)
    bodies_e = body_objs(ifl, sc)
    ge = make_solver(ifl, sc, prec, local_rank, bodies_e, args.pcg_cap)
    stream = torch.cuda.ExternalStream(g.stream, device=dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    for _ in range(args.warmup):
        step_host(g, sc, bodies)
        step_host(ge, sc, bodies_e)
    g.synchronize()
    ge.synchronize()
    g.set_timing(True)
    g.timing()  # reset accumulators
    launches0 = g.launch_count()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    with ClockSampler(local_rank) as clk:
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(float(k))  # > L2: evict the previous step's working set
                ev[k][0].record(stream)
            step_host(g, sc, bodies)
            with torch.cuda.stream(stream):
                ev[k][1].record(stream)
        g.synchronize()
        torch.cuda.synchronize(dev)
    dev_ms = sum(a.elapsed_time(b) for a, b in ev)
    launches = g.launch_count() - launches0
    kms, klaunch, iters = g.timing()
    g.set_timing(False)
    (pit, pst, perr), _, flags = g.stats()
    if flags & 1:
        raise RuntimeError("device-side wait timed out during the benchmark")
    check = None
    if args.field_check > 0 and rank == 0:  # one more (untimed) step against the FP64 reference
        job = (sc.variant, sc.w, sc.h, gpu_state(ifl, g, sc.variant), [b.as_tuple() for b in bodies],
               sc.inflows[:1], sc.dt)  # the scene generators use the reference's densities and diffusion
        step_host(g, sc, bodies)
        out = gpu_result(ifl, g, sc.variant)
        check = field_error_check([job], [out], [g.stats()[0][0]], 1)
        check["sample"] = f"the scene at update {args.warmup + args.steps + 1}"

    t_max = dev_ms
    if world > 1:
        t = torch.tensor([dev_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        t_max = float(t.item())
    value = world * cells * args.steps / (t_max / 1e3)

    # ---- end to end through the public API with pinned host buffers
    host_d = torch.empty((sc.h, sc.w), dtype=torch.float32 if prec == ifl.FP32 else torch.float64,
                         pin_memory=True).numpy()
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for k in range(args.steps):
        step_host(ge, sc, bodies_e)                     # body table: pinned upload inside update
        ge.read_field("d", dtype=host_d.dtype, out=host_d)  # result back to the host
    e2e_s = time.perf_counter() - t0
    ge.close()
    if world > 1:
        t = torch.tensor([e2e_s], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e = {"value": world * cells * args.steps / e2e_s, "unit": METRIC,
           "h2d_bytes_per_step": 96 * len(sc.bodies), "d2h_bytes_per_step": cells * fbytes}

    # ---- roofline of the persistent PCG kernel
    peak, peak_kind = load_peaks()
    n_solves = max(1, klaunch["pcg"])
    pcg_bytes = cells * n_solves * pcg_bytes_per_cell(fbytes, iters / n_solves)
    achieved = pcg_bytes / (kms["pcg"] / 1e3) / 1e9 if kms["pcg"] > 0 else 0.0
    roof = {"bound": "hbm", "kernel": "pcg_kernel", "achieved": round(achieved, 1), "peak": peak,
            "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_kind": f"of {peak_kind}",
            "traffic": None,
            "pcg_ms_per_launch": round(kms["pcg"] / max(1, klaunch["pcg"]), 3),
            "pcg_iterations_per_launch": round(iters / max(1, klaunch["pcg"]), 1),
            "kernel_ms_per_step": {k: round(v / args.steps, 3) for k, v in kms.items()}}

    # ---- FP64 drop-in on the same scene (reported beside the FP32 form)
    fp64 = None
    if prec == ifl.FP32 and args.fp64_steps > 0:
        g64 = make_solver(ifl, sc, ifl.FP64, local_rank, body_objs(ifl, sc))
        b64 = body_objs(ifl, sc)
        g64.set_bodies(b64)
        for _ in range(2):
            step_host(g64, sc, b64)
        g64.synchronize()
        s64 = torch.cuda.ExternalStream(g64.stream, device=dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(s64):
            e0.record(s64)
        for _ in range(args.fp64_steps):
            step_host(g64, sc, b64)
        with torch.cuda.stream(s64):
            e1.record(s64)
        g64.synchronize()
        fp64 = {"value": cells * args.fp64_steps / (e0.elapsed_time(e1) / 1e3), "unit": METRIC,
                "steps": args.fp64_steps, "pcg_iterations_last": g64.stats()[0][0]}
        g64.close()
    g.close()
    return {"value": value, "ms_per_step": t_max / args.steps, "e2e": e2e, "roofline": roof,
            "field_error": check,
            "gpu_launches": launches, "clocks": clk.summary(), "pcg_iterations_last": pit,
            "pcg_status_last": pst, "fp64_dropin": fp64, "cells": cells, "scene": sc}


# ----------------------------------------------------------- FLIP workload
FLIP_BOX = (0.5, 0.6, 0.7, 0.1, math.pi * 0.25, 0.0, 0.0, 0.0)   # 8-flip/Fluid.cpp:1489
FLIP_INFLOW = (0.45, 0.2, 0.2, 0.05, 1.0, 294.0, 0.0, 0.0)       # 8-flip/Fluid.cpp:1368
FLIP_RHO = (0.1, 0.25, 0.01)                                     # 8-flip/Fluid.cpp:1479-1481
FLIP_DT = 0.0025


def cpu_baseline_flip(n: int, steps: int, warmup: int):
    """Step 8 on one host core (single thread, as the reference) on the same scene,
    timed after `warmup` updates (the first places the particles)."""
    from oracle import oracle as O
    kind = "reference" if O.ref_available(8) else "port"
    s = cpu_solver(kind)(O.FLIP, n, n, *FLIP_RHO)
    s.set_bodies([(0,) + FLIP_BOX])
    for _ in range(max(1, warmup)):
        s.add_inflow(*FLIP_INFLOW)
        s.update(FLIP_DT)
    t0 = time.perf_counter()
    for _ in range(steps):
        s.add_inflow(*FLIP_INFLOW)
        s.update(FLIP_DT)
    t = time.perf_counter() - t0
    return {"value": n * n * steps / t, "unit": METRIC, "cores": 1, "kind": kind,
            "sample": f"updates {max(1, warmup) + 1}..{max(1, warmup) + steps} of the {n}x{n} FLIP scene, "
                      f"{cpu_kind_text(kind)}, {s.particle_count()} particles",
            "seconds": round(t, 3), "steps": steps, "warmup": max(1, warmup), "particles": s.particle_count()}


def time_handle(args, local_rank, make, step, cells):
    """Device time of K steps of one handle (CUDA events on its stream, L2
    flushed between steps), then an identical twin through the public API
    with the density read back into pinned host memory every step."""
    import torch
    dev = torch.device("cuda", local_rank)
    torch.cuda.set_device(local_rank)
    g, ge = make(), make()
    stream = torch.cuda.ExternalStream(g.stream, device=dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    for _ in range(max(1, args.warmup)):
        step(g)
        step(ge)
    g.synchronize()
    ge.synchronize()
    g.set_timing(True)
    g.timing()
    launches0 = g.launch_count()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    torch.cuda.synchronize(dev)
    with ClockSampler(local_rank) as clk:
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(float(k))
                ev[k][0].record(stream)
            step(g)
            with torch.cuda.stream(stream):
                ev[k][1].record(stream)
        g.synchronize()
        torch.cuda.synchronize(dev)
    step_ms = [a.elapsed_time(b) for a, b in ev]
    dev_ms = sum(step_ms)
    launches = g.launch_count() - launches0
    kms, klaunch, iters = g.timing()
    g.set_timing(False)
    stats = g.stats()
    if stats[2] & 1:
        raise RuntimeError("device-side wait timed out during the benchmark")
    n, m = g.shape(0)
    host_d = torch.empty((n, m), dtype=torch.float64, pin_memory=True).numpy()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step(ge)
        ge.read_field("d", dtype=host_d.dtype, out=host_d)
    e2e_s = time.perf_counter() - t0
    ge.close()
    return {"g": g, "dev_ms": dev_ms, "step_ms": step_ms, "launches": launches, "kms": kms, "klaunch": klaunch,
            "iters": iters, "stats": stats, "clocks": clk.summary(),
            "e2e": {"value": cells * args.steps / e2e_s, "unit": METRIC, "h2d_bytes_per_step": 96,
                    "d2h_bytes_per_step": cells * 8}}


def run_flip(args, local_rank):
    import ifluids as ifl
    n = args.size

    prec = ifl.FP32 if args.precision == "fp32" else ifl.FP64

    def make(precision=None):
        box = ifl.SolidBox(*FLIP_BOX)
        return ifl.FluidSolver(n, n, *FLIP_RHO, [box], variant=ifl.FLIP, device=local_rank,
                               precision=prec if precision is None else precision)

    def step(s):
        s.addInflow(*FLIP_INFLOW)
        s.update(FLIP_DT)

    cells = n * n
    T = time_handle(args, local_rank, make, step, cells)
    g, kms = T["g"], T["kms"]
    (pit, _, _), (hit, _, _), _ = T["stats"]
    particles = g.particle_count()
    # particle kernels: algorithmic bytes per particle and step (FP64 state of
    # x, y and four carried values = 48 B): transfer reads x, y, the carried
    # value of the grid's quantities once per grid kind and writes a bucket
    # rank and index (3 x (16 + 8)), the per-node gather reads x, y and the
    # carried values once more (3 x 16 + 32), count reads x, y (16), the
    # grid -> particle update reads x, y and reads/writes the four values
    # (16 + 64), advection reads/writes x, y (32): 312 B
    part_bytes = 312.0 * particles
    pk_ms = kms.get("particles", 0.0) / args.steps
    peak, peak_kind = load_peaks()
    achieved = part_bytes / (pk_ms / 1e3) / 1e9 if pk_ms > 0 else 0.0
    roof = {"bound": "hbm", "kernel": "particle kernels (transfer, seeding, update, advection)",
            "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
            "peak_kind": f"of {peak_kind}", "traffic": None,
            "kernel_ms_per_step": {k: round(v / args.steps, 3) for k, v in kms.items()},
            "pcg_iterations_last_step": [pit, hit]}
    g.close()
    dev_ms = T["dev_ms"]
    fp64 = None
    if prec == ifl.FP32 and args.fp64_steps > 0:  # the FP64 drop-in of the same scene beside it
        import torch
        g64 = make(ifl.FP64)
        for _ in range(2):
            step(g64)
        g64.synchronize()
        s64 = torch.cuda.ExternalStream(g64.stream, device=torch.device("cuda", local_rank))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(s64):
            e0.record(s64)
        for _ in range(args.fp64_steps):
            step(g64)
        with torch.cuda.stream(s64):
            e1.record(s64)
        g64.synchronize()
        fp64 = {"value": cells * args.fp64_steps / (e0.elapsed_time(e1) / 1e3), "unit": METRIC,
                "steps": args.fp64_steps}
        g64.close()
    return {"value": cells * args.steps / (dev_ms / 1e3), "ms_per_step": dev_ms / args.steps, "e2e": T["e2e"],
            "roofline": roof, "gpu_launches": T["launches"], "clocks": T["clocks"], "fp64_dropin": fp64,
            "particles": particles, "particle_steps_per_s": particles * args.steps / (dev_ms / 1e3),
            "latency_ms": {"p50": round(statistics.median(T["step_ms"]), 3), "max": round(max(T["step_ms"]), 3)}}


# ---------------------------------------------------- Gauss-Seidel steps 1-2
GS_INFLOW = {1: (0.45, 0.2, 0.1, 0.01, 1.0, 0.0, 3.0),      # 1-matrixless/Fluid.cpp:353
             2: (0.45, 0.2, 0.15, 0.03, 1.0, 0.0, 3.0)}     # 2-better-advection/Fluid.cpp:370
GS_DT = 0.005


def cpu_baseline_gs(variant: int, n: int, steps: int, warmup: int):
    """Steps 1-2 on one host core (single thread, as the reference) on the same
    scene, timed after `warmup` updates."""
    from oracle import oracle as O
    kind = "reference" if O.ref_available(variant) else "port"
    s = cpu_solver(kind)(variant, n, n)
    d, u, v = GS_INFLOW[variant][4:]
    x, y, w, h = GS_INFLOW[variant][:4]
    for _ in range(max(1, warmup)):
        s.add_inflow(x, y, w, h, d, 0.0, u, v)
        s.update(GS_DT)
    t0 = time.perf_counter()
    sweeps = 0
    for _ in range(steps):
        s.add_inflow(x, y, w, h, d, 0.0, u, v)
        s.update(GS_DT)
        sweeps += s.stats()[0][0]
    t = time.perf_counter() - t0
    return {"value": n * n * steps / t, "unit": METRIC, "cores": 1, "kind": kind,
            "sample": f"updates {max(1, warmup) + 1}..{max(1, warmup) + steps} of the {n}x{n} step-{variant} "
                      f"scene ({sweeps} Gauss-Seidel sweeps), {cpu_kind_text(kind)}",
            "seconds": round(t, 3), "steps": steps, "warmup": max(1, warmup)}


def run_gs(args, local_rank):
    import ifluids as ifl
    n, variant = args.size, args.gs_variant

    def make():
        return ifl.FluidSolver(n, n, 0.1, variant=variant, device=local_rank)

    def step(s):
        s.addInflow(*GS_INFLOW[variant])
        s.update(GS_DT)

    cells = n * n
    T = time_handle(args, local_rank, make, step, cells)
    kms, klaunch, iters = T["kms"], T["klaunch"], T["iters"]
    # Gauss-Seidel sweep: reads r, p (own, right, upper) and writes p: 24 B per
    # cell per sweep at the lower bound (p and r once each, p written once)
    gs_ms = kms.get("pcg", 0.0)
    peak, peak_kind = load_peaks()
    gs_bytes = 24.0 * cells * iters
    achieved = gs_bytes / (gs_ms / 1e3) / 1e9 if gs_ms > 0 else 0.0
    roof = {"bound": "hbm", "kernel": "gs_kernel", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "peak_kind": f"of {peak_kind}", "traffic": None,
            "sweeps_per_step": round(iters / args.steps, 1),
            "us_per_sweep": round(1e3 * gs_ms / max(1, iters), 2),
            "kernel_ms_per_step": {k: round(v / args.steps, 3) for k, v in kms.items()}}
    T["g"].close()
    dev_ms = T["dev_ms"]
    return {"value": cells * args.steps / (dev_ms / 1e3), "ms_per_step": dev_ms / args.steps, "e2e": T["e2e"],
            "roofline": roof, "gpu_launches": T["launches"], "clocks": T["clocks"], "fp64_dropin": None,
            "latency_ms": {"p50": round(statistics.median(T["step_ms"]), 3), "max": round(max(T["step_ms"]), 3)}}


# ----------------------------------------------------- batched workload
BATCH_COUNT, BATCH_SEED = 512, 2


def stratified(scs, k):
    """k scenes spread evenly over the size-sorted list (indices into scs)."""
    order = sorted(range(len(scs)), key=lambda i: scs[i].cells)
    if k >= len(order):
        return order
    return [order[int((j + 0.5) * len(order) / k)] for j in range(k)]


# ------------------------------------------------ per-field error check
# The benchmark spec reports every field with its error against the reference's
# own FP64 solve from the same state.  After the timed region the GPU state of
# a sample of scenes is taken just before one more update; the reference's own
# solver (oracle/_ref, built on this host from the staged sources; else the
# oracle, pinned bit-for-bit to it) then runs that update in spawned processes
# and the GPU's fields are compared with its result.  Nothing here is timed.
def gpu_state(ifl, g, variant):
    qs = [0, 2, 3] + ([1] if variant >= 6 else [])
    return {(q, a): np.asarray(g.read_field(ifl.field_id(q, a)), dtype=np.float64) for q in qs for a in (0, 1)}


def gpu_result(ifl, g, variant):
    qs = [0, 2, 3] + ([1] if variant >= 6 else [])
    out = {q: np.asarray(g.read_field(ifl.field_id(q, 0)), dtype=np.float64) for q in qs}
    out["p"] = np.asarray(g.read_field("p"), dtype=np.float64)
    return out


def field_error_check(jobs, outs, gpu_iters, procs):
    """Per-field max-norm errors of the GPU steps against the FP64 reference steps."""
    from oracle import oracle as O
    kind = "reference" if O.ref_available(jobs[0][0]) else "oracle"
    jobs = [j + (kind,) for j in jobs]
    t0 = time.perf_counter()
    with mp.get_context("spawn").Pool(max(1, min(procs, len(jobs)))) as pool:
        refs = pool.starmap(O.step_from_state, jobs)
    per = []
    for j, out, ref, it in zip(jobs, outs, refs, gpu_iters):
        e = O.field_errors(out, ref, j[0])
        per.append({"grid": [j[1], j[2]], "pcg_iterations": {"gpu": it, "fp64": ref["stats"][0][0]},
                    **{k: float(f"{v:.3e}") for k, v in e.items()}})
    worst = {k: max(x[k] for x in per) for k in per[0] if k not in ("grid", "pcg_iterations")}
    return {"against": "the reference's own FP64 solver" if kind == "reference" else
            "the FP64 oracle (pinned bit-for-bit to the reference)",
            "method": "one update from the GPU's state; max-norm error: p over fluid cells / max|p|, u and v / "
                      "the largest velocity component, d / max d",
            "max": worst, "scenes": per, "seconds": round(time.perf_counter() - t0, 1)}


def _cpu_batch_worker(args):
    idx, steps, warmup, count, seed, kind = args
    from ifluids import scenes
    scs = scenes.batch_scenes(count=count, seed=seed)
    spent, cells, its = 0.0, 0, []
    for i in idx:
        sc = scs[i]
        o = cpu_solver(kind)(sc.variant, sc.w, sc.h)
        if sc.bodies:
            o.set_bodies(sc.bodies)
        for k in range(warmup + steps):  # untimed warm-up updates, then the timed ones
            for r in sc.inflows:
                o.add_inflow(*r)
            t0 = time.perf_counter()
            o.update(sc.dt)
            if k >= warmup:
                spent += time.perf_counter() - t0
                cells += sc.cells
                its.append(o.stats()[0][0])
            o.advance_bodies(sc.dt)
    return spent, cells, its


def cpu_baseline_batch(procs: int, steps: int = 1, warmup: int = 3, sample: int = 32):
    """The CPU solver over a size-stratified sample of the batch on `procs`
    processes, timed at the GPU's step indices: every sampled scene runs
    `warmup` untimed updates, then `steps` timed ones."""
    from ifluids import scenes
    kind = cpu_kind()
    scs = scenes.batch_scenes(count=BATCH_COUNT, seed=BATCH_SEED)
    pick = stratified(scs, sample)
    pick.sort(key=lambda i: -scs[i].cells)
    shares = [[] for _ in range(procs)]
    load = [0] * procs
    for i in pick:  # largest first onto the least-loaded process
        j = load.index(min(load))
        shares[j].append(i)
        load[j] += scs[i].cells
    jobs = [(sh, steps, warmup, BATCH_COUNT, BATCH_SEED, kind) for sh in shares if sh]
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(len(jobs)) as pool:
        res = pool.map(_cpu_batch_worker, jobs)
    wall = time.perf_counter() - t0
    slowest = max(r[0] for r in res)
    cells = sum(r[1] for r in res)
    return {"value": cells / slowest, "unit": METRIC, "cores": len(jobs), "kind": kind,
            "sample": f"{len(pick)} of the {BATCH_COUNT} batch scenes (size-stratified), updates "
                      f"{warmup + 1}..{warmup + steps} of each (after {warmup} untimed), {cpu_kind_text(kind)}, "
                      f"FP64, scenes spread over {len(jobs)} processes (value = timed cells / slowest "
                      f"process's timed seconds)",
            "seconds": round(slowest, 2), "wall_seconds": round(wall, 2), "steps": steps, "warmup": warmup,
            "sample_cells": cells // max(1, steps)}


def run_batch(args, rank, world, local_rank):
    import torch
    import ifluids as ifl
    from ifluids import scenes

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    prec = ifl.FP32 if args.precision == "fp32" else ifl.FP64
    fbytes = 4 if prec == ifl.FP32 else 8
    # N ranks: the generator's first count x N scenes, split into disjoint,
    # balanced shares (per-GPU work stays about one count-scene batch: weak
    # scaling); scenes exchange nothing, so no collective touches the data path
    allscs = scenes.batch_scenes(count=args.count * world, seed=BATCH_SEED)
    mine = shard_scenes([scene_work(x.w, x.h) for x in allscs], rank, world) if world > 1 else range(len(allscs))
    scs = [allscs[i] for i in mine]
    cells = sum(s.cells for s in scs)
    cells_all = sum_over_ranks(float(cells), world, dev)

    def build(use_graph=True):
        members, bodies = [], []
        for sc in scs:
            bs = body_objs(ifl, sc)
            members.append(ifl.FluidSolver(sc.w, sc.h, sc.density, bs, variant=sc.variant, precision=prec,
                                           device=local_rank))
            bodies.append(bs)
        t, k, st = (int(v) for v in args.shape.split(",")) if args.shape else (0, 0, 0)
        b = ifl.Batch(members, use_graph=use_graph, max_team_blocks=args.max_team_blocks, threads=t,
                      strips_per_block=k, stages=st)
        for i, sc in enumerate(scs):
            b.set_inflows(i, sc.inflows)
        return b, members, bodies

    def step(b, bodies, dt):
        b.update(dt)
        for bs in bodies:
            for x in bs:
                x.update(dt)

    dt = scs[0].dt
    b, members, bodies = build()
    be, members_e, bodies_e = build()
    for _ in range(args.warmup):
        step(b, bodies, dt)
        step(be, bodies_e, dt)
    info0 = b.info()
    step_ms, pcg_ms, pcg_bytes, kernel_bytes = [], [], 0.0, 0.0
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    launches0 = info0["launches"]
    with ClockSampler(local_rank) as clk:
        for k in range(args.steps):
            step(b, bodies, dt)
            inf = b.info()
            step_ms.append(inf["last_step_ms"])
            pcg_ms.append(inf["last_pcg_ms"])
            st = b.stats()
            for sc, x in zip(scs, st):
                if x[2] & 1:
                    raise RuntimeError("device-side wait timed out during the benchmark")
                pcg_bytes += sc.cells * pcg_bytes_per_cell(fbytes, x[0][0])
                kernel_bytes += sc.cells * pcg_kernel_bytes_per_cell(fbytes, x[0][0])
    torch.cuda.synchronize(dev)
    info = b.info()
    launches = info["launches"] - launches0
    iters = [x[0][0] for x in b.stats()]
    dev_ms = sum(step_ms)
    t_max = max_over_ranks(dev_ms, world, dev)
    value = cells_all * args.steps / (t_max / 1e3)

    # ---- per-field error of one more (untimed) step of a size-stratified sample
    check = None
    if args.field_check > 0 and rank == 0:
        pick = stratified(scs, args.field_check)
        jobs = [(scs[i].variant, scs[i].w, scs[i].h, gpu_state(ifl, members[i], scs[i].variant),
                 [x.as_tuple() for x in bodies[i]], scs[i].inflows, dt) for i in pick]
        step(b, bodies, dt)
        st = b.stats()
        outs = [gpu_result(ifl, members[i], scs[i].variant) for i in pick]
        check_args = (jobs, outs, [st[i][0][0] for i in pick])

    # ---- end to end through the public API: pinned density readback of every scene
    host = [torch.empty((sc.h, sc.w), dtype=torch.float32, pin_memory=True).numpy() for sc in scs]
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    h2d = 0
    for k in range(args.steps):
        step(be, bodies_e, dt)
        h2d += be.info()["h2d_bytes_last_step"]
        for m, hb in zip(members_e, host):
            m.read_field("d", dtype=np.float32, out=hb)
    e2e_s = max_over_ranks(time.perf_counter() - t0, world, dev)
    e2e = {"value": cells_all * args.steps / e2e_s, "unit": METRIC,
           "h2d_bytes_per_step": int(h2d / args.steps),
           "d2h_bytes_per_step": int(cells * 4 + be.info()["d2h_bytes_last_step"])}
    be.close()
    del members_e

    # ---- roofline of the batched PCG kernel
    peak, peak_kind = load_peaks()
    achieved = pcg_bytes / (sum(pcg_ms) / 1e3) / 1e9 if sum(pcg_ms) > 0 else 0.0
    # DRAM traffic of one launch: the full batch is too large to capture under
    # the profiler's size rule, so it is scaled from a DRAM-only capture of 32
    # tall scenes (6.9 M cells, working set ~4x the L2, 20 pinned iterations),
    # where the kernel moved 1.00x its algorithmic bytes
    traffic_ratio = 1.00
    roof = {"bound": "hbm", "kernel": "pcg_batch_kernel", "achieved": round(achieved, 1), "peak": peak,
            "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_kind": f"of {peak_kind}",
            "traffic": round(traffic_ratio * pcg_bytes / args.steps),
            "traffic_source": "scaled from a 32-scene DRAM capture: 1.00 x algorithmic bytes",
            "algorithmic_bytes_per_step": round(pcg_bytes / args.steps),
            "kernel_bytes_per_step": round(kernel_bytes / args.steps),
            "kernel_bytes_gbs": round(kernel_bytes / (sum(pcg_ms) / 1e3) / 1e9, 1) if sum(pcg_ms) > 0 else 0.0,
            "pcg_ms_per_step": round(sum(pcg_ms) / args.steps, 2),
            "share_of_step": round(sum(pcg_ms) / max(dev_ms, 1e-9), 4),
            "pcg_iterations": {"max": max(iters), "mean": round(sum(iters) / len(iters), 1),
                               "cell_weighted_mean": round(sum(s.cells * i for s, i in zip(scs, iters)) / cells, 1)}}

    # ---- plain FP64 drop-in, one scene at a time, on a stratified sample
    fp64 = None
    if args.fp64_sample > 0:
        pick = stratified(scs, args.fp64_sample)
        spent, done = 0.0, 0
        for i in pick:
            sc = scs[i]
            bs = body_objs(ifl, sc)
            g = ifl.FluidSolver(sc.w, sc.h, sc.density, bs, variant=sc.variant, precision=ifl.FP64,
                                device=local_rank)
            timed = min(args.steps, 2)
            for k in range(args.warmup + timed):  # the batch's step indices: warm-up, then timed
                for r in sc.inflows:
                    g.addInflow(*r[:5], *r[6:])
                s0 = torch.cuda.ExternalStream(g.stream, device=dev)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                with torch.cuda.stream(s0):
                    e0.record(s0)
                g.update(sc.dt)
                with torch.cuda.stream(s0):
                    e1.record(s0)
                g.synchronize()
                if k >= args.warmup:
                    spent += e0.elapsed_time(e1) / 1e3
                    done += sc.cells
                for x in bs:
                    x.update(sc.dt)
            g.close()
        fp64 = {"value": done / spent, "unit": METRIC,
                "sample": f"{len(pick)} of the {len(scs)} scenes (size-stratified), FP64 drop-in "
                          f"(ifl_update), one scene at a time, updates {args.warmup + 1}..{args.warmup + timed} "
                          f"of each timed (after {args.warmup} untimed, as the batch)"}
    b.close()
    if args.field_check > 0 and rank == 0:
        check = field_error_check(*check_args, procs=min(16, os.cpu_count() or 1))
        check["sample"] = (f"{len(check_args[0])} size-stratified scenes of the batch at update "
                           f"{args.warmup + args.steps + 1}")
    lat = sorted(step_ms)
    pct = lambda q: lat[min(len(lat) - 1, int(math.ceil(q * len(lat))) - 1)]
    return {"value": value, "ms_per_step": t_max / args.steps, "e2e": e2e, "roofline": roof,
            "field_error": check, "shard": {"scenes": len(scs), "of": len(allscs), "cells": cells,
                                            "cells_all_ranks": int(cells_all)},
            "gpu_launches": launches, "clocks": clk.summary(), "fp64_dropin": fp64, "cells": cells,
            "latency_ms": {"p50": round(pct(0.50), 1), "p99": round(pct(0.99), 1)},
            "batch": {k: info[k] for k in ("members", "threads", "strips_per_block", "stages", "grid", "graph",
                                           "candidate_ms", "tiles", "tile_ms")}}


# ------------------------------------------------------------- serving
def run_serve(args, local_rank):
    """Open-loop Poisson arrivals of batch-generator scenes through ifl_server_*,
    against the plain FP64 drop-in serving one request at a time (FCFS)."""
    import torch
    import ifluids as ifl
    from ifluids import scenes

    rng = np.random.default_rng(4)
    scs = scenes.batch_scenes(count=args.serve_requests, seed=4)
    steps = [max(1, int(round(int(rng.integers(50, 501)) * args.serve_steps_scale))) for _ in scs]
    gaps = rng.exponential(1.0 / args.serve_rate, size=len(scs))
    offsets = np.cumsum(gaps) - gaps[0]
    prec = ifl.FP32 if args.precision == "fp32" else ifl.FP64
    srv = ifl.Server(precision=prec, device=local_rank, hbm_budget_bytes=int(args.serve_budget_gb * 2**30))
    t0 = srv.now() + 0.05
    nxt, lat, cell_steps, finished, peak = 0, [], 0, 0, 0
    while finished < len(scs):
        now = srv.now()
        while nxt < len(scs) and t0 + offsets[nxt] <= now:
            sc = scs[nxt]
            srv.submit(sc.w, sc.h, steps[nxt], sc.bodies, sc.inflows, arrival=t0 + offsets[nxt])
            nxt += 1
        a, q = srv.step()
        peak = max(peak, a)
        for c in srv.completions():
            lat.append(c["finished"] - c["arrival"])
            cell_steps += c["w"] * c["h"] * c["steps"]
            srv.release(c["id"])
            finished += 1
        if a == 0 and q == 0 and nxt < len(scs):
            time.sleep(max(0.0, t0 + offsets[nxt] - srv.now()))
    wall = srv.now() - t0
    info = srv.info()
    srv.close()

    # plain FP64 drop-in serving one request at a time, for real on the same
    # arrivals: requests in arrival order, each waits for its arrival and for
    # the previous one, then runs all its updates through ifl_update
    lat64, work = [], 0
    t64 = time.perf_counter()
    for k, sc in enumerate(scs):
        if args.serve_no_fp64:
            work += sc.cells * steps[k]
            continue
        wait = offsets[k] - (time.perf_counter() - t64)
        if wait > 0:
            time.sleep(wait)
        bs = body_objs(ifl, sc)
        g = ifl.FluidSolver(sc.w, sc.h, sc.density, bs, variant=sc.variant, precision=ifl.FP64, device=local_rank)
        for _ in range(steps[k]):
            for r in sc.inflows:
                g.addInflow(*r[:5], *r[6:])
            g.update(sc.dt)
            for x in bs:
                x.update(sc.dt)
        g.synchronize()
        g.close()
        lat64.append(time.perf_counter() - t64 - offsets[k])
        work += sc.cells * steps[k]
    wall64 = time.perf_counter() - t64

    def pct(v, q):
        v = sorted(v)
        return v[min(len(v) - 1, int(math.ceil(q * len(v))) - 1)]
    span = float(offsets[-1] - offsets[0]) if len(offsets) > 1 else 0.0
    offered = work / span if span > 0 else float("inf")
    served = cell_steps / wall
    return {"requests": len(scs), "arrival_rate_per_s": args.serve_rate,
            "steps_per_request": f"U[50,500] x {args.serve_steps_scale}",
            "p50_latency_s": round(pct(lat, 0.5), 3), "p99_latency_s": round(pct(lat, 0.99), 3),
            "cell_steps_per_s": round(served, 1), "wall_s": round(wall, 2), "peak_active": peak,
            "admitted": info["admitted"], "completed": info["completed"], "peak_queued": info["peak_queued"],
            "offered_cell_steps_per_s": round(offered, 1),
            "overload": bool(offered > served),
            "load_note": ("offered load above what one GPU serves: requests queue and latency grows with the run"
                          if offered > served else "offered load within capacity"),
            "batch_rebuilds": info["rebuilds"], "rebuild_ms_total": round(info["rebuild_ms"], 1),
            "rebuild_ms_per_membership_change": round(info["rebuild_ms"] / max(1, info["rebuilds"]), 2),
            "hbm_budget_gb": args.serve_budget_gb,
            "fp64_one_at_a_time": None if args.serve_no_fp64 else
            {"p50_latency_s": round(pct(lat64, 0.5), 3), "p99_latency_s": round(pct(lat64, 0.99), 3),
             "cell_steps_per_s": round(work / wall64, 1), "wall_s": round(wall64, 2),
             "how": "run: FP64 drop-in (ifl_update), one request at a time in arrival order on the same arrivals"}}


# ------------------------------------------------------- profiler case
def run_profile_case(args):
    """A small, reproducible batched-PCG launch for profiler captures (not a
    benchmark): the tall scenes (more than 512 rows) among the first
    --case-pool scenes of the batched-form generator (the class that dominates
    a full step), every PCG solve pinned to --case-iterations iterations so a
    launch is short and identical from run to run, three updates; prints the
    PCG time of each update."""
    import ifluids as ifl
    from ifluids import scenes
    threads, k, stages = (int(x) for x in (args.shape or "64,1,2").split(","))
    sc = [x for x in scenes.batch_scenes(count=args.case_pool, seed=BATCH_SEED) if x.h > 512][:args.count]
    print("scenes", len(sc), "cells", sum(x.w * x.h for x in sc), flush=True)
    members = [ifl.FluidSolver(x.w, x.h, x.density, body_objs(ifl, x), precision=ifl.FP32) for x in sc]
    for m in members:
        m.set_pinned_iterations(args.case_iterations, -1)
    b = ifl.Batch(members, threads=threads, strips_per_block=k, stages=stages, use_graph=False)
    for i, x in enumerate(sc):
        b.set_inflows(i, x.inflows)
    for u in range(3):
        b.update(sc[0].dt)
        print(u, round(b.info()["last_pcg_ms"], 3), "ms", [x[0][0] for x in b.stats()], flush=True)
    b.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--workload", choices=("batch", "single", "c3", "flip", "gs", "case"), default="batch",
                    help="case: the small pinned batch used for profiler captures (prints timings, no bench line)")
    ap.add_argument("--case-pool", type=int, default=64, help="case: generator scenes the tall ones are taken from")
    ap.add_argument("--case-iterations", type=int, default=20, help="case: PCG iterations per solve")
    ap.add_argument("--gs-variant", type=int, choices=(1, 2), default=1, help="gs workload: tutorial step 1 or 2")
    ap.add_argument("--count", type=int, default=BATCH_COUNT, help="scenes of the batched workload")
    ap.add_argument("--size", type=int, default=0, help="side of the single-scene workload (1024; c3: 2048)")
    ap.add_argument("--precision", choices=("fp32", "fp64"), default="fp32")
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--fp64-steps", type=int, default=3, help="single workload: FP64 drop-in steps")
    ap.add_argument("--fp64-sample", type=int, default=32, help="batch workload: scenes of the FP64 sample")
    ap.add_argument("--serve-requests", type=int, default=16, help="batch workload: requests of the serving run")
    ap.add_argument("--serve-rate", type=float, default=200.0, help="Poisson arrivals per second")
    ap.add_argument("--serve-steps-scale", type=float, default=0.1, help="scale of the U[50,500] steps per request")
    ap.add_argument("--serve-budget-gb", type=float, default=64.0, help="HBM budget of the serving run")
    ap.add_argument("--serve-no-fp64", action="store_true",
                    help="skip the FP64 one-at-a-time serving leg (it takes about 10x the batched leg's time)")
    ap.add_argument("--cpu-procs", type=int, default=0, help="host processes for the CPU legs (0 = auto)")
    ap.add_argument("--cpu-sample", type=int, default=32, help="batch: scenes of the CPU sample (size-stratified)")
    ap.add_argument("--max-team-blocks", type=int, default=0, help="batch: largest PCG team in blocks (0 = library default)")
    ap.add_argument("--shape", default="", help="batch: fixed PCG shape threads,strips_per_block,stages (default: autotuned)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline leg")
    ap.add_argument("--pcg-cap", type=int, default=0,
                    help="single / c3: cap the pressure PCG at this many iterations (a short launch for profiler "
                         "captures; the line then names the cap and is not the benchmark)")
    ap.add_argument("--field-check", type=int, default=-1,
                    help="scenes whose next update is compared with the FP64 reference after the timed region "
                         "(default: 8 for the batch, 1 for the 1024^2 scene, 0 otherwise)")
    args = ap.parse_args()
    if args.workload == "case":
        if args.count == BATCH_COUNT:
            args.count = 8
        run_profile_case(args)
        return
    if not args.size:
        args.size = {"c3": 2048, "flip": 128, "gs": 128}.get(args.workload, 1024)
    if args.field_check < 0:
        args.field_check = {"batch": 8, "single": 1}.get(args.workload, 0)

    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # one process per GPU: start the ranks through torch.distributed.run
        import socket
        with socket.socket() as sk:
            sk.bind(("127.0.0.1", 0))
            port = sk.getsockname()[1]
        cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={args.gpus}",
               "--master-addr=127.0.0.1", f"--master-port={port}", os.path.abspath(__file__)] + sys.argv[1:]
        sys.exit(subprocess.call(cmd))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    procs = args.cpu_procs or max(1, min(16, os.cpu_count() or 1))
    batch = args.workload == "batch"
    if batch:
        config = {"workload": f"batched form: {args.count} independent ragged scenes (sides log-uniform in "
                              f"[64, 1024], 1-3 inflow rectangles, 0-4 seeded bodies), 4-solid-boundaries, "
                              f"dt=0.0025 (configs[2])",
                  "variant": "4-solid-boundaries", "scenes": args.count, "seed": BATCH_SEED,
                  "sharding": "one GPU per rank; N ranks split the generator's first count x N scenes into "
                              "disjoint shares balanced by estimated work (no collective on the data path)",
                  "precision_form": args.precision,
                  "l2": "inputs larger than L2 (about 6 GB of scene state)", "scene_data": "seeded synthetic scenes"}
    elif args.workload == "flip":
        config = {"workload": f"FLIP particles (8-flip) on the reference main's scene {args.size}x{args.size}: "
                              f"rotated box, fixed inflow d=1 T=294 K, rhoAir 0.1, rhoSoot 0.25, diffusion 0.01, "
                              f"dt=0.0025",
                  "variant": "8-flip", "grid": [args.size, args.size], "precision_form": args.precision,
                  "precision_note": "FP64 fields and particles in both forms; fp32 = FP32-form solves",
                  "l2": "flushed between timed steps (512 MiB write)", "scene_data": "the reference's own scene"}
    elif args.workload == "gs":
        name = {1: "1-matrixless", 2: "2-better-advection"}[args.gs_variant]
        config = {"workload": f"Gauss-Seidel step {name} on the reference main's scene {args.size}x{args.size}: "
                              f"density 0.1, dt=0.005, its inflow, 600-sweep cap",
                  "variant": name, "grid": [args.size, args.size], "precision_form": "fp64",
                  "l2": "flushed between timed steps (512 MiB write)", "scene_data": "the reference's own scene"}
        args.precision = "fp64"
    elif args.workload == "c3":
        config = {"workload": f"heat + variable density scene {args.size}x{args.size} (7-variable-density), "
                              f"ambient 294 K, inflow d=1 T=700 K, the reference main's box, dt=0.001 (configs[3])",
                  "variant": "7-variable-density", "grid": [args.size, args.size], "precision_form": args.precision,
                  "l2": "flushed between timed steps (512 MiB write)", "scene_data": "seeded synthetic scene"}
        args.no_cpu = True  # one oracle update of this scene takes minutes: no bounded CPU sample
    else:
        config = {"workload": f"solid-boundary scene {args.size}x{args.size}, 3 seeded bodies, "
                              f"dt=0.0025, config-0 inflow (configs[1])",
                  "variant": "4-solid-boundaries", "grid": [args.size, args.size], "bodies": 3, "seed": args.seed,
                  "precision_form": args.precision, "l2": "flushed between timed steps (512 MiB write)",
                  "scene_data": "seeded synthetic scene"}
    if args.pcg_cap > 0 and args.workload in ("single", "c3"):
        config["pcg_cap"] = f"pressure PCG capped at {args.pcg_cap} iterations (profiling case, not the benchmark)"

    if args.impl == "reference":
        if rank != 0:
            return
        # Each step is a bounded sample of the workload, timed at the same step
        # indices as the GPU arm (after args.warmup untimed updates).
        if args.workload == "flip":
            cb = cpu_baseline_flip(args.size, args.steps, args.warmup)
            note = "step 8 on one host core, as the reference runs"
        elif args.workload == "gs":
            cb = cpu_baseline_gs(args.gs_variant, args.size, args.steps, args.warmup)
            note = "steps 1-2 on one host core, as the reference runs"
        elif batch:
            cb = cpu_baseline_batch(procs, steps=args.steps, warmup=args.warmup, sample=args.cpu_sample)
            note = ("one reference solver per sampled scene, the sample spread over the host cores; "
                    "ms_per_step is one step of the sample on its slowest process")
        else:
            steps = max(1, min(args.steps, 2))  # one update of this scene takes ~25 s per process
            cb = cpu_baseline(args.size, steps, args.warmup, procs, args.seed)
            note = ("one copy of the scene per host core; steps capped at 2 to keep the run within minutes; "
                    "ms_per_step is one update on the slowest process")
        line = {"metric": METRIC, "value": cb["value"], "unit": METRIC, "n_gpus": args.gpus,
                "steps": cb["steps"], "warmup": cb["warmup"], "ms_per_step": 1e3 * cb["seconds"] / cb["steps"],
                "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config,
                "impl": "reference", "cpu_baseline": cb,
                "e2e": {"value": cb["value"], "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "note": note}
        print(json.dumps(line), flush=True)
        return

    cb = None
    if rank == 0 and world == 1 and not args.no_cpu:  # before any GPU work (spawned pool)
        if args.workload == "flip":
            cb = cpu_baseline_flip(args.size, 10, args.warmup)
        elif args.workload == "gs":
            cb = cpu_baseline_gs(args.gs_variant, args.size, 5, args.warmup)
        elif batch:
            cb = cpu_baseline_batch(procs, steps=1, warmup=args.warmup, sample=args.cpu_sample)
        else:
            cb = cpu_baseline(args.size, 1, args.warmup, procs, args.seed)
    if world > 1:
        import torch.distributed as dist
        import torch
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    if args.workload == "flip":
        r = run_flip(args, local_rank)
    elif args.workload == "gs":
        r = run_gs(args, local_rank)
    else:
        r = run_batch(args, rank, world, local_rank) if batch else run_gpu(args, rank, world, local_rank)
    if rank != 0:
        return
    line = {"metric": METRIC, "value": r["value"], "unit": METRIC, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32" if args.precision == "fp32" else "f64",
            "data": "synthetic", "config": config, "e2e": r["e2e"], "roofline": r["roofline"],
            "cpu_baseline": cb, "gpu_launches": r["gpu_launches"], "clocks": r["clocks"],
            "fp64_dropin": r["fp64_dropin"]}
    if r.get("field_error") is not None:
        line["field_error"] = r["field_error"]
    if batch:
        line["latency_ms"] = r["latency_ms"]
        line["batch"] = r["batch"]
        line["shard"] = r["shard"]
        if args.serve_requests > 0 and world == 1:
            line["serving"] = run_serve(args, local_rank)
    elif args.workload == "gs":
        line["latency_ms"] = r["latency_ms"]
    elif args.workload == "flip":
        line["particles"] = r["particles"]
        line["particle_steps_per_s"] = r["particle_steps_per_s"]
        line["latency_ms"] = r["latency_ms"]
    else:
        line["pcg"] = {"iterations_last_step": r["pcg_iterations_last"], "status_last_step": r["pcg_status_last"]}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
