#!/usr/bin/env python
"""Benchmark of the GB300-native WCSPH step (one JSON line on rank 0).

Workload: the 1,000,000-particle dam break (100^3 lattice, spacing 0.005 m,
in [0,0.5]^3 of a 2x1x1 m box, h = 0.01 m, dt = 1e-4 s), synthetic seeded
inputs.  A step is one WCSPH substep of that scene (advance(dt, 1)).

  value      particle-steps/s with the state resident in HBM: K substeps
             replayed as a CUDA graph, CUDA events on the library's stream.
  roofline   dominant kernel from a per-pass CUDA-event region of the same
             workload (50 substeps from the middle of the timed run, replayed
             from its start state); algorithmic bytes per launch / mean
             launch time, against the measured HBM copy bandwidth.
  e2e        the fluidtest frame loop through the C ABI with host buffers
             (pinned): setupFromData (H2D) then K x (advance + exportToData
             of positions, colours, velocities to the host).
  cpu_baseline  the CPU oracle (OpenMP restatement of the reference step)
             on a bounded sample of the same scene, on this host's cores.
  large_tension  the ~8M-particle scene with surface tension (200x200x180
             pool and two falling spheres), 200 substeps, device-resident.
  batched    256 mixed-size dam breaks (2,048-65,536 particles) advanced by
             one launch per pass for 200 substeps, against the same scenes
             stepped one at a time over the same substeps.
  served     1,000 requests (1,024-262,144 particles, 50-500 substeps) under
             open-loop Poisson arrivals at 50, 100 and 2,000 requests/s:
             p50/p99 latency and aggregate particle-steps/s, against the
             plain sequential step.

--impl reference times the reference's step on host cores (the oracle port:
the reference has no CPU implementation of its own and its CUDA sources do
not travel to the GPU host).  Under torchrun every rank runs an independent
replica (the plain step does not shard); only rank 0 prints.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s at 1M; batched/served particle-steps/s & p99 vs plain"
# algorithmic bytes per particle for each pass (vec3 = 12 B, scalar = 4 B;
# each array read or written once per pass)
ALG_BYTES = {"hash": 16, "sort": 48 + 72 + 4, "density": 20, "normals": 28, "force_integrate": 80, "xsph": 40}
CELL_BYTES = 8


def _env_int(k, d):
    try:
        return int(os.environ.get(k, d))
    except ValueError:
        return d


class Dist:
    def __init__(self):
        self.world = _env_int("WORLD_SIZE", 1)
        self.rank = _env_int("RANK", 0)
        self.local = _env_int("LOCAL_RANK", 0)
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v: float) -> float:
        if not self.pg:
            return v
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v: float) -> float:
        if not self.pg:
            return v
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.pg.all_reduce(t)
        return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int, path: str | None = None):
        self.gpu = gpu
        self.proc = None
        # the raw samples: where --clocks-csv says, else a temporary file
        self.path = path or os.path.join(tempfile.gettempdir(), f"sph_clocks_{os.getpid()}_{gpu}.csv")

    def start(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self) -> dict | None:
        if not self.proc:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.fh.close()
        sm, mx, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "samples": len(sm),
                "power_w_max": max(power) if power else None, "reasons": sorted(reasons)}


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return None


def profile_traffic(kernel: str, workload: str):
    """DRAM bytes per launch from the committed ncu summary, or None."""
    path = os.path.join(ROOT, "profiles", f"traffic_{workload}.txt")
    try:
        for line in open(path):
            p = line.split()
            if len(p) >= 2 and p[0] == kernel:
                return float(p[1])
    except OSError:
        pass
    return None


def profile_counters(kernel: str, workload: str):
    """Issue-side ncu counters of a kernel from the committed summary, or None:
    the neighbour passes are bound by instruction issue and gather latency,
    which the HBM fraction alone does not show."""
    path = os.path.join(ROOT, "profiles", f"counters_{workload}.txt")
    keys = ("issue_active_pct", "lanes_per_inst", "fma_pipe_pct", "alu_pipe_pct", "dram_pct", "l1tex_pct",
            "lts_pct")
    try:
        for line in open(path):
            p = line.split()
            if len(p) == 1 + len(keys) and p[0] == kernel:
                d = {k: float(v) for k, v in zip(keys, p[1:])}
                d["source"] = f"profiles/counters_{workload}.txt (ncu --set full)"
                return d
    except OSError:
        pass
    return None


def configure(fs, spec, pos, vel):
    fs.init(spec.n, spec.unit_cube_res or 1)
    if not spec.unit_cube_res:
        fs.setDomain(*spec.box, spec.h)
    p = spec.params()
    fs.setParams(rest_density=p["rest_density"], mass=p["mass"], gamma=p["gamma"], gas_constant=p["gas_constant"],
                 viscosity=p["viscosity"], xsph=p["xsph"], surface_tension=p["surface_tension"],
                 adhesion=p["adhesion"], vdamp=p["vdamp"], particle_size=p["particle_size"],
                 vel_limit=p["vel_limit"], acc_limit=p["acc_limit"], gravity=p["gravity"], dt=p["dt"])
    fs.setState(pos, vel)


def configure_oracle(o, spec, pos, vel):
    o.init(spec.n, spec.unit_cube_res or 1)
    if not spec.unit_cube_res:
        o.set_domain(*spec.box, spec.h)
    for k, v in spec.params().items():
        if k == "gravity":
            o.set_gravity(*v)
        elif k not in ("vel_limit", "acc_limit"):
            o.set_param(k, v)
    o.set_limits(spec.vel_limit, spec.acc_limit)
    o.set_state(pos, vel)


def workload(name: str):
    from libfluid_gb300 import workloads as W
    if name == "dam_break_1m":
        return W.dam_break_1m(), ("1M dam break: 100^3 lattice, spacing 0.005 m, in [0,0.5]^3 of a 2x1x1 m box, "
                                  "h=0.01 m, dt=1e-4 s, c0=20 m/s, visc 0.01, XSPH 0.5, no surface tension")
    if name == "dam_break_1m_cube":
        return W.dam_break_1m(unit_cube=True), "1M dam break in the reference's unit cube (res 100, h=0.01 m)"
    if name == "small_dam_break":
        return W.small_dam_break(), "32,768-particle dam break in a 1.0x0.6x0.6 m box, h=0.02 m, dt=2e-4 s"
    if name == "small_dam_break_cube":
        return (W.small_dam_break(unit_cube=True),
                "32,768-particle dam break in the reference's unit cube (res 50, h=0.02 m)")
    if name == "large_tension":
        return W.large_tension(), ("8,005,232 particles with surface tension 0.0728: 200x200x180 lattice pool plus "
                                   "falling spheres, h=0.01 m, dt=8e-5 s")
    raise SystemExit(f"unknown workload {name}")


def cpu_oracle_rate(spec, pos, vel, budget_s: float, max_steps: int, warmup: int = 1):
    """Time the oracle on this host's cores; returns (rate, steps, seconds, threads)."""
    import oracle
    threads = oracle.set_threads(os.cpu_count() or 1)
    o = oracle.Oracle(32)
    configure_oracle(o, spec, pos, vel)
    for _ in range(warmup):
        o.advance(spec.dt, 1)
    t0 = time.perf_counter()
    o.advance(spec.dt, 1)
    t1 = time.perf_counter() - t0
    steps = 1
    target = max(1, min(max_steps - 1, int(budget_s / max(t1, 1e-6)) - 1))
    t0 = time.perf_counter()
    for _ in range(target):
        o.advance(spec.dt, 1)
    tt = time.perf_counter() - t0 + t1
    steps += target
    return spec.n * steps / tt, steps, tt, threads


def run_reference(args, dist):
    spec, desc = workload(args.workload)
    if dist.rank != 0:
        return
    pos, vel = spec.positions(), spec.velocities()
    budget = float(os.environ.get("SPH_REF_BUDGET_S", "120"))
    rate, steps, secs, threads = cpu_oracle_rate(spec, pos, vel, budget, max(1, args.steps), warmup=min(args.warmup, 1))
    sample = (f"{steps} substeps of the {spec.n}-particle scene in {secs:.1f} s "
              f"(of {args.steps} requested; capped at ~{budget:.0f} s of CPU work)")
    line = {"metric": METRIC, "value": rate, "unit": "particle-steps/s", "n_gpus": args.gpus, "steps": steps,
            "warmup": min(args.warmup, 1), "ms_per_step": 1e3 * secs / steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": desc, "particles": spec.n, "substeps_per_step": 1},
            "cpu_baseline": {"value": rate, "unit": "particle-steps/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": rate, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "the reference has no CPU step; this is the oracle's OpenMP restatement of its cudasrc kernels"}
    print(json.dumps(line), flush=True)


def reference_cuda_compare(args, fs):
    """Time NCCA/libfluid's own device code (compiled unmodified from its
    sources, driven by oracle/ref_runner.cu) and this library on the same
    1M-particle scene in the reference's unit cube (res 100, h = 0.01 m)."""
    from oracle import ref_cuda
    if not ref_cuda.available():
        return {"unavailable": "oracle/_ref/libfluid_ref.cubin not built (needs the reference sources)"}
    # the unit-cube form of the workload measured (the reference has no other domain)
    spec, desc = workload("small_dam_break_cube" if args.workload == "small_dam_break" else "dam_break_1m_cube")
    pos, vel = spec.positions(), spec.velocities()
    p = spec.params()
    rp = dict(p)
    rp["gx"], rp["gy"], rp["gz"] = p["gravity"]
    k = max(10, min(args.steps, 200))
    try:
        t = ref_cuda.time_steps(pos, vel, spec.unit_cube_res, spec.dt, rp, warmup=3, steps=k)
    except Exception as e:  # the reference's failure is reported, not raised
        return {"unavailable": f"reference runner failed: {str(e)[:200]}"}
    ref_rate = spec.n * t["steps"] / (t["ms"] * 1e-3)
    configure(fs, spec, pos, vel)
    for _ in range(3):
        fs.advance(spec.dt, 1)
    fs.sync()
    fs.timerMark(2)
    for _ in range(k):
        fs.advanceAsync(spec.dt, 1)
    fs.timerMark(3)
    ms = fs.timerElapsed(2, 3)
    fs.sync()
    ours = spec.n * k / (ms * 1e-3)
    return {"workload": desc, "steps": k, "value": ref_rate, "unit": "particle-steps/s",
            "ms_per_step": t["ms"] / t["steps"], "ours_value": ours, "ours_ms_per_step": ms / k,
            "speedup": ours / ref_rate,
            "how": "reference cudasrc kernels + thrust hash/sort/scan/reduce, its 4 syncs and blocking reduce per "
                   "substep (oracle/ref_runner.cu); CUDA events around both loops after 3 warm-up substeps"}


def run_ours(args, dist):
    from libfluid_gb300 import FluidSystem, _capi
    spec, desc = workload(args.workload)
    pos, vel = spec.positions(), spec.velocities()
    n = spec.n
    fs = FluidSystem(dist.local)
    configure(fs, spec, pos, vel)
    L = _capi.lib()
    if args.variant is not None or args.tile is not None or args.persistent is not None:
        fs.setExec(tile=args.tile or 128, persistent=args.persistent or 0,
                   variant=63 if args.variant is None else args.variant)

    # ---- warm-up ----
    for _ in range(args.warmup):
        fs.advance(spec.dt, 1)
    fs.sync()
    start_state = fs.snapshot()   # the per-pass region below replays the timed run from here

    # ---- timed region: K substeps as CUDA-graph replays, state resident ----
    clocks = ClockSampler(dist.local, args.clocks_csv)
    clocks.start()
    dist.barrier()
    fs.sync()
    fs.timerMark(0)
    for _ in range(args.steps):
        fs.advanceAsync(spec.dt, 1)
    fs.timerMark(1)
    ms = fs.timerElapsed(0, 1)
    fs.sync()
    dist.barrier()
    clk = clocks.stop()
    ms_max = dist.max(ms)
    total = dist.sum(float(n) * args.steps)
    value = total / (ms_max * 1e-3)

    # ---- per-pass region: CUDA events around every pass (eager launches) ----
    # over substeps from the middle of the timed run (the scene compresses as
    # it runs, so its first or last substeps would misstate the average one):
    # the timed run's start state, advanced half of its substeps, untimed
    prof_steps = max(3, min(args.steps, 50))
    fs.restore(start_state)
    for _ in range(max(0, args.steps // 2 - prof_steps // 2)):
        fs.advanceAsync(spec.dt, 1)
    fs.sync()
    fs.setProfiling(True)
    for _ in range(prof_steps):
        fs.advance(spec.dt, 1)
    passes, nsub = fs.passTimes()
    fs.setProfiling(False)
    per_launch = {k: v / max(nsub, 1) for k, v in passes.items()}
    cells = int(np.prod([int(np.ceil(b / spec.h - 1e-3)) for b in spec.box])) if not spec.unit_cube_res else \
        spec.unit_cube_res ** 3
    kern = {k: v for k, v in per_launch.items() if k not in ("substep",) and v > 0}
    dom = max(kern, key=kern.get)
    alg_bytes = dict(ALG_BYTES)
    if per_launch.get("hash", 0.0) < 0.05 * per_launch.get("force_integrate", 1.0):
        # the force pass hashed its output (reads nothing more; key and slot
        # written, 8 B) and the hash pass only cleared the substep scalars
        alg_bytes["force_integrate"] += 8
    if per_launch.get("xsph", 0.0) < 0.05 * per_launch.get("density", 1.0):
        # deferred XSPH: the update runs inside the density pass (its reads and
        # writes: P, V, rho 28 B, V 12 B) and there is no XSPH pass
        alg_bytes["density"] += alg_bytes["xsph"]
    alg = alg_bytes.get(dom, 0) * n + (CELL_BYTES * cells if dom == "scan" else 0)
    peaks = measured_peaks()
    peak = peaks["hbm_gbs"] if peaks else 6800.0
    achieved = alg / (per_launch[dom] * 1e-3) / 1e9
    traffic = profile_traffic(dom, args.workload)
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic,
                "alg_bytes_per_launch": alg, "mean_launch_ms": per_launch[dom],
                "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if peaks else "fallback 6.8 TB/s",
                "step_alg_bytes": sum(ALG_BYTES[k] for k in ("hash", "sort", "density", "force_integrate", "xsph"))
                * n + CELL_BYTES * cells,
                "pass_share": {k: v / per_launch["substep"] for k, v in kern.items()},
                "issue": profile_counters(dom, args.workload),
                "window": f"{prof_steps} eager substeps from substep {args.warmup + max(0, args.steps // 2 - prof_steps // 2)} "
                          f"of the timed run (the middle of its {args.steps}), CUDA events around every pass"}
    roofline["step_frac"] = roofline["step_alg_bytes"] / (ms_max / args.steps * 1e-3) / 1e9 / peak

    # ---- end to end through the C ABI with pinned host buffers ----
    e2e = None
    if not args.skip_e2e:
        hp = np.ascontiguousarray(pos)
        hv = np.ascontiguousarray(vel)
        outs = [np.empty((n, 3), np.float32) for _ in range(3)]
        bufs = [hp, hv] + outs
        for b in bufs:
            L.sph_host_register(b.ctypes.data, b.nbytes)
        k_e2e = args.steps
        fs.sync()
        dist.barrier()
        t0 = time.perf_counter()
        fs.setState(hp, hv)
        for _ in range(k_e2e):
            fs.advance(spec.dt, 1)
            fs.exportToData(*outs)
        t1 = time.perf_counter()
        for b in bufs:
            L.sph_host_unregister(b.ctypes.data)
        secs = dist.max(t1 - t0)
        e2e = {"value": dist.sum(float(n) * k_e2e) / secs, "unit": "particle-steps/s",
               "h2d_bytes_per_step": int((hp.nbytes + hv.nbytes) / k_e2e), "d2h_bytes_per_step": 3 * n * 12,
               "loop": "setupFromData then per step advance(dt,1) + exportToData (fluidtest frame loop)"}

    # ---- CPU baseline (rank 0 at N=1 only) ----
    cpu = None
    if not args.skip_cpu and dist.world == 1:
        rate, steps, secs, threads = cpu_oracle_rate(spec, pos, vel, float(os.environ.get("SPH_CPU_BUDGET_S", "20")),
                                                     1000)
        cpu = {"value": rate, "unit": "particle-steps/s", "cores": threads, "kind": "port",
               "sample": f"{steps} substeps of the same {n}-particle scene on the host, {secs:.1f} s"}

    # ---- the reference's own CUDA step on its unit-cube domain, beside ours ----
    refcuda = None
    if not args.skip_refcuda and dist.world == 1:
        refcuda = reference_cuda_compare(args, fs)

    # ---- the two systems forms, on their own workloads (rank 0 at N=1) ----
    batched = served = tension = None
    if not args.skip_systems and dist.world == 1:
        # the third plain configuration: ~8M particles with surface tension
        tension = measure_plain(dist, "large_tension", args.batched_steps, 5)
        batched = measure_batched(dist, args.scenes, args.batched_steps, 3)
        served = measure_served(dist, args.served_requests, args.served_rates)

    # the one-pass scan, scatter, rank+gather, density, force+integrate (which
    # also hashes the next substep) (+ normals with surface tension, + the
    # XSPH pass when it is not deferred into the next density pass); the
    # memsets are not kernels, and the warm-up's first substep ran the hash
    deferred = per_launch.get("xsph", 0.0) < 0.05 * per_launch.get("density", 1.0)
    launches_per_substep = 5 + (1 if spec.surface_tension != 0.0 else 0) + (0 if deferred else 1)
    line = {"metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": dist.world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": desc, "particles": n, "cells": cells, "substeps_per_step": 1,
                       "l2": "inputs larger than L2 (%.0f MB resident state+grid > 129 MB L2)" %
                             ((n * 160 + cells * 8) / 1e6),
                       "parallelism": "replicas" if dist.world > 1 else "single GPU",
                       "timing": "CUDA events on the library stream, graph replay"},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "reference_cuda": refcuda,
            "large_tension": tension, "batched": batched, "served": served,
            "gpu_launches": launches_per_substep * args.steps, "clocks": clk,
            "passes_ms_per_substep": per_launch,
            "published_reference": {"value": 7.7e7, "unit": "particle-steps/s",
                                    "note": "README: 1M particles at 77 FPS on an RTX 2080; grid, dt and substeps "
                                            "unstated, so not the same configuration"}}
    if dist.rank == 0:
        print(json.dumps(line), flush=True)


def measure_plain(dist, workload_name: str, steps: int, warmup: int) -> dict:
    """Another plain scene of the same library (device-resident state, graph
    replay, CUDA events on the library's stream)."""
    from libfluid_gb300 import FluidSystem
    spec, desc = workload(workload_name)
    fs = FluidSystem(dist.local)
    configure(fs, spec, spec.positions(), spec.velocities())
    for _ in range(warmup):
        fs.advance(spec.dt, 1)
    fs.sync()
    fs.timerMark(0)
    for _ in range(steps):
        fs.advanceAsync(spec.dt, 1)
    fs.timerMark(1)
    ms = fs.timerElapsed(0, 1)
    fs.sync()
    fs.close()
    return {"workload": desc, "particles": spec.n, "value": spec.n * steps / (ms * 1e-3), "unit": "particle-steps/s",
            "steps": steps, "warmup": warmup, "ms_per_step": ms / steps,
            "timing": "CUDA events on the library stream, graph replay"}


BATCH_DESC = ("dam-break scenes, particles log-uniform [2048, 65536], aspect [0.5,2], box 2x/1.2x the block, "
              "visc U[0.005,0.05], tension U[0,0.07], spacing 0.01 m, h 0.02 m, dt 2e-4 s")


def measure_batched(dist, num_scenes: int, steps: int, warmup: int, clocks_csv=None, manifest=None) -> dict:
    """Mixed-size dam breaks (2,048-65,536 particles each) advanced by one
    launch per pass, against the plain step run one scene at a time over the
    same substeps (each scene alone after the same warm-up)."""
    from libfluid_gb300 import workloads as W
    from libfluid_gb300.batch import Batch
    from libfluid_gb300 import autotune
    specs = W.batch_manifest(num_scenes=num_scenes, seed=7)
    if manifest and dist.rank == 0:
        write_manifest(manifest, W.manifest(specs, workload="batched", seed=7))
    exe = autotune.load("batched") or {}
    b = Batch(dist.local)
    b.set_exec(**exe)
    for s in specs:
        b.add_scene(s)
    total_n = sum(s.n for s in specs)
    for _ in range(warmup):
        b.step(1)
    clocks = ClockSampler(dist.local, clocks_csv)
    clocks.start()
    b.sync()
    b.timer_mark(0)
    for _ in range(steps):
        b.step_async(1)
    b.timer_mark(1)
    ms = b.timer_elapsed(0, 1)
    b.sync()
    clk = clocks.stop()
    value = total_n * steps / (ms * 1e-3)
    b.close()
    # the plain step, one scene at a time: each scene in its own engine, the
    # same warm-up, then the same substeps timed (graph replay).  A scene
    # alone is small enough for the split density scan (variant bit 0x20),
    # which the batch's own launches are too large to take.
    plain_exe = dict(exe)
    plain_exe["variant"] = exe.get("variant", 63) | 0x20
    plain_ms = 0.0
    for s in specs:
        one = Batch(dist.local)
        one.set_exec(**plain_exe)
        one.add_scene(s)
        for _ in range(warmup):
            one.step(1)
        one.sync()
        one.timer_mark(0)
        for _ in range(steps):
            one.step_async(1)
        one.timer_mark(1)
        plain_ms += one.timer_elapsed(0, 1)
        one.close()
    plain = total_n * steps / (plain_ms * 1e-3)
    return {"value": value, "unit": "particle-steps/s", "steps": steps, "warmup": warmup, "ms_per_step": ms / steps,
            "scenes": len(specs), "particles": total_n,
            "workload": f"{len(specs)} {BATCH_DESC}",
            "timing": "CUDA events, graph replay, one launch per pass",
            "exec": exe or "engine defaults",
            "plain_one_at_a_time": {"value": plain, "steps": steps, "warmup": warmup, "exec": plain_exe,
                                    "how": "each scene alone in its own engine, the same warm-up and the same "
                                           "substeps, graph replay, summed device time"},
            "speedup_vs_plain": value / plain, "clocks": clk}


def run_batched(args, dist):
    r = measure_batched(dist, args.scenes, args.steps, args.warmup, args.clocks_csv, args.manifest)
    line = {"metric": METRIC, "workload": "batched", "value": r["value"], "unit": "particle-steps/s",
            "n_gpus": dist.world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": r["workload"], "scenes": r["scenes"], "particles": r["particles"],
                       "timing": r["timing"], "exec": r["exec"]},
            "plain_one_at_a_time": r["plain_one_at_a_time"], "speedup_vs_plain": r["speedup_vs_plain"],
            "clocks": r["clocks"]}
    if dist.rank == 0:
        print(json.dumps(line), flush=True)


def write_manifest(path: str, m: dict) -> None:
    """The workload's scenes (and arrival times) as JSON (workloads.manifest)."""
    with open(path, "w") as f:
        json.dump(m, f)


def served_requests(count: int, seed: int):
    """Requests of the served workload: dam breaks as in the batched set but
    with particles log-uniform in [1,024, 262,144] and substeps uniform in
    [50, 500]."""
    from libfluid_gb300 import workloads as W
    specs = W.batch_manifest(num_scenes=count, seed=seed, nmin=1024, nmax=262144)
    rng = np.random.default_rng(seed + 1)
    steps = rng.integers(50, 501, size=count)
    return specs, [int(x) for x in steps]


def measure_served(dist, num_requests: int, rates, manifest=None, plain_sample: int = 1 << 30) -> dict:
    """Open-loop Poisson arrivals at each rate; p50/p99 latency (arrival to
    final state on the host) and aggregate particle-steps/s, against the
    plain sequential step on the same requests."""
    import threading
    from libfluid_gb300 import workloads as W
    from libfluid_gb300.batch import Batch
    from libfluid_gb300.server import Server
    specs, steps = served_requests(num_requests, seed=13)
    work = sum(s.n * k for s, k in zip(specs, steps))
    # plain sequential step: each request alone, from its initial state for
    # all of its substeps (graph replay), device time; every request by
    # default (a sample of a few hundred moved the rate by 10-15%: it follows
    # the mean scene size).  One engine serves them in turn, each scene alone
    # in it; step_async(0) brings its layout and graphs up to date first, so
    # the timed region holds the substeps alone.
    plain_ms = 0.0
    sample = list(range(0, len(specs), max(1, len(specs) // max(1, plain_sample))))
    sample_work = 0
    one = Batch(dist.local)
    for i in sample:
        sid = one.add_scene(specs[i])
        one.step_async(0)
        one.timer_mark(0)
        one.step_async(steps[i])
        one.timer_mark(1)
        plain_ms += one.timer_elapsed(0, 1)
        sample_work += specs[i].n * steps[i]
        one.remove_scene(sid)
    one.close()
    plain_rate = sample_work / (plain_ms * 1e-3)
    results = []
    rng = np.random.default_rng(99)
    all_gaps = [rng.exponential(1.0 / rate, size=len(specs)) for rate in rates]
    if manifest and dist.rank == 0:
        arrivals = {str(rate): np.cumsum(g).tolist() for rate, g in zip(rates, all_gaps)}
        write_manifest(manifest, W.manifest(specs, steps, workload="served", seed=13,
                                            arrival_seconds_per_rate=arrivals))
    for rate, gaps in zip(rates, all_gaps):
        srv = Server(dist.local, memory_budget=100 << 30)
        ids = [None] * len(specs)
        t0 = time.perf_counter()

        def producer():
            t = t0
            for i, (s, k) in enumerate(zip(specs, steps)):
                t += gaps[i]
                d = t - time.perf_counter()
                if d > 0:
                    time.sleep(d)
                ids[i] = srv.submit(s, k)

        th = threading.Thread(target=producer)
        th.start()
        th.join()
        srv.drain(-1)
        wall = time.perf_counter() - t0
        lat = []
        first, last = 1e30, 0.0
        for rid in ids:
            ts, ta, td = srv.times(rid)
            lat.append(td - ts)
            first, last = min(first, ts), max(last, td)
        st = srv.stats()
        srv.close()
        lat = np.asarray(lat)
        results.append({"rate_req_s": rate, "requests": len(specs), "p50_s": float(np.percentile(lat, 50)),
                        "p99_s": float(np.percentile(lat, 99)), "mean_s": float(lat.mean()),
                        "throughput": work / (last - first), "offered": rate * work / len(specs),
                        "wall_s": wall, "busy_frac": st["busy_seconds"] / max(last - first, 1e-9),
                        "peak_live_particles": st["peak_live_particles"], "iterations": st["iterations"],
                        "host_seconds": {"admit": st["admit_seconds"], "read": st["read_seconds"],
                                         "layout": st["layout_seconds"]},
                        "admit_retries": st["admit_retries"]})
    best = max(r["throughput"] for r in results)
    return {"value": best, "unit": "particle-steps/s",
            "workload": f"{len(specs)} requests: dam breaks as in the batched set, particles log-uniform "
                        "[1024, 262144], substeps U[50,500], open-loop Poisson arrivals, 100 GB budget",
            "requests": len(specs), "offered_particle_steps": work,
            "plain_sequential": {"value": plain_rate, "requests": len(sample),
                                 "how": f"{len(sample)} of the {len(specs)} requests alone in one engine, each "
                                        "from its initial state for all of its substeps, device time (graph "
                                        "replay)"},
            "speedup_vs_plain": best / plain_rate, "rates": results}


def run_served(args, dist):
    r = measure_served(dist, args.requests, args.rates, args.manifest, plain_sample=args.plain_sample)
    line = {"metric": METRIC, "workload": "served", "unit": "particle-steps/s", "value": r["value"],
            "higher_is_better": True, "n_gpus": dist.world, "dtype": "f32", "data": "synthetic",
            "config": {"workload": r["workload"], "requests": r["requests"], "memory_budget_bytes": 100 << 30,
                       "offered_particle_steps": r["offered_particle_steps"]},
            "plain_sequential": r["plain_sequential"], "speedup_vs_plain": r["speedup_vs_plain"],
            "rates": r["rates"]}
    if dist.rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="dam_break_1m")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--skip-refcuda", action="store_true")
    ap.add_argument("--manifest", default=None,
                    help="batched/served workloads: write their scenes (and arrival times) to this JSON file")
    ap.add_argument("--clocks-csv", default=None,
                    help="keep the nvidia-smi clock samples of the timed region in this CSV file")
    ap.add_argument("--tile", type=int, default=None, choices=[64, 128, 256],
                    help="plain workload: particles per tile (threads per block; default: the compiled default)")
    ap.add_argument("--persistent", type=int, default=None,
                    help="plain workload: persistent blocks per SM of the neighbour passes (default: one block per tile)")
    ap.add_argument("--variant", type=int, default=None,
                    help="plain workload: kernel variant bits (SPH_VARIANT_*; default: the compiled default)")
    ap.add_argument("--skip-systems", action="store_true",
                    help="plain workload: leave out the batched and served measurements")
    ap.add_argument("--batched-steps", type=int, default=200,
                    help="plain workload: substeps of its batched measurement")
    ap.add_argument("--served-requests", type=int, default=1000,
                    help="plain workload: requests of its served measurement")
    ap.add_argument("--served-rates", type=float, nargs="+", default=[50, 100, 2000],
                    help="plain workload: arrival rates (req/s) of its served measurement")
    ap.add_argument("--scenes", type=int, default=256, help="batched workload: number of scenes")
    ap.add_argument("--requests", type=int, default=400, help="served workload: number of requests")
    ap.add_argument("--plain-sample", type=int, default=1 << 30,
                    help="served workload: requests timed alone for the plain sequential rate (evenly spaced; "
                         "default: all of them)")
    # the knee is near 55 req/s (mean request 1.25e7 particle-steps, ~7e8 particle-steps/s
    # served): two rates below it show unloaded latency, the rest saturation
    ap.add_argument("--rates", type=float, nargs="+", default=[10, 25, 50, 200, 1000],
                    help="served workload: Poisson arrival rates (req/s)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    dist = Dist()
    if args.impl == "reference":
        run_reference(args, dist)
    elif args.workload == "batched":
        run_batched(args, dist)
    elif args.workload == "served":
        run_served(args, dist)
    else:
        run_ours(args, dist)


if __name__ == "__main__":
    main()
