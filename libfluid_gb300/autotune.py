"""Autotuner of the substep's launch configuration.

Sweeps, on a GPU, the execution choices that do not change results (every
choice computes bit-identical values; tests/test_exec_configs_gpu.py checks
it): particles per tile (= threads per block), persistent blocks per SM for
the neighbour passes (0 = one block per tile), the neighbour-mask skin, and
then, on the best of those, the kernel-variant bits (per-row density and XSPH
walks, the force kernel's register budget, row-table walks of the force and
normal passes, and for launches small enough to take it the density scan
split over three threads per particle, which sets how many particles a warp
scans: 32, or about 10).  Each candidate is timed with CUDA events over graph-replayed
substeps after warm-up.  The best configuration per workload is written to
tuned.json next to this file; the engine's compiled-in defaults (ExecConfig
in csrc/engine.h) follow that record.

    python -m libfluid_gb300.autotune [--workload batched|dam_break_1m|large_tension|all]
                                      [--steps 20] [--variants-only]
"""
from __future__ import annotations

import argparse
import itertools
import json
import os
import time

HERE = os.path.dirname(os.path.abspath(__file__))
TUNED = os.path.join(HERE, "tuned.json")

TILES = (128, 256)
PERSISTENT = (0, 2, 4)
SKINS = (0.1, 0.15, 0.2, 0.3)
VARIANTS = tuple(range(64))
# Launches of at most this many particles take the split density scan
# (SPH_VARIANT_DENSITY_SPLIT, bit 0x20; SPH_DENSITY_SPLIT_MAX in
# csrc/sph_types.h); above it the bit changes nothing and is not swept.
DENSITY_SPLIT_MAX = 49152


def variants_for(particles: int, persistent: int) -> tuple:
    """The variant values worth timing for a launch of `particles` particles:
    all 64 where the split density scan can apply (one block per tile and a
    small enough launch), else the 32 without its bit, which would change
    nothing there."""
    split = particles <= DENSITY_SPLIT_MAX and persistent == 0
    return VARIANTS if split else VARIANTS[:32]


def load(workload: str) -> dict | None:
    try:
        return json.load(open(TUNED))[workload]["best"]
    except (OSError, KeyError, ValueError):
        return None


def _scenes(workload: str):
    from . import workloads as W
    if workload == "batched":
        return W.batch_manifest(num_scenes=256, seed=7)
    if workload == "dam_break_1m":
        return [W.dam_break_1m()]
    if workload == "small_dam_break":
        return [W.small_dam_break()]
    if workload == "large_tension":
        return [W.large_tension()]
    raise ValueError(workload)


def time_config(scenes, tile: int, persistent: int, skin: float, steps: int, warmup: int = 5,
                device: int = 0, variant: int = 0) -> float:
    from .batch import Batch
    b = Batch(device)
    b.set_exec(tile=tile, persistent=persistent, skin=skin, variant=variant)
    for s in scenes:
        b.add_scene(s)
    for _ in range(warmup):
        b.step(1)
    b.sync()
    b.timer_mark(0)
    for _ in range(steps):
        b.step_async(1)
    b.timer_mark(1)
    ms = b.timer_elapsed(0, 1) / steps
    b.sync()
    b.close()
    return ms


def tune(workload: str, steps: int = 20, device: int = 0, variants_only: bool = False) -> dict:
    scenes = _scenes(workload)
    n = sum(s.n for s in scenes)
    trials = []
    grid = [(128, 0, 0.1)] if variants_only else itertools.product(TILES, PERSISTENT, SKINS)
    for tile, pers, skin in grid:
        ms = time_config(scenes, tile, pers, skin, steps, device=device)
        trials.append({"tile": tile, "persistent": pers, "skin": skin, "variant": 0, "ms_per_step": ms,
                       "particle_steps_per_s": n / (ms * 1e-3)})
    best = min(trials, key=lambda t: t["ms_per_step"])
    for v in variants_for(n, best["persistent"])[1:]:
        ms = time_config(scenes, best["tile"], best["persistent"], best["skin"], steps, device=device, variant=v)
        trials.append({"tile": best["tile"], "persistent": best["persistent"], "skin": best["skin"], "variant": v,
                       "ms_per_step": ms, "particle_steps_per_s": n / (ms * 1e-3)})
    best = min(trials, key=lambda t: t["ms_per_step"])
    return {"workload": workload, "particles": n, "scenes": len(scenes), "steps": steps,
            "when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime()),
            "best": {k: best[k] for k in ("tile", "persistent", "skin", "variant")}, "trials": trials}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="all")
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--out", default=TUNED)
    ap.add_argument("--variants-only", action="store_true",
                    help="keep tile 128, persistent 0, skin 0.1 and sweep the kernel variants only")
    args = ap.parse_args()
    names = ["dam_break_1m", "batched", "small_dam_break"] if args.workload == "all" else [args.workload]
    try:
        tuned = json.load(open(args.out))
    except (OSError, ValueError):
        tuned = {}
    for w in names:
        r = tune(w, args.steps, variants_only=args.variants_only)
        tuned[w] = r
        print(w, r["best"], "%.4f ms/step" % min(t["ms_per_step"] for t in r["trials"]), flush=True)
    with open(args.out, "w") as f:
        json.dump(tuned, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
