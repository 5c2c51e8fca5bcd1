"""Generate the golden vectors that pin the oracle to the reference's own code.

Runs NCCA/libfluid's device code (oracle/_ref/libfluid_ref.cubin, compiled
from its cudasrc by oracle/ref_build.sh) through oracle/_ref/ref_runner on a
GPU, for three small scenes in the reference's unit-cube domain, and writes
tests/golden/<scene>.npz with the scene's inputs and the intermediates of one
substep:

  hash (sorted m_Hash), perm, cellocc, cellstart (m_ScatterAddress),
  nbrcount, density, pressure, soundspeed, normal, fpressure, ftension,
  fadhesion, fviscosity, pos, vel, acc (after the substep), colour,
  vel_int (velocity after integration, before XSPH)

Usage (on a GPU host, after build()):  python tests/golden/make_golden.py [--out DIR]
"""
from __future__ import annotations

import argparse
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from libfluid_gb300 import workloads as W  # noqa: E402

from oracle import ref_cuda  # noqa: E402


def scenes() -> dict:
    out = {}
    # 1. the small dam break's lattice and parameters, 16^3 particles, unit cube res 50
    lat = W.Lattice(lo=(0.0, 0.0, 0.0), spacing=0.01, nx=16, ny=16, nz=16, jitter=5e-4, seed=11)
    p = lat.positions()
    out["dam_cube_res50"] = dict(
        res=50, dt=2e-4, pos=p, vel=np.zeros_like(p),
        params=dict(rest_density=1000.0, gas_constant=400.0, gamma=7.0, mass=1e-3, particle_size=0.005, xsph=0.5,
                    surface_tension=0.0, viscosity=0.01, adhesion=0.0, vdamp=0.5, vel_limit=5.0, acc_limit=150.0,
                    gx=0.0, gy=-9.8, gz=0.0, unused=0.0))
    # 2. FluidSystem::setup-style block with the reference's init defaults
    #    (gas constant 100, gamma 7, rho0 1000) and createFluidBlock's placement,
    #    mass and particle size; tension, viscosity and adhesion on.
    import oracle
    o = oracle.Oracle(32)
    o.init(4000, 16)
    o.create_block(0, 4000, 0.1, 0.1, 0.1, 0.9, 0.9, 0.9)
    pos = o.get("pos", np.float32)
    prm = o.params()
    out["block_res16_tension"] = dict(
        res=16, dt=0.002, pos=pos, vel=np.zeros_like(pos),
        params=dict(rest_density=1000.0, gas_constant=100.0, gamma=7.0, mass=float(np.float32(prm[14])),
                    particle_size=float(np.float32(prm[15])), xsph=0.5, surface_tension=1.0, viscosity=0.2,
                    adhesion=0.1, vdamp=0.5, vel_limit=5.0, acc_limit=150.0, gx=0.0, gy=-9.8, gz=0.0, unused=0.0))
    # 3. edge cases: points on cell faces, at 1.0 and outside the unit cube
    #    (NULL_HASH), a dense clump, a lone particle, moving particles
    rng = np.random.default_rng(5)
    res = 10
    faces = (rng.integers(0, res, size=(200, 3)) / res).astype(np.float32)
    faces[:, 1] += np.float32(0.013)
    clump = (np.float32(0.5) + rng.uniform(-0.02, 0.02, size=(300, 3))).astype(np.float32)
    bulk = rng.uniform(0.05, 0.95, size=(400, 3)).astype(np.float32)
    outside = np.array([[1.0, 0.5, 0.5], [-0.01, 0.5, 0.5], [0.5, 1.2, 0.5], [0.5, 0.5, -3.0], [0.999, 0.999, 0.999],
                        [0.0, 0.0, 0.0]], np.float32)
    lone = np.array([[0.93, 0.07, 0.41]], np.float32)
    pos = np.concatenate([faces, clump, bulk, outside, lone])
    vel = rng.uniform(-2, 2, size=pos.shape).astype(np.float32)
    out["edges_res10"] = dict(
        res=res, dt=1e-3, pos=pos, vel=vel,
        params=dict(rest_density=1000.0, gas_constant=50.0, gamma=7.0, mass=0.02, particle_size=0.01, xsph=0.5,
                    surface_tension=0.5, viscosity=0.1, adhesion=0.5, vdamp=0.3, vel_limit=5.0, acc_limit=150.0,
                    gx=0.0, gy=-9.8, gz=0.0, unused=0.0))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=HERE, help="output directory (default tests/golden)")
    args = ap.parse_args()
    if not ref_cuda.available():
        raise SystemExit("oracle/_ref/ref_runner missing: build() with the reference cubin present")
    os.makedirs(args.out, exist_ok=True)
    meta = {}
    for name, sc in scenes().items():
        out = ref_cuda.run(sc["pos"], sc["vel"], sc["res"], sc["dt"], sc["params"])
        arrays = {f"in_{k}": v for k, v in (("pos", sc["pos"]), ("vel", sc["vel"]))}
        arrays.update({f"ref_{k}": v for k, v in out.items()})
        np.savez_compressed(os.path.join(args.out, f"{name}.npz"), **arrays)
        meta[name] = {"res": sc["res"], "dt": sc["dt"], "params": sc["params"], "n": int(sc["pos"].shape[0])}
        print(name, "n =", sc["pos"].shape[0], "block =", int(out["block"]))
    with open(os.path.join(args.out, "scenes.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
