"""Driver of oracle/_ref/ref_runner: the reference's own device code
(NCCA/libfluid cudasrc compiled from its sources) on the GPU.

TEST INFRASTRUCTURE ONLY: used by tests/golden/make_golden.py to produce the
golden vectors and by bench.py to time the reference's CUDA step beside ours.
"""
from __future__ import annotations

import json
import os
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
RUNNER = os.path.join(REF_DIR, "ref_runner")
PARAM_ORDER = ["rest_density", "gas_constant", "gamma", "mass", "particle_size", "xsph", "surface_tension",
               "viscosity", "adhesion", "vdamp", "vel_limit", "acc_limit", "gx", "gy", "gz", "unused"]


def available() -> bool:
    return os.path.exists(RUNNER) and os.path.exists(os.path.join(REF_DIR, "libfluid_ref.cubin"))


def write_input(path: str, pos, vel, res: int, dt: float, params: dict, substeps: int = 1) -> None:
    pos = np.ascontiguousarray(pos, np.float32)
    vel = np.ascontiguousarray(vel, np.float32)
    with open(path, "wb") as f:
        f.write(struct.pack("<4I", 0x53504831, pos.shape[0], res, substeps))
        f.write(struct.pack("<f", dt))
        f.write(struct.pack("<16f", *[float(params.get(k, 0.0)) for k in PARAM_ORDER]))
        f.write(pos.tobytes())
        f.write(vel.tobytes())


def run(pos, vel, res: int, dt: float, params: dict, substeps: int = 1) -> dict:
    n = pos.shape[0]
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        write_input(fin, pos, vel, res, dt, params, substeps)
        r = subprocess.run([RUNNER, REF_DIR, "run", fin, fout], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(r.stdout + r.stderr)
        raw = open(fout, "rb").read()
    n_, cells, block = struct.unpack_from("<3I", raw, 0)
    assert n_ == n
    off = 12
    res_ = {"block": np.uint32(block)}

    def take(name, dtype, count, shape=None):
        nonlocal off
        a = np.frombuffer(raw, dtype=dtype, count=count, offset=off).copy()
        off += a.nbytes
        res_[name] = a if shape is None else a.reshape(shape)

    for name in ("hash", "perm"):
        take(name, np.uint32, n)
    take("cellocc", np.uint32, cells)
    take("cellstart", np.uint32, cells)
    take("nbrcount", np.uint32, n)
    for name in ("density", "pressure", "soundspeed"):
        take(name, np.float32, n)
    for name in ("normal", "fpressure", "ftension", "fadhesion", "fviscosity", "pos", "vel", "acc", "colour",
                 "vel_int"):
        take(name, np.float32, 3 * n, (n, 3))
    assert off == len(raw)
    return res_


def time_steps(pos, vel, res: int, dt: float, params: dict, warmup: int, steps: int, timeout: float = 600) -> dict:
    """Device time of `steps` reference substeps (CUDA events around the loop,
    the reference's synchronisations included)."""
    with tempfile.TemporaryDirectory() as td:
        fin = os.path.join(td, "in.bin")
        write_input(fin, pos, vel, res, dt, params)
        r = subprocess.run([RUNNER, REF_DIR, "time", fin, str(warmup), str(steps)], capture_output=True, text=True,
                           timeout=timeout)
        if r.returncode != 0:
            raise RuntimeError(r.stdout + r.stderr)
    return json.loads(r.stdout.strip().splitlines()[-1])
