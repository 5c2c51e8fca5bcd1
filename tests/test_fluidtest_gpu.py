"""The C++ drop-in end to end: libfluid_gb300/bin/fluidtest (the reference's
demo driver on this library: FluidSystem subclass, double dam break,
advance + exportToData + .geo per frame) against the oracle running the same
scene.  fluidtest's defaults turn on surface tension, viscosity and adhesion,
so the normals pass and every force term are exercised."""
import os
import subprocess

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def read_geo(path):
    lines = open(path).read().splitlines()
    n = int(lines[1].split()[1])
    start = lines.index("pscale 1 float 1") + 1
    pos, col, vel = [], [], []
    for ln in lines[start:start + n]:
        head, attr = ln.split("(")
        x, y, z, _ = head.split()
        a = [float(t) for t in attr.rstrip(")").split()]
        pos.append((float(x), float(y), float(z)))
        col.append(a[0:3])
        vel.append(a[3:6])
    assert lines[start + n] == "PrimitiveAttrib"
    return np.array(pos), np.array(col), np.array(vel), float(a[6])


def test_fluidtest_double_dam_break_matches_oracle(tmp_path):
    n, res, steps, dt = 3000, 16, 3, 0.002
    exe = os.path.join(ROOT, "libfluid_gb300", "bin", "fluidtest")
    r = subprocess.run([exe, "-n", str(n), "-g", str(res), "-q", str(steps), "-t", str(dt), "-f",
                        str(tmp_path / "sim")], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "TOTAL TIME" in r.stdout
    files = sorted(os.listdir(tmp_path))
    assert files == [f"sim.{i:04d}.geo" for i in range(1, steps + 1)]
    pos, col, vel, pscale = read_geo(str(tmp_path / f"sim.{steps:04d}.geo"))

    o = oracle.Oracle(32)
    o.init(n, res)
    for k, v in (("adhesion", 0.1), ("viscosity", 0.2), ("surface_tension", 1.0), ("vdamp", 0.5)):
        o.set_param(k, v)
    o.create_block(0, n // 2, 0.0, 0.0, 0.0, 0.33, 0.9, 0.33)
    o.create_block(n // 2, n - n // 2, 0.66, 0.0, 0.66, 1.0, 0.9, 1.0)
    for _ in range(steps):
        o.advance(dt, 1)
    o.stage("colour")
    ps = float(np.float32(o.params()[15]))
    assert abs(pscale - ps) <= 1e-6 * ps
    # .geo prints 6 significant digits
    ref = o.get("pos")
    assert np.max(np.abs(pos - ref) / np.maximum(np.abs(ref), 1e-3)) < 2e-5
    vref = o.get("vel")
    vs = float(np.sqrt((vref ** 2).sum(1).mean()))
    assert np.max(np.linalg.norm(vel - vref, axis=1)) < 1e-3 * vs + 1e-5
    assert np.max(np.abs(col - o.get("colour"))) < 1e-4
