"""Multi-step runs against the oracle, compared on conserved and aggregate
quantities.

After a few dozen substeps per-particle states diverge chaotically: every
rounding difference (summation order, approximate reciprocals, the FP32
versus FP64 oracle) grows.  So long runs are compared on total mass, kinetic
energy, centre of mass and the largest density deviation from rest.  The
bound for each is stated against the divergence of the two oracles from each
other: the GPU may differ from the FP64 oracle by at most a few times what
the FP32 oracle does (KIN_FACTOR and friends below), or by a small absolute
floor where the oracles agree to rounding.
"""
import numpy as np
import pytest

import oracle
from helpers import configure_gpu, configure_oracle, scene_invariants
from libfluid_gb300 import FluidSystem, workloads as W

pytestmark = pytest.mark.gpu

FACTOR = 4.0          # GPU-vs-FP64 difference allowed, in units of FP32-vs-FP64
KIN_FLOOR = 1e-4      # relative, kinetic energy
COM_FLOOR = 1e-5      # metres, centre of mass
RHO_FLOOR = 2e-3      # absolute, max |rho/rho0 - 1|


def _invariants_oracle(o, spec):
    return scene_invariants(o.get("pos"), o.get("vel"), spec.mass, rho=o.get("density"), rho0=spec.rest_density)


def gpu_density(fs, n):
    """Densities of the last substep: the w component of the positions in a
    snapshot (128-byte header, then n float4 positions)."""
    snap = fs.snapshot()
    return np.frombuffer(snap, np.float32, count=4 * n, offset=128).reshape(n, 4)[:, 3]


@pytest.mark.parametrize("unit_cube,steps", [(False, 200), (True, 200), (False, 1000)])
def test_dam_break_multistep(unit_cube, steps):
    """The 32,768-particle dam break (substeps of 2e-4 s), in the 1.0x0.6x0.6 m
    box and in the reference's unit cube; 1000 substeps take the collapse
    well into the chaotic regime."""
    spec = W.small_dam_break(seed=21, unit_cube=unit_cube)
    fs = FluidSystem(0)
    configure_gpu(fs, spec)
    o32 = configure_oracle(oracle.Oracle(32), spec)
    o64 = configure_oracle(oracle.Oracle(64), spec)
    try:
        for _ in range(steps):
            assert fs.advance(spec.dt, 1) == 1
            o32.advance(spec.dt, 1)
            o64.advance(spec.dt, 1)
        pos, _, vel = fs.exportToData()
        g = scene_invariants(pos, vel, spec.mass, rho=gpu_density(fs, spec.n), rho0=spec.rest_density)
        a = _invariants_oracle(o32, spec)
        d = _invariants_oracle(o64, spec)
        print(f"unit_cube={unit_cube} steps={steps}")
        for key in ("mass", "kinetic", "max_rho_dev"):
            print(f"  {key}: gpu {g[key]:.6e}  fp32 {a[key]:.6e}  fp64 {d[key]:.6e}")
        print(f"  com: gpu {g['com']}  fp32 {a['com']}  fp64 {d['com']}")
        assert g["mass"] == pytest.approx(d["mass"], rel=1e-12)
        kin_ref = abs(a["kinetic"] - d["kinetic"])
        assert abs(g["kinetic"] - d["kinetic"]) <= max(FACTOR * kin_ref, KIN_FLOOR * d["kinetic"])
        com_ref = float(np.max(np.abs(a["com"] - d["com"])))
        assert float(np.max(np.abs(g["com"] - d["com"]))) <= max(FACTOR * com_ref, COM_FLOOR)
        rho_ref = abs(a["max_rho_dev"] - d["max_rho_dev"])
        assert abs(g["max_rho_dev"] - d["max_rho_dev"]) <= max(FACTOR * rho_ref, RHO_FLOOR)
    finally:
        fs.close()


def test_dam_break_1m_multistep():
    """The 1,000,000-particle dam break of the benchmark (2x1x1 m box,
    substeps of 1e-4 s) for 100 substeps on the benchmarked path (deferred
    XSPH, CUDA graphs), against both oracles on the same bounds."""
    spec = W.dam_break_1m(seed=23)
    steps = 100
    fs = FluidSystem(0)
    configure_gpu(fs, spec)
    o32 = configure_oracle(oracle.Oracle(32), spec)
    o64 = configure_oracle(oracle.Oracle(64), spec)
    try:
        for _ in range(steps):
            assert fs.advance(spec.dt, 1) == 1
            o32.advance(spec.dt, 1)
            o64.advance(spec.dt, 1)
        pos, _, vel = fs.exportToData()
        g = scene_invariants(pos, vel, spec.mass, rho=gpu_density(fs, spec.n), rho0=spec.rest_density)
        a = _invariants_oracle(o32, spec)
        d = _invariants_oracle(o64, spec)
        print(f"1M dam break, {steps} substeps")
        for key in ("mass", "kinetic", "max_rho_dev"):
            print(f"  {key}: gpu {g[key]:.6e}  fp32 {a[key]:.6e}  fp64 {d[key]:.6e}")
        print(f"  com: gpu {g['com']}  fp32 {a['com']}  fp64 {d['com']}")
        assert g["mass"] == pytest.approx(d["mass"], rel=1e-12)
        kin_ref = abs(a["kinetic"] - d["kinetic"])
        assert abs(g["kinetic"] - d["kinetic"]) <= max(FACTOR * kin_ref, KIN_FLOOR * d["kinetic"])
        com_ref = float(np.max(np.abs(a["com"] - d["com"])))
        assert float(np.max(np.abs(g["com"] - d["com"]))) <= max(FACTOR * com_ref, COM_FLOOR)
        rho_ref = abs(a["max_rho_dev"] - d["max_rho_dev"])
        assert abs(g["max_rho_dev"] - d["max_rho_dev"]) <= max(FACTOR * rho_ref, RHO_FLOOR)
    finally:
        fs.close()
