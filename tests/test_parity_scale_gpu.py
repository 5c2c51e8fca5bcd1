"""GPU parity at the benchmarked sizes, through the C ABI.

The same bar as the 32,768-particle tests, at the scenes the throughput is
quoted on (the reference step being matched is fluidsystem.cu:301-398):

* 1,000,000-particle dam break in its 2x1x1 m box (2,000,000 cells), one
  substep from the initial state and one substep after 50 substeps of
  compression (the GPU state handed to the oracle exactly: positions,
  velocities and accelerations): hash, sort permutation, cell start and
  occupancy, neighbour counts bit-exact against the FP32 oracle; density
  within 1e-5, forces within 1e-4, positions within 1e-6 relative, each
  result's error against the FP64 oracle printed beside the FP32 oracle's.
* The same 1M particles in the reference's own domain (unit cube, res 100):
  integer fields bit-exact against the reference's own device code
  (oracle/ref_runner driving the unmodified cudasrc kernels), density within
  1e-5 and forces within 1e-4 of it (relative to the pair terms' magnitude).
* The ~8M-particle tension scene after three substeps: the GPU state of a
  spatial window (the pool's free surface and the bottom of the first
  sphere) handed to the oracle; hashes and the order of the window's
  particles bit-exact, neighbour counts, density, normals, forces and
  positions compared on the particles far enough inside the window that
  their neighbourhoods (and their neighbours') lie in it.
"""
import numpy as np
import pytest

import oracle
from helpers import (SCALE_FIELD, by_particle, check_vector_field, configure_gpu, configure_oracle,
                     oracle_from_state, pair_scale, rel_err, scaled_err, snapshot_state)
from libfluid_gb300 import FluidSystem, workloads as W

pytestmark = pytest.mark.gpu

RTOL_DENSITY = 1e-5
RTOL_FORCE = 1e-4
RTOL_POS = 1e-6
FORCES = ("fpressure", "fviscosity", "fadhesion", "ftension")
INT_FIELDS = ("hash", "perm", "nbrcount")


def _check_full(fs, o32, o64, label):
    """Every field of one substep of the whole scene, GPU against oracles."""
    for f in INT_FIELDS:
        g, r = fs.debug(f), o32.get(f)
        assert np.array_equal(g, r), f"{label} {f}: {np.count_nonzero(g != r)} mismatches"
    for f in ("cellstart", "cellocc"):
        g, r = fs.debug(f, ncells=o32.ncells), o32.get(f)
        assert np.array_equal(g, r), f"{label} {f}: {np.count_nonzero(g != r)} mismatches"
    rho_g, rho_o, rho_d = fs.debug("density"), o32.get("density"), o64.get("density")
    e = rel_err(rho_g, rho_o, 1.0)
    print(f"{label} density: gpu-vs-fp32 {e:.2e}, gpu-vs-fp64 {rel_err(rho_g, rho_d, 1.0):.2e}, "
          f"fp32-vs-fp64 {rel_err(rho_o, rho_d, 1.0):.2e}")
    assert e < RTOL_DENSITY
    for f in FORCES:
        S = pair_scale(o32, o64, f) if f in SCALE_FIELD else None
        check_vector_field(f"{label} {f}", fs.debug(f), o32.get(f), o64.get(f), S, RTOL_FORCE)
    pos, _, vel = fs.exportToData()
    ep = rel_err(pos, o32.get("pos"), 1e-3)
    print(f"{label} pos: gpu-vs-fp32 {ep:.2e}, fp32-vs-fp64 {rel_err(o32.get('pos'), o64.get('pos'), 1e-3):.2e}; "
          f"vel {rel_err(vel, o32.get('vel'), 1e-3):.2e}")
    assert ep < RTOL_POS
    assert rel_err(vel, o32.get("vel"), 1e-3) < RTOL_FORCE


def _one_substep(spec, fs, pos, vel, acc):
    o32 = oracle_from_state(32, spec, pos, vel, acc)
    o64 = oracle_from_state(64, spec, pos, vel, acc)
    assert fs.advance(spec.dt, 1) == 1
    assert o32.advance(spec.dt, 1) == 1
    assert o64.advance(spec.dt, 1) == 1
    return o32, o64


def test_dam_break_1m_first_substep():
    spec = W.dam_break_1m()
    assert spec.n == 1_000_000
    fs = FluidSystem(0)
    fs.debugEnable(True)
    configure_gpu(fs, spec)
    o32 = configure_oracle(oracle.Oracle(32), spec)
    o64 = configure_oracle(oracle.Oracle(64), spec)
    o32.track_scales(True)
    o64.track_scales(True)
    assert o32.ncells == 2_000_000
    assert fs.advance(spec.dt, 1) == 1
    o32.advance(spec.dt, 1)
    o64.advance(spec.dt, 1)
    _check_full(fs, o32, o64, "1M substep 1")
    fs.close()


def test_dam_break_1m_after_50_substeps():
    """50 substeps on the benchmarked path (deferred XSPH, CUDA graphs), then
    the exact state (the pending XSPH update applied, as the snapshot does)
    to the oracles and one substep on both with the taps on."""
    spec = W.dam_break_1m(seed=2)
    fs = FluidSystem(0)
    configure_gpu(fs, spec)
    for _ in range(50):
        assert fs.advance(spec.dt, 1) == 1
    pos, vel, acc = snapshot_state(fs)
    fs.debugEnable(True)
    o32, o64 = _one_substep(spec, fs, pos, vel, acc)
    nbr = fs.debug("nbrcount")
    print(f"1M after 50: neighbours mean {nbr.mean():.1f} max {nbr.max()}")
    _check_full(fs, o32, o64, "1M substep 51")
    fs.close()


def test_dam_break_1m_unit_cube_against_reference_device_code():
    from oracle import ref_cuda
    if not ref_cuda.available():
        pytest.skip("the reference's device build (oracle/_ref) is absent")
    spec = W.dam_break_1m(unit_cube=True)
    pos, vel = spec.positions(), spec.velocities()
    p = spec.params()
    ref = ref_cuda.run(pos, vel, spec.unit_cube_res, spec.dt,
                       dict(p, gx=p["gravity"][0], gy=p["gravity"][1], gz=p["gravity"][2]))
    fs = FluidSystem(0)
    fs.debugEnable(True)
    configure_gpu(fs, spec)
    assert fs.advance(spec.dt, 1) == 1
    for f in INT_FIELDS:
        g = fs.debug(f)
        assert np.array_equal(g, ref[f]), f"{f}: {np.count_nonzero(g != ref[f])} mismatches against the reference"
    nc = spec.unit_cube_res ** 3
    for f in ("cellstart", "cellocc"):
        assert np.array_equal(fs.debug(f, ncells=nc), ref[f]), f
    o32 = configure_oracle(oracle.Oracle(32), spec)
    o64 = configure_oracle(oracle.Oracle(64), spec)
    o32.track_scales(True)
    o64.track_scales(True)
    o32.advance(spec.dt, 1)
    o64.advance(spec.dt, 1)
    rho_g = fs.debug("density")
    e = rel_err(rho_g, ref["density"], 1.0)
    print(f"1M unit cube density: gpu-vs-reference {e:.2e}, "
          f"fp32-oracle-vs-reference {rel_err(o32.get('density'), ref['density'], 1.0):.2e}")
    assert e < RTOL_DENSITY
    for f in FORCES:
        g, r, o = fs.debug(f), ref[f], o32.get(f)
        scale = float(np.sqrt((r.astype(np.float64) ** 2).sum(1).mean()))
        floor = max(1e-2 * scale, 1e-30)
        msg = (f"1M unit cube {f}: |F|-relative gpu-vs-reference {rel_err(g, r, floor):.2e}, "
               f"fp32-oracle-vs-reference {rel_err(o, r, floor):.2e}")
        if f in SCALE_FIELD:
            S = pair_scale(o32, o64, f)
            e_g, e_o = scaled_err(g, r, S), scaled_err(o, r, S)
            msg += f"; pair-scale-relative gpu-vs-reference {e_g:.2e}, fp32-oracle-vs-reference {e_o:.2e}"
        else:
            e_g = rel_err(g, r, floor)
        print(msg)
        assert e_g < RTOL_FORCE, msg
    pos_g, _, _ = fs.exportToData()
    assert rel_err(pos_g, ref["pos"], 1e-3) < RTOL_POS
    fs.close()


# The window of the tension scene: the pool's free surface (z = 0.9 m) and
# the bottom of the first sphere (centre (0.27, 0.5, 1.3), radius 0.229 m).
WINDOW_LO = np.array([0.15, 0.35, 0.75])
WINDOW_HI = np.array([0.45, 0.65, 1.15])


def test_large_tension_window_after_three_substeps():
    spec = W.large_tension()
    h = spec.h
    fs = FluidSystem(0)
    fs.debugEnable(True)
    configure_gpu(fs, spec)
    for _ in range(3):
        assert fs.advance(spec.dt, 1) == 1
    pos, vel, acc = snapshot_state(fs)
    n = pos.shape[0]
    assert n > 7_900_000
    inside = np.all((pos >= WINDOW_LO) & (pos <= WINDOW_HI), axis=1)
    win = np.flatnonzero(inside)              # state slots, ascending: the window in slot order
    depth = np.minimum(pos[win] - WINDOW_LO, WINDOW_HI - pos[win]).min(1)
    print(f"tension window: {win.size} particles")
    assert win.size > 100_000

    assert fs.advance(spec.dt, 1) == 1        # substep 4 on the whole scene
    o32, o64 = _one_substep_window(spec, pos[win], vel[win], acc[win])

    perm_g = fs.debug("perm")
    in_win = np.zeros(n, bool)
    in_win[win] = True
    sel_sorted = in_win[perm_g]
    # the stable sort keeps the window's particles in the same relative order
    perm_o = o32.get("perm")
    assert np.array_equal(perm_g[sel_sorted], win[perm_o]), "order of the window's particles"
    assert np.array_equal(fs.debug("hash")[sel_sorted], o32.get("hash")), "hash"

    def gpu(f):
        return by_particle(fs.debug(f), perm_g)[win]

    def orc(o, f):
        return by_particle(o.get(f), perm_o)

    # neighbourhoods complete: 1 h inside; neighbours' densities: 2 h;
    # neighbours' normals (tension): 3 h
    d1, d2, d3 = depth > 1.05 * h, depth > 2.05 * h, depth > 3.05 * h
    print(f"interior particles: {d1.sum()} / {d2.sum()} / {d3.sum()}")
    assert np.array_equal(gpu("nbrcount")[d1], orc(o32, "nbrcount")[d1]), "neighbour counts"
    rho_g, rho_o, rho_d = gpu("density")[d1], orc(o32, "density")[d1], orc(o64, "density")[d1]
    e = rel_err(rho_g, rho_o, 1.0)
    print(f"window density: gpu-vs-fp32 {e:.2e}, gpu-vs-fp64 {rel_err(rho_g, rho_d, 1.0):.2e}, "
          f"fp32-vs-fp64 {rel_err(rho_o, rho_d, 1.0):.2e}")
    assert e < RTOL_DENSITY
    def scale(f):
        return np.maximum(orc(o32, SCALE_FIELD[f]), orc(o64, SCALE_FIELD[f]))

    check_vector_field("window normal", gpu("normal")[d2], orc(o32, "normal")[d2], orc(o64, "normal")[d2],
                       scale("normal")[d2], RTOL_FORCE)
    for f in FORCES:
        S = scale(f)[d3] if f in SCALE_FIELD else None
        check_vector_field(f"window {f}", gpu(f)[d3], orc(o32, f)[d3], orc(o64, f)[d3], S, RTOL_FORCE)
    # positions after the integrator: the exported state is in sorted order
    pos_g, _, _ = fs.exportToData()
    pos_g = by_particle(pos_g, perm_g)[win]
    ep = rel_err(pos_g[d3], orc(o32, "pos")[d3], 1e-3)
    print(f"window pos: gpu-vs-fp32 {ep:.2e}")
    assert ep < RTOL_POS
    fs.close()


def _one_substep_window(spec, pos, vel, acc):
    o32 = oracle_from_state(32, spec, pos, vel, acc)
    o64 = oracle_from_state(64, spec, pos, vel, acc)
    assert o32.advance(spec.dt, 1) == 1
    assert o64.advance(spec.dt, 1) == 1
    return o32, o64
