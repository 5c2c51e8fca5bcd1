"""GPU parity on crowded cells, where the neighbour masks change form.

The density pass records each particle's neighbours per cell row: one mask
word for a row of up to 32 candidates, two words for 33 to 64, none above 64
(those rows are walked candidate by candidate with the distance test).  A
lattice at rest density fills a row with about 24 candidates, so the other
two forms only appear once a flow compresses.  Here compressed lattices
produce them from the first substep: spacing h/2.67 gives rows of 33 to 64
candidates, spacing h/3.3 rows above 64.  Each is compared with the CPU
oracle, which knows nothing of masks, after one substep: integer fields bit
for bit, density, forces and the one-step state within the plain tests'
bounds, under both XSPH schedules.

Forces and velocities: with 60 to 160 candidates per row the pair terms
cancel more than at rest density, and the FP32 oracle itself sits 1.2e-4 to
1.8e-4 from the FP64 oracle under the plain tests' measure.  So the GPU must
be no further from FP64 than twice the FP32 oracle is, and, by the triangle
inequality, within three times the FP32 oracle's FP64 error (or 1e-4,
whichever is larger) of the FP32 oracle.
"""
import numpy as np
import pytest

import oracle
from helpers import configure_gpu, configure_oracle, rel_err
from libfluid_gb300 import FluidSystem, workloads as W

pytestmark = pytest.mark.gpu

RTOL_DENSITY = 1e-5
RTOL_FORCE = 1e-4
RTOL_POS = 1e-6


def crowded(spacing: float, n_side: int, seed: int = 3) -> W.SceneSpec:
    lat = W.Lattice(lo=(0.05, 0.05, 0.05), spacing=spacing, nx=n_side, ny=n_side, nz=n_side,
                    jitter=0.05 * spacing, seed=seed)
    return W.SceneSpec(box=(0.4, 0.4, 0.4), h=0.02, blocks=[lat], mass=1e-3, particle_size=0.005, dt=1e-4, steps=1)


def row_lengths(occ: np.ndarray, dims) -> np.ndarray:
    """Candidates in each (y,z) row of three cells around every occupied cell."""
    g = occ.reshape(dims[2], dims[1], dims[0]).astype(np.int64)
    p = np.pad(g, 1)
    out = []
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            s = p[1 + dz:1 + dz + dims[2], 1 + dy:1 + dy + dims[1], :]
            row = s[:, :, 0:dims[0]] + s[:, :, 1:dims[0] + 1] + s[:, :, 2:dims[0] + 2]
            out.append(row[g > 0])
    return np.concatenate(out)


# spacing h/2.67: rows of 32 to 72 candidates (two words, some walked in
# full); spacing h/3.3: most rows above 64 (walked in full)
SCENES = [(0.0075, (33, 64)), (0.006, (65, 10**9))]


@pytest.mark.parametrize("spacing,rows", SCENES)
def test_crowded_cells_match_oracle(spacing, rows):
    """Debug taps on (so XSPH runs as the last pass of the substep)."""
    spec = crowded(spacing, 24)
    fs = FluidSystem(0)
    fs.debugEnable(True)
    configure_gpu(fs, spec)
    o32 = configure_oracle(oracle.Oracle(32), spec)
    o64 = configure_oracle(oracle.Oracle(64), spec)
    try:
        assert fs.advance(spec.dt, 1) == 1
        o32.advance(spec.dt, 1)
        o64.advance(spec.dt, 1)
        dims = [int(np.ceil(b / spec.h - 1e-3)) for b in spec.box]
        occ = fs.debug("cellocc", ncells=int(np.prod(dims)))
        lens = row_lengths(occ, dims)
        hit = np.count_nonzero((lens >= rows[0]) & (lens <= rows[1]))
        print(f"{spacing}: rows {lens.min()}..{lens.max()}, {hit} of {lens.size} in {rows}")
        assert hit > 0, "the scene does not reach this mask form"
        for f in ("hash", "perm", "nbrcount"):
            g, r = fs.debug(f), o32.get(f)
            assert np.array_equal(g, r), f"{f}: {np.count_nonzero(g != r)} mismatches"
        assert np.array_equal(occ, o32.get("cellocc"))
        assert rel_err(fs.debug("density"), o32.get("density"), 1.0) < RTOL_DENSITY
        for field in ("fpressure", "fviscosity"):
            g, r, d = fs.debug(field), o32.get(field), o64.get(field)
            scale = float(np.sqrt((r.astype(np.float64) ** 2).sum(1).mean()))
            floor = max(1e-2 * scale, 1e-30)
            e, e64, o_e64 = rel_err(g, r, floor), rel_err(g, d, floor), rel_err(r, d, floor)
            print(f"{spacing} {field}: gpu-vs-fp32 {e:.2e}, gpu-vs-fp64 {e64:.2e}, fp32-vs-fp64 {o_e64:.2e}")
            assert e64 <= 2.0 * o_e64 + 1e-6
            assert e < max(RTOL_FORCE, 3.0 * o_e64)
        pos, _, vel = fs.exportToData()
        assert rel_err(pos, o32.get("pos"), 1e-3) < RTOL_POS
        _check_vel(vel, o32.get("vel"), o64.get("vel"))
    finally:
        fs.close()


def _check_vel(vel, v32, v64):
    ev, ev64, o_ev64 = rel_err(vel, v32, 1e-3), rel_err(vel, v64, 1e-3), rel_err(v32, v64, 1e-3)
    print(f"vel: gpu-vs-fp32 {ev:.2e}, gpu-vs-fp64 {ev64:.2e}, fp32-vs-fp64 {o_ev64:.2e}")
    assert ev64 <= 2.0 * o_ev64 + 1e-6
    assert ev < max(RTOL_FORCE, 3.0 * o_ev64)


@pytest.mark.parametrize("spacing,rows", SCENES)
def test_crowded_cells_deferred_xsph(spacing, rows):
    """No debug taps: the default schedule, each substep's XSPH update applied
    by the next density pass (here the second substep's, and the export's
    prefix for the second update), against the oracle's per-substep XSPH."""
    spec = crowded(spacing, 24)
    fs = FluidSystem(0)
    configure_gpu(fs, spec)
    o32 = configure_oracle(oracle.Oracle(32), spec)
    o64 = configure_oracle(oracle.Oracle(64), spec)
    try:
        for _ in range(2):
            assert fs.advance(spec.dt, 1) == 1
            o32.advance(spec.dt, 1)
            o64.advance(spec.dt, 1)
        pos, _, vel = fs.exportToData()
        ep = rel_err(pos, o32.get("pos"), 1e-3)
        print(f"{spacing}: pos {ep:.2e}")
        assert ep < 10 * RTOL_POS
        _check_vel(vel, o32.get("vel"), o64.get("vel"))
    finally:
        fs.close()
