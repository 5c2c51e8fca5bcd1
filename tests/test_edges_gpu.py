"""Edge cases of the plain step on the GPU, each against the oracle: an empty
system, one particle, a particle count that leaves the last tile ragged, and
a cell at exactly the supported occupancy (8192 particles, which the
reference could not launch at all: fluidsystem.cu:322 allows 1024 threads
per cell block) next to one particle over it (SPH_ECELL)."""
import ctypes as C

import numpy as np
import pytest

import oracle
from helpers import configure_gpu, configure_oracle, rel_err
from libfluid_gb300 import FluidSystem, _capi, workloads as W

pytestmark = pytest.mark.gpu

RTOL_DENSITY = 1e-5
RTOL_POS = 1e-6


def _spec(pos, vel=None, box=(1.0, 1.0, 1.0), h=0.05):
    pos = np.asarray(pos, np.float32).reshape(-1, 3)
    return W.SceneSpec(box=box, h=h, blocks=[], mass=1e-3, particle_size=0.005, dt=1e-4, steps=1,
                       extra_pos=pos, extra_vel=np.zeros_like(pos) if vel is None else np.asarray(vel, np.float32))


def _one_substep(spec):
    """GPU (debug taps on) and FP32 oracle after one substep."""
    fs = FluidSystem(0)
    fs.debugEnable(True)
    configure_gpu(fs, spec)
    o = configure_oracle(oracle.Oracle(32), spec)
    assert fs.advance(spec.dt, 1) == 1
    o.advance(spec.dt, 1)
    return fs, o


def _check_fields(fs, o, n):
    for f in ("hash", "perm", "nbrcount"):
        g, r = fs.debug(f), o.get(f)
        assert np.array_equal(g, r), f"{f}: {np.count_nonzero(g != r)} of {n} differ"
    assert rel_err(fs.debug("density"), o.get("density"), 1.0) < RTOL_DENSITY
    pos, _, _ = fs.exportToData()
    assert rel_err(pos, o.get("pos"), 1e-3) < RTOL_POS


def test_empty_system():
    """No particles: every call succeeds and nothing is stepped."""
    fs = FluidSystem(0)
    try:
        fs.init(0, 16)
        assert fs.numParticles() == 0
        assert fs.advance(1e-3, 4) == 0
        pos, colour, vel = fs.exportToData()
        assert pos.shape == colour.shape == vel.shape == (0, 3)
    finally:
        fs.close()


def test_single_particle_falls_like_the_oracle():
    """One particle: no neighbours, gravity and the integrator only, for 20
    substeps."""
    spec = _spec([[0.5, 0.5, 0.5]], [[0.1, 0.0, -0.2]])
    fs = FluidSystem(0)
    configure_gpu(fs, spec)
    o = configure_oracle(oracle.Oracle(32), spec)
    try:
        for _ in range(20):
            assert fs.advance(spec.dt, 1) == 1
            o.advance(spec.dt, 1)
        pos, _, vel = fs.exportToData()
        assert rel_err(pos, o.get("pos"), 1e-3) < RTOL_POS
        assert rel_err(vel, o.get("vel"), 1e-3) < RTOL_POS
    finally:
        fs.close()


@pytest.mark.parametrize("n", [1037, 129])
def test_ragged_last_tile(n):
    """A particle count that is no multiple of the tile size (the last tile
    holds 13 or 1 particles), particles scattered in a small box."""
    rng = np.random.default_rng(n)
    spec = _spec(rng.uniform(0.05, 0.25, (n, 3)), box=(0.3, 0.3, 0.3), h=0.02)
    fs, o = _one_substep(spec)
    try:
        _check_fields(fs, o, n)
    finally:
        fs.close()


def _cell_block(n, seed=9):
    """n particles inside one 0.05 m cell of a 20^3 grid."""
    rng = np.random.default_rng(seed)
    return rng.uniform(0.505, 0.545, (n, 3))


def test_cell_at_the_occupancy_limit():
    """8192 particles in one cell: supported, and equal to the oracle."""
    spec = _spec(_cell_block(8192))
    fs, o = _one_substep(spec)
    try:
        occ = fs.debug("cellocc", ncells=20 ** 3)
        assert occ.max() == 8192
        _check_fields(fs, o, 8192)
    finally:
        fs.close()


def test_cell_one_over_the_limit():
    """8193 particles in one cell: the step reports SPH_ECELL and leaves the
    particles where they were."""
    spec = _spec(_cell_block(8193))
    fs = FluidSystem(0)
    configure_gpu(fs, spec)
    try:
        with pytest.raises(_capi.SphError) as err:
            fs.advance(spec.dt, 1)
        assert err.value.code == _capi.SPH_ECELL
        # positions alone: velocities would need the next substep's sort,
        # which fails on the same cell until the state is replaced
        pos = np.empty((spec.n, 3), np.float32)
        assert _capi.lib().sph_export(fs._h, pos.ctypes.data_as(C.c_void_p), None, None, spec.n) == _capi.SPH_OK
        assert np.array_equal(pos, spec.positions().astype(np.float32))
    finally:
        fs.close()
