"""GPU tests of the one-pass cell scan (k_scan_single, decoupled look-back).

The scan turns per-cell particle counts into cell starts across the whole
packed cell arena (the grid's cells and one bucket for particles outside
it).  Its tiles of 4096 cells each add up the tiles before them while those
are still running, so the interesting cases are grids of many tiles, and the
edges: an arena that ends exactly at a 16-cell vector (the vector path writes
the total) and one that ends one cell into a new tile.  The cell starts and occupancies the step reports (sph_debug_get) are
compared with the histogram of the sorted cell keys and its exclusive
cumulative sum, and, on the first substep (particles placed at cell centres),
with the cells computed on the host.  Two substeps in a row check that the
scan's per-substep tile counter and look-back words start from zero.
"""
import numpy as np
import pytest

from libfluid_gb300 import FluidSystem

pytestmark = pytest.mark.gpu


def _check_scan(fs, dims, n):
    nc = int(np.prod(dims))
    occ = fs.debug("cellocc", ncells=nc).astype(np.int64)
    start = fs.debug("cellstart", ncells=nc).astype(np.int64)
    keys = fs.debug("hash").astype(np.int64)
    inside = keys < nc                       # keys of particles outside the grid are nc
    hist = np.bincount(keys[inside], minlength=nc)
    np.testing.assert_array_equal(occ, hist)
    excl = np.concatenate([[0], np.cumsum(hist)[:-1]])
    np.testing.assert_array_equal(start, excl)
    assert occ.sum() == inside.sum() <= n
    return occ


@pytest.mark.parametrize("dims,n", [((13, 7, 5), 3000),          # one partial tile
                                    ((31, 11, 3), 2000),         # arena of 1024 cells
                                    ((64, 32, 4), 20000),        # arena of 8193 cells: 3 tiles
                                    ((200, 160, 100), 1_000_000)])  # 782 tiles
def test_scan_many_tiles(dims, n):
    h = 0.01
    rng = np.random.default_rng(11)
    nc = int(np.prod(dims))
    # particles in coincident pairs: a particle alone in its cell, with no
    # wall within h, gets only the near-zero poly6 weights of neighbours at
    # r = h (less rounding) as its density, and the reference's EOS then
    # gives forces that overflow in the next substep
    cells = np.repeat(rng.integers(0, nc, size=n // 2), 2)
    cx = cells % dims[0]
    cy = (cells // dims[0]) % dims[1]
    cz = cells // (dims[0] * dims[1])
    # cell centres, so host and device agree on every cell
    pos = (np.stack([cx, cy, cz], 1).astype(np.float64) + 0.5) * h
    pos = pos.astype(np.float32)
    fs = FluidSystem(0)
    fs.debugEnable(True)   # the sort fields then describe the substep just run
    fs.init(n, 1)
    fs.setDomain(dims[0] * h, dims[1] * h, dims[2] * h, h)
    fs.setParams(mass=2e-4, particle_size=0.0025, dt=1e-5)
    fs.setState(pos, np.zeros_like(pos))
    try:
        assert fs.advance(1e-5, 1) == 1
        occ = _check_scan(fs, dims, n)
        np.testing.assert_array_equal(occ, np.bincount(cells, minlength=nc))
        # a second substep: the particles have moved, the scan starts afresh
        assert fs.advance(1e-5, 1) == 1
        _check_scan(fs, dims, n)
    finally:
        fs.close()
