"""GPU test of sph_scan_cells_noalloc, the allocation-free cell-start scan.

Callers that cannot call cudaMalloc (an application that owns every byte of
device memory through its own arena, or a real-time frame loop where an
allocation would stall the device) use this entry point: it turns per-cell
particle counts into cell starts with its scratch in a fixed array inside
the library.  The test hands it caller-owned device buffers and checks its
output against the cell starts the normal step produced (sph_advance, then
sph_debug_get), bit for bit as for every integer field, on two calls in a
row with different inputs (the second call must not see the first call's
scratch).  Synthetic count arrays of more than 1,024 tiles and of the
largest accepted size reach every thread and warp of the tile-sum scan and
are checked against numpy's cumulative sum; free device memory is the same
before and after a call.  It lives in its own file, collected last.
"""
import ctypes as C

import numpy as np
import pytest

from cudart import DeviceBuffer, mem_get_info, synchronize
from helpers import configure_gpu
from libfluid_gb300 import FluidSystem, _capi, workloads as W

pytestmark = pytest.mark.gpu


def _cells_from_step(spec):
    fs = FluidSystem(0)
    configure_gpu(fs, spec)
    assert fs.advance(spec.dt, 1) == 1
    nc = (spec.unit_cube_res ** 3) if spec.unit_cube_res else int(
        np.prod([int(np.ceil(b / spec.h - 1e-3)) for b in spec.box]))
    occ = fs.debug("cellocc", ncells=nc)
    start = fs.debug("cellstart", ncells=nc)
    fs.close()
    return occ, start


def test_noalloc_scan_matches_step_on_two_calls():
    L = _capi.lib()
    scenes = [W.small_dam_break(seed=5), W.small_dam_break(seed=9, unit_cube=True)]
    expected = [_cells_from_step(s) for s in scenes]
    cap = max(o.size for o, _ in expected)
    d_counts = DeviceBuffer(4 * cap)
    d_starts = DeviceBuffer(4 * (cap + 1))
    try:
        for occ, start in expected:
            d_starts.fill(0xAB)
            d_counts.upload(occ)
            rc = L.sph_scan_cells_noalloc(d_counts.ptr, occ.size, d_starts.ptr, None)
            assert rc == _capi.SPH_OK
            synchronize()
            out = np.empty(occ.size + 1, np.uint32)
            d_starts.download(out)
            assert np.array_equal(out[:-1], start)
            assert int(out[-1]) == int(occ.sum(dtype=np.uint64))
    finally:
        d_counts.free()
        d_starts.free()


def _scan_synthetic(counts):
    """Two calls in a row on the same caller-owned buffers (the second sees
    the first call's scratch); returns the free device bytes around the
    second call and whether both outputs matched numpy."""
    L = _capi.lib()
    n = counts.size
    expect = np.empty(n + 1, np.uint32)
    expect[0] = 0
    np.cumsum(counts, dtype=np.uint32, out=expect[1:])
    d_counts = DeviceBuffer(4 * n)
    d_starts = DeviceBuffer(4 * (n + 1))
    try:
        d_counts.upload(counts)
        out = np.empty(n + 1, np.uint32)
        frees = []
        for call in range(2):
            d_starts.fill(0xCD)
            synchronize()
            frees.append(mem_get_info()[0])
            assert L.sph_scan_cells_noalloc(d_counts.ptr, n, d_starts.ptr, None) == _capi.SPH_OK
            synchronize()
            frees.append(mem_get_info()[0])
            d_starts.download(out)
            bad = np.flatnonzero(out != expect)
            assert bad.size == 0, f"call {call}: {bad.size} wrong starts, first at cell {bad[0]}"
        return frees
    finally:
        d_counts.free()
        d_starts.free()


def test_noalloc_scan_across_threads_and_warps():
    """5,000,000 cells = 1,221 tiles: the tile sums span 39 threads and two
    warps of the single-block scan, so the carry between them is checked."""
    rng = np.random.default_rng(11)
    counts = rng.integers(0, 4, size=5_000_000, dtype=np.uint32)
    counts[rng.integers(0, counts.size, size=1000)] = 200   # a few crowded cells
    frees = _scan_synthetic(counts)
    # the second call allocates nothing: free memory is unchanged around it
    assert frees[2] == frees[3], f"free device memory changed by {frees[2] - frees[3]} bytes"


def test_noalloc_scan_at_the_size_limit():
    """SPH_NOALLOC_MAX_CELLS cells (32,768 tiles): every thread of the
    tile-sum scan holds 32 sums."""
    L = _capi.lib()
    n = 32768 * 4096
    rng = np.random.default_rng(12)
    counts = rng.integers(0, 3, size=n, dtype=np.uint8).astype(np.uint32)
    frees = _scan_synthetic(counts)
    assert frees[2] == frees[3]
    del counts
    p = C.c_void_p(16)  # never dereferenced: the size check comes first
    assert L.sph_scan_cells_noalloc(p, n + 1, p, None) == _capi.SPH_EINVAL


def test_noalloc_scan_rejects_out_of_range_sizes():
    L = _capi.lib()
    p = C.c_void_p(16)  # never dereferenced: the size check comes first
    assert L.sph_scan_cells_noalloc(p, 0, p, None) == _capi.SPH_EINVAL
    too_many = 32768 * 4096 + 1
    assert L.sph_scan_cells_noalloc(p, too_many, p, None) == _capi.SPH_EINVAL
