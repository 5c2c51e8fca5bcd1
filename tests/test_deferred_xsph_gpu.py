"""Deferred XSPH: a substep's XSPH update applied inside the next substep's
density pass.

* Reading the state (export) does not change the run: exporting after every
  substep and exporting once at the end give identical final states.
* The deferred schedule agrees with the per-substep schedule (the reference's)
  to rounding: the pairs are the same, only the order of the XSPH sums differs.
* Scenes that join later, a snapshot taken mid-run, and a parameter change on
  a scene with a pending update keep the bit-identity properties of a batch.
"""
import copy

import numpy as np
import pytest

from helpers import configure_gpu, rel_err
from libfluid_gb300 import FluidSystem, workloads as W
from libfluid_gb300.batch import Batch

pytestmark = pytest.mark.gpu


def _plain(spec, steps, export_every=False, deferred=True):
    fs = configure_gpu(FluidSystem(0), spec)
    fs.setDeferredXSPH(deferred)
    for _ in range(steps):
        fs.advance(spec.dt, 1)
        if export_every:
            fs.exportToData()
    out = [a.copy() for a in fs.exportToData()]
    fs.close()
    return out


def test_export_does_not_change_the_run():
    spec = W.small_dam_break(seed=31)
    spec.surface_tension = 0.04
    a = _plain(spec, 8, export_every=False)
    b = _plain(spec, 8, export_every=True)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_deferred_matches_per_substep_schedule():
    spec = W.small_dam_break(seed=32)
    d = _plain(spec, 6, deferred=True)
    p = _plain(spec, 6, deferred=False)
    assert rel_err(d[0], p[0], 1e-3) < 1e-6                      # positions
    vs = float(np.sqrt((p[2].astype(np.float64) ** 2).sum(1).mean()))
    assert rel_err(d[2], p[2], 1e-2 * vs) < 1e-4                  # velocities


def test_multi_substep_advance_and_snapshot_resume():
    spec = W.small_dam_break(seed=33)
    fs = configure_gpu(FluidSystem(0), spec)
    fs.advance(spec.dt * 3, 3)                   # three substeps, updates deferred between them
    snap = fs.snapshot()                         # applies the pending update
    for _ in range(4):
        fs.advance(spec.dt, 1)
    want = [a.copy() for a in fs.exportToData()]
    fs.close()
    other = FluidSystem(0)
    other.init(spec.n, 16)
    other.restore(snap)
    for _ in range(4):
        other.advance(spec.dt, 1)
    got = other.exportToData()
    for x, y in zip(got, want):
        assert np.array_equal(x, y)
    other.close()


def test_batch_join_and_param_change_with_pending_updates():
    specs = W.batch_manifest(num_scenes=3, seed=44, nmin=2000, nmax=6000)
    # reference: scene 0 alone, 4 substeps, viscosity changed after 2
    ref = Batch(0)
    r = ref.add_scene(specs[0])
    ref.step(2)
    visc = specs[0].viscosity
    changed = copy.deepcopy(specs[0])
    changed.viscosity = visc * 2.0
    ref.set_params(r, changed)
    ref.step(2)
    want = ref.get_state(r)
    ref.close()
    # the same scene in a batch, with another scene joining while it is pending
    b = Batch(0)
    s0 = b.add_scene(specs[0])
    b.add_scene(specs[1])
    b.step(2)
    b.add_scene(specs[2])
    b.set_params(s0, changed)
    b.step(2)
    got = b.get_state(s0)
    b.close()
    for x, y in zip(got, want):
        assert np.array_equal(x, y)


def test_reads_then_profiled_or_partial_prefixes_keep_the_run():
    """A full prefix's scan clears the cell counts that the force pass built;
    a prefix run again before the next force pass (profiled substeps after a
    read) must hash afresh, and a read of one scene of a batch (a prefix over
    that scene's tiles) must leave the counts for the full prefix.  Neither
    may change the trajectory."""
    spec = W.small_dam_break(seed=35)
    want = _plain(spec, 7)
    fs = configure_gpu(FluidSystem(0), spec)
    for _ in range(2):
        fs.advance(spec.dt, 1)
        fs.exportToData()                # the next prefix has run
    fs.setProfiling(True)                # profiled substeps recompute that prefix
    for _ in range(3):
        fs.advance(spec.dt, 1)
    fs.setProfiling(False)
    fs.exportToData()
    for _ in range(2):
        fs.advance(spec.dt, 1)
    got = fs.exportToData()
    fs.close()
    for x, y in zip(got, want):
        assert np.array_equal(x, y)

    specs = W.batch_manifest(num_scenes=2, seed=45, nmin=2000, nmax=6000)

    def run(mid_reads):
        b = Batch(0)
        ids = [b.add_scene(s) for s in specs]
        for k in range(5):
            b.step(1)
            if mid_reads and k in (1, 3):
                b.get_state(ids[1])      # a prefix over scene 1's tiles only
            if mid_reads and k == 3:
                b.set_profiling(True)
        b.set_profiling(False)
        out = [b.get_state(i) for i in ids]
        b.close()
        return out

    plain, read = run(False), run(True)
    for sa, sb in zip(plain, read):
        for x, y in zip(sa, sb):
            assert np.array_equal(x, y)
