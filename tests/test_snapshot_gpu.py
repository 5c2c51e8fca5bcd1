"""Snapshot / resume (sph_snapshot, sph_restore, sph_batch_snapshot,
sph_batch_restore): a restored system continues bit for bit as the
snapshotted one would have, in a fresh system, in another batch arena and
across scene placements; malformed snapshots are rejected with SPH_EINVAL."""
import struct

import numpy as np
import pytest

from helpers import configure_gpu
from libfluid_gb300 import FluidSystem, _capi, workloads as W
from libfluid_gb300.batch import Batch

pytestmark = pytest.mark.gpu


def _state(fs):
    p, c, v = fs.exportToData()
    return p.copy(), c.copy(), v.copy()


def _same(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a, b))


def test_plain_resume_bit_exact():
    spec = W.small_dam_break(seed=21)
    spec.surface_tension = 0.03
    fs = configure_gpu(FluidSystem(0), spec)
    fs.advance(spec.dt, 1)
    for _ in range(4):
        fs.advance(spec.dt, 1)
    snap = fs.snapshot()
    assert len(snap) == 128 + 48 * spec.n
    magic, version, n, hb = struct.unpack_from("<4I", snap, 0)
    assert (magic, version, n, hb) == (0x53485053, 1, spec.n, 128)
    for _ in range(6):
        fs.advance(spec.dt, 1)
    want = _state(fs)
    fs.close()

    other = FluidSystem(0)
    other.init(spec.n, 16)                     # different domain and defaults: restore replaces them
    other.restore(snap)
    assert other.getParams()["surface_tension"] == pytest.approx(0.03)
    for _ in range(6):
        other.advance(spec.dt, 1)
    assert _same(_state(other), want)
    other.close()


def test_batch_resume_in_another_arena():
    specs = W.batch_manifest(num_scenes=4, seed=41, nmin=2000, nmax=8000)
    b = Batch(0)
    ids = [b.add_scene(s) for s in specs]
    b.step(3)
    snaps = [b.snapshot(i) for i in ids]
    b.step(5)
    want = [b.get_state(i) for i in ids]
    b.close()

    c = Batch(0)                               # reversed order: other slots, other cell bases
    filler = c.add_scene(W.small_dam_break(seed=5))
    rid = {}
    for k in reversed(range(len(specs))):
        rid[k] = c.add_scene(specs[k], generate=False)
        c.restore(rid[k], snaps[k])
    c.remove_scene(filler)
    c.step(5)
    for k in range(len(specs)):
        assert _same(c.get_state(rid[k]), want[k])
    c.close()


def test_malformed_snapshots_rejected():
    spec = W.small_dam_break(seed=22)
    fs = configure_gpu(FluidSystem(0), spec)
    fs.advance(spec.dt, 1)
    snap = fs.snapshot()
    before = _state(fs)
    bad_magic = b"XXXX" + snap[4:]
    for bad in (snap[:100], snap[:-16], bad_magic, snap[:8] + struct.pack("<I", spec.n + 1) + snap[12:]):
        with pytest.raises(_capi.SphError) as e:
            fs.restore(bad)
        assert e.value.code == _capi.SPH_EINVAL
    assert _same(_state(fs), before)           # a rejected restore changes nothing
    fs.close()
