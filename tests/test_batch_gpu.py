"""Batched step: many scenes of uneven size, different domains and
parameters, advanced by one launch per pass.

Each scene's arithmetic is scene-local (its own cell ranges, sort order and
parameters), so a scene's results are bit-identical whether it runs alone or
in the mix; that is what is asserted, together with oracle parity and
scenes joining and leaving between steps."""
import numpy as np
import pytest

import oracle
from helpers import configure_oracle, rel_err
from libfluid_gb300 import FluidSystem, workloads as W
from libfluid_gb300.batch import Batch

pytestmark = pytest.mark.gpu


def _mix(count=6, seed=3):
    specs = W.batch_manifest(num_scenes=count, seed=seed, nmin=1500, nmax=9000)
    specs[1].unit_cube_res = 25          # one scene in the reference's unit cube
    specs[1].box = (1.0, 1.0, 1.0)
    specs[2].surface_tension = 0.0
    specs[3].surface_tension = 0.05
    if count > 4:
        specs[4].adhesion = 0.2
    return specs


def test_device_lattice_matches_host_generator():
    spec = W.small_dam_break(seed=17)
    b = Batch(0)
    sid = b.add_scene(spec)
    pos, _, vel = b.get_state(sid)
    assert np.array_equal(pos, spec.positions())
    assert np.array_equal(vel, spec.velocities())


def test_each_scene_identical_alone_and_in_the_mix():
    specs = _mix()
    steps = 4
    batch = Batch(0)
    ids = [batch.add_scene(s) for s in specs]
    for _ in range(steps):
        batch.step(1)
    for s, sid in zip(specs, ids):
        alone = Batch(0)
        aid = alone.add_scene(s)
        for _ in range(steps):
            alone.step(1)
        pa, ca, va = alone.get_state(aid)
        pb, cb, vb = batch.get_state(sid)
        assert np.array_equal(pa, pb) and np.array_equal(va, vb) and np.array_equal(ca, cb)
        alone.close()


def test_engine_reused_after_a_larger_scene():
    """A scene added to an engine after a larger one was removed gives the
    same results as in a fresh engine.  The slots past its end then hold the
    old scene's particles: a candidate scan that read one slot past an empty
    cell row (the row starts at the scene's last slot, an odd one) found
    three phantom neighbours there for nine particles of this scene."""
    specs = W.batch_manifest(num_scenes=256, seed=7)
    fresh = Batch(0)
    fid = fresh.add_scene(specs[175])
    fresh.step(10)
    want = fresh.get_state(fid)
    fresh.close()
    reused = Batch(0)
    pid = reused.add_scene(specs[174])
    reused.step(3)
    reused.get_state(pid)
    reused.remove_scene(pid)
    aid = reused.add_scene(specs[175])
    reused.step(10)
    got = reused.get_state(aid)
    reused.close()
    assert all(np.array_equal(x, y) for x, y in zip(got, want))


def test_benchmark_batch_identical_alone_and_in_the_mix():
    """The benchmarked batch (256 dam breaks of 2,048-65,536 particles, 4.5M
    in all, with viscosity and surface tension varying per scene): 10
    substeps with one launch per pass, then each scene run alone for the same
    substeps (in turn, in one engine) gives the same positions, colours and
    velocities to the bit."""
    specs = W.batch_manifest(num_scenes=256, seed=7)
    steps = 10
    batch = Batch(0)
    ids = [batch.add_scene(s) for s in specs]
    batch.step(steps)
    mixed = [batch.get_state(sid) for sid in ids]
    batch.close()
    alone = Batch(0)
    bad = []
    for k, s in enumerate(specs):
        aid = alone.add_scene(s)
        alone.step(steps)
        got = alone.get_state(aid)
        if not all(np.array_equal(x, y) for x, y in zip(got, mixed[k])):
            bad.append(k)
        alone.remove_scene(aid)
    alone.close()
    assert not bad, f"scenes differing alone and in the mix: {bad[:10]} ({len(bad)} of {len(specs)})"


def test_batch_matches_oracle_per_scene():
    specs = _mix(count=4, seed=11)
    b = Batch(0)
    ids = [b.add_scene(s) for s in specs]
    b.step(1)
    for s, sid in zip(specs, ids):
        o = configure_oracle(oracle.Oracle(32), s)
        o.advance(s.dt, 1)
        pos, _, vel = b.get_state(sid)
        assert rel_err(pos, o.get("pos"), 1e-3) < 1e-6
        vs = float(np.sqrt((o.get("vel") ** 2).sum(1).mean())) + 1e-9
        assert rel_err(vel, o.get("vel"), 1e-2 * vs) < 1e-4


def test_plain_system_equals_single_scene_batch():
    spec = W.small_dam_break(seed=4)
    fs = FluidSystem(0)
    fs.init(spec.n, 1)
    fs.setDomain(*spec.box, spec.h)
    p = spec.params()
    fs.setParams(**{k: v for k, v in p.items()})
    fs.setState(spec.positions(), spec.velocities())
    b = Batch(0)
    sid = b.add_scene(spec)
    for _ in range(3):
        fs.advance(spec.dt, 1)
        b.step(1)
    pf, cf, vf = fs.exportToData()
    pb, cb, vb = b.get_state(sid)
    assert np.array_equal(pf, pb) and np.array_equal(vf, vb)


def test_scenes_join_and_leave_between_steps():
    specs = _mix(count=5, seed=21)
    b = Batch(0)
    ids = [b.add_scene(s) for s in specs[:3]]
    b.step(2)
    b.remove_scene(ids[1])
    late = b.add_scene(specs[3])
    b.step(2)
    b.remove_scene(ids[0])
    b.add_scene(specs[4])
    b.step(1)
    # scene 2 ran 5 substeps through three different batch layouts
    ref = Batch(0)
    rid = ref.add_scene(specs[2])
    ref.step(5)
    assert np.array_equal(b.get_state(ids[2])[0], ref.get_state(rid)[0])
    # the late joiner ran 3 substeps
    ref2 = Batch(0)
    r2 = ref2.add_scene(specs[3])
    ref2.step(3)
    assert np.array_equal(b.get_state(late)[2], ref2.get_state(r2)[2])
    assert b.num_scenes == 3
