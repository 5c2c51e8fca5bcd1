"""Export ahead (sph_set_export_ahead) and the cell-overflow error path.

An export of velocities after a blocking advance waits for the next
substep's density pass (it computes the deferred XSPH update).  With export
ahead on, that export also starts the next substep's normal and force
passes; the next advance takes them when nothing changed, and every other
call undoes them first.  Two systems, one with the option and one without,
go through the same calls here, and every export, snapshot, debug tap and
error must agree bit for bit.

A grid cell of more than 8192 particles (SPH_ECELL) is the error that the
prefix an export waits on can raise; the passes run ahead must then do
nothing.  The reference has no such limit to report: its launch of more than
1024 threads per cell block fails silently (fluidsystem.cu:322).
"""
import ctypes as C

import numpy as np
import pytest

from helpers import configure_gpu
from libfluid_gb300 import FluidSystem, _capi, workloads as W

pytestmark = pytest.mark.gpu


def _pair(spec, **exec_kw):
    out = []
    for on in (True, False):
        fs = configure_gpu(FluidSystem(0), spec)
        if exec_kw:
            fs.setExec(**exec_kw)
        fs.setExportAhead(on)
        out.append(fs)
    return out


def _export(fs):
    return [a.copy() for a in fs.exportToData()]


def _same(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a, b))


def _positions_only(fs):
    """An export of positions alone (no velocities: nothing waits for a
    density pass), through the C ABI."""
    n = fs.numParticles()
    pos = np.empty((n, 3), np.float32)
    rc = _capi.lib().sph_export(fs._h, pos.ctypes.data_as(C.c_void_p), None, None, n)
    assert rc == _capi.SPH_OK
    return pos


def _ops(spec, snap_box, last):
    """Calls that take the passes run ahead (advances at an unchanged time
    step: 2 * dt over 2 substeps is dt exactly) and calls that undo them (a
    return from half the time step to the whole one is such a call too), each
    undoing call followed by advances that take the next ones: two undone in
    a row would pause the option (Engine::settle)."""
    dt = spec.dt

    def snapshot(fs):
        snap_box[fs] = fs.snapshot()
        return snap_box[fs]

    def adv(fs):
        return fs.advance(dt, 1)

    def half(fs):
        return fs.advance(0.5 * dt, 1)

    # each undoing call with the advance that follows it twice: the first
    # runs passes ahead again (if the call left nothing pending), the second
    # takes them
    undoing = [
        ("export again", lambda fs: None, adv),
        ("snapshot", snapshot, adv),
        ("viscosity", lambda fs: fs.setViscosity(spec.viscosity * 1.5), adv),
        ("half dt", half, half),
        ("whole dt", adv, adv),   # back from half the time step: undoes those run with it
        ("density tap", lambda fs: fs.debug("density"), adv),
        ("sync", lambda fs: fs.sync(), adv),   # the export after it undoes them
        ("per-substep xsph", lambda fs: (fs.setDeferredXSPH(False), fs.advance(dt, 1), fs.setDeferredXSPH(True)),
         adv),
        ("tile 64", lambda fs: fs.setExec(**{**fs.getExec(), "tile": 64}), adv),
        ("restore", lambda fs: fs.restore(snap_box[fs]), adv),
        ("set state", lambda fs: fs.setState(last[fs][0], last[fs][2]), adv),
    ]
    ops = [("advance", adv), ("advance x2", lambda fs: fs.advance(2 * dt, 2))]
    for name, call, follow in undoing:
        ops += [(name, call), ("advance", follow), ("advance", follow)]
    # an async step takes them too; its export runs nothing ahead
    ops += [("async + sync", lambda fs: (fs.advanceAsync(dt, 2), fs.sync())), ("advance", adv), ("advance", adv)]
    return ops


@pytest.mark.parametrize("case", ["dam", "tension", "persistent"])
def test_export_ahead_changes_nothing(case):
    """Every call after an export that ran the next force pass ahead sees
    the system exactly as without it: an advance that takes the passes, and
    parameter changes, other time steps, taps, snapshots, restores, state
    uploads, schedule and launch changes that undo them."""
    spec = W.small_dam_break(seed=31)
    kw = {}
    if case == "tension":
        spec.surface_tension = 0.03
    if case == "persistent":
        kw = {"persistent": 2}
    on, off = _pair(spec, **kw)
    snaps, last = {}, {}
    try:
        for fs in (on, off):
            fs.advance(spec.dt, 1)
            last[fs] = _export(fs)
        assert _same(last[on], last[off])
        for name, op in _ops(spec, snaps, last):
            r_on, r_off = op(on), op(off)
            if isinstance(r_on, (bytes, np.ndarray)):
                assert np.array_equal(np.frombuffer(r_on, np.uint8) if isinstance(r_on, bytes) else r_on,
                                      np.frombuffer(r_off, np.uint8) if isinstance(r_off, bytes) else r_off), name
            last[on], last[off] = _export(on), _export(off)
            assert _same(last[on], last[off]), name
        # the passes ran ahead after most exports, and both fates were met
        st = on.exportAheadStats()
        print(case, st)
        assert st["started"] >= 15 and st["taken"] >= 8 and st["undone"] >= 8
        assert off.exportAheadStats() == {"started": 0, "taken": 0, "undone": 0}
    finally:
        on.close()   # with passes run ahead still in flight
        off.close()


def test_export_ahead_frame_loop_matches():
    """The benchmark's frame loop (advance(dt, 1) then exportToData, every
    substep) for 40 frames, with and without export ahead."""
    spec = W.small_dam_break(seed=32)
    on, off = _pair(spec)
    try:
        for _ in range(40):
            on.advance(spec.dt, 1)
            off.advance(spec.dt, 1)
            assert _same(_export(on), _export(off))
        # every export ran the next force pass ahead and each advance took it
        assert on.exportAheadStats() == {"started": 40, "taken": 39, "undone": 0}
    finally:
        on.close()
        off.close()


def test_export_ahead_with_a_changing_time_step():
    """A time step that changes every frame: every pass run ahead is undone,
    so the option pauses after two and tries again after 16 exports; 60
    frames, the same bits as without the option."""
    spec = W.small_dam_break(seed=33)
    on, off = _pair(spec)
    try:
        for f in range(60):
            dt = spec.dt * (1.0 + 0.01 * (f % 7))
            on.advance(dt, 1)
            off.advance(dt, 1)
            assert _same(_export(on), _export(off)), f
        # two undone, a pause of 16 exports, one more try: a handful in 60 frames
        st = on.exportAheadStats()
        print(st)
        assert st["taken"] == 0 and 3 <= st["started"] <= 8 and st["started"] - 1 <= st["undone"] <= st["started"]
    finally:
        on.close()
        off.close()


def _overflow_system(ahead, converge):
    """8,400 particles, all in one cell of 0.05 m (a 20^3 grid) when
    `converge` is False; otherwise 4,200 in that cell and 4,200 just across
    its +x face moving at -2 m/s, which enter it during the first substep."""
    rng = np.random.default_rng(5)
    a = rng.uniform(0.505, 0.545, (4200, 3))
    b = rng.uniform(0.505, 0.545, (4200, 3))
    if converge:
        b[:, 0] = rng.uniform(0.5502, 0.5508, 4200)
    pos = np.concatenate([a, b]).astype(np.float32)
    vel = np.zeros_like(pos)
    if converge:
        vel[4200:, 0] = -2.0
    fs = FluidSystem(0)
    fs.init(pos.shape[0], 1)
    fs.setDomain(1.0, 1.0, 1.0, 0.05)
    # the dam break's fluid (particle size 5 mm: the walls stay out of reach)
    p = W.small_dam_break().params()
    p["dt"] = 1e-3
    fs.setParams(**p)
    fs.setState(pos, vel)
    fs.setExportAhead(ahead)
    return fs, pos


def test_cell_overflow_leaves_the_particles():
    """A cell of 8,400 particles: the step reports SPH_ECELL and no pass
    after the rank pass touches the particles."""
    fs, pos = _overflow_system(True, converge=False)
    try:
        with pytest.raises(_capi.SphError) as err:
            fs.advance(1e-3, 1)
        assert err.value.code == _capi.SPH_ECELL
        assert np.array_equal(_positions_only(fs), pos)
        with pytest.raises(_capi.SphError) as err:
            fs.advance(1e-3, 1)
        assert err.value.code == _capi.SPH_ECELL
        assert np.array_equal(_positions_only(fs), pos)
    finally:
        fs.close()


def test_cell_overflow_in_the_prefix_of_an_export():
    """The first substep fills one cell past 8192 particles, so the prefix
    that the export waits on (started by the advance) fails: with and without
    export ahead the export reports SPH_ECELL, and the particles stay where
    the substep left them (the passes run ahead did nothing)."""
    moved, res = {}, {}
    for ahead in (True, False):
        fs, pos = _overflow_system(ahead, converge=True)
        try:
            assert fs.advance(1e-3, 1) == 1
            with pytest.raises(_capi.SphError) as err:
                fs.exportToData()
            assert err.value.code == _capi.SPH_ECELL
            # the passes launched ahead found the prefix failed: none ran
            assert fs.exportAheadStats()["started"] == 0
            moved[ahead] = _positions_only(fs)
            assert np.all(moved[ahead][4200:, 0] < 0.55)   # all 8,400 in the one cell
            with pytest.raises(_capi.SphError) as err:
                fs.advance(1e-3, 1)
            assert err.value.code == _capi.SPH_ECELL
            assert np.array_equal(_positions_only(fs), moved[ahead])
            # spread out again, the system steps on
            fs.setState(pos, np.zeros_like(pos))
            assert fs.advance(1e-3, 1) == 1
            res[ahead] = _export(fs)
        finally:
            fs.close()
    assert np.array_equal(moved[True], moved[False])
    assert _same(res[True], res[False])
