"""Served step: continuous batching.

Requests arrive while others run, are admitted against a device-memory
budget as slots free up, run overlapped in the batched step, and each result
must be bit-identical to the same scene run alone.  Faults are injected on
the host: malformed and over-budget requests, a wait that times out."""
import time

import numpy as np
import pytest

from libfluid_gb300 import SphError, workloads as W
from libfluid_gb300.batch import Batch
from libfluid_gb300.server import DONE, Server

pytestmark = pytest.mark.gpu


def _alone(spec, steps):
    b = Batch(0)
    sid = b.add_scene(spec)
    b.step(steps)
    pos, _, vel = b.get_state(sid)
    b.close()
    return pos, vel


def test_results_identical_alone_and_in_the_mix():
    specs = W.batch_manifest(num_scenes=6, seed=5, nmin=1024, nmax=8000, steps=12)
    steps = [7, 12, 3, 9, 5, 11]
    srv = Server(0, memory_budget=2 << 30)
    ids = []
    for k, (s, n) in enumerate(zip(specs, steps)):
        ids.append(srv.submit(s, n))
        if k % 2 == 1:
            time.sleep(0.01)   # later requests arrive while earlier ones are running
    assert srv.drain(60000)
    st = srv.stats()
    assert st["completed"] == 6 and st["failed"] == 0
    assert st["particle_steps"] == sum(s.n * n for s, n in zip(specs, steps))
    for rid, s, n in zip(ids, specs, steps):
        assert srv.state(rid) == DONE
        t_sub, t_adm, t_done = srv.times(rid)
        assert 0.0 <= t_sub <= t_adm <= t_done
        pos, vel = srv.fetch(rid)
        pa, va = _alone(s, n)
        assert np.array_equal(pos, pa) and np.array_equal(vel, va)
    srv.close()


def _request_bytes(s):
    # the server's footprint of a scene: particle slots, cells + NULL bucket, tile entries
    cells = int(np.prod([int(np.ceil(b / s.h - 1e-3)) for b in s.box]))
    return s.n * 196 + (cells + 1) * 8 + (s.n // 64 + 1) * 16


def test_admission_respects_memory_budget():
    specs = W.batch_manifest(num_scenes=5, seed=9, nmin=4000, nmax=4100, steps=6)
    per_scene = max(_request_bytes(s) for s in specs)
    # room for two scenes, never three
    srv = Server(0, memory_budget=int(2.5 * per_scene))
    ids = [srv.submit(s, 6) for s in specs]
    assert srv.drain(60000)
    st = srv.stats()
    assert st["completed"] == 5
    assert st["peak_live_particles"] <= 2 * max(s.n for s in specs)
    assert st["device_bytes"] <= int(2.5 * per_scene)
    for rid, s in zip(ids, specs):
        pos, vel = srv.fetch(rid)
        pa, va = _alone(s, 6)
        assert np.array_equal(pos, pa)
    srv.close()


def test_host_side_fault_injection():
    srv = Server(0, memory_budget=64 << 20)
    big = W.dam_break_1m()                      # 1M particles cannot fit 64 MiB
    with pytest.raises(SphError) as e:
        srv.submit(big, 10)
    assert e.value.code == 8                    # SPH_EBUSY
    bad = W.small_dam_break()
    bad.h = -1.0                                # malformed domain
    with pytest.raises(SphError) as e:
        srv.submit(bad, 10)
    assert e.value.code == 1                    # SPH_EINVAL
    ok = W.small_dam_break()
    rid = srv.submit(ok, 400)
    assert srv.wait(rid, timeout_ms=1) is False  # bounded wait runs out, request still pending
    assert srv.wait(rid, timeout_ms=120000)
    st = srv.stats()
    assert st["rejected"] == 1 and st["completed"] == 1
    srv.close()


def test_request_with_host_arrays():
    spec = W.small_dam_break(seed=2)
    pos0, vel0 = spec.positions(), spec.velocities()
    srv = Server(0, memory_budget=1 << 30)
    rid = srv.submit(spec, 5, pos=pos0, vel=vel0)
    assert srv.wait(rid, 60000)
    pos, vel = srv.fetch(rid)
    pa, va = _alone(spec, 5)
    assert np.array_equal(pos, pa) and np.array_equal(vel, va)
    srv.close()
