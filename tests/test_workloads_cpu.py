"""Workload manifests: the batched and served scene sets written as JSON are
deterministic for a seed and rebuild the same scenes (positions bit for bit,
parameters and substeps equal), so a run can be replayed from its manifest."""
import json
import os
import sys

import numpy as np

from libfluid_gb300 import workloads as W

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _roundtrip(specs, steps=None):
    m = W.manifest(specs, steps, workload="test")
    text = json.dumps(m)
    specs2, steps2 = W.from_manifest(json.loads(text))
    assert len(specs2) == len(specs)
    for a, b in zip(specs, specs2):
        assert a.n == b.n and a.params() == b.params() and tuple(a.box) == tuple(b.box) and a.h == b.h
    for a, b in zip(specs[:4], specs2[:4]):
        assert np.array_equal(a.positions(), b.positions())
        assert np.array_equal(a.velocities(), b.velocities())
    if steps is not None:
        assert steps2 == list(steps)
    return text, m


def test_batched_manifest_is_deterministic_and_replays():
    text, m = _roundtrip(W.batch_manifest(256, seed=7))
    again = json.dumps(W.manifest(W.batch_manifest(256, seed=7), workload="test"))
    assert text == again
    assert len(m["scenes"]) == 256 and m["total_particles"] == sum(s["n"] for s in m["scenes"])
    assert 2048 * 0.5 < min(s["n"] for s in m["scenes"]) and max(s["n"] for s in m["scenes"]) < 65536 * 1.5


def test_served_manifest_replays():
    sys.path.insert(0, ROOT)
    import bench
    specs, steps = bench.served_requests(64, seed=13)
    _roundtrip(specs, steps)
    assert all(50 <= k <= 500 for k in steps)
