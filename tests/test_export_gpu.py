"""exportToData into host buffers registered with sph_host_register: the pack
kernel writes them directly (mapped pinned memory); results are identical to
the export into pageable buffers (staging + copy), also when only some of the
three buffers are registered."""
import numpy as np
import pytest

from helpers import configure_gpu
from libfluid_gb300 import FluidSystem, _capi, workloads as W

pytestmark = pytest.mark.gpu


def test_registered_export_matches_pageable():
    spec = W.small_dam_break(seed=12)
    fs = configure_gpu(FluidSystem(0), spec)
    for _ in range(3):
        fs.advance(spec.dt, 1)
    want = [a.copy() for a in fs.exportToData()]
    L = _capi.lib()
    n = spec.n
    for registered in ((0, 1, 2), (1,), ()):
        outs = [np.full((n, 3), np.nan, np.float32) for _ in range(3)]
        for i in registered:
            assert L.sph_host_register(outs[i].ctypes.data, outs[i].nbytes) == 0
        try:
            got = fs.exportToData(*outs)
        finally:
            for i in registered:
                L.sph_host_unregister(outs[i].ctypes.data)
        for g, w in zip(got, want):
            assert np.array_equal(g, w)
    fs.close()
