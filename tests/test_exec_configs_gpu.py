"""Every launch configuration computes the same values bit for bit: tile
size, persistent tile scheduling, neighbour-mask skin (including a skin so
small that XSPH falls back to the full candidate walk), graph or eager."""
import numpy as np
import pytest

from libfluid_gb300 import workloads as W
from libfluid_gb300.batch import Batch

pytestmark = pytest.mark.gpu


def _run(specs, steps, graph=True, deferred=True, **exe):
    b = Batch(0)
    b.set_exec(**exe)
    b.set_use_graph(graph)
    b.set_deferred_xsph(deferred)
    ids = [b.add_scene(s) for s in specs]
    b.step(steps)
    out = [b.get_state(i) for i in ids]
    b.close()
    return out


@pytest.mark.parametrize("exe", [dict(tile=128, persistent=0, skin=0.2), dict(tile=64, persistent=2, skin=0.2),
                                 dict(tile=256, persistent=4, skin=0.1), dict(tile=256, persistent=0, skin=0.3),
                                 dict(tile=128, persistent=1, skin=0.01)])
def test_configs_bit_identical(exe):
    specs = W.batch_manifest(num_scenes=4, seed=31, nmin=2000, nmax=12000)
    specs.append(W.small_dam_break(seed=8))
    base = _run(specs, 6, tile=256, persistent=0, skin=0.2)
    other = _run(specs, 6, **exe)
    for (pa, ca, va), (pb, cb, vb) in zip(base, other):
        assert np.array_equal(pa, pb) and np.array_equal(va, vb) and np.array_equal(ca, cb)


@pytest.mark.parametrize("tile", [64, 128, 256])
def test_split_scan_bit_identical(tile):
    """The density scan split over three threads per particle (launches of
    at most 49,152 particles; this one holds 40,928), at every tile size,
    against the one-thread scan, with surface tension in one scene."""
    specs = [W.small_dam_break(seed=12)] + W.batch_manifest(num_scenes=1, seed=43, nmin=8000, nmax=8000)
    assert sum(s.n for s in specs) <= 49152
    base = _run(specs, 6, tile=tile, persistent=0, skin=0.1, variant=31)
    other = _run(specs, 6, tile=tile, persistent=0, skin=0.1, variant=63)
    for (pa, ca, va), (pb, cb, vb) in zip(base, other):
        assert np.array_equal(pa, pb) and np.array_equal(va, vb) and np.array_equal(ca, cb)


@pytest.mark.parametrize("variant", [1, 2, 4, 7, 8, 12, 15, 16, 31, 33, 63])
def test_variants_bit_identical(variant):
    """Per-row density/XSPH walks, the density scan split over three
    threads per particle (in the single-scene runs below), the 64-register
    force kernel and the force kernel's row-table walk visit neighbours in
    the same order as the default walks: identical results, with and without
    surface tension."""
    specs = W.batch_manifest(num_scenes=3, seed=37, nmin=2000, nmax=9000)
    specs.append(W.small_dam_break(seed=10))
    base = _run(specs, 6, tile=128, persistent=0, skin=0.1, variant=0)
    other = _run(specs, 6, tile=128, persistent=0, skin=0.1, variant=variant)
    for (pa, ca, va), (pb, cb, vb) in zip(base, other):
        assert np.array_equal(pa, pb) and np.array_equal(va, vb) and np.array_equal(ca, cb)
    plain = [W.small_dam_break(seed=11)]        # no tension anywhere: the tension-free force kernel
    a = _run(plain, 6, variant=0)
    b = _run(plain, 6, variant=variant)
    assert np.array_equal(a[0][0], b[0][0]) and np.array_equal(a[0][2], b[0][2])


def test_eager_equals_graph():
    specs = [W.small_dam_break(seed=9)]
    a = _run(specs, 5, graph=True)
    b = _run(specs, 5, graph=False)
    assert np.array_equal(a[0][0], b[0][0]) and np.array_equal(a[0][2], b[0][2])


@pytest.mark.parametrize("deferred", [True, False])
@pytest.mark.parametrize("variant", [1, 2, 8, 16, 31, 33, 63])
def test_variants_bit_identical_crowded(variant, deferred):
    """The same on compressed lattices whose cell rows hold 33 to 160
    candidates, so the two-word masks and the rows walked in full meet every
    walk (the table walks and the mask walks of the normal and force passes,
    both density loops, and, without deferral, the per-substep XSPH pass's
    skin walks), with surface tension so the normal pass runs."""
    specs = []
    for k, spacing in enumerate((0.0075, 0.006)):
        lat = W.Lattice(lo=(0.05, 0.05, 0.05), spacing=spacing, nx=20, ny=20, nz=20, jitter=0.05 * spacing,
                        seed=41 + k)
        specs.append(W.SceneSpec(box=(0.4, 0.4, 0.4), h=0.02, blocks=[lat], mass=1e-3, particle_size=0.005,
                                 dt=1e-4, steps=4, surface_tension=0.05))
    base = _run(specs, 4, deferred=deferred, tile=128, persistent=0, skin=0.1, variant=0)
    other = _run(specs, 4, deferred=deferred, tile=128, persistent=0, skin=0.1, variant=variant)
    for (pa, ca, va), (pb, cb, vb) in zip(base, other):
        assert np.array_equal(pa, pb) and np.array_equal(va, vb) and np.array_equal(ca, cb)
