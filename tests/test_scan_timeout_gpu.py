"""The cell scan's bounded look-back wait, made to run out on the GPU.

The one wait inside a kernel of the substep is the scan's look-back on the
tiles before it (k_scan_single).  The test control sph_debug_scan_fault
lowers its poll limit and withholds the first tile (no block takes it), so
every wait that reaches that tile gives up: the step must return
SPH_ETIMEOUT, every pass after the scan must leave the particles alone (their
cell starts are invalid), and once the control is cleared the system must
continue exactly as a system that never failed.  The reference's scan is
thrust's (fluidsystem.cu:316) and has no such failure; its closest failure,
a launch of more than 1024 threads per cell (fluidsystem.cu:322), goes
unreported.
"""
import numpy as np
import pytest

from helpers import configure_gpu
from libfluid_gb300 import FluidSystem, _capi, workloads as W

pytestmark = pytest.mark.gpu

SPIN_LIMIT = 256   # polls per wait: the failed scan ends within milliseconds


def _system(spec):
    fs = FluidSystem(0)
    configure_gpu(fs, spec)
    return fs


def _state(fs):
    return [a.copy() for a in fs.exportToData()]


def _same(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a, b))


@pytest.mark.parametrize("substeps", [1, 4])
def test_scan_timeout_is_reported_and_the_state_kept(substeps):
    spec = W.small_dam_break(seed=21)   # 45,001 cells: 11 scan tiles
    clean, faulty = _system(spec), _system(spec)
    for fs in (clean, faulty):
        for _ in range(3):
            assert fs.advance(spec.dt, 1) == 1
    before = _state(faulty)
    assert _same(before, _state(clean))

    faulty.debugScanFault(SPIN_LIMIT, True)
    with pytest.raises(_capi.SphError) as err:
        faulty.advance(spec.dt * substeps, substeps)
    assert err.value.code == _capi.SPH_ETIMEOUT
    faulty.debugScanFault(0, False)

    # nothing after the failed scan touched the particles
    assert _same(_state(faulty), before)

    # and the system carries on as one that never failed, bit for bit
    for _ in range(5):
        assert faulty.advance(spec.dt, 1) == 1
        assert clean.advance(spec.dt, 1) == 1
    assert _same(_state(faulty), _state(clean))
    faulty.close()
    clean.close()


def test_scan_timeout_then_a_second_fault_and_recovery():
    """Two failed steps in a row, then recovery: the control takes effect on
    every step it is set for, and clearing it is enough to go on."""
    spec = W.small_dam_break(seed=22)
    clean, faulty = _system(spec), _system(spec)
    for fs in (clean, faulty):
        assert fs.advance(spec.dt, 1) == 1
    faulty.debugScanFault(SPIN_LIMIT, True)
    for _ in range(2):
        with pytest.raises(_capi.SphError) as err:
            faulty.advance(spec.dt, 1)
        assert err.value.code == _capi.SPH_ETIMEOUT
    faulty.debugScanFault(0, False)
    for _ in range(3):
        assert faulty.advance(spec.dt, 1) == 1
        assert clean.advance(spec.dt, 1) == 1
    assert _same(_state(faulty), _state(clean))
    faulty.close()
    clean.close()
