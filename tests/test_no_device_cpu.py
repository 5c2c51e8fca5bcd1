"""Without a visible CUDA device every entry point that creates a system,
a batch or a server fails with SPH_ECUDA and says so; there is no CPU
fallback (the oracle is test infrastructure, never the product path)."""
import pytest

from libfluid_gb300 import FluidSystem
from libfluid_gb300._capi import SPH_ECUDA, SphError, lib
from libfluid_gb300.batch import Batch
from libfluid_gb300.server import Server


def _device_visible() -> bool:
    torch = pytest.importorskip("torch")
    return torch.cuda.is_available()


@pytest.mark.skipif(_device_visible(), reason="a CUDA device is visible")
@pytest.mark.parametrize("make", [lambda: FluidSystem(0), lambda: Batch(0), lambda: Server(0)])
def test_create_without_device_fails_loudly(make):
    lib()   # the library itself loads
    with pytest.raises(SphError) as e:
        make()
    assert e.value.code == SPH_ECUDA
    assert "no CPU path" in str(e.value)
