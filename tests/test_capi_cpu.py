"""CPU checks of the C ABI boundary: the library loads and exports every
function include/sph_c.h declares; host-only entry points behave like the
reference.  No kernel is launched here."""
import ctypes as C
import os
import re

import numpy as np

from libfluid_gb300 import _capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header: str) -> list[str]:
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_ \*]*?\b(sph_[a-z0-9_]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(_capi.LIB_PATH)
    names = _declared("sph_c.h")
    assert len(names) > 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_ctypes_signatures_cover_header():
    names = set(_declared("sph_c.h"))
    bound = {n for n, _, _ in _capi.SIGNATURES + _capi._extra_signatures()}
    assert names == bound, (names - bound, bound - names)


def test_substep_count_matches_reference_loop():
    L = _capi.lib()
    # fluidsystem.cu:301 float loop: advance(0.01, 10) runs 9 substeps
    assert L.sph_substep_count(C.c_float(0.01), 10) == 9
    assert L.sph_substep_count(C.c_float(2e-4), 1) == 1
    assert L.sph_substep_count(C.c_float(0.002), 1) == 1
    assert L.sph_substep_count(C.c_float(0.0), 0) == 0
    # a loop whose accumulator stalls never ends in the reference
    assert L.sph_substep_count(C.c_float(1.0), 1 << 30) == -1
    # brute-force the rule in numpy float32 for a sweep
    for full, sub in [(0.01, 3), (0.033, 7), (1.0, 10), (0.1, 25), (0.002, 4)]:
        part = np.float32(full) / np.float32(sub)
        t, cnt = part, 0
        while t <= np.float32(full):
            cnt += 1
            t = np.float32(t + part)
        assert L.sph_substep_count(C.c_float(full), sub) == cnt


def test_version_string():
    assert b"sm_103a" in _capi.lib().sph_version()
