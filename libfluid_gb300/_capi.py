"""ctypes bindings of include/sph_c.h (libsph_gb300.so).

The product path is the native library; there is no Python or CPU fallback.
Loading fails loudly if the library has not been built.
"""
from __future__ import annotations

import ctypes as C
import os

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libsph_gb300.so")

SPH_OK, SPH_EINVAL, SPH_ENOMEM, SPH_ECUDA, SPH_ENAN, SPH_ETIMEOUT, SPH_ENOTINIT, SPH_ECELL, SPH_EBUSY = range(9)
STATUS_NAMES = {0: "SPH_OK", 1: "SPH_EINVAL", 2: "SPH_ENOMEM", 3: "SPH_ECUDA", 4: "SPH_ENAN",
                5: "SPH_ETIMEOUT", 6: "SPH_ENOTINIT", 7: "SPH_ECELL", 8: "SPH_EBUSY"}

FIELDS = {
    "hash": 0, "perm": 1, "cellstart": 2, "cellocc": 3, "nbrcount": 4, "density": 5, "pressure": 6,
    "soundspeed": 7, "fpressure": 8, "ftension": 9, "fadhesion": 10, "fviscosity": 11, "normal": 12,
    "pos_sorted": 13, "acc": 14, "vel_int": 15,
}


class SphParams(C.Structure):
    _fields_ = [("box_mode", C.c_uint32), ("res", C.c_uint32), ("lx", C.c_float), ("ly", C.c_float),
                ("lz", C.c_float), ("h", C.c_float), ("rest_density", C.c_float), ("gas_constant", C.c_float),
                ("gamma", C.c_float), ("mass", C.c_float), ("particle_size", C.c_float), ("xsph", C.c_float),
                ("surface_tension", C.c_float), ("viscosity", C.c_float), ("adhesion", C.c_float),
                ("vdamp", C.c_float), ("vel_limit", C.c_float), ("acc_limit", C.c_float), ("dt", C.c_float),
                ("gravity", C.c_float * 3)]


class SphExec(C.Structure):
    _fields_ = [("tile", C.c_uint32), ("persistent", C.c_uint32), ("skin", C.c_float), ("variant", C.c_uint32)]


# sph_exec_config.variant bits (include/sph_c.h)
VARIANT_DENSITY_ROWS = 0x1
VARIANT_XSPH_ROWS = 0x2
VARIANT_FORCE_OCC = 0x4
VARIANT_FORCE_TABLE = 0x8
VARIANT_NORMALS_TABLE = 0x10


class SphError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


_lib = None

_P = C.c_void_p
_F = C.c_float
_U32 = C.c_uint32
_I = C.c_int
_FP = C.POINTER(C.c_float)

# (name, restype, argtypes) of every exported C function of include/sph_c.h
SIGNATURES = [
    ("sph_create", _I, [C.POINTER(_P), _I]),
    ("sph_destroy", _I, [_P]),
    ("sph_clear", _I, [_P]),
    ("sph_init", _I, [_P, _U32, _U32]),
    ("sph_setup", _I, [_P, _U32, _U32]),
    ("sph_setup_from_data", _I, [_P, _P, _P, _U32, _U32]),
    ("sph_create_block", _I, [_P, _U32, _U32, _F, _F, _F, _F, _F, _F]),
    ("sph_set_state", _I, [_P, _P, _P, _U32]),
    ("sph_advance", _I, [_P, _F, _U32, C.POINTER(_U32)]),
    ("sph_advance_async", _I, [_P, _F, _U32, C.POINTER(_U32)]),
    ("sph_sync", _I, [_P]),
    ("sph_substep_count", C.c_int64, [_F, _U32]),
    ("sph_export", _I, [_P, _P, _P, _P, _U32]),
    ("sph_get_pscale", _I, [_P, _FP]),
    ("sph_num_particles", _U32, [_P]),
    ("sph_is_init", _I, [_P]),
    ("sph_snapshot_bytes", C.c_uint64, [_U32]),
    ("sph_snapshot", _I, [_P, _P, C.c_uint64, C.POINTER(C.c_uint64)]),
    ("sph_restore", _I, [_P, _P, C.c_uint64]),
    ("sph_set_rest_density", _I, [_P, _F]),
    ("sph_set_particle_size", _I, [_P, _F]),
    ("sph_set_gas_constant", _I, [_P, _F]),
    ("sph_set_limits", _I, [_P, _F, _F]),
    ("sph_set_xsph_scale", _I, [_P, _F]),
    ("sph_set_surface_tension", _I, [_P, _F]),
    ("sph_set_viscosity", _I, [_P, _F]),
    ("sph_set_adhesion", _I, [_P, _F]),
    ("sph_set_vdamp", _I, [_P, _F]),
    ("sph_set_gamma", _I, [_P, _F]),
    ("sph_set_mass", _I, [_P, _F]),
    ("sph_set_gravity", _I, [_P, _F, _F, _F]),
    ("sph_set_domain", _I, [_P, _F, _F, _F, _F]),
    ("sph_set_boundary", _I, [_P, _I]),
    ("sph_get_boundary", _I, [_P, C.POINTER(_I)]),
    ("sph_get_params", _I, [_P, C.POINTER(SphParams)]),
    ("sph_set_params", _I, [_P, C.POINTER(SphParams)]),
    ("sph_get_derived", _I, [_P, C.POINTER(C.c_double), _I]),
    ("sph_derive_params", _I, [C.POINTER(SphParams), C.POINTER(C.c_double), _I]),
    ("sph_debug_enable", _I, [_P, _I]),
    ("sph_debug_scan_fault", _I, [_P, _U32, _I]),
    ("sph_debug_get", _I, [_P, _I, _P, C.c_uint64]),
    ("sph_set_use_graph", _I, [_P, _I]),
    ("sph_set_export_ahead", _I, [_P, _I]),
    ("sph_export_ahead_stats", _I, [_P, C.POINTER(C.c_uint64)]),
    ("sph_set_profiling", _I, [_P, _I]),
    ("sph_set_exec", _I, [_P, C.POINTER(SphExec)]),
    ("sph_set_deferred_xsph", _I, [_P, _I]),
    ("sph_get_exec", _I, [_P, C.POINTER(SphExec)]),
    ("sph_get_pass_times", _I, [_P, C.POINTER(C.c_double), _I, C.POINTER(C.c_uint64)]),
    ("sph_pass_name", C.c_char_p, [_I]),
    ("sph_host_register", _I, [_P, C.c_uint64]),
    ("sph_host_unregister", _I, [_P]),
    ("sph_timer_mark", _I, [_P, _I]),
    ("sph_timer_elapsed", _I, [_P, _I, _I, _FP]),
    ("sph_last_error", C.c_char_p, [_P]),
    ("sph_version", C.c_char_p, []),
    ("sph_scan_cells_noalloc", _I, [_P, _U32, _P, _P]),
    ("sph_write_geo", _I, [C.c_char_p, _P, _P, _P, _U32, _F]),
    ("sph_geo_path", _I, [C.c_char_p, C.c_uint64, C.c_char_p, _U32]),
]


def lib() -> C.CDLL:
    """Load libsph_gb300.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run `python -c 'import __graft_entry__ as g; g.build()'`")
        L = C.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES + _extra_signatures():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _extra_signatures():
    from . import _capi_batch
    return _capi_batch.SIGNATURES


# what a failure without a handle to ask (a failed create) means
_NO_HANDLE_MSG = {
    SPH_ECUDA: "no CUDA device is visible or the CUDA runtime failed; the library has no CPU path",
    SPH_EINVAL: "invalid argument (for a create: a device index out of range or an invalid configuration)",
}


def check(code: int, handle=None) -> None:
    if code != SPH_OK:
        msg = ""
        if handle is not None:
            raw = lib().sph_last_error(handle)
            msg = raw.decode() if raw else ""
        else:
            msg = _NO_HANDLE_MSG.get(code, "")
        raise SphError(code, msg)
