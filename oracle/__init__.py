"""ctypes wrapper of the CPU oracle (oracle/oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline legs of bench.py, as the checker or the timed CPU baseline of
NCCA/libfluid's WCSPH step.  The product library never uses it.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "liboracle.so")

PARAMS = {"rest_density": 0, "particle_size": 1, "gas_constant": 2, "xsph": 3, "surface_tension": 4,
          "viscosity": 5, "adhesion": 6, "vdamp": 7, "gamma": 8, "mass": 9, "dt": 10}
VEC_FIELDS = {"pos": 0, "vel": 1, "acc": 2, "normal": 3, "fpressure": 4, "ftension": 5, "fadhesion": 6,
              "fviscosity": 7, "colour": 8, "vel_int": 9}
SCALAR_FIELDS = {"density": 16, "pressure": 17, "soundspeed": 18, "rho_sum": 19,
                 # test scales (track_scales): sum over pairs of each pair term's magnitude
                 "fpressure_scale": 20, "fviscosity_scale": 21, "ftension_scale": 22, "normal_scale": 23}
U32_FIELDS = {"hash_pre": 32, "hash": 33, "perm": 34, "cellstart": 35, "cellocc": 36, "nbrcount": 37}
STAGES = {"hash_sort": 0, "density": 1, "normals": 2, "forces": 3, "integrate": 4, "xsph": 5, "colour": 6}

_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} missing: build with libfluid_gb300/build.py")
        L = C.CDLL(LIB_PATH)
        P, F, U = C.c_void_p, C.c_float, C.c_uint32
        sig = {
            "orc_create": (P, [C.c_int]), "orc_destroy": (None, [P]), "orc_precision": (C.c_int, [P]),
            "orc_init": (C.c_int, [P, U, U]), "orc_set_domain": (C.c_int, [P, F, F, F, F]),
            "orc_set_boundary": (C.c_int, [P, C.c_int]),
            "orc_set_param": (C.c_int, [P, C.c_int, F]), "orc_set_limits": (C.c_int, [P, F, F]),
            "orc_set_gravity": (C.c_int, [P, F, F, F]),
            "orc_create_block": (C.c_int, [P, U, U, F, F, F, F, F, F]),
            "orc_set_state": (C.c_int, [P, P, P, U]), "orc_set_state_f64": (C.c_int, [P, P, P, P, U]),
            "orc_substep_count": (C.c_int64, [F, U]), "orc_advance": (C.c_int64, [P, F, U]),
            "orc_stage": (C.c_int, [P, C.c_int]), "orc_num_particles": (U, [P]), "orc_num_cells": (U, [P]),
            "orc_get_params": (C.c_int, [P, P, C.c_int]), "orc_get": (C.c_int, [P, C.c_int, P, P, P, C.c_uint64]),
            "orc_set_threads": (C.c_int, [C.c_int]), "orc_track_scales": (C.c_int, [P, C.c_int]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def set_threads(n: int) -> int:
    return int(lib().orc_set_threads(n))


def substep_count(full_dt: float, substeps: int) -> int:
    return int(lib().orc_substep_count(C.c_float(full_dt), substeps))


class Oracle:
    """One scene of the reference algorithm on the CPU (precision 32 or 64)."""

    def __init__(self, precision: int = 32):
        self._L = lib()
        self._h = self._L.orc_create(precision)
        self.precision = precision

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._L.orc_destroy(h)
            self._h = None

    def _ck(self, rc):
        if rc != 0:
            raise RuntimeError(f"oracle call failed ({rc})")

    def init(self, n: int, res: int):
        self._ck(self._L.orc_init(self._h, n, res))

    def set_domain(self, lx, ly, lz, h):
        self._ck(self._L.orc_set_domain(self._h, lx, ly, lz, h))

    def set_boundary(self, shape: int):
        """0: the box (the reference's boundary); 1: the sphere of radius min
        half extent about the box centre."""
        self._ck(self._L.orc_set_boundary(self._h, shape))

    def track_scales(self, on: bool = True):
        """Also record, per particle, the sum of the magnitudes of the pair
        terms of the pressure, viscosity and tension forces and of the normal
        (fields *_scale): the scale of a cancelling sum's rounding error."""
        self._ck(self._L.orc_track_scales(self._h, 1 if on else 0))

    def set_param(self, name: str, v: float):
        self._ck(self._L.orc_set_param(self._h, PARAMS[name], v))

    def set_limits(self, vel: float, acc: float):
        self._ck(self._L.orc_set_limits(self._h, vel, acc))

    def set_gravity(self, gx, gy, gz):
        self._ck(self._L.orc_set_gravity(self._h, gx, gy, gz))

    def create_block(self, first, n, mnx, mny, mnz, mxx, mxy, mxz):
        self._ck(self._L.orc_create_block(self._h, first, n, mnx, mny, mnz, mxx, mxy, mxz))

    def set_state(self, pos, vel=None):
        p = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
        v = None if vel is None else np.ascontiguousarray(vel, np.float32).reshape(-1, 3)
        self._ck(self._L.orc_set_state(self._h, p.ctypes.data, None if v is None else v.ctypes.data, p.shape[0]))

    def set_state_f64(self, pos, vel=None, acc=None):
        arrs = [None if a is None else np.ascontiguousarray(a, np.float64).reshape(-1, 3) for a in (pos, vel, acc)]
        ptrs = [None if a is None else a.ctypes.data for a in arrs]
        self._ck(self._L.orc_set_state_f64(self._h, *ptrs, arrs[0].shape[0]))

    def advance(self, full_dt: float, substeps: int) -> int:
        r = int(self._L.orc_advance(self._h, C.c_float(full_dt), substeps))
        if r < 0:
            raise RuntimeError("substep loop would not terminate")
        return r

    def stage(self, name: str):
        self._ck(self._L.orc_stage(self._h, STAGES[name]))

    @property
    def n(self) -> int:
        return int(self._L.orc_num_particles(self._h))

    @property
    def ncells(self) -> int:
        return int(self._L.orc_num_cells(self._h))

    def params(self) -> np.ndarray:
        buf = (C.c_double * 64)()
        k = self._L.orc_get_params(self._h, buf, 64)
        return np.array(buf[:k])

    def get(self, field: str, dtype=np.float64) -> np.ndarray:
        n = self.n
        if field in VEC_FIELDS:
            out = np.empty((n, 3), dtype)
            f = VEC_FIELDS[field]
        elif field in SCALAR_FIELDS:
            out = np.empty(n, dtype)
            f = SCALAR_FIELDS[field]
        else:
            f = U32_FIELDS[field]
            size = self.ncells if field in ("cellstart", "cellocc") else n
            out = np.empty(size, np.uint32)
            self._ck(self._L.orc_get(self._h, f, None, None, out.ctypes.data, out.size))
            return out
        p32 = out.ctypes.data if dtype == np.float32 else None
        p64 = out.ctypes.data if dtype == np.float64 else None
        self._ck(self._L.orc_get(self._h, f, p32, p64, None, out.size))
        return out
