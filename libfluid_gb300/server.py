"""Python host mirror of the served step (include/sph_c.h, sph_server_*)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._capi import SphError, SphParams, check, lib
from ._capi_batch import SphLattice
from .batch import lattice_struct, params_struct
from .workloads import SceneSpec

QUEUED, RUNNING, DONE, FAILED, UNKNOWN = range(5)


class ServerConfig(C.Structure):
    _fields_ = [("device", C.c_int), ("memory_budget", C.c_uint64), ("max_live_scenes", C.c_uint32),
                ("substeps_per_iteration", C.c_uint32)]


class Request(C.Structure):
    _fields_ = [("params", SphParams), ("n", C.c_uint32), ("steps", C.c_uint32), ("pos", C.c_void_p),
                ("vel", C.c_void_p), ("blocks", C.POINTER(SphLattice)), ("num_blocks", C.c_uint32),
                ("pad_", C.c_uint32)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("admitted", C.c_uint64), ("completed", C.c_uint64),
                ("failed", C.c_uint64), ("rejected", C.c_uint64), ("iterations", C.c_uint64),
                ("particle_steps", C.c_uint64), ("busy_seconds", C.c_double), ("live_scenes", C.c_uint32),
                ("queued", C.c_uint32), ("live_particles", C.c_uint64), ("device_bytes", C.c_uint64),
                ("peak_live_particles", C.c_uint64), ("admit_seconds", C.c_double), ("read_seconds", C.c_double),
                ("layout_seconds", C.c_double), ("admit_retries", C.c_uint64)]


class Server:
    """Continuous-batching request loop on one GPU."""

    def __init__(self, device: int = -1, memory_budget: int = 100 << 30, max_live_scenes: int = 0,
                 substeps_per_iteration: int = 1):
        self._L = lib()
        cfg = ServerConfig(device, memory_budget, max_live_scenes, substeps_per_iteration)
        h = C.c_void_p()
        check(self._L.sph_server_create(C.byref(h), C.byref(cfg)))
        self._h = h
        self._n: dict[int, int] = {}

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._L.sph_server_destroy(h)
            self._h = None

    def close(self):
        self.__del__()

    def _ck(self, rc):
        if rc != 0:
            raw = self._L.sph_server_last_error(self._h)
            raise SphError(rc, raw.decode() if raw else "")

    def submit(self, spec: SceneSpec, steps: int, pos=None, vel=None) -> int:
        req = Request()
        req.params = params_struct(spec)
        req.n = spec.n
        req.steps = steps
        keep = []
        if pos is not None:
            p = np.ascontiguousarray(pos, np.float32)
            keep.append(p)
            req.pos = p.ctypes.data
            if vel is not None:
                v = np.ascontiguousarray(vel, np.float32)
                keep.append(v)
                req.vel = v.ctypes.data
        else:
            arr = (SphLattice * len(spec.blocks))(*[lattice_struct(b) for b in spec.blocks])
            keep.append(arr)
            req.blocks = arr
            req.num_blocks = len(spec.blocks)
        rid = C.c_uint64(0)
        self._ck(self._L.sph_server_submit(self._h, C.byref(req), C.byref(rid)))
        self._n[rid.value] = spec.n
        return rid.value

    def state(self, rid: int) -> int:
        return int(self._L.sph_server_state(self._h, rid))

    def wait(self, rid: int, timeout_ms: int = -1) -> bool:
        rc = self._L.sph_server_wait(self._h, rid, timeout_ms)
        if rc == 5:
            return False
        self._ck(rc)
        return True

    def times(self, rid: int):
        a, b, c = C.c_double(), C.c_double(), C.c_double()
        self._ck(self._L.sph_server_times(self._h, rid, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def fetch(self, rid: int):
        n = self._n.pop(rid)
        pos = np.empty((n, 3), np.float32)
        vel = np.empty((n, 3), np.float32)
        self._ck(self._L.sph_server_fetch(self._h, rid, pos.ctypes.data, vel.ctypes.data, n))
        return pos, vel

    def stats(self) -> dict:
        s = ServerStats()
        self._ck(self._L.sph_server_get_stats(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in ServerStats._fields_}

    def drain(self, timeout_ms: int = -1) -> bool:
        rc = self._L.sph_server_drain(self._h, timeout_ms)
        if rc == 5:
            return False
        self._ck(rc)
        return True
