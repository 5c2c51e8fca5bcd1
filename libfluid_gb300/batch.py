"""Python host mirror of the batched step (include/sph_c.h, sph_batch_*)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._capi import SphParams, check, lib
from ._capi_batch import SphLattice
from .workloads import Lattice, SceneSpec


def params_struct(spec: SceneSpec) -> SphParams:
    p = SphParams()
    if spec.unit_cube_res:
        p.box_mode, p.res = 0, spec.unit_cube_res
        p.lx = p.ly = p.lz = 1.0
        p.h = 1.0 / spec.unit_cube_res
    else:
        p.box_mode, p.res = 1, 0
        p.lx, p.ly, p.lz = spec.box
        p.h = spec.h
    d = spec.params()
    for k in ("rest_density", "gas_constant", "gamma", "mass", "particle_size", "xsph", "surface_tension",
              "viscosity", "adhesion", "vdamp", "vel_limit", "acc_limit", "dt"):
        setattr(p, k, float(d[k]))
    for i in range(3):
        p.gravity[i] = float(d["gravity"][i])
    return p


def lattice_struct(b: Lattice) -> SphLattice:
    s = SphLattice()
    for i in range(3):
        s.lo[i] = float(b.lo[i])
        s.vel[i] = float(b.vel[i])
    s.spacing, s.jitter = float(b.spacing), float(b.jitter)
    s.nx, s.ny, s.nz = b.nx, b.ny, b.nz
    s.seed = int(b.seed)
    return s


class Batch:
    """Many independent scenes advanced with one launch per pass."""

    def __init__(self, device: int = -1):
        self._L = lib()
        h = C.c_void_p()
        check(self._L.sph_batch_create(C.byref(h), device))
        self._h = h
        self.scenes: dict[int, SceneSpec] = {}

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._L.sph_batch_destroy(h)
            self._h = None

    def close(self):
        self.__del__()

    def _ck(self, code):
        if code != 0:
            raw = self._L.sph_batch_last_error(self._h)
            from ._capi import SphError
            raise SphError(code, raw.decode() if raw else "")

    def add_scene(self, spec: SceneSpec, generate: bool = True) -> int:
        sid = C.c_int(-1)
        p = params_struct(spec)
        self._ck(self._L.sph_batch_add_scene(self._h, C.byref(p), spec.n, C.byref(sid)))
        self.scenes[sid.value] = spec
        if getattr(spec, "boundary", 0):
            self._ck(self._L.sph_batch_set_boundary(self._h, sid.value, spec.boundary))
        if generate and getattr(spec, "extra_pos", None) is not None:
            # particles beyond the lattice blocks come from the host (the
            # lattice part is identical to the device generator's)
            self.set_state(sid.value, spec.positions(), spec.velocities())
        elif generate:
            first = 0
            for b in spec.blocks:
                s = lattice_struct(b)
                self._ck(self._L.sph_batch_generate_lattice(self._h, sid.value, C.byref(s), first))
                first += b.n
        return sid.value

    def remove_scene(self, sid: int) -> None:
        self._ck(self._L.sph_batch_remove_scene(self._h, sid))
        self.scenes.pop(sid, None)

    def set_params(self, sid: int, spec: SceneSpec) -> None:
        """Replace a scene's parameters with those of `spec` (state is kept)."""
        p = params_struct(spec)
        self._ck(self._L.sph_batch_set_params(self._h, sid, C.byref(p)))
        self.scenes[sid] = spec

    def set_state(self, sid: int, pos, vel=None) -> None:
        p = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
        v = None if vel is None else np.ascontiguousarray(vel, np.float32).reshape(-1, 3)
        self._ck(self._L.sph_batch_set_state(self._h, sid, p.ctypes.data, None if v is None else v.ctypes.data,
                                             p.shape[0]))

    def step(self, substeps: int = 1) -> None:
        self._ck(self._L.sph_batch_step(self._h, substeps))

    def step_async(self, substeps: int = 1) -> None:
        self._ck(self._L.sph_batch_step_async(self._h, substeps))

    def sync(self) -> None:
        self._ck(self._L.sph_batch_sync(self._h))

    def get_state(self, sid: int):
        n = self.scenes[sid].n
        outs = [np.empty((n, 3), np.float32) for _ in range(3)]
        self._ck(self._L.sph_batch_get_state(self._h, sid, *[o.ctypes.data for o in outs], n))
        return tuple(outs)

    def snapshot(self, sid: int) -> bytes:
        """Exact snapshot of one scene (sph_snapshot format)."""
        size = int(self._L.sph_snapshot_bytes(self.scenes[sid].n))
        buf = C.create_string_buffer(size)
        written = C.c_uint64(0)
        self._ck(self._L.sph_batch_snapshot(self._h, sid, buf, size, C.byref(written)))
        return buf.raw[:written.value]

    def restore(self, sid: int, snap: bytes) -> None:
        self._ck(self._L.sph_batch_restore(self._h, sid, snap, len(snap)))

    @property
    def num_scenes(self) -> int:
        return int(self._L.sph_batch_num_scenes(self._h))

    @property
    def num_particles(self) -> int:
        return int(self._L.sph_batch_num_particles(self._h))

    def debug_enable(self, on: bool = True) -> None:
        self._ck(self._L.sph_batch_debug_enable(self._h, 1 if on else 0))

    def debug(self, sid: int, field: str, ncells: int | None = None) -> np.ndarray:
        from ._capi import FIELDS
        n = self.scenes[sid].n
        if field in ("cellstart", "cellocc"):
            out = np.empty(int(ncells), np.uint32)
        elif field in ("hash", "perm", "nbrcount"):
            out = np.empty(n, np.uint32)
        elif field in ("density", "pressure", "soundspeed"):
            out = np.empty(n, np.float32)
        else:
            out = np.empty((n, 3), np.float32)
        self._ck(self._L.sph_batch_debug_get(self._h, sid, FIELDS[field], out.ctypes.data, out.size))
        return out

    def set_use_graph(self, on: bool) -> None:
        self._ck(self._L.sph_batch_set_use_graph(self._h, 1 if on else 0))

    def set_exec(self, tile: int = 128, persistent: int = 0, skin: float = 0.1, variant: int = 63) -> None:
        from ._capi import SphExec
        e = SphExec(tile, persistent, skin, variant)
        self._ck(self._L.sph_batch_set_exec(self._h, C.byref(e)))

    def set_deferred_xsph(self, on: bool) -> None:
        self._ck(self._L.sph_batch_set_deferred_xsph(self._h, 1 if on else 0))

    def set_profiling(self, on: bool) -> None:
        """Per-pass CUDA events around each pass (replaces graph replay)."""
        self._ck(self._L.sph_batch_set_profiling(self._h, 1 if on else 0))

    def pass_times(self) -> tuple[dict, int]:
        """Accumulated per-pass milliseconds and the substeps they cover."""
        buf = (C.c_double * 8)()
        n = C.c_uint64(0)
        self._ck(self._L.sph_batch_get_pass_times(self._h, buf, 8, C.byref(n)))
        return {self._L.sph_pass_name(i).decode(): buf[i] for i in range(8)}, n.value

    def timer_mark(self, slot: int) -> None:
        self._ck(self._L.sph_batch_timer_mark(self._h, slot))

    def timer_elapsed(self, a: int, b: int) -> float:
        ms = C.c_float(0.0)
        self._ck(self._L.sph_batch_timer_elapsed(self._h, a, b, C.byref(ms)))
        return ms.value
