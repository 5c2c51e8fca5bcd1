"""GB300-native WCSPH step with NCCA/libfluid's FluidSystem interface.

`FluidSystem` mirrors libfluid/include/fluidsystem.h:16-126 method for method
(same names, argument meaning and defaults) over the C ABI in
include/sph_c.h.  Particle arrays are numpy float32 arrays of shape (n, 3),
the layout of std::vector<float3>.  Everything runs in libsph_gb300.so on
the GPU; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._capi import FIELDS, SphError, SphParams, check, lib

__all__ = ["FluidSystem", "SphError", "DEFAULT_TIMESTEP", "substep_count"]

DEFAULT_TIMESTEP = 0.01  # fluiddefines.h:4


def _f32x3(a, n=None) -> np.ndarray:
    arr = np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(-1, 3))
    if n is not None and arr.shape[0] != n:
        raise ValueError(f"expected {n} rows, got {arr.shape[0]}")
    return arr


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def substep_count(full_dt: float, substeps: int) -> int:
    """Substeps FluidSystem::advance runs (fluidsystem.cu:301 float loop)."""
    return int(lib().sph_substep_count(C.c_float(full_dt), substeps))


class FluidSystem:
    """Drop-in for libfluid's FluidSystem (fluidsystem.h:16-126)."""

    STATIC, DYNAMIC = 1, 2  # ParticleState (fluidsystem.h:19-23)

    def __init__(self, device: int = -1):
        self._L = lib()
        h = C.c_void_p()
        check(self._L.sph_create(C.byref(h), device))
        self._h = h
        self.m_isInit = False

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._L.sph_destroy(h)
            self._h = None

    def close(self) -> None:
        self.__del__()

    def _ck(self, code: int) -> None:
        check(code, self._h)

    # ---- lifetime (fluidsystem.cu:132-265) -------------------------------
    def init(self, num_points: int, res: int) -> None:
        self._ck(self._L.sph_init(self._h, num_points, res))
        self.m_isInit = True

    def clear(self) -> None:
        self._ck(self._L.sph_clear(self._h))

    def setup(self, num_points: int, res: int) -> None:
        self._ck(self._L.sph_setup(self._h, num_points, res))
        self.m_isInit = True

    def setupFromData(self, points, velocity, res: int = 32) -> None:
        p = _f32x3(points)
        v = _f32x3(velocity, p.shape[0])
        self._ck(self._L.sph_setup_from_data(self._h, _ptr(p), _ptr(v), p.shape[0], res))
        self.m_isInit = True

    def createFluidBlock(self, first: int, num_points: int, min_x: float, min_y: float, min_z: float,
                         max_x: float, max_y: float, max_z: float) -> None:
        self._ck(self._L.sph_create_block(self._h, first, num_points, min_x, min_y, min_z, max_x, max_y, max_z))

    def setState(self, points, velocity=None) -> None:
        p = _f32x3(points, self.numParticles())
        v = None if velocity is None else _f32x3(velocity, p.shape[0])
        self._ck(self._L.sph_set_state(self._h, _ptr(p), _ptr(v), p.shape[0]))

    # ---- stepping ---------------------------------------------------------
    def advance(self, dt: float = DEFAULT_TIMESTEP, substeps: int = 10) -> int:
        """FluidSystem::advance; returns the number of substeps executed."""
        if not self.m_isInit:
            return 0  # fluidsystem.cu:276-277
        ex = C.c_uint32(0)
        self._ck(self._L.sph_advance(self._h, C.c_float(dt), substeps, C.byref(ex)))
        return ex.value

    def advanceAsync(self, dt: float = DEFAULT_TIMESTEP, substeps: int = 10) -> int:
        ex = C.c_uint32(0)
        self._ck(self._L.sph_advance_async(self._h, C.c_float(dt), substeps, C.byref(ex)))
        return ex.value

    def sync(self) -> None:
        self._ck(self._L.sph_sync(self._h))

    # ---- readback ---------------------------------------------------------
    def numParticles(self) -> int:
        return int(self._L.sph_num_particles(self._h))

    def exportToData(self, points=None, colour=None, velocity=None):
        """FluidSystem::exportToData; returns (points, colour, velocity)."""
        n = self.numParticles()
        outs = []
        for a in (points, colour, velocity):
            if a is None:
                a = np.empty((n, 3), np.float32)
            if a.dtype != np.float32 or a.shape != (n, 3) or not a.flags.c_contiguous:
                raise ValueError("export buffers must be C-contiguous float32 arrays of shape (n, 3)")
            outs.append(a)
        self._ck(self._L.sph_export(self._h, _ptr(outs[0]), _ptr(outs[1]), _ptr(outs[2]), n))
        return tuple(outs)

    def getPscale(self) -> float:
        out = C.c_float(0.0)
        self._ck(self._L.sph_get_pscale(self._h, C.byref(out)))
        return out.value

    # ---- snapshot / resume (no reference counterpart) ----------------------
    def snapshot(self) -> bytes:
        """Exact snapshot (header + positions, velocities, accelerations)."""
        n = self.numParticles()
        size = int(self._L.sph_snapshot_bytes(n))
        buf = C.create_string_buffer(size)
        written = C.c_uint64(0)
        self._ck(self._L.sph_snapshot(self._h, buf, size, C.byref(written)))
        return buf.raw[:written.value]

    def restore(self, snap: bytes) -> None:
        """Replace parameters and state with a snapshot of the same particle count."""
        self._ck(self._L.sph_restore(self._h, snap, len(snap)))

    # ---- setters (fluidsystem.cu:412-475) ---------------------------------
    def setRestDensity(self, v: float) -> None: self._ck(self._L.sph_set_rest_density(self._h, v))
    def setParticleSize(self, v: float) -> None: self._ck(self._L.sph_set_particle_size(self._h, v))
    def setGasConstant(self, v: float) -> None: self._ck(self._L.sph_set_gas_constant(self._h, v))
    def setLimits(self, vel: float, acc: float) -> None: self._ck(self._L.sph_set_limits(self._h, vel, acc))
    def setXSPHScale(self, v: float) -> None: self._ck(self._L.sph_set_xsph_scale(self._h, v))
    def setSurfaceTension(self, v: float) -> None: self._ck(self._L.sph_set_surface_tension(self._h, v))
    def setViscosity(self, v: float) -> None: self._ck(self._L.sph_set_viscosity(self._h, v))
    def setAdhesion(self, v: float) -> None: self._ck(self._L.sph_set_adhesion(self._h, v))
    def setVDamp(self, v: float) -> None: self._ck(self._L.sph_set_vdamp(self._h, v))
    def setGamma(self, v: float) -> None: self._ck(self._L.sph_set_gamma(self._h, v))
    def setMass(self, v: float) -> None: self._ck(self._L.sph_set_mass(self._h, v))
    # additions
    def setGravity(self, gx: float, gy: float, gz: float) -> None: self._ck(self._L.sph_set_gravity(self._h, gx, gy, gz))
    def setDomain(self, lx: float, ly: float, lz: float, h: float) -> None:
        self._ck(self._L.sph_set_domain(self._h, lx, ly, lz, h))

    def setBoundary(self, shape: int) -> None:
        """0: the box (the reference's boundary); 1: the sphere of radius the
        box's smallest half extent about its centre."""
        self._ck(self._L.sph_set_boundary(self._h, shape))

    def getBoundary(self) -> int:
        out = C.c_int(0)
        self._ck(self._L.sph_get_boundary(self._h, C.byref(out)))
        return out.value

    def getParams(self) -> dict:
        p = SphParams()
        self._ck(self._L.sph_get_params(self._h, C.byref(p)))
        d = {k: getattr(p, k) for k, _ in SphParams._fields_ if k != "gravity"}
        d["gravity"] = tuple(p.gravity)
        return d

    def setParams(self, **kw) -> None:
        p = SphParams()
        self._ck(self._L.sph_get_params(self._h, C.byref(p)))
        for k, v in kw.items():
            if k == "gravity":
                for i in range(3):
                    p.gravity[i] = float(v[i])
            else:
                setattr(p, k, v)
        self._ck(self._L.sph_set_params(self._h, C.byref(p)))

    def derived(self) -> np.ndarray:
        buf = (C.c_double * 64)()
        k = self._L.sph_get_derived(self._h, buf, 64)
        return np.array(buf[:k])

    # ---- parity taps --------------------------------------------------------
    def debugEnable(self, on: bool = True) -> None:
        self._ck(self._L.sph_debug_enable(self._h, 1 if on else 0))

    def debugScanFault(self, spin_limit: int = 0, withhold_first_tile: bool = False) -> None:
        """Test control of the cell scan's bounded waits (sph_debug_scan_fault):
        with withhold_first_tile the next substep's scan gives up after
        spin_limit polls per wait and the step raises SPH_ETIMEOUT."""
        self._ck(self._L.sph_debug_scan_fault(self._h, spin_limit, 1 if withhold_first_tile else 0))

    def debug(self, field: str, ncells: int | None = None) -> np.ndarray:
        f = FIELDS[field]
        n = self.numParticles()
        if field in ("cellstart", "cellocc"):
            out = np.empty(int(ncells), np.uint32)
        elif field in ("hash", "perm", "nbrcount"):
            out = np.empty(n, np.uint32)
        elif field in ("density", "pressure", "soundspeed"):
            out = np.empty(n, np.float32)
        else:
            out = np.empty((n, 3), np.float32)
        self._ck(self._L.sph_debug_get(self._h, f, _ptr(out), out.size))
        return out

    # ---- execution options ----------------------------------------------------
    def setUseGraph(self, on: bool) -> None:
        self._ck(self._L.sph_set_use_graph(self._h, 1 if on else 0))

    def setExportAhead(self, on: bool) -> None:
        """Let an export of velocities start the next substep's force pass
        (default on; results are identical either way)."""
        self._ck(self._L.sph_set_export_ahead(self._h, 1 if on else 0))

    def exportAheadStats(self) -> dict:
        """Exports that ran passes ahead, and how many were taken or undone."""
        out = (C.c_uint64 * 3)()
        self._ck(self._L.sph_export_ahead_stats(self._h, out))
        return {"started": out[0], "taken": out[1], "undone": out[2]}

    def setExec(self, tile: int = 128, persistent: int = 0, skin: float = 0.1, variant: int = 63) -> None:
        from ._capi import SphExec
        e = SphExec(tile, persistent, skin, variant)
        self._ck(self._L.sph_set_exec(self._h, C.byref(e)))

    def setDeferredXSPH(self, on: bool) -> None:
        """XSPH applied by the next substep's density pass (default) or at the
        end of every substep, as the reference does."""
        self._ck(self._L.sph_set_deferred_xsph(self._h, 1 if on else 0))

    def getExec(self) -> dict:
        from ._capi import SphExec
        e = SphExec()
        self._ck(self._L.sph_get_exec(self._h, C.byref(e)))
        return {"tile": e.tile, "persistent": e.persistent, "skin": e.skin, "variant": e.variant}

    def setProfiling(self, on: bool) -> None:
        self._ck(self._L.sph_set_profiling(self._h, 1 if on else 0))

    def timerMark(self, slot: int) -> None:
        self._ck(self._L.sph_timer_mark(self._h, slot))

    def timerElapsed(self, a: int, b: int) -> float:
        ms = C.c_float(0.0)
        self._ck(self._L.sph_timer_elapsed(self._h, a, b, C.byref(ms)))
        return ms.value

    def passTimes(self) -> tuple[dict, int]:
        buf = (C.c_double * 8)()
        n = C.c_uint64(0)
        self._ck(self._L.sph_get_pass_times(self._h, buf, 8, C.byref(n)))
        return {self._L.sph_pass_name(i).decode(): buf[i] for i in range(8)}, n.value
