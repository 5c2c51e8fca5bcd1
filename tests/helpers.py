"""Shared set-up for parity tests: one scene on the GPU (through the C ABI)
and the same scene in the CPU oracle."""
from __future__ import annotations

import numpy as np

import oracle
from libfluid_gb300 import workloads as W


def configure_oracle(o: "oracle.Oracle", spec: W.SceneSpec, pos=None, vel=None):
    n = spec.n if pos is None else int(np.asarray(pos).reshape(-1, 3).shape[0])
    o.init(n, spec.unit_cube_res or 1)
    if not spec.unit_cube_res:
        o.set_domain(*spec.box, spec.h)
    if spec.boundary:
        o.set_boundary(spec.boundary)
    for k, v in spec.params().items():
        if k == "gravity":
            o.set_gravity(*v)
        elif k in ("vel_limit", "acc_limit"):
            continue
        else:
            o.set_param(k, v)
    o.set_limits(spec.vel_limit, spec.acc_limit)
    o.set_state(spec.positions() if pos is None else pos, spec.velocities() if vel is None else vel)
    return o


def configure_gpu(fs, spec: W.SceneSpec, pos=None, vel=None):
    n = spec.n if pos is None else int(np.asarray(pos).reshape(-1, 3).shape[0])
    fs.init(n, spec.unit_cube_res or 1)
    if not spec.unit_cube_res:
        fs.setDomain(*spec.box, spec.h)
    if spec.boundary:
        fs.setBoundary(spec.boundary)
    p = spec.params()
    fs.setParams(rest_density=p["rest_density"], mass=p["mass"], gamma=p["gamma"],
                 gas_constant=p["gas_constant"], viscosity=p["viscosity"], xsph=p["xsph"],
                 surface_tension=p["surface_tension"], adhesion=p["adhesion"], vdamp=p["vdamp"],
                 particle_size=p["particle_size"], vel_limit=p["vel_limit"], acc_limit=p["acc_limit"],
                 gravity=p["gravity"], dt=p["dt"])
    fs.setState(spec.positions() if pos is None else pos, spec.velocities() if vel is None else vel)
    return fs


def rel_err(a, b, floor):
    """max_i |a_i - b_i| / max(|b_i|, floor)  (row norms for vector fields)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    if a.ndim == 2:
        d = np.linalg.norm(a - b, axis=1)
        m = np.linalg.norm(b, axis=1)
    else:
        d = np.abs(a - b)
        m = np.abs(b)
    return float(np.max(d / np.maximum(m, floor))) if d.size else 0.0


def scene_invariants(pos, vel, mass, rho=None, rho0=1000.0):
    pos = np.asarray(pos, np.float64)
    vel = np.asarray(vel, np.float64)
    out = {
        "mass": mass * pos.shape[0],
        "kinetic": 0.5 * mass * float((vel ** 2).sum()),
        "com": pos.mean(0),
    }
    if rho is not None:
        out["max_rho_dev"] = float(np.max(np.abs(np.asarray(rho, np.float64) / rho0 - 1.0)))
    return out


SNAPSHOT_HEADER_BYTES = 128


def snapshot_state(fs):
    """Exact state of a system (sph_snapshot): positions, velocities and
    accelerations as (n, 3) float32, in the system's slot order."""
    snap = fs.snapshot()
    n = fs.numParticles()
    a = np.frombuffer(snap, np.float32, count=12 * n, offset=SNAPSHOT_HEADER_BYTES).reshape(3, n, 4)
    return a[0, :, :3].copy(), a[1, :, :3].copy(), a[2, :, :3].copy()


def oracle_from_state(precision, spec, pos, vel, acc, scales=True):
    """An oracle of the scene's parameters holding exactly this state (with
    the force and normal test scales recorded)."""
    o = configure_oracle(oracle.Oracle(precision), spec, pos=pos, vel=vel)
    o.set_state_f64(pos, vel, acc)
    if scales:
        o.track_scales(True)
    return o


def by_particle(arr, perm):
    """A field in sorted order (entry f belongs to the particle that sat in
    slot perm[f] before the sort) re-indexed by that slot."""
    out = np.empty_like(arr)
    out[perm] = arr
    return out


def force_err(g, r, d, sel=None):
    """(gpu-vs-fp32, gpu-vs-fp64, fp32-vs-fp64) errors of a force field,
    each relative to max(|F_i|, 1% of the RMS force of the FP32 oracle)."""
    if sel is not None:
        g, r, d = g[sel], r[sel], d[sel]
    scale = float(np.sqrt((r.astype(np.float64) ** 2).sum(1).mean())) if r.size else 0.0
    floor = max(1e-2 * scale, 1e-30)
    return rel_err(g, r, floor), rel_err(g, d, floor), rel_err(r, d, floor)


# The oracle field holding, per particle, the sum over its pairs of the
# magnitude of each pair's term (oracle.Oracle.track_scales).
SCALE_FIELD = {"fpressure": "fpressure_scale", "fviscosity": "fviscosity_scale", "ftension": "ftension_scale",
               "normal": "normal_scale"}


def pair_scale(o32, o64, field):
    """The pair-term magnitude sum of a field (sorted order), the larger of
    the FP32 and FP64 oracles' (a pair at r = h that FP32 arithmetic counts
    and FP64 does not belongs to the FP32 result's scale)."""
    return np.maximum(o32.get(SCALE_FIELD[field]), o64.get(SCALE_FIELD[field]))


def scaled_err(a, b, S):
    """max_i |a_i - b_i| / S_i, S_i the sum of the magnitudes of particle i's
    pair terms: a force (or normal) is a sum of about 30 pair terms that
    largely cancel, so FP32 rounding is proportional to S_i, not to the net
    |F_i|; a single missing or wrong pair changes F_i by about S_i / 30."""
    d = np.linalg.norm(np.asarray(a, np.float64) - np.asarray(b, np.float64), axis=1)
    return float(np.max(d / np.maximum(np.asarray(S, np.float64), 1e-30))) if d.size else 0.0


def check_vector_field(label, g, r, d, S, rtol):
    """A force or normal field, GPU (g) against the FP32 (r) and FP64 (d)
    oracles.  The bar: within rtol of the FP32 oracle relative to the pair
    terms' magnitude S (relative to max(|F_i|, 1% RMS) where the field is no
    pair sum, S None: adhesion), and no further from FP64 than twice the
    FP32 oracle is.  Both measures are printed."""
    e_old, e64_old, o64_old = force_err(g, r, d)
    msg = f"{label}: |F|-relative gpu-vs-fp32 {e_old:.2e}, gpu-vs-fp64 {e64_old:.2e}, fp32-vs-fp64 {o64_old:.2e}"
    if S is not None:
        e, e64, o64 = scaled_err(g, r, S), scaled_err(g, d, S), scaled_err(r, d, S)
        msg += f"; pair-scale-relative gpu-vs-fp32 {e:.2e}, gpu-vs-fp64 {e64:.2e}, fp32-vs-fp64 {o64:.2e}"
    else:
        e = e_old
    print(msg)
    assert e < rtol, msg
    assert e64_old <= 2.0 * o64_old + 1e-6, msg
