"""Shared set-up for parity tests: one scene on the GPU (through the C ABI)
and the same scene in the CPU oracle."""
from __future__ import annotations

import numpy as np

import oracle
from libfluid_gb300 import workloads as W


def configure_oracle(o: "oracle.Oracle", spec: W.SceneSpec, pos=None, vel=None):
    n = spec.n
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
    n = spec.n
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
