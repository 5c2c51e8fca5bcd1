"""Pins: the oracle (CPU) and the GPU step against golden vectors produced by
the reference's own device code (tests/golden/make_golden.py runs NCCA/libfluid's
cudasrc, compiled unmodified from its sources, on a GB300).

Integer fields (hash, permutation, cell occupancy and starts, neighbour
counts) must match bit for bit.  Float fields are compared with tolerances:
the reference build fuses multiply-adds where nvcc chooses and uses the GPU's
powf/rsqrtf, so its results differ from any restatement by a few ulp.
Rows that overflow to inf/NaN (the edge scene's deliberately over-packed
clump) must be the same rows on both sides.

Velocities: the reference's XSPH (fluidphysics.cu:355-409) updates velocity
in place while neighbours read it, so a particle sees some neighbours' XSPH
corrections already applied.  The velocity after integration and before XSPH
is compared tightly; the final velocity may differ from a race-free result by
at most xsph * (largest XSPH correction among the particle's neighbours),
which is the bound used.
"""
import json
import os

import numpy as np
import pytest

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
META = os.path.join(GOLD, "scenes.json")
SCENES = sorted(json.load(open(META)).keys()) if os.path.exists(META) else []

INT_FIELDS = ["hash", "perm", "cellocc", "cellstart", "nbrcount"]
RTOL_DENSITY = 1e-5
RTOL_FORCE = 1e-4


def _load(name):
    meta = json.load(open(META))[name]
    z = np.load(os.path.join(GOLD, f"{name}.npz"))
    return meta, z


def _oracle(meta, z, precision=32, scales=False):
    o = oracle.Oracle(precision)
    p = meta["params"]
    o.init(meta["n"], meta["res"])
    for k in ("rest_density", "gas_constant", "gamma", "mass", "particle_size", "xsph", "surface_tension",
              "viscosity", "adhesion", "vdamp"):
        o.set_param(k, p[k])
    o.set_limits(p["vel_limit"], p["acc_limit"])
    o.set_gravity(p["gx"], p["gy"], p["gz"])
    o.set_state(z["in_pos"], z["in_vel"])
    if scales:
        o.track_scales(True)
    assert o.advance(meta["dt"], 1) == 1
    return o


_SCALES = {}


def _scales(name, meta, z):
    """Per particle, the sum over its pairs of each pair term's magnitude for
    the pressure, viscosity and tension forces and the normal (oracles on the
    golden input): the scale of the rounding error of these cancelling
    sums, and so of a meaningful relative bound on them."""
    if name not in _SCALES:
        # the larger of the FP32 and FP64 sums: a pair at r = h that FP32
        # arithmetic counts and FP64 does not is part of the FP32 result's scale
        o32, o64 = _oracle(meta, z, 32, scales=True), _oracle(meta, z, 64, scales=True)
        _SCALES[name] = {f: np.maximum(o32.get(f"{f}_scale"), o64.get(f"{f}_scale"))
                         for f in ("fpressure", "fviscosity", "ftension", "normal")}
    return _SCALES[name]


NULL_HASH = 0xFFFFFFFF


def finite_scaled_err(a, b, S, hashes):
    """Same non-finite rows on both sides; on the rows where both and the
    scale are finite, max |a_i - b_i| / S_i.  Particles outside the grid
    (null hash) are left out: the reference leaves their fields as they were
    (fluidphysics.cu's passes skip them), this library and the oracle zero
    them (a listed deviation)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    S = np.asarray(S, np.float64)
    fa, fb = np.isfinite(a).all(1), np.isfinite(b).all(1)
    assert np.array_equal(fa, fb), f"non-finite rows differ: {np.count_nonzero(fa != fb)}"
    ok = fa & np.isfinite(S) & (np.asarray(hashes) != NULL_HASH)
    if not ok.any():
        return 0.0
    d = np.linalg.norm(a[ok] - b[ok], axis=1)
    return float(np.max(d / np.maximum(S[ok], 1e-300)))


def finite_rel_err(a, b, floor_frac=1e-2, floor_abs=0.0):
    """Same non-finite rows on both sides; on the finite rows the max of
    |a-b| / max(|b|, floor_frac * rms(b), floor_abs) (row norms for vectors)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    a2, b2 = (a, b) if a.ndim == 2 else (a[:, None], b[:, None])
    fa, fb = np.isfinite(a2).all(1), np.isfinite(b2).all(1)
    assert np.array_equal(fa, fb), f"non-finite rows differ: {np.count_nonzero(fa != fb)}"
    a2, b2 = a2[fa], b2[fb]
    if a2.size == 0:
        return 0.0
    d = np.linalg.norm(a2 - b2, axis=1)
    m = np.linalg.norm(b2, axis=1)
    rms = float(np.sqrt((m ** 2).mean()))
    return float(np.max(d / np.maximum(np.maximum(m, floor_frac * rms), max(floor_abs, 1e-300))))


def _check(get, z, meta, who, scales=None):
    p = meta["params"]
    ref = lambda f: z[f"ref_{f}"]
    e = finite_rel_err(get("density"), ref("density"), 0.0, 1e-3 * p["rest_density"])
    assert e < RTOL_DENSITY, f"{who} density {e}"
    k = p["gas_constant"] * p["rest_density"] / p["gamma"]
    assert finite_rel_err(get("pressure"), ref("pressure"), 0.0, 1e-2 * k) < 1e-4, f"{who} pressure"
    assert finite_rel_err(get("soundspeed"), ref("soundspeed"), 0.0, 1e-3 * p["gas_constant"]) < 1e-4
    for f in ("fpressure", "fviscosity", "fadhesion", "ftension"):
        e = finite_rel_err(get(f), ref(f))
        assert e < 1e-3, f"{who} {f} {e}"
        if scales is not None and f in scales:
            # the force bar, 1e-4, relative to the pair terms' magnitude
            es = finite_scaled_err(get(f), ref(f), scales[f], ref("hash"))
            print(f"{who} {f} against the reference: |F|-relative {e:.2e}, pair-scale-relative {es:.2e}")
            assert es < RTOL_FORCE, f"{who} {f} pair-scale-relative {es}"
    if scales is not None and p["surface_tension"] != 0.0:
        es = finite_scaled_err(get("normal"), ref("normal"), scales["normal"], ref("hash"))
        print(f"{who} normal against the reference: pair-scale-relative {es:.2e}")
        assert es < RTOL_FORCE, f"{who} normal {es}"
    assert finite_rel_err(get("pos"), ref("pos"), 0.0, 1e-3) < 1e-6, f"{who} pos"
    assert finite_rel_err(get("acc"), ref("acc"), 1e-2) < 1e-3, f"{who} acc"
    vint = get("vel_int")
    assert finite_rel_err(vint, ref("vel_int"), 1e-2) < 1e-4, f"{who} velocity before XSPH"
    _check_final_velocity(get("vel"), vint, z, meta, who)


def _check_final_velocity(vfin, vint, z, meta, who):
    """Final velocities against the reference's within the bound its racy
    in-place XSPH update allows (module docstring)."""
    p = meta["params"]
    ref = lambda f: z[f"ref_{f}"]
    from scipy.spatial import cKDTree
    vfin, vref = np.asarray(vfin, np.float64), ref("vel").astype(np.float64)
    pos = ref("pos").astype(np.float64)
    ok = np.isfinite(vfin).all(1) & np.isfinite(vref).all(1) & np.isfinite(pos).all(1)
    corr = np.linalg.norm(vfin - np.asarray(vint, np.float64), axis=1)
    corr[~ok] = 0.0
    h = 1.0 / meta["res"]
    tree = cKDTree(np.where(ok[:, None], pos, 1e9))
    scale = float(np.sqrt((vref[ok] ** 2).sum(1).mean()))
    bad = 0
    for i in np.nonzero(ok)[0]:
        nb = tree.query_ball_point(pos[i], 1.05 * h)
        bound = abs(p["xsph"]) * 1.05 * float(corr[nb].max()) + 1e-4 * (np.linalg.norm(vref[i]) + 1e-2 * scale)
        if np.linalg.norm(vfin[i] - vref[i]) > bound:
            bad += 1
    assert bad == 0, f"{who}: {bad} final velocities outside the XSPH-race bound"


@pytest.mark.skipif(not SCENES, reason="golden vectors not generated")
@pytest.mark.parametrize("name", SCENES)
def test_oracle_matches_reference_device_code(name):
    meta, z = _load(name)
    if "ref_vel_int" not in z:
        pytest.skip("golden vectors predate the pre-XSPH velocity tap")
    o = _oracle(meta, z)
    for f in INT_FIELDS:
        g = o.get(f)
        assert np.array_equal(g, z[f"ref_{f}"]), f"{f}: {np.count_nonzero(g != z['ref_' + f])} mismatches"
    _check(lambda f: o.get(f), z, meta, "oracle", _scales(name, meta, z))
    if meta["params"]["surface_tension"] != 0.0:
        assert finite_rel_err(o.get("normal"), z["ref_normal"]) < 1e-4


@pytest.mark.gpu
@pytest.mark.skipif(not SCENES, reason="golden vectors not generated")
@pytest.mark.parametrize("name", SCENES)
def test_gpu_deferred_xsph_matches_reference_device_code(name):
    """The default schedule (XSPH applied by the next substep's density pass,
    computed on demand for the export) against the reference's own substep:
    positions, and final velocities within the XSPH-race bound."""
    from libfluid_gb300 import FluidSystem
    meta, z = _load(name)
    if "ref_vel_int" not in z:
        pytest.skip("golden vectors predate the pre-XSPH velocity tap")
    p = meta["params"]
    fs = FluidSystem(0)
    fs.init(meta["n"], meta["res"])
    fs.setParams(rest_density=p["rest_density"], gas_constant=p["gas_constant"], gamma=p["gamma"],
                 mass=p["mass"], particle_size=p["particle_size"], xsph=p["xsph"],
                 surface_tension=p["surface_tension"], viscosity=p["viscosity"], adhesion=p["adhesion"],
                 vdamp=p["vdamp"], vel_limit=p["vel_limit"], acc_limit=p["acc_limit"],
                 gravity=(p["gx"], p["gy"], p["gz"]))
    fs.setState(z["in_pos"], z["in_vel"])
    assert fs.advance(meta["dt"], 1) == 1
    pos, _, vel = fs.exportToData()
    assert finite_rel_err(pos, z["ref_pos"], 0.0, 1e-3) < 1e-6
    _check_final_velocity(vel, z["ref_vel_int"], z, meta, "gpu deferred")
    fs.close()


@pytest.mark.gpu
@pytest.mark.skipif(not SCENES, reason="golden vectors not generated")
@pytest.mark.parametrize("name", SCENES)
def test_gpu_matches_reference_device_code(name):
    from libfluid_gb300 import FluidSystem
    meta, z = _load(name)
    if "ref_vel_int" not in z:
        pytest.skip("golden vectors predate the pre-XSPH velocity tap")
    p = meta["params"]
    fs = FluidSystem(0)
    fs.debugEnable(True)
    fs.init(meta["n"], meta["res"])
    fs.setParams(rest_density=p["rest_density"], gas_constant=p["gas_constant"], gamma=p["gamma"],
                 mass=p["mass"], particle_size=p["particle_size"], xsph=p["xsph"],
                 surface_tension=p["surface_tension"], viscosity=p["viscosity"], adhesion=p["adhesion"],
                 vdamp=p["vdamp"], vel_limit=p["vel_limit"], acc_limit=p["acc_limit"],
                 gravity=(p["gx"], p["gy"], p["gz"]))
    fs.setState(z["in_pos"], z["in_vel"])
    assert fs.advance(meta["dt"], 1) == 1
    for f in INT_FIELDS:
        g = fs.debug(f, ncells=meta["res"] ** 3)
        assert np.array_equal(g, z[f"ref_{f}"]), f"{f}: {np.count_nonzero(g != z['ref_' + f])} mismatches"
    pos, _, vel = fs.exportToData()
    got = {"pos": pos, "vel": vel}
    _check(lambda f: got[f] if f in got else fs.debug(f), z, meta, "gpu", _scales(name, meta, z))
