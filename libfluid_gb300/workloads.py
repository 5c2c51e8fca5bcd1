"""Synthetic workloads of the WCSPH step (dam-break scenes) and their inputs.

No public dataset exists for this path: every workload is a seeded lattice
block with uniform jitter, generated identically on the host (numpy, here)
and on the device (k_lattice in csrc/sph_kernels.cu).

Lattice site (ix, iy, iz), x outermost and z innermost, is particle
(ix*ny + iy)*nz + iz with coordinate, in float32 arithmetic,
    lo + (i + 0.5) * spacing + (2u - 1) * jitter,
u = uniform01(seed, 3*particle + axis) (splitmix64, top 24 bits).
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)
_CTR = np.uint64(0xD1B54A32D192ED03)


def splitmix64(x: np.ndarray) -> np.ndarray:
    """splitmix64 finaliser (Steele, Lea, Flood, OOPSLA 2014) on uint64 arrays."""
    with np.errstate(over="ignore"):
        z = np.asarray(x, np.uint64) + _GAMMA
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def uniform01(seed: int, ctr: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = splitmix64(np.uint64(seed) ^ (np.asarray(ctr, np.uint64) * _CTR))
    return (z >> np.uint64(40)).astype(np.float32) * np.float32(1.0 / 16777216.0)


@dataclasses.dataclass
class Lattice:
    lo: tuple
    spacing: float
    nx: int
    ny: int
    nz: int
    jitter: float
    vel: tuple = (0.0, 0.0, 0.0)
    seed: int = 1

    @property
    def n(self) -> int:
        return self.nx * self.ny * self.nz

    def positions(self) -> np.ndarray:
        n = self.n
        i = np.arange(n, dtype=np.int64)
        iz = i % self.nz
        iy = (i // self.nz) % self.ny
        ix = i // (self.nz * self.ny)
        out = np.empty((n, 3), np.float32)
        sp = np.float32(self.spacing)
        jit = np.float32(self.jitter)
        for a, idx in enumerate((ix, iy, iz)):
            u = uniform01(self.seed, 3 * i + a)
            j = (np.float32(2.0) * u - np.float32(1.0)) * jit
            base = np.float32(self.lo[a]) + (idx.astype(np.float32) + np.float32(0.5)) * sp
            out[:, a] = base + j
        return out

    def velocities(self) -> np.ndarray:
        return np.tile(np.asarray(self.vel, np.float32), (self.n, 1))


@dataclasses.dataclass
class SceneSpec:
    """One dam-break scene: domain, parameters and its fluid blocks."""
    box: tuple
    h: float
    blocks: list
    rest_density: float = 1000.0
    mass: float = 1e-3
    gamma: float = 7.0
    gas_constant: float = 400.0     # c0^2: p = B*rho0/gamma*((rho/rho0)^gamma - 1) (fluidphysics.cu:78)
    viscosity: float = 0.01
    xsph: float = 0.5
    surface_tension: float = 0.0
    adhesion: float = 0.0
    vdamp: float = 0.5
    particle_size: float = 0.005
    vel_limit: float = 5.0
    acc_limit: float = 150.0
    gravity: tuple = (0.0, -9.81, 0.0)
    dt: float = 2e-4
    steps: int = 200
    unit_cube_res: int = 0          # >0: the reference's unit cube with res cells instead of box/h
    extra_pos: np.ndarray | None = None   # host-generated particles after the blocks (e.g. spheres)
    extra_vel: np.ndarray | None = None
    boundary: int = 0               # 0: the box; 1: the sphere of radius min half extent about its centre

    @property
    def n(self) -> int:
        return sum(b.n for b in self.blocks) + (0 if self.extra_pos is None else int(self.extra_pos.shape[0]))

    def positions(self) -> np.ndarray:
        parts = [b.positions() for b in self.blocks]
        if self.extra_pos is not None:
            parts.append(np.asarray(self.extra_pos, np.float32))
        return np.concatenate(parts)

    def velocities(self) -> np.ndarray:
        parts = [b.velocities() for b in self.blocks]
        if self.extra_pos is not None:
            parts.append(np.asarray(self.extra_vel, np.float32))
        return np.concatenate(parts)

    def params(self) -> dict:
        return dict(rest_density=self.rest_density, mass=self.mass, gamma=self.gamma,
                    gas_constant=self.gas_constant, viscosity=self.viscosity, xsph=self.xsph,
                    surface_tension=self.surface_tension, adhesion=self.adhesion, vdamp=self.vdamp,
                    particle_size=self.particle_size, vel_limit=self.vel_limit, acc_limit=self.acc_limit,
                    gravity=tuple(self.gravity), dt=self.dt)


def small_dam_break(seed: int = 1, unit_cube: bool = False) -> SceneSpec:
    """32,768 particles: 32^3 lattice, spacing 0.01 m, in [0,0.32]^3 of a
    1.0x0.6x0.6 m box; h = 0.02 m; dt = 2e-4 s for 200 steps.  The unit-cube
    variant (the reference's own domain) uses res = 50 and g = -9.8."""
    lat = Lattice(lo=(0.0, 0.0, 0.0), spacing=0.01, nx=32, ny=32, nz=32, jitter=0.05 * 0.01, seed=seed)
    s = SceneSpec(box=(1.0, 0.6, 0.6), h=0.02, blocks=[lat], mass=1e-3, particle_size=0.005, dt=2e-4, steps=200)
    if unit_cube:
        s.box, s.unit_cube_res, s.gravity = (1.0, 1.0, 1.0), 50, (0.0, -9.8, 0.0)
    return s


def sphere_tank(seed: int = 1) -> SceneSpec:
    """The sphere boundary: lattice sites (spacing 0.01 m, jittered) inside a
    sphere of radius 0.34 m about (0.35, 0.35, 0.35), below its centre, in a
    0.7 m cube whose boundary is the inscribed sphere (radius 0.35 m, so the
    outer particles feel the wall); h = 0.02 m, dt = 2e-4 s.  About 82,000
    particles."""
    sites = sphere_sites((0.35, 0.35, 0.35), 0.34, 0.01)
    sites = sites[sites[:, 1] <= 0.35]
    ctr = np.arange(3 * sites.shape[0], dtype=np.uint64).reshape(-1, 3)
    jit = ((np.float32(2.0) * uniform01(int(np.uint64(seed) * np.uint64(2654435761)), ctr) - np.float32(1.0)) *
           np.float32(0.05 * 0.01)).astype(np.float32)
    pos = (sites + jit).astype(np.float32)
    return SceneSpec(box=(0.7, 0.7, 0.7), h=0.02, blocks=[], mass=1e-3, particle_size=0.005, dt=2e-4, steps=200,
                     extra_pos=pos, extra_vel=np.zeros_like(pos), boundary=1)


def dam_break_1m(seed: int = 1, unit_cube: bool = False) -> SceneSpec:
    """1,000,000 particles: 100^3 lattice, spacing 0.005 m, in [0,0.5]^3 of a
    2x1x1 m box; h = 0.01 m; dt = 1e-4 s for 1000 steps.  Unit-cube variant:
    res = 100 (the same h), g = -9.8."""
    lat = Lattice(lo=(0.0, 0.0, 0.0), spacing=0.005, nx=100, ny=100, nz=100, jitter=0.05 * 0.005, seed=seed)
    s = SceneSpec(box=(2.0, 1.0, 1.0), h=0.01, blocks=[lat], mass=1.25e-4, particle_size=0.0025, dt=1e-4,
                  steps=1000)
    if unit_cube:
        s.box, s.unit_cube_res, s.gravity = (1.0, 1.0, 1.0), 100, (0.0, -9.8, 0.0)
    return s


def large_tension(seed: int = 1) -> SceneSpec:
    """~8M particles with surface tension: a 200x200x180 lattice pool (depth
    0.9 m, z up) plus two spheres of radius 0.229 m falling at 1 m/s, spacing
    0.005 m, h = 0.01 m, box 1x1x2 m, c0 = 25 m/s, dt = 8e-5 s."""
    pool = Lattice(lo=(0.0, 0.0, 0.0), spacing=0.005, nx=200, ny=200, nz=180, jitter=0.05 * 0.005, seed=seed)
    spheres = [sphere_sites(c, 0.229, 0.005) for c in ((0.27, 0.5, 1.3), (0.73, 0.5, 1.6))]
    sp = np.concatenate(spheres)
    rng_seed = np.uint64(seed) * np.uint64(2654435761)
    ctr = np.arange(3 * sp.shape[0], dtype=np.uint64).reshape(-1, 3)
    jit = ((np.float32(2.0) * uniform01(int(rng_seed), ctr) - np.float32(1.0)) *
           np.float32(0.05 * 0.005)).astype(np.float32)
    sp = (sp + jit).astype(np.float32)
    sv = np.tile(np.asarray((0.0, 0.0, -1.0), np.float32), (sp.shape[0], 1))
    return SceneSpec(box=(1.0, 1.0, 2.0), h=0.01, blocks=[pool], mass=1.25e-4, particle_size=0.0025,
                     gas_constant=625.0, surface_tension=0.0728, gravity=(0.0, 0.0, -9.81), dt=8e-5, steps=500,
                     extra_pos=sp, extra_vel=sv)


def sphere_sites(center, radius, spacing):
    """Global lattice sites (i+0.5)*spacing inside a sphere, x outermost."""
    lo = [int(math.floor((c - radius) / spacing)) for c in center]
    hi = [int(math.ceil((c + radius) / spacing)) for c in center]
    ax = [np.arange(l, h + 1) for l, h in zip(lo, hi)]
    g = np.stack(np.meshgrid(*ax, indexing="ij"), -1).reshape(-1, 3)
    pos = (g.astype(np.float32) + np.float32(0.5)) * np.float32(spacing)
    d2 = ((pos.astype(np.float64) - np.asarray(center)) ** 2).sum(1)
    return pos[d2 <= radius * radius]


def batch_manifest(num_scenes: int = 256, seed: int = 7, nmin: int = 2048, nmax: int = 65536,
                   spacing: float = 0.01, steps: int = 500) -> list:
    """Mixed-size dam breaks: particle count log-uniform in [nmin, nmax],
    block aspect ratios uniform in [0.5, 2], box 2x the block in x and 1.2x in
    y/z, viscosity uniform [0.005, 0.05], surface tension uniform [0, 0.07]."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(num_scenes):
        target = math.exp(rng.uniform(math.log(nmin), math.log(nmax)))
        ay, az = rng.uniform(0.5, 2.0, size=2)
        nx = max(2, int(round((target / (ay * az)) ** (1.0 / 3.0))))
        ny = max(2, int(round(nx * ay)))
        nz = max(2, int(round(nx * az)))
        lat = Lattice(lo=(0.0, 0.0, 0.0), spacing=spacing, nx=nx, ny=ny, nz=nz, jitter=0.05 * spacing,
                      seed=seed * 100003 + k)
        box = (2.0 * nx * spacing, 1.2 * ny * spacing, 1.2 * nz * spacing)
        out.append(SceneSpec(box=box, h=2.0 * spacing, blocks=[lat], mass=1000.0 * spacing ** 3,
                             particle_size=0.5 * spacing, viscosity=float(rng.uniform(0.005, 0.05)),
                             surface_tension=float(rng.uniform(0.0, 0.07)), dt=2e-4, steps=steps))
    return out


def manifest(specs: list, steps: list | None = None, **extra) -> dict:
    """A JSON-ready record of a scene set: per scene its particle count,
    domain, parameters, fluid blocks (with their seeds) and substeps, so that
    a run can be inspected or replayed without the generator that drew it
    (`from_manifest`).  `extra` entries (workload name, seed, arrival times)
    are stored beside the scenes."""
    scenes = []
    for k, s in enumerate(specs):
        if s.extra_pos is not None:
            raise ValueError("a scene with host-generated particles has no manifest form")
        blocks = []
        for b in s.blocks:
            d = dataclasses.asdict(b)
            blocks.append({key: (list(v) if isinstance(v, tuple) else v) for key, v in d.items()})
        params = {key: (list(v) if isinstance(v, tuple) else v) for key, v in s.params().items()}
        scenes.append({"n": s.n, "box": list(s.box), "h": s.h, "unit_cube_res": s.unit_cube_res,
                       "boundary": s.boundary, "params": params, "blocks": blocks,
                       "steps": int(steps[k]) if steps is not None else int(s.steps)})
    out = {"scenes": scenes, "total_particles": sum(sc["n"] for sc in scenes)}
    out.update(extra)
    return out


def from_manifest(m: dict) -> tuple[list, list]:
    """The scenes and substep counts of a `manifest` record."""
    specs, steps = [], []
    for sc in m["scenes"]:
        p = dict(sc["params"])
        p["gravity"] = tuple(p["gravity"])
        blocks = [Lattice(**{k: (tuple(v) if isinstance(v, list) else v) for k, v in b.items()})
                  for b in sc["blocks"]]
        specs.append(SceneSpec(box=tuple(sc["box"]), h=sc["h"], blocks=blocks, steps=sc["steps"],
                               unit_cube_res=sc["unit_cube_res"], boundary=sc["boundary"], **p))
        steps.append(sc["steps"])
    return specs, steps
