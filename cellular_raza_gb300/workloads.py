"""Seeded synthetic workloads for the mechanics/interaction step.

Every generator returns plain numpy arrays in the host layout of the C ABI
([n][n_vertices][dim] doubles) plus a ``Model`` describing the domain and the agent
parameters.  The same arrays feed the device path and the oracle, so both see identical
inputs.  Seeds use numpy's PCG64.

Named workloads (sizes and parameter values of the benchmark configurations):
  spheres_3d        3D NewtonDamped3D + MorsePotential spheres, 4,096 agents in [0,200)^3,
                    voxel side 15, Euler dt 0.01, 1,000 steps
  rods_2d           2D bacterial rods, 100,000 rods x 6 vertices, 3,000 x 3,000 box,
                    voxel side 12, Euler dt 0.005, 500 steps
  spheres_3d_large  2^23 spheres at the density of spheres_3d, mixed precision, 200 steps
  ensemble          1,024 independent 3D Morse simulations with log-uniform sizes
  request_stream    Poisson stream of simulation requests (serving)
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional, Tuple

import numpy as np

DENSITY_3D = 4096 / 200.0 ** 3  # 5.12e-4 agents per unit^3


def host_threads() -> int:
    """Cores this process may run on: chili's n_threads for a run on all of them (one
    subdomain per thread, chili/setup.rs:17-27), which also fixes chili's pair weights."""
    import os

    try:
        return max(1, len(os.sched_getaffinity(0)))
    except AttributeError:
        return max(1, os.cpu_count() or 1)


@dataclasses.dataclass
class Model:
    """Domain + agent parameters of one simulation (mirrors crg_domain + crg_model)."""

    kind: str = "sphere"  # "sphere" (NewtonDamped) | "rod" | "brownian" | "langevin"
    dim: int = 3
    n_vertices: int = 1
    domain_min: Tuple[float, ...] = (0.0, 0.0, 0.0)
    domain_max: Tuple[float, ...] = (200.0, 200.0, 200.0)
    interaction_range: Optional[float] = 15.0  # CartesianCuboid::from_boundaries_and_interaction_range
    n_voxels: Optional[Tuple[int, ...]] = None  # CartesianCuboid::from_boundaries_and_n_voxels
    n_subdomains: int = 1  # chili Settings::n_threads
    weight_mode: int = 0  # 0 chili weights, 1 physical
    solver_order: int = 1  # 1 Euler, 2 AB2, 3 AB3
    precision: str = "f64"  # "f64" | "mixed"
    # NewtonDamped / Langevin (mass, damping gamma)
    mass: float = 1.0
    damping: float = 1.5
    # Brownian / Langevin k_B T; seed of the stochastic mechanics' random stream
    kb_temperature: float = 0.0
    rng_seed: int = 0
    # RodMechanics
    spring_tension: float = 0.0
    rigidity: float = 0.0
    spring_length: float = 0.0
    diffusion: float = 0.0  # RodMechanics / Brownian diffusion constant
    # MorsePotential
    radius: float = 5.0
    stiffness: float = 0.4
    cutoff: float = 15.0
    strength: float = 0.5
    dt: float = 0.01
    # Cell cycle of the bacterial-rods agent (rods only): growth limited by neighbour
    # sensing, division past division_length
    cycle: bool = False
    growth_rate: float = 0.0
    division_length: float = 0.0
    sense_range: float = 0.0
    sense_saturation: float = 8.0

    @property
    def nc(self) -> int:
        return self.n_vertices * self.dim

    def replace(self, **kw) -> "Model":
        return dataclasses.replace(self, **kw)


@dataclasses.dataclass
class Workload:
    name: str
    model: Model
    pos: np.ndarray  # [n][nv][dim]
    vel: np.ndarray
    n_steps: int
    spring_length: Optional[np.ndarray] = None  # cell cycle: per-rod initial spring lengths

    @property
    def n(self) -> int:
        return self.pos.shape[0]


def spheres(n: int, side: float, seed: int = 0, dim: int = 3, **model_kw) -> Workload:
    """n spheres uniform in (0, side)^dim with zero velocity (NewtonDamped + Morse)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    pos = rng.uniform(0.0, side, size=(n, 1, dim))
    pos[pos <= 0.0] = side * 1e-9  # CartesianCuboid rejects pos <= min at insertion
    vel = np.zeros_like(pos)
    kw = dict(kind="sphere", dim=dim, n_vertices=1, domain_min=(0.0,) * dim,
              domain_max=(side,) * dim, interaction_range=15.0)
    kw.update(model_kw)
    m = Model(**kw)
    return Workload("spheres", m, pos, vel, 0)


def spheres_3d(seed: int = 0, n: int = 4096, n_subdomains: int = 1, **kw) -> Workload:
    """3D soft spheres: N=4,096 in [0,200)^3, NewtonDamped3D (m 1, damping 1.5), Morse
    (radius 5, stiffness 0.4, cutoff 15, strength 0.5), voxel side 15, Euler dt 0.01."""
    side = 200.0 * (n / 4096.0) ** (1.0 / 3.0)
    w = spheres(n, side, seed, 3, n_subdomains=n_subdomains, **kw)
    w.name, w.n_steps = "spheres_3d", 1000
    return w


def spheres_3d_large(seed: int = 0, n: int = 2 ** 23, **kw) -> Workload:
    """2^23 spheres at density 5.12e-4 (cube side 200 * 2048^(1/3)), mixed precision."""
    side = (n / DENSITY_3D) ** (1.0 / 3.0)
    kw.setdefault("precision", "mixed")
    w = spheres(n, side, seed, 3, **kw)
    w.name, w.n_steps = "spheres_3d_large", 200
    return w


def rods(n: int, side: float, seed: int = 0, n_vertices: int = 6, spring_length: float = 3.0,
         dim: int = 2, **model_kw) -> Workload:
    """n rods with centres uniform in (0, side)^dim and orientation angle uniform in
    [0, 2 pi) (in the x-y plane), vertices spaced spring_length along the rod.  Vertices
    may stick out of the box; like the reference, only the centroid decides the voxel and
    the first apply_boundary reflects them."""
    rng = np.random.Generator(np.random.PCG64(seed))
    centres = rng.uniform(0.0, side, size=(n, dim))
    theta = rng.uniform(0.0, 2.0 * math.pi, size=n)
    direction = np.zeros((n, dim))
    direction[:, 0] = np.cos(theta)
    direction[:, 1] = np.sin(theta)
    k = np.arange(n_vertices) - (n_vertices - 1) / 2.0
    pos = centres[:, None, :] + k[None, :, None] * spring_length * direction[:, None, :]
    # centroids must lie strictly inside (min, max) for insertion; nudge the rare exceptions
    cen = pos.sum(axis=1) / n_vertices
    bad = np.any(cen <= 0.0, axis=1) | np.any(cen >= side, axis=1)
    if bad.any():
        pos[bad] += (side / 2.0 - cen[bad])[:, None, :] * 1e-3
    vel = np.zeros_like(pos)
    kw = dict(kind="rod", dim=dim, n_vertices=n_vertices, domain_min=(0.0,) * dim,
              domain_max=(side,) * dim, interaction_range=12.0, mass=1.0,
              spring_tension=1.0, rigidity=2.0, spring_length=spring_length, damping=1.0,
              diffusion=0.0, radius=3.0, stiffness=0.5, cutoff=6.0, strength=0.1, dt=0.005)
    kw.update(model_kw)
    return Workload("rods", Model(**kw), pos, vel, 0)


def rods_2d(seed: int = 0, n: int = 100_000, n_subdomains: int = 1, **kw) -> Workload:
    """2D bacterial rods: 100,000 rods x 6 vertices at spring length 3 in a 3,000^2 box,
    RodMechanics (tension 1, rigidity 2, damping 1, diffusion 0), RodInteraction(Morse
    radius 3, stiffness 0.5, cutoff 6, strength 0.1), voxel side 12, Euler dt 0.005."""
    side = 3000.0 * math.sqrt(n / 100_000.0)
    w = rods(n, side, seed, n_subdomains=n_subdomains, **kw)
    w.name, w.n_steps = "rods_2d", 500
    return w


def rod_colony(n: int = 200, side: float = 300.0, seed: int = 0, dim: int = 2,
               n_vertices: int = 5, growth_rate: float = 2.0, **model_kw) -> Workload:
    """A growing colony with the bacterial-rods example's agent (cellular_raza-examples/
    bacterial_rods/src/main.rs:114-150, units dropped): RodMechanics (tension 10, rigidity 1,
    damping 1.5), RodInteraction(Morse radius 3, stiffness 0.5, strength 0.1, cutoff 5),
    division past spring length 6, neighbour sensing of vertex pairs closer than 2 x radius
    with saturation 8.  dt is 0.01 rather than the example's 0.1: forward Euler on the
    spring chain is stable only while omega^2 dt < damping (omega^2 up to ~4 x tension).
    Spring lengths start uniform in [1.5, 5.5] (the vertices spaced accordingly) and the
    base growth rate is raised from 0.1 so that divisions start within tens of steps."""
    rng = np.random.Generator(np.random.PCG64(seed))
    slen = rng.uniform(1.5, 5.5, size=n)
    centres = rng.uniform(0.2 * side, 0.8 * side, size=(n, dim))
    theta = rng.uniform(0.0, 2.0 * math.pi, size=n)
    direction = np.zeros((n, dim))
    direction[:, 0] = np.cos(theta)
    direction[:, 1] = np.sin(theta)
    k = np.arange(n_vertices) - (n_vertices - 1) / 2.0
    pos = centres[:, None, :] + k[None, :, None] * slen[:, None, None] * direction[:, None, :]
    vel = np.zeros_like(pos)
    kw = dict(kind="rod", dim=dim, n_vertices=n_vertices, domain_min=(0.0,) * dim,
              domain_max=(side,) * dim, interaction_range=20.0, spring_tension=10.0,
              rigidity=1.0, spring_length=3.0, damping=1.5, diffusion=0.0, radius=3.0,
              stiffness=0.5, cutoff=5.0, strength=0.1, dt=0.01, cycle=True,
              growth_rate=growth_rate, division_length=6.0, sense_range=6.0,
              sense_saturation=8.0)
    kw.update(model_kw)
    return Workload("rod_colony", Model(**kw), pos, vel, 200, slen)


def ensemble(seed: int = 0, n_sims: int = 1024, n_lo: int = 256, n_hi: int = 65536,
             precision: str = "mixed", n_steps: int = 500) -> List[Workload]:
    """Independent 3D Morse simulations: N log-uniform in [n_lo, n_hi], Morse strength
    U[0.1, 1], damping U[0.5, 2], cube sized for density 5.12e-4."""
    rng = np.random.Generator(np.random.PCG64(seed))
    ns = np.exp(rng.uniform(math.log(n_lo), math.log(n_hi), size=n_sims)).astype(np.int64)
    strength = rng.uniform(0.1, 1.0, size=n_sims)
    damping = rng.uniform(0.5, 2.0, size=n_sims)
    out = []
    for s in range(n_sims):
        side = (ns[s] / DENSITY_3D) ** (1.0 / 3.0)
        w = spheres(int(ns[s]), side, seed * 100003 + s + 1, 3, strength=float(strength[s]),
                    damping=float(damping[s]), precision=precision)
        w.name, w.n_steps = f"ensemble[{s}]", n_steps
        out.append(w)
    return out


@dataclasses.dataclass
class Request:
    rid: int
    arrival_s: float
    workload: Workload


def request_stream(seed: int = 0, n_requests: int = 20_000, rate_hz: float = 100.0,
                   n_lo: int = 128, n_hi: int = 262_144, steps_lo: int = 100,
                   steps_hi: int = 2000) -> List[Request]:
    """Poisson arrivals; N log-uniform, steps uniform, 2D or 3D Morse spheres (50/50),
    FP64 or mixed (50/50).  2D density: the 3D mean neighbour count within the cutoff
    (4/3 pi 15^3 * 5.12e-4 = 7.24) over the disc pi 15^2 gives 0.01024 agents per unit^2."""
    rng = np.random.Generator(np.random.PCG64(seed))
    t = np.cumsum(rng.exponential(1.0 / rate_hz, size=n_requests))
    ns = np.exp(rng.uniform(math.log(n_lo), math.log(n_hi), size=n_requests)).astype(np.int64)
    steps = rng.integers(steps_lo, steps_hi + 1, size=n_requests)
    dims = np.where(rng.uniform(size=n_requests) < 0.5, 2, 3)
    prec = np.where(rng.uniform(size=n_requests) < 0.5, "f64", "mixed")
    dens2 = 4.0 / 3.0 * math.pi * 15.0 ** 3 * DENSITY_3D / (math.pi * 15.0 ** 2)
    out = []
    for r in range(n_requests):
        d = int(dims[r])
        side = (ns[r] / (DENSITY_3D if d == 3 else dens2)) ** (1.0 / d)
        w = spheres(int(ns[r]), side, seed * 7919 + r + 1, d, precision=str(prec[r]))
        w.name, w.n_steps = f"request[{r}]", int(steps[r])
        out.append(Request(r, float(t[r]), w))
    return out
