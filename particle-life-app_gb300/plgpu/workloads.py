"""Seeded synthetic workloads for the batched and served forms.

Reference units are the unit box [0,1)^d; a config quoted in a [-1,1]^d box
has its lengths halved here.  Generators use numpy's Philox4x32
counter-based PRNG (Salmon et al. 2011), so a seed fixes every world.
"""
from __future__ import annotations

import math

import numpy as np

from .batch import WorldDesc


def friction_of_half_life(t_half: float) -> float:
    """Per-1/60 s velocity factor whose pow(f, 60 t) halves in t_half seconds."""
    return 0.5 ** (1.0 / (60.0 * t_half))


def random_world(rng: np.random.Generator, dim: int, n: int, ntypes: int, rmax: float, friction: float,
                 dt: float) -> WorldDesc:
    pos = np.zeros((n, 3))
    pos[:, :dim] = rng.random((n, dim), dtype=np.float32)
    types = rng.integers(0, ntypes, n).astype(np.int32)
    m = np.asarray(2 * rng.random((ntypes, ntypes)) - 1, np.float32).astype(np.float64)
    return WorldDesc(pos=pos, types=types, matrix=m, rmax=rmax, friction=friction, dt=dt)


def batched_worlds(count: int = 512, seed: int = 7, n_lo: int = 1_000, n_hi: int = 200_000) -> list[WorldDesc]:
    """The batched configuration: `count` 2D periodic worlds, N log-uniform in
    [n_lo, n_hi], types uniform in 3..12, matrix uniform in [-1,1], rmax
    uniform in [0.01, 0.06] of a [-1,1]^2 box (0.005..0.03 here), friction
    half-life uniform in [0.02, 0.1] s, dt = 0.02, positions uniform,
    velocities zero."""
    rng = np.random.Generator(np.random.Philox(seed))
    out = []
    for _ in range(count):
        n = int(round(math.exp(rng.uniform(math.log(n_lo), math.log(n_hi)))))
        ntypes = int(rng.integers(3, 13))
        rmax = float(rng.uniform(0.01, 0.06)) / 2
        friction = friction_of_half_life(float(rng.uniform(0.02, 0.1)))
        out.append(random_world(rng, 2, n, ntypes, rmax, friction, 0.02))
    return out


def cells_of(w: WorldDesc, dim: int) -> int:
    return int(math.floor(1.0 / w.rmax)) ** dim


def serving_request(rng: np.random.Generator, n_lo: int = 1_000, n_hi: int = 2_000_000, steps_lo: int = 100,
                    steps_hi: int = 5_000) -> tuple[int, WorldDesc, int]:
    """One request of the served configuration: 2D or 3D (50/50), N
    log-uniform in [n_lo, n_hi], types uniform in 3..16, matrix uniform in
    [-1,1], rmax giving k uniform in [10, 50] expected neighbours
    (2D: k = pi n rmax^2, 3D: k = 4/3 pi n rmax^3), friction half-life
    0.043 s, dt 0.02, step count uniform in [steps_lo, steps_hi]."""
    dim = 2 if rng.random() < 0.5 else 3
    n = int(round(math.exp(rng.uniform(math.log(n_lo), math.log(n_hi)))))
    ntypes = int(rng.integers(3, 17))
    k = float(rng.uniform(10, 50))
    if dim == 2:
        rmax = math.sqrt(k / (math.pi * n))
    else:
        rmax = (3 * k / (4 * math.pi * n)) ** (1 / 3)
    rmax = min(rmax, 0.3)
    steps = int(rng.integers(steps_lo, steps_hi + 1))
    return dim, random_world(rng, dim, n, ntypes, rmax, friction_of_half_life(0.043), 0.02), steps


def serving_request_generated(rng: np.random.Generator, n_lo: int = 1_000, n_hi: int = 2_000_000,
                              steps_lo: int = 100, steps_hi: int = 5_000):
    """One request of the served configuration as a world spec the server
    generates on the device: the distributions of serving_request (2D or 3D
    50/50, N log-uniform in [n_lo, n_hi], types uniform in 3..16, matrix
    uniform in [-1,1], rmax for k uniform in [10, 50] neighbours, friction
    half-life 0.043 s, dt 0.02, steps uniform in [steps_lo, steps_hi]),
    positions uniform and types uniform from a per-request seed."""
    from .serve import GeneratedWorld

    dim = 2 if rng.random() < 0.5 else 3
    n = int(round(math.exp(rng.uniform(math.log(n_lo), math.log(n_hi)))))
    ntypes = int(rng.integers(3, 17))
    k = float(rng.uniform(10, 50))
    if dim == 2:
        rmax = math.sqrt(k / (math.pi * n))
    else:
        rmax = (3 * k / (4 * math.pi * n)) ** (1 / 3)
    rmax = min(rmax, 0.3)
    steps = int(rng.integers(steps_lo, steps_hi + 1))
    m = np.asarray(2 * rng.random((ntypes, ntypes)) - 1, np.float32).astype(np.float64)
    seed = int(rng.integers(0, 2**63))
    return dim, GeneratedWorld(n=n, matrix=m, rmax=rmax, friction=friction_of_half_life(0.043), dt=0.02,
                               seed=seed), steps


# rmax of the 3D blob configuration: bisection (30 halvings) of the mean
# neighbour count within rmax over a 1% sample of the 4M-particle world below
# (periodic KD-tree), to 40 neighbours.
BLOB3D_RMAX = 0.004711


def blob_world_3d(n: int = 4_000_000, ntypes: int = 16, nblobs: int = 64, sigma: float = 0.025, seed: int = 3,
                  rmax: float = BLOB3D_RMAX) -> WorldDesc:
    """The 3D configuration: n particles in `nblobs` isotropic Gaussian blobs
    (sigma 0.05 of a [-1,1]^3 box = 0.025 here), centres uniform, wrapped
    into the unit cube; types uniform, matrix uniform in [-1,1], velocities
    zero, friction half-life 0.043 s, dt = 0.01."""
    rng = np.random.Generator(np.random.Philox(seed))
    centres = rng.random((nblobs, 3))
    which = rng.integers(0, nblobs, n)
    p = centres[which] + rng.standard_normal((n, 3)) * sigma
    p = p - np.floor(p)
    p = np.asarray(p, np.float32)
    p[p >= 1.0] = 0.0
    types = rng.integers(0, ntypes, n).astype(np.int32)
    m = np.asarray(2 * rng.random((ntypes, ntypes)) - 1, np.float32).astype(np.float64)
    return WorldDesc(pos=p.astype(np.float64), types=types, matrix=m, rmax=rmax,
                     friction=friction_of_half_life(0.043), dt=0.01)
