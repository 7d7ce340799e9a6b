"""Seeded synthetic worlds and comparison helpers shared by the tests.

Positions, velocities and matrix entries are drawn as float32 and stored as
float64, so the GPU's FP32 state and the oracle's FP64 state start equal.
Generators use numpy's Philox4x32 counter-based PRNG (Salmon et al. 2011).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

FRICTION_T_HALF_0043 = 0.5 ** (1.0 / (60.0 * 0.043))  # 0.7644018106552037


@dataclass
class WorldSpec:
    dim: int
    pos: np.ndarray  # (n, 3) float64, FP32-exact
    vel: np.ndarray  # (n, 3) float64, FP32-exact
    types: np.ndarray  # (n,) int32
    matrix: np.ndarray  # (t, t) float64, FP32-exact
    rmax: float
    friction: float = FRICTION_T_HALF_0043
    force: float = 1.0
    dt: float = 0.02
    beta: float = 0.3
    wrap: bool = True

    @property
    def n(self) -> int:
        return self.pos.shape[0]


def rng_of(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.Philox(seed))


def f32(a) -> np.ndarray:
    return np.asarray(a, np.float32).astype(np.float64)


def uniform_world(n, ntypes, rmax, seed=0, dim=2, vel_scale=0.0, **kw) -> WorldSpec:
    rng = rng_of(seed)
    pos = np.zeros((n, 3))
    pos[:, :dim] = rng.random((n, dim), dtype=np.float32)
    vel = np.zeros((n, 3))
    if vel_scale:
        vel[:, :dim] = f32(rng.standard_normal((n, dim)) * vel_scale)
    types = rng.integers(0, ntypes, n).astype(np.int32)
    m = f32(2 * rng.random((ntypes, ntypes)) - 1)
    return WorldSpec(dim, pos, vel, types, m, rmax, **kw)


def blob_world(n, ntypes, rmax, nblobs=64, sigma=0.025, seed=0, dim=3, **kw) -> WorldSpec:
    """Isotropic Gaussian blobs (sigma in reference units), centres uniform,
    positions wrapped into the unit box."""
    rng = rng_of(seed)
    centres = rng.random((nblobs, dim))
    which = rng.integers(0, nblobs, n)
    p = centres[which] + rng.standard_normal((n, dim)) * sigma
    p = p - np.floor(p)
    p = np.asarray(p, np.float32)
    p[p >= 1.0] = 0.0
    pos = np.zeros((n, 3))
    pos[:, :dim] = p
    vel = np.zeros((n, 3))
    types = rng.integers(0, ntypes, n).astype(np.int32)
    m = f32(2 * rng.random((ntypes, ntypes)) - 1)
    return WorldSpec(dim, pos, vel, types, m, rmax, **kw)


def min_image(d: np.ndarray, wrap: bool) -> np.ndarray:
    if not wrap:
        return d
    return d - np.round(d)


def norm_rel(a: np.ndarray, b: np.ndarray) -> float:
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / nb) if nb > 0 else float(np.linalg.norm(a - b))


def run_gpu_debug(spec: WorldSpec, capacity=None):
    """Upload spec, run one instrumented step, download; returns (debug, state)."""
    from plgpu.physics import GpuWorld

    w = GpuWorld(spec.dim, capacity or max(spec.n, 1))
    try:
        w.set_settings(spec.rmax, spec.friction, spec.force, spec.dt, beta=spec.beta, wrap=spec.wrap)
        w.set_matrix(spec.matrix)
        w.upload(spec.pos, spec.vel, spec.types)
        d = w.debug_step()
        st = w.download()
    finally:
        w.close()
    return d, st


def run_oracle_debug(spec: WorldSpec, threads=8, ids=None):
    import orc

    ids = np.arange(spec.n, dtype=np.int32) if ids is None else np.ascontiguousarray(ids, np.int32)
    o = orc.World(spec.dim, spec.pos, spec.vel, spec.types, ids, spec.matrix,
                  orc.settings(spec.rmax, spec.friction, spec.force, spec.dt, spec.beta, spec.wrap))
    d = o.step(threads=threads, debug=True)
    return d, o


def accel_errors(acc_gpu: np.ndarray, acc_ref: np.ndarray, abs_terms: np.ndarray | None = None) -> dict:
    """Norm-wise relative error and raw per-particle relative error."""
    e = np.linalg.norm(acc_gpu - acc_ref, axis=1)
    r = np.linalg.norm(acc_ref, axis=1)
    nz = r > 0
    raw = e[nz] / r[nz]
    out = dict(normwise=norm_rel(acc_gpu, acc_ref))
    if raw.size:
        out.update(p50=float(np.percentile(raw, 50)), p99=float(np.percentile(raw, 99)), max=float(raw.max()))
    return out


ACC_TOL = 1e-5
VEL_TOL = 1e-5
POS_ABS = 1.2e-7


def compare_with_oracle(spec: WorldSpec, g: dict, state, exact_only=False, normwise=True, ids=None):
    """Asserts one GPU step (debug outputs `g`, downloaded `state`) against
    the oracle's step of the same start state (particle ids `ids`, default
    0..n-1); returns error figures."""
    gpos, gvel, gtypes, gids = state
    d, o = run_oracle_debug(spec, ids=ids)
    assert np.array_equal(gids, o.ids), "sorted order (ids) differs from the oracle"
    assert np.array_equal(gtypes, o.types)
    assert np.array_equal(g["cell"], d["cell"]), "cell assignment differs"
    assert np.array_equal(g["pairs"], d["pairs"]), "interacting-pair counts differ"
    assert np.array_equal(g["hsum"], d["hsum"]), "interacting-pair sets differ (sum hash)"
    assert np.array_equal(g["hxor"], d["hxor"]), "interacting-pair sets differ (xor hash)"
    out = dict(pairs=float(d["pairs"].mean()) if spec.n else 0.0)
    if spec.n == 0 or d["pairs"].sum() == 0 or exact_only:
        return out
    acc_g = g["acc"].astype(np.float64)
    e = accel_errors(acc_g, d["acc"])
    if normwise:
        assert e["normwise"] <= ACC_TOL, e
    scale = np.where(d["fscale"] > 0, d["fscale"], 1.0)
    per = np.linalg.norm(acc_g - d["acc"], axis=1) / scale
    assert per.max() <= ACC_TOL, per.max()
    dim = spec.dim
    if normwise:
        assert norm_rel(gvel[:, :dim], o.vel[:, :dim]) <= VEL_TOL
    dp = np.abs(min_image(gpos[:, :dim] - o.pos[:, :dim], spec.wrap))
    dv = VEL_TOL * np.abs(o.vel[:, :dim]) + ACC_TOL * (spec.rmax * spec.force * spec.dt) * d["fscale"][:, None]
    bound = POS_ABS + spec.dt * dv
    assert np.all(dp <= bound), float((dp / bound).max())
    out.update(e)
    return out


def cursor_inside(pos: np.ndarray, x, y, z, size, shape, wrap: bool) -> np.ndarray:
    """Cursor.isInside (app/cursors/Cursor.java:16-35) in FP64: delta to the
    cursor, wrapped as val - floor(val + 0.5), divided by the size, then the
    shape's test (0 circle: length <= 0.5, 1 square: |x|, |y| <= 0.5,
    2 infinity)."""
    if size == 0.0:
        return np.zeros(pos.shape[0], bool)
    d = np.asarray(pos, np.float64) - np.array([x, y, z], np.float64)
    if wrap:
        d = d - np.floor(d + 0.5)
    d = d / size
    if shape == 0:
        return np.sqrt(d[:, 0] * d[:, 0] + (d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2])) <= 0.5
    if shape == 1:
        return (np.abs(d[:, 0]) <= 0.5) & (np.abs(d[:, 1]) <= 0.5)
    return np.ones(pos.shape[0], bool)


def ensure_position_f64(x: np.ndarray, wrap: bool) -> np.ndarray:
    """Range.wrap / Range.clamp (backend/Range.java:40-96) of FP64 values."""
    if wrap:
        x = x - np.floor(x)
        return np.where(x >= 1.0, 0.0, x)
    return np.clip(x, 0.0, 1.0)
