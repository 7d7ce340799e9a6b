"""The force kernel's paths give the same bits.

Plain steps run the force kernel as compiled for speed; the instrumented step
runs its instrumented instantiation (pair counts, hashes, accelerations) on
the same tiles.  Both evaluate every target's candidates in the same order
with the same arithmetic, so three steps of each from the same start state
must agree exactly: positions, velocities, types and the sorted order.  The
worlds cover what changes the staging: dense tiles (one staging per block),
windows that overflow a staging (chunks and the global-memory path), clamped
walls, the periodic boundary, coincident particles (the deferred FP64 pass),
more than 16 types (matrix in global memory), a small grid (the literal
path), 3D blobs, and a batch of uneven worlds.
"""
import numpy as np
import pytest

from worlds import blob_world, uniform_world

pytestmark = pytest.mark.gpu


def spec_for(case):
    if case == "2d_uniform":
        return uniform_world(120_000, 6, 0.004, seed=41, vel_scale=0.01)
    if case == "2d_overflow":
        return blob_world(60_000, 5, 0.01, nblobs=12, sigma=0.004, seed=14, dim=2)
    if case == "2d_clamp":
        spec = uniform_world(20_000, 5, 0.01, seed=3, vel_scale=0.05, wrap=False)
        spec.pos[:200, 0] = 0.0
        spec.pos[200:400, 0] = 1.0
        spec.pos[600:800, :2] = 1.0
        return spec
    if case == "2d_coincident":
        spec = uniform_world(5000, 4, 0.02, seed=9)
        spec.pos[100:140] = spec.pos[99]
        spec.pos[1000:1003] = spec.pos[2000]
        return spec
    if case == "2d_many_types":
        return uniform_world(40_000, 100, 0.01, seed=7, vel_scale=0.01)
    if case == "2d_small_grid":
        return uniform_world(3000, 4, 0.4, seed=5, vel_scale=0.01)  # nx = 2: the literal path
    if case == "3d_uniform":
        return uniform_world(100_000, 8, 0.03, seed=42, dim=3, vel_scale=0.01, dt=0.01)
    if case == "3d_blobs":
        return blob_world(300_000, 16, 0.0095, seed=12, dt=0.01)
    raise KeyError(case)


CASES = ["2d_uniform", "2d_overflow", "2d_clamp", "2d_coincident", "2d_many_types", "2d_small_grid", "3d_uniform",
         "3d_blobs"]


@pytest.mark.parametrize("case", CASES)
def test_plain_and_instrumented_steps_agree(gpu, case):
    from plgpu.physics import GpuWorld

    spec = spec_for(case)
    runs = []
    for instrumented in (False, True):
        w = GpuWorld(spec.dim, spec.n)
        w.set_settings(spec.rmax, spec.friction, spec.force, spec.dt, beta=spec.beta, wrap=spec.wrap)
        w.set_matrix(spec.matrix)
        w.upload(spec.pos, spec.vel, spec.types)
        for _ in range(3):
            if instrumented:
                w.debug_step()
            else:
                w.step(1)
        runs.append(w.download())
        w.close()
    for a, b in zip(*runs):
        assert np.array_equal(a, b)


def test_batched_plain_and_instrumented_steps_agree(gpu):
    from plgpu.batch import GpuBatch, WorldDesc

    specs = [uniform_world(20_000, 5, 0.01, seed=43), blob_world(30_000, 6, 0.01, nblobs=6, sigma=0.01, seed=44, dim=2),
             uniform_world(900, 3, 0.05, seed=45, wrap=False), uniform_world(5000, 20, 0.02, seed=46)]
    total = sum(s.n for s in specs)
    cells = sum(int(np.floor(1 / s.rmax)) ** 2 for s in specs)
    runs = []
    for instrumented in (False, True):
        b = GpuBatch(2, total + 1, len(specs), cells + 1)
        ids = b.update(add=[WorldDesc(pos=s.pos, types=s.types, matrix=s.matrix, rmax=s.rmax, friction=s.friction,
                                      force=s.force, dt=s.dt, beta=s.beta, wrap=s.wrap, vel=s.vel) for s in specs])
        b.set_tile(0)
        for _ in range(3):
            if instrumented:
                b.debug_step()
            else:
                b.step(1)
        runs.append([b.download(i) for i in ids])
        b.close()
    for wa, wb in zip(*runs):
        for a, c in zip(wa, wb):
            assert np.array_equal(a, c)
