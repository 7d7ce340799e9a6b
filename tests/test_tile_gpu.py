"""Force tile variants of a single world: every variant gives the same bits
(the same candidate order and arithmetic per target, only the block shape
and staging size change), and the autotuner leaves the world where it was
(the state it times is restored) while keeping the fastest variant."""
import numpy as np
import pytest

from worlds import blob_world, uniform_world

pytestmark = pytest.mark.gpu


def _world(spec):
    from plgpu.physics import GpuWorld

    w = GpuWorld(spec.dim, spec.n)
    w.set_settings(spec.rmax, spec.friction, spec.force, spec.dt, beta=spec.beta, wrap=spec.wrap)
    w.set_matrix(spec.matrix)
    w.upload(spec.pos, spec.vel, spec.types)
    return w


def spec_for(case):
    if case == "2d_uniform":
        return uniform_world(100_000, 6, 0.004, seed=61, vel_scale=0.01)
    if case == "2d_dense":  # variant 0's staging overflows, variant 1's fits
        return blob_world(88_000, 5, 0.01, nblobs=8, sigma=0.004, seed=62, dim=2)
    if case == "2d_clamp":
        return uniform_world(20_000, 5, 0.01, seed=63, vel_scale=0.05, wrap=False)
    if case == "3d_blobs":
        return blob_world(200_000, 16, 0.0095, seed=64, dt=0.01)
    if case == "3d_uniform":
        return uniform_world(60_000, 8, 0.03, seed=65, dim=3, vel_scale=0.01, dt=0.01)
    raise KeyError(case)


@pytest.mark.parametrize("case", ["2d_uniform", "2d_dense", "2d_clamp", "3d_blobs", "3d_uniform"])
def test_tile_variants_give_the_same_bits(gpu, case):
    from plgpu import _lib

    spec = spec_for(case)
    runs = []
    for v in range(_lib.PLG_TILE_VARIANTS):
        w = _world(spec)
        try:
            w.set_tile(v)
            assert w.tile() == v
            w.step(3)
            runs.append(w.download())
        finally:
            w.close()
    for other in runs[1:]:
        for a, b in zip(runs[0], other):
            assert np.array_equal(a, b)


@pytest.mark.parametrize("case", ["2d_uniform", "3d_blobs"])
def test_autotune_restores_the_world(gpu, case):
    from plgpu import _lib

    spec = spec_for(case)
    a, b = _world(spec), _world(spec)
    try:
        a.step(1)
        b.step(1)
        before = a.tile()
        chosen, ms = a.autotune(3)
        assert chosen in range(_lib.PLG_TILE_VARIANTS)
        assert a.tile() == chosen
        assert len(ms) == _lib.PLG_TILE_VARIANTS and all(t > 0 for t in ms)
        fastest = int(np.argmin(ms))
        # the fastest variant replaces the current one only when it is at least 2% faster
        assert chosen == (fastest if ms[fastest] < 0.98 * ms[before] else before)
        for x, y in zip(a.download(), b.download()):
            assert np.array_equal(x, y)
        a.step(2)
        b.step(2)
        for x, y in zip(a.download(), b.download()):
            assert np.array_equal(x, y)
    finally:
        a.close()
        b.close()


def test_tile_errors_and_small_grid(gpu):
    from plgpu import _lib
    from plgpu.physics import GpuWorld

    spec = uniform_world(2000, 4, 0.4, seed=66)  # nx = 2: the literal kernel, no tiles
    w = _world(spec)
    try:
        assert w.lib.plg_set_tile(w.ctx, _lib.PLG_TILE_VARIANTS) == _lib.PLG_E_INVALID_ARG
        assert w.lib.plg_set_tile(w.ctx, -1) == _lib.PLG_E_INVALID_ARG
        w.set_tile(1)
        chosen, _ = w.autotune(2)
        assert chosen == 1
    finally:
        w.close()
    fresh = GpuWorld(2, 10)
    try:
        c = _lib.C.c_int32()
        assert fresh.lib.plg_autotune(fresh.ctx, 2, _lib.C.byref(c), None) == _lib.PLG_E_STATE  # not ready
    finally:
        fresh.close()


def test_default_variant_follows_the_size(gpu):
    """Until a variant is set or tuned, 2D worlds under 300,000 particles
    take the 128-target tile (variant 2) and larger ones variant 0; 3D
    worlds variant 0.  Setting a variant overrides the default."""
    small, large = uniform_world(10_000, 6, 0.02, seed=71), uniform_world(400_000, 6, 0.004, seed=72)
    small3 = uniform_world(20_000, 6, 0.05, seed=73, dim=3)
    worlds = [_world(small), _world(large), _world(small3)]
    try:
        assert [w.tile() for w in worlds] == [2, 0, 0]
        worlds[0].set_tile(1)
        assert worlds[0].tile() == 1
        worlds[0].step(1)
        assert worlds[0].tile() == 1
    finally:
        for w in worlds:
            w.close()
