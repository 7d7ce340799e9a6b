"""Device-side edits (plg_cursor_*, plg_append, plg_permute, plg_set_types)
against the same edits done on a downloaded copy on the host, and a step
after the edits against the oracle."""
import numpy as np
import pytest

from worlds import (WorldSpec, compare_with_oracle, cursor_inside, ensure_position_f64, f32, rng_of,
                    uniform_world)

pytestmark = pytest.mark.gpu


def gpu_world(spec, capacity=None):
    from plgpu.physics import GpuWorld

    w = GpuWorld(spec.dim, capacity or 2 * spec.n)
    w.set_settings(spec.rmax, spec.friction, spec.force, spec.dt, beta=spec.beta, wrap=spec.wrap)
    w.set_matrix(spec.matrix)
    w.upload(spec.pos, spec.vel, spec.types)
    w.step(2)
    return w


CURSORS = [(0.1, 0.95, 0.0, 0.3, 0), (0.5, 0.5, 0.0, 0.25, 1), (0.02, 0.02, 0.0, 0.2, 1),
           (0.5, 0.5, 0.0, 1.0, 2), (0.3, 0.3, 0.0, 0.0, 0)]


@pytest.mark.parametrize("wrap", [True, False])
@pytest.mark.parametrize("dim", [2, 3])
def test_cursor_count_move_delete(gpu, wrap, dim):
    spec = uniform_world(20_000, 4, 0.03 if dim == 2 else 0.08, seed=101, dim=dim, vel_scale=0.01, wrap=wrap)
    w = gpu_world(spec)
    for x, y, z, size, shape in CURSORS:
        pos, vel, types, ids = w.download()
        inside = cursor_inside(pos, x, y, z, size, shape, wrap)
        assert w.cursor_count(x, y, z, size, shape) == inside.sum()
    # MOVE: the selection shifts, then wraps / clamps (FP64, stored as FP32)
    pos, vel, types, ids = w.download()
    x, y, z, size, shape = CURSORS[0]
    inside = cursor_inside(pos, x, y, z, size, shape, wrap)
    delta = np.array([0.37, -0.61, 0.2 if dim == 3 else 0.0])
    assert w.cursor_move(x, y, z, size, shape, *delta) == inside.sum()
    exp = pos.copy()
    for k in range(dim):
        exp[inside, k] = f32(ensure_position_f64(pos[inside, k] + delta[k], wrap))
    p2, v2, t2, i2 = w.download()
    assert np.array_equal(p2, exp) and np.array_equal(i2, ids) and np.array_equal(v2, vel)
    # DELETE: the rest stays in order
    x, y, z, size, shape = CURSORS[1]
    inside = cursor_inside(p2, x, y, z, size, shape, wrap)
    assert w.cursor_delete(x, y, z, size, shape) == inside.sum()
    p3, v3, t3, i3 = w.download()
    keep = ~inside
    assert np.array_equal(p3, p2[keep]) and np.array_equal(v3, v2[keep])
    assert np.array_equal(t3, t2[keep]) and np.array_equal(i3, i2[keep])
    w.step(2)  # the edited world steps on
    w.close()


def test_append_permute_set_types_then_step_matches_oracle(gpu):
    spec = uniform_world(15_000, 5, 0.02, seed=102, vel_scale=0.01)
    w = gpu_world(spec, capacity=40_000)
    rng = rng_of(103)
    # BRUSH-like growth: new particles at the end, ids after every id so far
    add = 4_000
    apos = np.zeros((add, 3))
    apos[:, :2] = f32(0.4 + 0.2 * rng.random((add, 2)))
    atyp = rng.integers(0, 5, add).astype(np.int32)
    w.append(apos, None, atyp)
    pos, vel, types, ids = w.download()
    assert pos.shape[0] == spec.n + add
    assert np.array_equal(ids[spec.n:], np.arange(spec.n, spec.n + add))
    assert np.array_equal(pos[spec.n:], apos) and not vel[spec.n:].any()
    # shuffle + truncate (setParticleCount shrink)
    src = rng.permutation(pos.shape[0])[:12_000].astype(np.int32)
    w.permute(src)
    p2, v2, t2, i2 = w.download()
    assert np.array_equal(p2, pos[src]) and np.array_equal(i2, ids[src]) and np.array_equal(t2, types[src])
    # new types (ensureTypes / setTypes)
    nt = rng.integers(0, 5, src.shape[0]).astype(np.int32)
    w.set_types(nt)
    p3, v3, t3, i3 = w.download()
    assert np.array_equal(t3, nt) and np.array_equal(p3, p2)
    # and a step from the edited state agrees with the oracle
    edited = WorldSpec(2, p3, v3, t3, spec.matrix, spec.rmax, spec.friction, spec.force, spec.dt, spec.beta,
                       spec.wrap)
    g = w.debug_step()
    compare_with_oracle(edited, g, w.download(), ids=i3)
    w.close()


def test_bad_edits_change_nothing(gpu):
    from plgpu import _lib

    spec = uniform_world(2_000, 3, 0.05, seed=104)
    w = gpu_world(spec, capacity=2_500)
    before = w.download()
    for bad in (lambda: w.permute(np.array([0, 0, 1], np.int32)),
                lambda: w.permute(np.array([5_000], np.int32)),
                lambda: w.set_types(np.full(2_000, 7, np.int32)),
                lambda: w.append(np.full((600, 3), 0.5), None, np.zeros(600, np.int32)),
                lambda: w.cursor_delete(0.5, 0.5, 0.0, 0.1, 9)):
        with pytest.raises(_lib.PlgError):
            bad()
    after = w.download()
    for a, b in zip(before, after):
        assert np.array_equal(a, b)
    w.close()
