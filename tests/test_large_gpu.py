"""Large worlds: 16M particles in 2D and 3D through a few steps, checked by
properties that hold at any size (an FP64 oracle step at this size takes
minutes): the ids stay a permutation of the upload order, types travel with
their particles, positions stay in the unit box, the order is the cell
order (cells nondecreasing), and plain and instrumented steps agree bit for
bit.  The parity against the oracle at full configuration size is in the
parity tests (1M 2D, 4M 3D)."""
import numpy as np
import pytest

from worlds import uniform_world

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dim, rmax", [(2, 0.0005), (3, 0.006)])
def test_sixteen_million_particles(gpu, dim, rmax):
    from plgpu.physics import GpuWorld

    n = 16_000_000
    spec = uniform_world(n, 8, rmax, seed=71, dim=dim, vel_scale=0.01)
    runs = []
    for instrumented in (False, True):
        w = GpuWorld(dim, n)
        w.set_settings(spec.rmax, spec.friction, spec.force, spec.dt, beta=spec.beta, wrap=spec.wrap)
        w.set_matrix(spec.matrix)
        w.upload(spec.pos, spec.vel, spec.types)
        w.step(2)
        cells = w.debug_step()["cell"] if instrumented else None
        if not instrumented:
            w.step(1)
        runs.append(w.download())
        w.close()
    pos, vel, types, ids = runs[0]
    for a, b in zip(runs[0], runs[1]):
        assert np.array_equal(a, b)
    assert np.array_equal(np.sort(ids), np.arange(n, dtype=np.int32))
    assert np.array_equal(types, spec.types[ids])
    assert np.all((pos[:, :dim] >= 0.0) & (pos[:, :dim] < 1.0))
    assert np.all(np.isfinite(vel))
    assert np.all(np.diff(cells.astype(np.int64)) >= 0)  # the step's sorted order is the cell order
