"""Known answers for the oracle, derived by hand from the reference formulas
(paths relative to src/main/java/com/particle_life/)."""
import math

import numpy as np
import pytest

from worlds import FRICTION_T_HALF_0043, f32


def test_accelerator_known_points(oracle):
    """app/Main.java:275-280: f(0+) = -1, f(beta) = 0, f((1+beta)/2) = a,
    f(1) = 0; the returned vector is pos * f / |pos|."""
    beta, a = 0.3, 0.7
    assert oracle.accel(a, beta, 1e-12) == pytest.approx(-1.0, abs=1e-11)
    assert oracle.accel(a, beta, beta) == pytest.approx(0.0, abs=1e-15)
    assert oracle.accel(a, beta, (1 + beta) / 2) == pytest.approx(a, abs=1e-15)
    assert oracle.accel(a, beta, 1.0) == pytest.approx(0.0, abs=1e-15)
    assert oracle.accel(-0.4, beta, 0.5) == pytest.approx(-0.4 * (1 - abs(1.3 - 1.0) / 0.7), rel=1e-15)
    # linear repulsion part does not depend on a
    assert oracle.accel(0.0, beta, 0.15) == pytest.approx(0.15 / 0.3 - 1, rel=1e-15)


def test_wrap_connection_half(oracle):
    """backend/Range.java:74-81: single wind onto [-0.5, 0.5)."""
    assert oracle.wrap_connection(0.5) == -0.5
    assert oracle.wrap_connection(-0.5) == -0.5
    assert oracle.wrap_connection(0.75) == -0.25
    assert oracle.wrap_connection(-0.75) == 0.25
    assert oracle.wrap_connection(0.4999) == 0.4999


def test_range_wrap_and_clamp(oracle):
    """backend/Range.java:46-57 and 89-96."""
    assert oracle.wrap(-0.3) == pytest.approx(0.7, abs=1e-16)
    assert oracle.wrap(2.0) == 0.0
    assert oracle.wrap(3.25) == 0.25
    assert oracle.wrap(-1e-20) == 1.0 - 1e-20  # rounds to 1.0 in FP64: the reference keeps it
    assert oracle.clamp(-0.1) == 0.0 and oracle.clamp(1.5) == 1.0 and oracle.clamp(1.0) == 1.0


def test_container_index_edges(oracle):
    """backend/Physics.java:362-375: truncation, cx == nx clamped to nx-1; the
    last partial cell [nx*cs, 1) maps to nx-1."""
    rmax = 0.3  # nx = 3, sliver [0.9, 1)
    assert oracle.grid_n(rmax) == 3
    assert oracle.container_index(2, 0.0, 0.0, 0, rmax) == 0
    assert oracle.container_index(2, 0.95, 0.0, 0, rmax) == 2
    assert oracle.container_index(2, 1.0, 1.0, 0, rmax) == 2 + 2 * 3
    assert oracle.container_index(2, 0.3, 0.0, 0, rmax) == 1
    assert oracle.container_index(3, 0.0, 0.0, 0.95, rmax) == 2 * 9
    assert oracle.grid_n(0.02) == 50 and oracle.grid_n(0.0025) == 400


def world(oracle, pos, types, matrix, rmax, friction=1.0, force=1.0, dt=0.02, wrap=True, vel=None, dim=2):
    n = len(types)
    p = np.zeros((n, 3))
    p[:, : len(pos[0])] = pos
    v = np.zeros((n, 3)) if vel is None else np.asarray(vel, float)
    return oracle.World(dim, p, v, np.asarray(types, np.int32), np.arange(n, dtype=np.int32), np.asarray(matrix, float),
                        oracle.settings(rmax, friction, force, dt, 0.3, wrap))


def test_two_particles_hand_computed(oracle):
    """Particle 1 at r = 0.5 rmax to the right of particle 0: particle 0 gets
    v += (a * (1 - |1.3 - 1| / 0.7)) * rmax * force * dt along +x."""
    rmax, dt = 0.1, 0.02
    m = [[0.0, 0.8], [-0.6, 0.0]]
    w = world(oracle, [(0.5, 0.5), (0.55, 0.5)], [0, 1], m, rmax, dt=dt)
    w.step()
    f01 = 0.8 * (1 - abs(1.3 - 1.0) / 0.7)
    f10 = -0.6 * (1 - abs(1.3 - 1.0) / 0.7)
    by_id = {int(i): k for k, i in enumerate(w.ids)}
    assert w.vel[by_id[0], 0] == pytest.approx(f01 * rmax * dt, rel=1e-12)
    assert w.vel[by_id[1], 0] == pytest.approx(-f10 * rmax * dt, rel=1e-12)
    assert w.pos[by_id[0], 0] == pytest.approx(0.5 + f01 * rmax * dt * dt, rel=1e-12)


def test_pair_across_periodic_border(oracle):
    rmax = 0.1
    w = world(oracle, [(0.01, 0.5), (0.98, 0.5)], [0, 0], [[1.0]], rmax)
    d = w.step(debug=True)
    assert list(d["pairs"]) == [1, 1]
    wc = world(oracle, [(0.01, 0.5), (0.98, 0.5)], [0, 0], [[1.0]], rmax, wrap=False)
    assert list(wc.step(debug=True)["pairs"]) == [0, 0]


def test_small_grid_multiplicity(oracle):
    """nx < 3 (backend/Physics.java:377-409): the 9 offsets wrap onto the same
    cells, so a pair is counted once per visit: 9x for nx = 1, 4x-per-axis
    pattern for nx = 2."""
    w = world(oracle, [(0.2, 0.2), (0.3, 0.25)], [0, 0], [[1.0]], 0.7)  # nx = 1
    assert list(w.step(debug=True)["pairs"]) == [9, 9]
    w = world(oracle, [(0.1, 0.1), (0.2, 0.1)], [0, 0], [[1.0]], 0.4)  # nx = 2, same cell
    # each axis visits cells {1, 0, 1} -> cell 0 once per axis -> 1 x 1 ... and cell 1 twice
    assert list(w.step(debug=True)["pairs"]) == [1, 1]
    w = world(oracle, [(0.1, 0.1), (0.45, 0.1)], [0, 0], [[1.0]], 0.4)  # cells 0 and 1 along x
    assert list(w.step(debug=True)["pairs"]) == [2, 2]


def test_counting_sort_is_stable(oracle):
    """makeContainers (backend/Physics.java:342-348) keeps the array order of
    particles of one cell."""
    rng = np.random.default_rng(0)
    n = 500
    pos = f32(rng.random((n, 2)))
    w = world(oracle, pos, np.zeros(n, int), [[0.0]], 0.1, friction=1.0)
    w.step()
    cells = (np.floor(pos[w.ids, 0] / 0.1) + 10 * np.floor(pos[w.ids, 1] / 0.1)).astype(int)
    assert np.all(np.diff(cells) >= 0)
    for c in np.unique(cells):
        ids = w.ids[cells == c]
        assert np.all(np.diff(ids) > 0)


def test_friction_factor(oracle):
    """v *= pow(friction, 60 dt) with no neighbours (backend/Physics.java:401-402)."""
    fr, dt = FRICTION_T_HALF_0043, 0.01
    w = world(oracle, [(0.5, 0.5)], [0], [[0.0]], 0.05, friction=fr, dt=dt, vel=[(0.3, -0.2, 0.0)])
    w.step()
    ff = fr ** (60 * dt)
    assert w.vel[0, 0] == pytest.approx(0.3 * ff, rel=1e-15)
    assert w.pos[0, 1] == pytest.approx(0.5 - 0.2 * ff * dt, rel=1e-15)
    # t_1/2 = 0.043 s: after 0.043 s of steps the speed halves
    assert fr ** (60 * 0.043) == pytest.approx(0.5, rel=1e-12)


def test_3d_extension_27_cells(oracle):
    rmax = 0.1
    w = world(oracle, [(0.5, 0.5, 0.01), (0.5, 0.5, 0.98)], [0, 0], [[1.0]], rmax, dim=3)
    assert list(w.step(debug=True)["pairs"]) == [1, 1]
