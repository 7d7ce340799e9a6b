"""Host-side logic of the Physics mirror (no GPU): the reference's mutators
and helpers behave as in src/main/java/com/particle_life/backend/Physics.java."""
import math

import numpy as np
import pytest

from plgpu import PlgError
from plgpu.physics import (DEFAULT_DT, DefaultMatrix, ParticleLifeAccelerator, Physics, PhysicsSettings,
                           matrix_to_array)


def make(**kw):
    return Physics(ParticleLifeAccelerator(0.3), seed=3, **kw)


def test_constructor_defaults():
    """Physics.java:65-80: default matrix size 6 (from PhysicsSettings), 10000
    particles from the position setter, zero velocities."""
    p = make()
    assert p.settings.matrix.size() == 6
    assert len(p.types) == 10000
    assert p.positions.shape == (10000, 3)
    assert np.all((p.positions[:, :2] >= 0) & (p.positions[:, :2] < 1)) and np.all(p.positions[:, 2] == 0)
    assert np.all(p.velocities == 0)
    assert p.types.min() >= 0 and p.types.max() < 6
    assert p.settings.dt == DEFAULT_DT == float(np.float32(0.02))
    m = matrix_to_array(p.settings.matrix)
    assert m.min() >= -1 and m.max() <= 1


def test_set_particle_count_grow_keeps_prefix_and_shrink_keeps_subset():
    p = make(initial_count=100)
    before = p.positions.copy()
    p.set_particle_count(150)
    assert len(p.types) == 150 and np.array_equal(p.positions[:100], before)
    assert len(set(p.ids.tolist())) == 150
    ids = set(p.ids.tolist())
    p.set_particle_count(40)
    assert len(p.types) == 40 and set(p.ids.tolist()) <= ids
    with pytest.raises(ValueError):
        p.set_particle_count(-1)


def test_set_matrix_size_copies_common_block_and_retypes():
    """Physics.java:238-258 and ensureTypes 266-272."""
    p = make(initial_count=2000)
    old = matrix_to_array(p.settings.matrix)
    p.set_matrix_size(9)
    new = matrix_to_array(p.settings.matrix)
    assert new.shape == (9, 9) and np.array_equal(new[:6, :6], old)
    p.types[:] = 8
    p.set_matrix_size(4)
    assert matrix_to_array(p.settings.matrix).shape == (4, 4)
    assert p.types.max() < 4
    p.set_matrix_size(4)  # same size keeps the matrix
    assert matrix_to_array(p.settings.matrix).shape == (4, 4)


def test_connection_distance_ensure_position():
    """Physics.java:460-505 with Range.java semantics."""
    p = make(initial_count=1)
    assert np.allclose(p.connection([0.9, 0.5, 0], [0.1, 0.5, 0]), [0.2, 0, 0])
    assert p.distance([0.0, 0.0, 0], [0.75, 0.0, 0]) == pytest.approx(0.25)
    assert p.connection([0.0, 0.0, 0], [0.5, 0.0, 0])[0] == -0.5
    x = np.array([1.25, -0.25, 0.7])
    p.ensure_position(x)
    assert np.allclose(x, [0.25, 0.75, 0.0])
    p.settings.wrap = False
    x = np.array([1.25, -0.25, 0.3])
    p.ensure_position(x)
    assert np.allclose(x, [1.0, 0.0, 0.0])
    assert np.allclose(p.connection([0.9, 0.5, 0], [0.1, 0.5, 0]), [-0.8, 0, 0])


def test_settings_deep_copy_and_equality():
    s = PhysicsSettings()
    c = s.deep_copy()
    assert c == s and c.matrix is not s.matrix
    c.matrix.set(0, 0, 0.5)
    assert c != s
    c2 = s.deep_copy()
    c2.rmax = 0.03
    assert c2 != s


def test_accelerator_matches_oracle(oracle):
    acc = ParticleLifeAccelerator(0.3)
    for a in (-0.7, 0.0, 0.4):
        for dist in (0.05, 0.3, 0.5, 0.65, 0.99):
            v = acc.accelerate(a, np.array([dist, 0.0, 0.0]))
            assert v[0] == pytest.approx(oracle.accel(a, 0.3, dist), rel=1e-15, abs=1e-16)


def test_unsupported_accelerator_is_rejected_without_fallback():
    class Custom:
        def accelerate(self, a, pos):
            return pos

    p = Physics(Custom(), seed=1, initial_count=10)
    with pytest.raises(PlgError) as e:
        p._beta()
    assert e.value.status == 2


def test_default_matrix_randomize_range():
    rng = np.random.Generator(np.random.Philox(0))
    m = DefaultMatrix(16)
    m.randomize(rng)
    assert m.values.min() >= -1 and m.values.max() < 1
    assert m == m.deep_copy()
