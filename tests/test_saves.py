"""Save format of the app (particles.tsv, physics.toml, matrix.tsv in a zip):
Java's double formatting, exact round trips, missing entries, and an
archive laid out as the app writes it."""
import io
import zipfile

import numpy as np
import pytest

from plgpu import saves


@pytest.mark.parametrize("x, s", [
    (1.0, "1.0"), (0.5, "0.5"), (-2.25, "-2.25"), (0.0, "0.0"), (-0.0, "-0.0"),
    (0.001, "0.001"), (0.0001, "1.0E-4"), (1e-5, "1.0E-5"), (1.5e-7, "1.5E-7"),
    (1e7, "1.0E7"), (9999999.0, "9999999.0"), (123456789.0, "1.23456789E8"),
    (0.1 + 0.2, "0.30000000000000004"), (1 / 3, "0.3333333333333333"), (100.0, "100.0"),
    (0.7644018106552037, "0.7644018106552037"), (2.5e-300, "2.5E-300"), (1.7976931348623157e308, "1.7976931348623157E308"),
])
def test_java_double_formatting(x, s):
    assert saves.java_double(x) == s
    assert float(s) == x


def test_round_trip_is_exact(tmp_path):
    rng = np.random.Generator(np.random.Philox(5))
    n = 500
    pos = np.zeros((n, 3))
    pos[:, :2] = rng.random((n, 2))
    vel = np.zeros((n, 3))
    vel[:, :2] = rng.standard_normal((n, 2)) * 1e-3
    vel[0, 0] = 1e-12
    typ = rng.integers(0, 6, n).astype(np.int32)
    m = 2 * rng.random((6, 6)) - 1
    f = tmp_path / "s.zip"
    saves.save_state(f, pos, vel, typ, wrap=False, rmax=0.035, friction=0.7644018106552037, force=1.25, matrix=m)
    st = saves.load_state(f)
    assert st.dim == 2 and st.wrap is False and st.rmax == 0.035 and st.friction == 0.7644018106552037
    assert st.force == 1.25
    assert np.array_equal(st.positions, pos) and np.array_equal(st.velocities, vel) and np.array_equal(st.types, typ)
    assert np.array_equal(st.matrix, m)


def test_3d_extension_round_trip(tmp_path):
    rng = np.random.Generator(np.random.Philox(6))
    pos = rng.random((50, 3))
    vel = rng.standard_normal((50, 3))
    typ = rng.integers(0, 3, 50).astype(np.int32)
    f = tmp_path / "s3.zip"
    saves.save_state(f, pos, vel, typ, wrap=True, rmax=0.1, friction=0.8, force=1.0, matrix=np.eye(3), dim=3)
    st = saves.load_state(f)
    assert st.dim == 3 and np.array_equal(st.positions, pos) and np.array_equal(st.velocities, vel)


def test_reads_an_archive_laid_out_like_the_apps(tmp_path):
    """Entries as Main.saveState writes them (including a thumbnail, which
    loading ignores); missing entries come back as None."""
    f = tmp_path / "app.zip"
    with zipfile.ZipFile(f, "w") as z:
        z.writestr("particles.tsv", "x\ty\tvx\tvy\tcolor\n0.25\t0.75\t1.0E-4\t-0.5\t2\n0.5\t1.0E-5\t0.0\t0.0\t0\n")
        z.writestr("physics.toml", 'boundaries = "clamped"\nradius = 0.04\nfriction = 0.85\nforce = 1.0\n')
        z.writestr("matrix.tsv", "0.5\t-1.0E-3\t0.0\n1.0\t0.25\t-0.75\n0.0\t0.0\t1.0\n")
        z.writestr("img.png", b"\x89PNG")
    st = saves.load_state(f)
    assert np.array_equal(st.positions, [[0.25, 0.75, 0.0], [0.5, 1e-5, 0.0]])
    assert np.array_equal(st.velocities, [[1e-4, -0.5, 0.0], [0.0, 0.0, 0.0]])
    assert np.array_equal(st.types, [2, 0])
    assert st.wrap is False and st.rmax == 0.04
    assert np.array_equal(st.matrix, [[0.5, -1e-3, 0.0], [1.0, 0.25, -0.75], [0.0, 0.0, 1.0]])
    g = tmp_path / "only_matrix.zip"
    with zipfile.ZipFile(g, "w") as z:
        z.writestr("matrix.tsv", "1.0\n")
    st = saves.load_state(g)
    assert st.positions is None and st.rmax is None and st.matrix.shape == (1, 1)


def test_written_text_matches_the_apps_layout():
    text = saves.particles_tsv(np.array([[0.5, 1e-4, 0.0]]), np.array([[0.0, -2.0, 0.0]]), np.array([3]))
    assert text == "x\ty\tvx\tvy\tcolor\n0.5\t1.0E-4\t0.0\t-2.0\t3\n"
    assert saves.matrix_tsv(np.array([[1.0, 0.5], [-0.25, 1e-8]])) == "1.0\t0.5\n-0.25\t1.0E-8\n"
    assert saves.settings_toml(True, 0.02, 0.85, 1.0) == 'boundaries = "periodic"\nradius = 0.02\nfriction = 0.85\nforce = 1.0\n'


def test_physics_mirror_save_and_load(tmp_path):
    from plgpu import Physics, ParticleLifeAccelerator

    a = Physics(ParticleLifeAccelerator(), seed=3, initial_count=300)
    a.settings.rmax, a.settings.wrap, a.settings.friction = 0.045, False, 0.61
    f = tmp_path / "mirror.zip"
    a.save_state(f)
    b = Physics(ParticleLifeAccelerator(), seed=4, initial_count=10)
    b.load_state(f)
    assert np.array_equal(a.positions, b.positions) and np.array_equal(a.types, b.types)
    assert (b.settings.rmax, b.settings.wrap, b.settings.friction) == (0.045, False, 0.61)
    assert np.array_equal(a.settings.matrix.as_array(), b.settings.matrix.as_array())


@pytest.mark.gpu
def test_a_loaded_save_continues_the_trajectory(gpu, tmp_path):
    from plgpu import Physics, ParticleLifeAccelerator

    a = Physics(ParticleLifeAccelerator(), seed=7, initial_count=20_000)
    a.settings.rmax = 0.03
    for _ in range(4):
        a.update()
    f = tmp_path / "run.zip"
    a.save_state(f)
    b = Physics(ParticleLifeAccelerator(), seed=8, initial_count=5)
    b.load_state(f)
    b.settings.dt = a.settings.dt  # dt is not part of a save (PhysicsSettingsToml.java:31-32)
    for _ in range(3):
        a.update()
        b.update()
    assert np.array_equal(a.positions, b.positions) and np.array_equal(a.velocities, b.velocities)
    a.close()
    b.close()


def test_png_round_trip():
    """The thumbnail encoder writes an 8-bit RGBA PNG that reads back exactly."""
    from plgpu import saves

    img = np.random.default_rng(2).integers(0, 256, size=(37, 53, 4), dtype=np.uint8)
    png = saves.png_rgba(img)
    assert png[:8] == b"\x89PNG\r\n\x1a\n" and png[12:16] == b"IHDR"
    assert np.array_equal(saves.read_png_rgba(png), img)
