"""plg_render (the headless splat of the default particle shaders) against
the numpy FP32 restatement in the oracle directory: bit-exact images."""
import numpy as np
import pytest

from worlds import blob_world, uniform_world

pytestmark = pytest.mark.gpu


def palette(k, seed=5):
    rng = np.random.default_rng(seed)
    p = rng.random((k, 4), dtype=np.float32)
    p[:, 3] = 1.0
    return p


def world_after(spec, steps):
    from plgpu.physics import GpuWorld

    w = GpuWorld(spec.dim, spec.n)
    w.set_settings(spec.rmax, spec.friction, spec.force, spec.dt, beta=spec.beta, wrap=spec.wrap)
    w.set_matrix(spec.matrix)
    w.upload(spec.pos, spec.vel, spec.types)
    w.step(steps)
    return w


@pytest.mark.parametrize("case", ["thumbnail", "zoom_wrap", "offset_wrap", "3d", "empty"])
def test_render_matches_restatement(gpu, case):
    import splat_ref

    kw = {}
    if case == "3d":
        spec = blob_world(1500, 5, 0.05, nblobs=4, sigma=0.08, seed=31, dim=3, dt=0.02)
    else:
        spec = uniform_world(0 if case == "empty" else 2000, 6, 0.03, seed=30, dt=0.02)
    if case == "zoom_wrap":  # a camera over a corner: the copies across the edges show
        kw = dict(cam=(0.1, 0.9, 0.4, 0.3), top_left=(0.0, 0.0), size=0.03, wrap=True)
    elif case == "offset_wrap":  # camTopLeft shifts the world before the mod
        kw = dict(cam=(0.5, 0.5, 1.0, 1.0), top_left=(0.3, -0.2), size=0.02, wrap=True)
    else:
        kw = dict(cam=(0.5, 0.5, 1.0, 1.0), top_left=(0.0, 0.0), size=0.015, wrap=False)
    w = world_after(spec, 3) if spec.n else None
    if w is None:
        from plgpu.physics import GpuWorld

        w = GpuWorld(2, 16)
        w.set_settings(0.03, 0.85, 1.0, 0.02, wrap=True)
        w.set_matrix(spec.matrix)
        w.upload(np.zeros((0, 3)), np.zeros((0, 3)), np.zeros(0, np.int32))
    pal = palette(spec.matrix.shape[0] - 1)  # one colour short: the last type takes the last colour
    width, height = (96, 64) if case == "zoom_wrap" else (80, 80)
    img = w.render(width, height, pal, **kw)
    pos, _, types, _ = w.download()
    w.close()
    ref = splat_ref.splat(pos.astype(np.float32), types, pal, width, height, **kw)
    diff = np.argwhere(np.any(img != ref, axis=2))
    assert diff.size == 0, f"{len(diff)} pixels differ, first {diff[:5].tolist()}"
    if spec.n:
        assert (img[:, :, 3] > 0).mean() > 0.02  # something was drawn


def test_thumbnail_png_in_save(gpu, tmp_path):
    from plgpu import saves
    from plgpu.physics import ParticleLifeAccelerator, Physics

    ph = Physics(ParticleLifeAccelerator(), seed=33, initial_count=3000)
    ph.update()
    pal = palette(ph.settings.matrix.size())
    thumb = ph.thumbnail(pal)
    assert thumb.shape == (256, 256, 4)
    path = tmp_path / "s.zip"
    ph.save_state(path, palette=pal)
    import zipfile

    with zipfile.ZipFile(path) as z:
        png = z.read(saves.IMAGE)
    assert np.array_equal(saves.read_png_rgba(png), thumb)
