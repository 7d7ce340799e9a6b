"""plg_step_download: a step whose force kernel also writes the snapshot
(page-locked or pageable host arrays written in place) against plg_step
followed by plg_download: the same particle state, bit for bit, for every
array subset, both dimensions, worlds whose particle count is not a multiple
of a warp or a tile, deferred FP64 targets and the small-grid path (which
never fuses).  The call keeps plg_step's errors and stop behaviour: a
stopped call writes nothing."""
import numpy as np
import pytest

from worlds import blob_world, uniform_world

pytestmark = pytest.mark.gpu

SHAPES = (((3,), np.float64), ((3,), np.float64), ((), np.int32), ((), np.int32))


def _pinned(shape, dtype):
    import torch

    t = torch.empty(shape, dtype={np.float64: torch.float64, np.int32: torch.int32}[dtype], pin_memory=True)
    return t, t.numpy()


def _world(spec):
    from plgpu.physics import GpuWorld

    w = GpuWorld(spec.dim, spec.n)
    w.set_settings(spec.rmax, spec.friction, spec.force, spec.dt, beta=spec.beta, wrap=spec.wrap)
    w.set_matrix(spec.matrix)
    w.upload(spec.pos, spec.vel, spec.types)
    return w


def _outputs(n, kinds, keep):
    """kinds: per array 'pinned', 'pageable' or None (not requested)."""
    outs = []
    for (tail, dt), kind in zip(SHAPES, kinds):
        shape = (n,) + tail
        if kind is None:
            outs.append(None)
        elif kind == "pinned":
            t, v = _pinned(shape, dt)
            v.fill(-7)  # the CPU touches every page before the device writes it
            keep.append(t)
            outs.append(v)
        else:
            outs.append(np.full(shape, -7, dt))
    return tuple(outs)


def _fuses(w, outs):
    from plgpu import _lib

    f = _lib.C.c_int32(-1)
    P, I = _lib.C.c_double, _lib.C.c_int32
    rc = w.lib.plg_step_download_fuses(w.ctx, _lib.ptr(outs[0], P), _lib.ptr(outs[1], P), _lib.ptr(outs[2], I),
                                       _lib.ptr(outs[3], I), _lib.C.byref(f))
    assert rc == 0
    return f.value


def spec_for(case):
    if case == "2d_uniform":
        return uniform_world(100_003, 6, 0.004, seed=51, vel_scale=0.01)
    if case == "2d_coincident":
        spec = uniform_world(5001, 4, 0.02, seed=52)
        spec.pos[100:140] = spec.pos[99]
        return spec
    if case == "2d_clamp_tiny":
        return uniform_world(37, 3, 0.05, seed=53, vel_scale=0.05, wrap=False)
    if case == "2d_small_grid":
        return uniform_world(3001, 4, 0.4, seed=54, vel_scale=0.01)  # nx = 2: the literal path
    if case == "3d_blobs":
        return blob_world(60_001, 8, 0.02, seed=55, dt=0.01)
    raise KeyError(case)


@pytest.mark.parametrize("case", ["2d_uniform", "2d_coincident", "2d_clamp_tiny", "2d_small_grid", "3d_blobs"])
@pytest.mark.parametrize("nsteps", [1, 3])
def test_step_download_equals_step_then_download(gpu, case, nsteps):
    spec = spec_for(case)
    a, b = _world(spec), _world(spec)
    keep = []
    try:
        a.step(nsteps)
        ref = a.download()
        outs = _outputs(spec.n, ("pinned",) * 4, keep)
        fused = _fuses(b, outs)
        assert fused == (0 if case == "2d_small_grid" else 1)
        got = b.step_download(nsteps, out=outs)
        for x, y in zip(ref, got):
            assert np.array_equal(x, y)
        # the context holds the same state afterwards
        for x, y in zip(ref, b.download()):
            assert np.array_equal(x, y)
    finally:
        a.close()
        b.close()


@pytest.mark.parametrize("kinds", [
    ("pageable",) * 4,
    ("pinned", "pageable", "pinned", "pageable"),
    ("pinned", None, None, "pinned"),
    (None, "pinned", "pinned", None),
    ("pageable", None, None, None),
])
def test_step_download_subsets_and_memory_kinds(gpu, kinds):
    spec = uniform_world(20_011, 5, 0.01, seed=56, vel_scale=0.02)
    a, b = _world(spec), _world(spec)
    keep = []
    try:
        a.step(2)
        ref = a.download()
        outs = _outputs(spec.n, kinds, keep)
        got = b.step_download(2, out=outs)
        for x, y, kind in zip(ref, got, kinds):
            if kind is None:
                assert y is None
            else:
                assert np.array_equal(x, y)
    finally:
        a.close()
        b.close()


def test_step_download_repeated_calls_follow_plain_steps(gpu):
    """Fused and plain steps interleave (the graph of the plain step is not
    disturbed by the plain launches of the fused one)."""
    spec = blob_world(40_000, 6, 0.01, nblobs=6, sigma=0.01, seed=57, dim=2)
    a, b = _world(spec), _world(spec)
    keep = []
    try:
        outs = _outputs(spec.n, ("pinned",) * 4, keep)
        for k in range(4):
            a.step(1 + k % 2)
            ref = a.download()
            got = b.step_download(1 + k % 2, out=outs)
            for x, y in zip(ref, got):
                assert np.array_equal(x, y)
        a.step(2)
        b.step(2)
        for x, y in zip(a.download(), b.download()):
            assert np.array_equal(x, y)
    finally:
        a.close()
        b.close()


def test_step_download_errors_and_stop(gpu):
    from plgpu import _lib
    from plgpu.physics import GpuWorld

    spec = uniform_world(5000, 4, 0.02, seed=58)
    keep = []
    outs = _outputs(spec.n, ("pinned",) * 4, keep)
    P, I = _lib.C.c_double, _lib.C.c_int32
    args = tuple(_lib.ptr(o, t) for o, t in zip(outs, (P, P, I, I)))
    w = GpuWorld(spec.dim, spec.n)
    try:
        assert w.lib.plg_step_download(w.ctx, 1, *args) == _lib.PLG_E_STATE  # before settings
        w.set_settings(spec.rmax, spec.friction, spec.force, spec.dt, beta=spec.beta, wrap=spec.wrap)
        w.set_matrix(spec.matrix)
        assert w.lib.plg_step_download(w.ctx, 1, *args) == _lib.PLG_E_STATE  # before an upload
        w.upload(spec.pos, spec.vel, spec.types)
        assert w.lib.plg_step_download(w.ctx, -1, *args) == _lib.PLG_E_INVALID_ARG
        before = w.download()
        # a requested stop ends the call before its first step: nothing written
        for nsteps in (1, 3):
            assert w.lib.plg_request_stop(w.ctx) == 0
            assert w.lib.plg_step_download(w.ctx, nsteps, *args) == _lib.PLG_E_STOPPED
            assert (outs[0] == -7).all() and (outs[3] == -7).all()
            for x, y in zip(before, w.download()):
                assert np.array_equal(x, y)
        # zero steps: a download
        assert w.lib.plg_step_download(w.ctx, 0, *args) == 0
        for x, y in zip(before, outs):
            assert np.array_equal(x, y)
    finally:
        w.close()


@pytest.mark.parametrize("dim", [2, 3])
def test_host_mirror_sync_policies_agree(gpu, dim):
    """Physics.update() with sync_policy 'every' (plg_step_download each
    update) and 'manual' (plain steps, one read-back at the end) leave the
    same host arrays, ids included."""
    from plgpu import ParticleLifeAccelerator, Physics

    runs = []
    for policy in ("every", "manual"):
        p = Physics(ParticleLifeAccelerator(), dim=dim, seed=11, initial_count=30_000, sync_policy=policy)
        p.settings.rmax = 0.02 if dim == 2 else 0.05
        for _ in range(4):
            p.update()
        p.sync_host()
        runs.append((p.positions.copy(), p.velocities.copy(), p.types.copy(), p.ids.copy()))
        p.close()
    for a, b in zip(*runs):
        assert np.array_equal(a, b)
