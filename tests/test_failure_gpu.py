"""Failure detection without a GPU fault: a bounded device wait that runs out
reports through the error word and leaves the context usable; the host-side
waits (plg_sync with a timeout) and the stop flag end calls cleanly."""
import numpy as np
import pytest

from worlds import uniform_world

pytestmark = pytest.mark.gpu

K_DEV_SPIN_LIMIT = 1 << 3


def _world(spec):
    from plgpu.physics import GpuWorld

    w = GpuWorld(spec.dim, spec.n)
    w.set_settings(spec.rmax, spec.friction, spec.force, spec.dt, beta=spec.beta, wrap=spec.wrap)
    w.set_matrix(spec.matrix)
    w.upload(spec.pos, spec.vel, spec.types)
    return w


def test_scan_wait_runs_out_and_the_context_stays_usable(gpu):
    from plgpu import _lib

    lib = _lib.load()
    status = _lib.C.c_uint32(0)
    secs = _lib.C.c_double(0.0)
    assert lib.plg_test_scan_wait(_lib.C.byref(status), _lib.C.byref(secs)) == 0
    assert status.value & K_DEV_SPIN_LIMIT
    assert 0.0 < secs.value < 30.0
    # the device still steps a world exactly like a fresh context
    spec = uniform_world(20_000, 5, 0.01, seed=71, vel_scale=0.01)
    a, b = _world(spec), _world(spec)
    try:
        a.step(2)
        b.step(2)
        for x, y in zip(a.download(), b.download()):
            assert np.array_equal(x, y)
    finally:
        a.close()
        b.close()


def test_async_steps_and_bounded_sync(gpu):
    from plgpu import _lib

    spec = uniform_world(200_000, 6, 0.004, seed=72, vel_scale=0.01)
    a, b = _world(spec), _world(spec)
    try:
        assert a.lib.plg_step_async(a.ctx, 20) == 0
        rc = a.lib.plg_sync(a.ctx, 1e-6)  # may or may not be done: either answer is clean
        assert rc in (0, _lib.PLG_E_TIMEOUT)
        assert a.lib.plg_sync(a.ctx, 60.0) == 0
        b.step(20)
        for x, y in zip(a.download(), b.download()):
            assert np.array_equal(x, y)
    finally:
        a.close()
        b.close()


def test_stop_flag_ends_a_multi_step_call_before_its_next_step(gpu):
    from plgpu import _lib

    spec = uniform_world(20_000, 5, 0.01, seed=73, vel_scale=0.01)
    w = _world(spec)
    try:
        before = w.download()
        assert w.lib.plg_request_stop(w.ctx) == 0
        assert w.lib.plg_step(w.ctx, 5) == _lib.PLG_E_STOPPED
        for x, y in zip(before, w.download()):
            assert np.array_equal(x, y)
        # the flag was cleared: the next call runs
        assert w.lib.plg_step(w.ctx, 1) == 0
    finally:
        w.close()
