"""plg_upload / plg_download with page-locked host buffers (read and written
in place by the conversion kernels) against pageable buffers (staged through
device memory): the same particle state, bit for bit, in any mix."""
import numpy as np
import pytest

from worlds import uniform_world

pytestmark = pytest.mark.gpu


def _pinned(shape, dtype):
    import torch

    t = torch.empty(shape, dtype={np.float64: torch.float64, np.int32: torch.int32}[dtype], pin_memory=True)
    return t, t.numpy()


def _run(spec, pin_in, pin_out, steps=3):
    from plgpu import _lib
    from plgpu.physics import GpuWorld

    keep = []
    n = spec.n

    def arr(a, dtype, pin):
        if not pin:
            return np.ascontiguousarray(a, dtype=dtype)
        t, v = _pinned(a.shape, dtype)
        v[...] = a
        keep.append(t)
        return v

    w = GpuWorld(spec.dim, n)
    try:
        w.set_settings(spec.rmax, spec.friction, spec.force, spec.dt, beta=spec.beta, wrap=spec.wrap)
        w.set_matrix(spec.matrix)
        w.upload(arr(spec.pos, np.float64, pin_in[0]), arr(spec.vel, np.float64, pin_in[1]),
                 arr(spec.types, np.int32, pin_in[2]))
        w.step(steps)
        outs = []
        shapes = (((n, 3), np.float64), ((n, 3), np.float64), ((n,), np.int32), ((n,), np.int32))
        assert len(pin_out) == len(shapes)
        for (shape, dt), pin in zip(shapes, pin_out):
            if pin:
                t, v = _pinned(shape, dt)
                keep.append(t)
            else:
                v = np.empty(shape, dt)
            outs.append(v)
        P, I = _lib.C.c_double, _lib.C.c_int32
        rc = w.lib.plg_download(w.ctx, _lib.ptr(outs[0], P), _lib.ptr(outs[1], P), _lib.ptr(outs[2], I),
                                _lib.ptr(outs[3], I))
        assert rc == 0, w.lib.plg_last_error(w.ctx)
        return [o.copy() for o in outs]
    finally:
        w.close()


@pytest.mark.parametrize("dim", [2, 3])
def test_pinned_and_pageable_buffers_give_the_same_state(gpu, dim):
    spec = uniform_world(60_000, 5, 0.02 if dim == 2 else 0.05, seed=31, dim=dim, vel_scale=0.01)
    ref = _run(spec, (False, False, False), (False, False, False, False))
    for pin_in, pin_out in (((True, True, True), (True, True, True, True)),
                            ((True, False, True), (False, True, True, False)),
                            ((False, True, False), (True, False, False, True))):
        got = _run(spec, pin_in, pin_out)
        for a, b in zip(ref, got):
            assert np.array_equal(a, b)
