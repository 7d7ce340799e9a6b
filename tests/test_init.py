"""Initialiser catalogues: the Philox restatement against numpy's Philox
(an independent implementation), the host matrix generators against it, and
(GPU) the device setters against it."""
import numpy as np
import pytest

import init_ref


def test_philox_restatement_matches_numpy():
    # numpy's Philox generates block `counter + 1` first.
    for key, ctr in (([12345, 678], [0, 0, 0, 0]), ([2**64 - 1, 5], [7, 1, 3, 9])):
        bg = np.random.Philox(key=np.array(key, np.uint64), counter=np.array(ctr, np.uint64))
        raw = [int(x) for x in bg.random_raw(4)]
        nxt = list(ctr)
        nxt[0] += 1
        assert raw == init_ref.philox4x64(nxt, key)


@pytest.mark.parametrize("kind", range(7))
def test_matrix_generators(lib, kind):
    from plgpu import _lib

    for size in (1, 2, 5, 9):
        out = np.zeros((size, size))
        assert lib.plg_generate_matrix(kind, size, 2024, _lib.ptr(out, _lib.C.c_double)) == 0
        assert np.array_equal(out, init_ref.matrix(kind, size, 2024))
    assert lib.plg_generate_matrix(7, 3, 0, _lib.ptr(np.zeros(9), _lib.C.c_double)) == _lib.PLG_E_INVALID_ARG


@pytest.mark.gpu
@pytest.mark.parametrize("dim", [2, 3])
def test_device_setters_match_the_restatement(gpu, dim):
    from plgpu.physics import GpuWorld

    n, ntypes, seed = 3_000, 6, 77
    w = GpuWorld(dim, n)
    w.set_settings(0.05, 0.8, 1.0, 0.02, wrap=True)
    m = np.zeros((ntypes, ntypes))
    w.set_matrix(m)
    for ps in range(11):
        for ts in (0, 2, 3, 4, 5, 6):
            w.generate(n, ps, ts, seed)
            pos, vel, types, ids = w.download()
            assert np.array_equal(ids, np.arange(n)) and not vel.any()
            for i in range(0, n, 37):
                t = init_ref.type_of(ts, seed, i, (0.0, 0.0, 0.0), (0.0, 0.0, 0.0), 0, ntypes)
                assert types[i] == t, (ps, ts, i)
                x, y = init_ref.position(ps, seed, i, t, ntypes)
                exp = np.float32([init_ref.ensure(x, True), init_ref.ensure(y, True)])
                assert np.allclose(pos[i, :2], exp, rtol=0, atol=2e-7), (ps, i, pos[i], exp)
    # type setters applied to the current state (Physics.setTypes)
    w.generate(n, 1, 0, seed)
    w.step(3)
    pos0, vel0, types0, _ = w.download()
    for ts in range(8):
        w.apply_type_setter(ts, seed + ts)
        pos1, vel1, types1, _ = w.download()
        for i in range(0, n, 29):
            assert types1[i] == init_ref.type_of(ts, seed + ts, i, pos1[i], vel1[i], types0[i], ntypes), (ts, i)
        types0 = types1
    w.close()
