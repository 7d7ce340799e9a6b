"""plg_sort_cells_noalloc (cell sort over caller device buffers, static
scratch, no allocation) against the cell-sorted order of the context path.

The context path (plg_upload + plg_debug_step) reports, per slot of the
step's cell-sorted order, the particle id (= upload index) and its cell; the
no-allocation call must give the same order (perm) and the cell offsets those
cells imply, bit-exact, on two calls in a row.  This file sorts last so the
calls also run after every other GPU test has used the device.
"""
import ctypes as C

import numpy as np
import pytest

from worlds import blob_world, f32, run_gpu_debug, uniform_world

pytestmark = pytest.mark.gpu


def _noalloc(lib, dim, rmax, pos, n, ncells, status_word=True):
    import torch

    dev = torch.device("cuda:0")
    p = torch.from_numpy(np.ascontiguousarray(pos[:n])).to(dev) if n else None
    perm = torch.full((max(n, 1),), -1, dtype=torch.int32, device=dev)
    cstart = torch.full((ncells + 1,), -1, dtype=torch.int32, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev) if status_word else None
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.plg_sort_cells_noalloc(dim, rmax, n, C.c_void_p(p.data_ptr() if p is not None else 0),
                                    C.c_void_p(perm.data_ptr()), C.c_void_p(cstart.data_ptr()),
                                    C.c_void_p(status.data_ptr() if status is not None else 0), stream)
    torch.cuda.synchronize()
    st = int(status.item()) if status is not None else 0
    return rc, perm[:n].cpu().numpy().astype(np.int64), cstart.cpu().numpy().astype(np.int64), st


def _expected(spec):
    d, (_, _, _, ids) = run_gpu_debug(spec)
    nx = int(np.floor(1 / spec.rmax))
    ncells = nx ** spec.dim
    counts = np.bincount(d["cell"].astype(np.int64), minlength=ncells)
    return ids.astype(np.int64), np.concatenate([[0], np.cumsum(counts)]), ncells


def _check_twice(lib, spec):
    ids, cstart, ncells = _expected(spec)
    for _ in range(2):
        rc, perm, cs, st = _noalloc(lib, spec.dim, spec.rmax, spec.pos, spec.n, ncells)
        assert rc == 0, lib.plg_status_string(rc)
        assert st == 0
        assert np.array_equal(cs, cstart), "cell offsets differ from the context path"
        assert np.array_equal(perm, ids), "sorted order differs from the context path"


def test_noalloc_2d_matches_context_order(lib, gpu):
    rmax = 0.0031  # 1/rmax not an integer: sliver beyond the last full cell
    spec = uniform_world(200_000, 4, rmax, seed=21, wrap=False)  # clamp mode allows x == 1
    spec.pos[:300, 0] = 1.0
    spec.pos[300:600, 1] = 0.0
    spec.pos[600:900, :2] = 1.0
    spec.pos[900:1200, :2] = f32(np.full((300, 2), 0.5))  # one crowded cell
    _check_twice(lib, spec)


def test_noalloc_3d_matches_context_order(lib, gpu):
    _check_twice(lib, blob_world(150_000, 8, 0.02, seed=22))


def test_noalloc_limits_and_bad_pointers(lib, gpu):
    from plgpu import _lib

    spec = uniform_world(1000, 3, 0.05, seed=23)
    too_many = _lib.PLG_NOALLOC_MAX_PARTICLES + 1
    assert lib.plg_sort_cells_noalloc(2, 0.05, too_many, None, None, None, None, None) == _lib.PLG_E_CAPACITY
    # rmax = 0.001: 1000^2 cells > the scratch's cell capacity.
    assert lib.plg_sort_cells_noalloc(2, 0.001, 10, None, None, None, None, None) == _lib.PLG_E_CAPACITY
    assert lib.plg_sort_cells_noalloc(3, 0.01, 10, None, None, None, None, None) == _lib.PLG_E_CAPACITY
    assert lib.plg_sort_cells_noalloc(4, 0.05, 10, None, None, None, None, None) == _lib.PLG_E_INVALID_ARG
    assert lib.plg_sort_cells_noalloc(2, 0.0, 10, None, None, None, None, None) == _lib.PLG_E_INVALID_ARG
    host_pos = np.ascontiguousarray(spec.pos)
    host_out = np.zeros(1000, np.uint32)
    host_cs = np.zeros(401, np.uint32)
    assert lib.plg_sort_cells_noalloc(2, 0.05, 1000, C.c_void_p(host_pos.ctypes.data),
                                      C.c_void_p(host_out.ctypes.data), C.c_void_p(host_cs.ctypes.data),
                                      None, None) == _lib.PLG_E_INVALID_ARG
    # Still usable after the rejections; empty input gives all-zero offsets.
    rc, perm, cs, st = _noalloc(lib, 2, 0.05, spec.pos, 0, 400)
    assert rc == 0 and st == 0 and perm.size == 0 and not cs.any()
    _check_twice(lib, spec)


def test_noalloc_flags_positions_outside_the_box(lib, gpu):
    spec = uniform_world(5000, 3, 0.05, seed=24)
    pos = spec.pos.copy()
    pos[7, 0] = 1.5
    pos[8, 1] = -0.25
    pos[9, 0] = np.nan
    rc, perm, cs, st = _noalloc(lib, 2, 0.05, pos, spec.n, 400)
    assert rc == 0
    assert st & 1
    assert np.array_equal(np.sort(perm), np.arange(spec.n)) and cs[-1] == spec.n
