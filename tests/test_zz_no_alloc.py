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


def _java_order(pos, dim, rmax):
    """The reference's binning restated on the CPU in FP64: per axis
    (int)(x / containerSize) with the quotient correctly rounded, cx == nx
    clamped to nx - 1 (backend/Physics.java:362-375), then a stable counting
    sort by cell (the sequential fill of Physics.java:342-348).  Positions
    outside [0, 1] or NaN are clamped as the library clamps them (to 1 above
    the box, 0 below or NaN)."""
    nx = int(np.floor(1 / rmax))
    x = np.nan_to_num(pos[:, :dim], nan=0.0)
    x = np.where(x > 1.0, 1.0, np.where(x < 0.0, 0.0, x))
    c = np.minimum((x / rmax).astype(np.int64), nx - 1)
    cell = c[:, 0] + (c[:, 1] * nx if dim > 1 else 0) + (c[:, 2] * nx * nx if dim > 2 else 0)
    order = np.argsort(cell, kind="stable")
    counts = np.bincount(cell, minlength=nx ** dim)
    return order, np.concatenate([[0], np.cumsum(counts)]), nx ** dim


def test_noalloc_fp64_cell_boundaries_against_the_java_rule(lib, gpu):
    """Double positions one ulp either side of k * rmax (not float32-exact:
    the FP64 quotient decides their cell), the last partial cell and the box
    edges, against the CPU restatement of getContainerIndex."""
    rmax = 0.0031
    nx = int(np.floor(1 / rmax))
    rng = np.random.default_rng(25)
    ks = rng.integers(1, nx + 1, 20_000).astype(np.float64)
    edge = ks * rmax
    xs = np.concatenate([np.nextafter(edge, -np.inf), edge, np.nextafter(edge, np.inf), [0.0, 1.0, nx * rmax]])
    xs = xs[(xs >= 0) & (xs <= 1)]
    pos = np.zeros((len(xs), 3))
    pos[:, 0] = xs
    pos[:, 1] = rng.permutation(np.concatenate([xs[: len(xs) // 2], rng.random(len(xs) - len(xs) // 2)]))
    order, cstart, ncells = _java_order(pos, 2, rmax)
    for _ in range(2):
        rc, perm, cs, st = _noalloc(lib, 2, rmax, pos, len(pos), ncells)
        assert rc == 0 and st == 0
        assert np.array_equal(cs, cstart) and np.array_equal(perm, order)


def test_noalloc_one_crowded_cell(lib, gpu):
    """100,000 particles on one point (a corner) among 31,072 others: the
    crowded cell's members keep index order like every other cell.  The
    ordering work of a cell grows with the square of its population, shared
    by the lanes of a warp; this case takes about a millisecond."""
    import time

    rng = np.random.default_rng(26)
    n = 131_072
    pos = np.zeros((n, 3))
    pos[:, :2] = rng.random((n, 2))
    crowd = rng.choice(n, 100_000, replace=False)
    pos[crowd, :2] = 0.0
    rmax = 0.01
    order, cstart, ncells = _java_order(pos, 2, rmax)
    _noalloc(lib, 2, rmax, pos, n, ncells)  # warm
    t0 = time.perf_counter()
    rc, perm, cs, st = _noalloc(lib, 2, rmax, pos, n, ncells)
    dt = time.perf_counter() - t0
    print(f"crowded cell of 100,000: {1e3 * dt:.2f} ms (call, copies and synchronisation included)")
    assert rc == 0 and st == 0
    assert np.array_equal(cs, cstart) and np.array_equal(perm, order)
    assert dt < 1.0
