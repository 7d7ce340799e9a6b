"""The C-ABI library without a GPU: it loads, exports every symbol that
include/*.h declares, and its host-only functions behave (no compute calls)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from plgpu import _lib

REPO = Path(__file__).resolve().parent.parent


def declared_symbols():
    names = set()
    for h in (REPO / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(plg_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_every_declared_symbol_is_exported(lib):
    names = declared_symbols()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    assert set(declared_symbols()) <= set(_lib.SIGNATURES), set(declared_symbols()) - set(_lib.SIGNATURES)


def test_version_and_status_strings(lib):
    assert b"sm_103a" in lib.plg_version()
    assert lib.plg_status_string(0) == b"ok"
    assert lib.plg_status_string(_lib.PLG_E_UNSUPPORTED) == b"unsupported"
    assert lib.plg_status_string(999) == b"unknown status"
    assert [lib.plg_kernel_name(k).decode() for k in range(len(_lib.KERNELS))] == _lib.KERNELS
    assert lib.plg_kernel_name(3) == b"force"
    assert lib.plg_kernel_name(99) == b""


def settings(**kw):
    d = dict(rmax=0.02, friction=0.85, force=1.0, dt=0.02, beta=0.3, wrap=1, accel_kind=_lib.PLG_ACCEL_PARTICLE_LIFE)
    d.update(kw)
    return _lib.plg_settings(**d)


@pytest.mark.parametrize(
    "kw,dim,expect",
    [
        ({}, 2, 0),
        ({}, 3, 0),
        ({}, 4, _lib.PLG_E_INVALID_ARG),
        ({"accel_kind": 7}, 2, _lib.PLG_E_UNSUPPORTED),
        ({"rmax": 0.0}, 2, _lib.PLG_E_INVALID_ARG),
        ({"rmax": 1.5}, 2, _lib.PLG_E_INVALID_ARG),
        ({"rmax": float("nan")}, 2, _lib.PLG_E_INVALID_ARG),
        ({"rmax": 1e-6}, 3, _lib.PLG_E_INVALID_ARG),  # too many cells
        ({"beta": 1.0}, 2, _lib.PLG_E_INVALID_ARG),
        ({"beta": 0.0}, 2, _lib.PLG_E_INVALID_ARG),
        ({"friction": -0.1}, 2, _lib.PLG_E_INVALID_ARG),
        ({"dt": float("inf")}, 2, _lib.PLG_E_INVALID_ARG),
        ({"wrap": 2}, 2, _lib.PLG_E_INVALID_ARG),
        ({"rmax": 1.0}, 2, 0),
    ],
)
def test_validate_settings(lib, kw, dim, expect):
    s = settings(**kw)
    assert lib.plg_validate_settings(dim, C.byref(s)) == expect


def cell_bounds(lib, rmax):
    nx = C.c_int32()
    assert lib.plg_cell_bounds(rmax, C.byref(nx), None, 0) == 0
    b = np.zeros(nx.value + 1, np.float32)
    assert lib.plg_cell_bounds(rmax, None, _lib.ptr(b, C.c_float), b.size) == 0
    return nx.value, b


def device_rule(x32, b, nx):
    """The device's table lookup: #(k >= 1 with x >= b[k]), clamped."""
    c = np.searchsorted(b[1:], x32, side="right")
    return np.minimum(c, nx - 1), c


@pytest.mark.parametrize("rmax", [0.02, 0.0025, 0.0031, 0.3, 0.1, 1.0 / 3.0, 2.0 ** -6, 0.00474, 0.4, 0.7])
def test_cell_table_matches_fp64_division(lib, rmax):
    """(int)((double)x / rmax) (backend/Physics.java:363) for FP32 x equals
    the table rule, on random floats and on every boundary float and its
    neighbours."""
    nx, b = cell_bounds(lib, rmax)
    assert nx == int(np.floor(1 / rmax))
    assert b[0] == 0 and np.all(np.diff(b) > 0)
    rng = np.random.default_rng(1)
    xs = [rng.random(200_000).astype(np.float32), b[1:]]
    xs.append(np.nextafter(b[1:], np.float32(-1)))
    xs.append(np.nextafter(b[1:], np.float32(2)))
    xs.append(np.array([0.0, 1.0, np.nextafter(np.float32(1), np.float32(0))], np.float32))
    x32 = np.concatenate(xs)
    x32 = x32[(x32 >= 0) & (x32 <= 1)]
    ref = np.trunc(x32.astype(np.float64) / rmax).astype(np.int64)
    got_clamped, got = device_rule(x32, b, nx)
    assert np.array_equal(got, ref)
    assert np.array_equal(got_clamped, np.minimum(ref, nx - 1))


def test_cell_bounds_rejects_bad_input(lib):
    assert lib.plg_cell_bounds(0.0, None, None, 0) == _lib.PLG_E_INVALID_ARG
    b = np.zeros(3, np.float32)
    assert lib.plg_cell_bounds(0.02, None, _lib.ptr(b, C.c_float), 3) == _lib.PLG_E_INVALID_ARG


def test_null_context_calls_fail_cleanly(lib):
    assert lib.plg_destroy(None) == _lib.PLG_E_INVALID_ARG
    assert lib.plg_step(None, 1) == _lib.PLG_E_INVALID_ARG
    assert lib.plg_request_stop(None) == _lib.PLG_E_INVALID_ARG
    assert lib.plg_last_error(None) == b"null context"
    assert lib.plg_step_download(None, 1, None, None, None, None) == _lib.PLG_E_INVALID_ARG
    f = C.c_int32(-1)
    assert lib.plg_step_download_fuses(None, None, None, None, None, C.byref(f)) == _lib.PLG_E_INVALID_ARG
    assert lib.plg_set_tile(None, 0) == _lib.PLG_E_INVALID_ARG
    assert lib.plg_get_tile(None, C.byref(f)) == _lib.PLG_E_INVALID_ARG
    assert lib.plg_autotune(None, 2, C.byref(f), None) == _lib.PLG_E_INVALID_ARG
    out = C.c_void_p()
    assert lib.plg_create(5, 10, C.byref(out)) == _lib.PLG_E_INVALID_ARG
    assert lib.plg_create(2, 0, C.byref(out)) == _lib.PLG_E_INVALID_ARG
