"""ctypes wrapper and build recipe of the oracle (plg_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline / reference arm, as the checker.  The product path
(libplgpu.so) never uses it.

Parity status: unpinned (see plg_oracle.c) — cross-checked against the
pure-Python restatement in tests/golden/make_golden.py and hand-derived
known answers.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

ORACLE_DIR = Path(__file__).resolve().parent
SRC = ORACLE_DIR / "plg_oracle.c"
LIB = ORACLE_DIR / "liborc.so"

# IEEE double without contraction: gcc contracts a*b+c into FMA by default on
# aarch64, which would change the reference's rounding.
CFLAGS = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread", "-std=c11"]


def build(force: bool = False) -> Path:
    if force or not LIB.exists() or LIB.stat().st_mtime < SRC.stat().st_mtime:
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [os.environ.get("CC", "gcc")] + CFLAGS + [str(SRC), "-o", str(tmp), "-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


class _Settings(C.Structure):
    _fields_ = [
        ("rmax", C.c_double),
        ("friction", C.c_double),
        ("force", C.c_double),
        ("dt", C.c_double),
        ("beta", C.c_double),
        ("wrap", C.c_int32),
        ("pad", C.c_int32),
    ]


class _Debug(C.Structure):
    _fields_ = [
        ("cell", C.POINTER(C.c_int32)),
        ("pairs", C.POINTER(C.c_int32)),
        ("hsum", C.POINTER(C.c_uint64)),
        ("hxor", C.POINTER(C.c_uint64)),
        ("acc", C.POINTER(C.c_double)),
        ("fscale", C.POINTER(C.c_double)),
        ("candidates", C.c_int64),
    ]


_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        lib = C.CDLL(str(build()))
        D = C.POINTER(C.c_double)
        I = C.POINTER(C.c_int32)
        lib.orc_step.restype = C.c_int
        lib.orc_step.argtypes = [C.c_int, C.c_int64, D, D, I, I, C.c_int32, D, C.POINTER(_Settings), C.c_int32,
                                 C.POINTER(_Debug)]
        lib.orc_run.restype = C.c_double
        lib.orc_run.argtypes = [C.c_int, C.c_int64, D, D, I, I, C.c_int32, D, C.POINTER(_Settings), C.c_int32,
                                C.c_int32]
        lib.orc_accel_scalar.restype = C.c_double
        lib.orc_accel_scalar.argtypes = [C.c_double, C.c_double, C.c_double]
        lib.orc_grid_n.restype = C.c_int32
        lib.orc_grid_n.argtypes = [C.c_double]
        lib.orc_container_index.restype = C.c_int32
        lib.orc_container_index.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_double]
        for nm in ("orc_range_wrap", "orc_range_wrap_connection", "orc_range_clamp"):
            getattr(lib, nm).restype = C.c_double
            getattr(lib, nm).argtypes = [C.c_double]
        lib.orc_mix64.restype = C.c_uint64
        lib.orc_mix64.argtypes = [C.c_uint64]
        _lib = lib
    return _lib


def settings(rmax, friction, force, dt, beta=0.3, wrap=True) -> _Settings:
    return _Settings(rmax, friction, force, dt, beta, 1 if wrap else 0, 0)


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


class World:
    """Host state for the oracle: double positions/velocities (n, 3), int32
    types and ids.  ``step`` permutes the arrays like Physics.update()."""

    def __init__(self, dim, pos, vel, types, ids, matrix, st: _Settings):
        self.dim = dim
        self.pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3).copy()
        self.vel = np.ascontiguousarray(vel, np.float64).reshape(-1, 3).copy()
        self.types = np.ascontiguousarray(types, np.int32).copy()
        self.ids = np.ascontiguousarray(ids, np.int32).copy()
        self.matrix = np.ascontiguousarray(matrix, np.float64)
        self.st = st

    @property
    def n(self) -> int:
        return self.pos.shape[0]

    def step(self, threads: int = 1, debug: bool = False):
        lib = load()
        n = self.n
        dbg = None
        out = None
        if debug:
            out = dict(
                cell=np.zeros(n, np.int32),
                pairs=np.zeros(n, np.int32),
                hsum=np.zeros(n, np.uint64),
                hxor=np.zeros(n, np.uint64),
                acc=np.zeros((n, self.dim), np.float64),
                fscale=np.zeros(n, np.float64),
            )
            dbg = _Debug(
                _p(out["cell"], C.c_int32),
                _p(out["pairs"], C.c_int32),
                _p(out["hsum"], C.c_uint64),
                _p(out["hxor"], C.c_uint64),
                _p(out["acc"], C.c_double),
                _p(out["fscale"], C.c_double),
                0,
            )
        rc = lib.orc_step(self.dim, n, _p(self.pos, C.c_double), _p(self.vel, C.c_double), _p(self.types, C.c_int32),
                          _p(self.ids, C.c_int32), self.matrix.shape[0], _p(self.matrix, C.c_double),
                          C.byref(self.st), threads, C.byref(dbg) if dbg is not None else None)
        if rc != 0:
            raise RuntimeError("orc_step failed")
        if debug:
            out["candidates"] = dbg.candidates
        return out

    def run(self, steps: int, threads: int) -> float:
        lib = load()
        return lib.orc_run(self.dim, self.n, _p(self.pos, C.c_double), _p(self.vel, C.c_double),
                           _p(self.types, C.c_int32), _p(self.ids, C.c_int32), self.matrix.shape[0],
                           _p(self.matrix, C.c_double), C.byref(self.st), threads, steps)


def accel(a: float, beta: float, dist: float) -> float:
    return load().orc_accel_scalar(a, beta, dist)


def grid_n(rmax: float) -> int:
    return load().orc_grid_n(rmax)


def container_index(dim, x, y, z, rmax) -> int:
    return load().orc_container_index(dim, x, y, z, rmax)


def wrap(v: float) -> float:
    return load().orc_range_wrap(v)


def wrap_connection(v: float) -> float:
    return load().orc_range_wrap_connection(v)


def clamp(v: float) -> float:
    return load().orc_range_clamp(v)


def mix64(i: int) -> int:
    return load().orc_mix64(i)
