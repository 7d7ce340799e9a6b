"""Host-side mirror of the reference's physics API over the GPU C ABI.

Same names, argument meanings and error behaviour as the Java backend of
tom-mohr/particle-life-app (paths relative to
src/main/java/com/particle_life/backend/):

  PhysicsSettings  PhysicsSettings.java:8-72
  Matrix           Matrix.java:3-8, DefaultMatrix.java:3-69
  Accelerator      Accelerator.java:16 (+ the default lambda, app/Main.java:275-280)
  PositionSetter / TypeSetter / MatrixGenerator   PositionSetter.java:6,
                   TypeSetter.java:14, MatrixGenerator.java:9 and their
                   Default* implementations
  Physics          Physics.java:9-512

Particles are held as arrays (the structure-of-arrays view of
``Particle[]``): ``positions`` and ``velocities`` are float64 (n, 3), ``types``
int32 (n,), ``ids`` int32 (n,).  ``update()`` runs the step on the GPU: the
host state is uploaded when a mutator touched it, one step runs, and the new
state (in the new cell-sorted order, as ``Physics.particles`` is permuted by
every update) is read back according to ``sync_policy``.

Only :class:`ParticleLifeAccelerator` has a device implementation; any other
accelerator makes ``update()`` raise (no CPU fallback).
"""
from __future__ import annotations

import copy
import math
from dataclasses import dataclass, field
from typing import Callable, Optional, Protocol

import numpy as np

from . import _lib


# ---------------------------------------------------------------- matrix --


class Matrix(Protocol):
    """backend/Matrix.java:3-8."""

    def size(self) -> int: ...

    def get(self, i: int, j: int) -> float: ...

    def set(self, i: int, j: int, value: float) -> None: ...

    def deep_copy(self) -> "Matrix": ...


class DefaultMatrix:
    """backend/DefaultMatrix.java: n x n doubles, zero-initialised."""

    def __init__(self, size: int):
        self.values = np.zeros((size, size), dtype=np.float64)

    @property
    def size_(self) -> int:
        return self.values.shape[0]

    def size(self) -> int:
        return self.values.shape[0]

    def zero(self) -> None:
        self.values[:] = 0.0

    def randomize(self, rng: np.random.Generator) -> None:
        """values[i][j] = 2 * random() - 1 (DefaultMatrix.java:25-31), seeded."""
        self.values[:] = 2.0 * rng.random(self.values.shape) - 1.0

    def get(self, i: int, j: int) -> float:
        return float(self.values[i, j])

    def set(self, i: int, j: int, value: float) -> None:
        self.values[i, j] = value

    def deep_copy(self) -> "DefaultMatrix":
        m = DefaultMatrix(self.size())
        m.values[:] = self.values
        return m

    def __eq__(self, other) -> bool:
        if not hasattr(other, "size") or other.size() != self.size():
            return False
        n = self.size()
        return all(other.get(i, j) == self.get(i, j) for i in range(n) for j in range(n))

    def as_array(self) -> np.ndarray:
        return np.ascontiguousarray(self.values, dtype=np.float64)


def matrix_to_array(m) -> np.ndarray:
    if isinstance(m, DefaultMatrix):
        return m.as_array()
    n = m.size()
    return np.array([[m.get(i, j) for j in range(n)] for i in range(n)], dtype=np.float64)


# -------------------------------------------------------------- settings --

# `public double dt = 0.02f;` (PhysicsSettings.java:37): a float literal.
DEFAULT_DT = float(np.float32(0.02))


@dataclass
class PhysicsSettings:
    """backend/PhysicsSettings.java:8-38."""

    wrap: bool = True
    rmax: float = 0.02
    friction: float = 0.85
    force: float = 1.0
    dt: float = DEFAULT_DT
    matrix: object = field(default_factory=lambda: DefaultMatrix(6))

    def deep_copy(self) -> "PhysicsSettings":
        return PhysicsSettings(self.wrap, self.rmax, self.friction, self.force, self.dt, self.matrix.deep_copy())

    def __eq__(self, o) -> bool:
        if not isinstance(o, PhysicsSettings):
            return False
        return (
            o.wrap == self.wrap
            and o.rmax == self.rmax
            and o.friction == self.friction
            and o.force == self.force
            and o.dt == self.dt
            and o.matrix == self.matrix
        )


# ----------------------------------------------------------- accelerator --


class Accelerator(Protocol):
    """backend/Accelerator.java:16: acceleration for matrix entry a and r/rmax."""

    def accelerate(self, a: float, pos: np.ndarray) -> np.ndarray: ...


@dataclass(frozen=True)
class ParticleLifeAccelerator:
    """The default lambda of app/Main.java:275-280, with beta as a parameter.

    ``accelerate`` evaluates it on the host for callers that want the value;
    the GPU step uses the same formula in its force kernel.
    """

    beta: float = 0.3

    def accelerate(self, a: float, pos: np.ndarray) -> np.ndarray:
        pos = np.asarray(pos, dtype=np.float64)
        dist = math.sqrt(pos[0] * pos[0] + (pos[1] * pos[1] + pos[2] * pos[2]))
        beta = self.beta
        f = (dist / beta - 1) if dist < beta else a * (1 - abs(1 + beta - 2 * dist) / (1 - beta))
        return pos * (f / dist)


# ---------------------------------------------------- setters / generator --


class PositionSetter(Protocol):
    def set(self, position: np.ndarray, type_: int, n_types: int) -> None: ...


class TypeSetter(Protocol):
    def get_type(self, position: np.ndarray, velocity: np.ndarray, type_: int, n_types: int) -> int: ...


class MatrixGenerator(Protocol):
    def make_matrix(self, size: int): ...


class DefaultPositionSetter:
    """DefaultPositionSetter.java: uniform in [0,1)^2 (z = 0), seeded here."""

    def __init__(self, rng: np.random.Generator, dim: int = 2):
        self.rng = rng
        self.dim = dim

    def set(self, position: np.ndarray, type_: int, n_types: int) -> None:
        position[0] = self.rng.random()
        position[1] = self.rng.random()
        position[2] = self.rng.random() if self.dim == 3 else 0.0


class DefaultTypeSetter:
    """DefaultTypeSetter.java: floor(random() * nTypes), seeded here."""

    def __init__(self, rng: np.random.Generator):
        self.rng = rng

    def get_type(self, position, velocity, type_: int, n_types: int) -> int:
        return int(math.floor(self.rng.random() * n_types))


class DefaultMatrixGenerator:
    """DefaultMatrixGenerator.java: a randomized DefaultMatrix."""

    def __init__(self, rng: np.random.Generator):
        self.rng = rng

    def make_matrix(self, size: int) -> DefaultMatrix:
        m = DefaultMatrix(size)
        m.randomize(self.rng)
        return m


# ---------------------------------------------------------------- world --


def check(status: int, ctx=None, what: str = "") -> None:
    if status != _lib.PLG_OK:
        lib = _lib.load()
        msg = lib.plg_last_error(ctx).decode() if ctx else ""
        raise _lib.PlgError(status, f"{what}: {lib.plg_status_string(status).decode()}: {msg}")


def _resident(shape, dtype) -> np.ndarray:
    """An uninitialised array whose pages the CPU has written once (one byte
    per page, and the last byte: the array rarely starts on a page
    boundary, so its last page may begin less than a page before its end),
    so that they are resident before the device writes the array in place;
    far cheaper than filling it."""
    a = np.empty(shape, dtype)
    if a.size:
        b = a.reshape(-1).view(np.uint8)
        b[::4096] = 0
        b[-1] = 0
    return a


class GpuWorld:
    """Thin owner of one plg_ctx (one world on the current CUDA device)."""

    def __init__(self, dim: int, capacity: int):
        self.lib = _lib.load()
        self.dim = dim
        self.capacity = int(capacity)
        h = _lib.C.c_void_p()
        check(self.lib.plg_create(dim, self.capacity, _lib.C.byref(h)), None, "plg_create")
        self.ctx = h

    def close(self) -> None:
        if getattr(self, "ctx", None):
            self.lib.plg_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _c(self, status: int, what: str) -> None:
        check(status, self.ctx, what)

    def set_settings(self, rmax, friction, force, dt, beta=0.3, wrap=True, accel_kind=_lib.PLG_ACCEL_PARTICLE_LIFE):
        s = _lib.plg_settings(rmax, friction, force, dt, beta, 1 if wrap else 0, accel_kind)
        self._c(self.lib.plg_set_settings(self.ctx, _lib.C.byref(s)), "plg_set_settings")

    def set_matrix(self, m: np.ndarray) -> None:
        m = np.ascontiguousarray(m, dtype=np.float64)
        self._c(self.lib.plg_set_matrix(self.ctx, m.shape[0], _lib.ptr(m, _lib.C.c_double)), "plg_set_matrix")

    def upload(self, pos: np.ndarray, vel: Optional[np.ndarray], types: np.ndarray) -> None:
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        n = pos.shape[0]
        velp = None
        if vel is not None:
            vel = np.ascontiguousarray(vel, dtype=np.float64).reshape(-1, 3)
            velp = _lib.ptr(vel, _lib.C.c_double)
        types = np.ascontiguousarray(types, dtype=np.int32)
        self._c(
            self.lib.plg_upload(self.ctx, n, _lib.ptr(pos, _lib.C.c_double), velp, _lib.ptr(types, _lib.C.c_int32)),
            "plg_upload",
        )

    def step(self, n: int = 1) -> None:
        self._c(self.lib.plg_step(self.ctx, n), "plg_step")

    def count(self) -> int:
        v = _lib.C.c_int64()
        self._c(self.lib.plg_particle_count(self.ctx, _lib.C.byref(v)), "plg_particle_count")
        return v.value

    def download(self):
        n = self.count()
        pos = np.empty((n, 3), np.float64)
        vel = np.empty((n, 3), np.float64)
        types = np.empty(n, np.int32)
        ids = np.empty(n, np.int32)
        self._c(
            self.lib.plg_download(
                self.ctx,
                _lib.ptr(pos, _lib.C.c_double),
                _lib.ptr(vel, _lib.C.c_double),
                _lib.ptr(types, _lib.C.c_int32),
                _lib.ptr(ids, _lib.C.c_int32),
            ),
            "plg_download",
        )
        return pos, vel, types, ids

    def step_download(self, nsteps: int = 1, out=None):
        """`nsteps` steps, then the state in the download() layout
        (plg_step_download: the last step's force kernel writes the arrays
        when they are page-locked, or pageable on a device that accesses
        pageable memory).  `out`: optional (pos, vel, types, ids) arrays of
        the download() shapes and dtypes to fill (any may be None)."""
        n = self.count()
        if out is None:
            out = (_resident((n, 3), np.float64), _resident((n, 3), np.float64), _resident((n,), np.int32),
                   _resident((n,), np.int32))
        pos, vel, types, ids = out
        for a, shape, dt in ((pos, (n, 3), np.float64), (vel, (n, 3), np.float64),
                             (types, (n,), np.int32), (ids, (n,), np.int32)):
            if a is not None and (a.shape != shape or a.dtype != dt or not a.flags.c_contiguous):
                raise ValueError("step_download: output arrays must be C-contiguous with the download() shapes")
        self._c(
            self.lib.plg_step_download(
                self.ctx,
                nsteps,
                _lib.ptr(pos, _lib.C.c_double),
                _lib.ptr(vel, _lib.C.c_double),
                _lib.ptr(types, _lib.C.c_int32),
                _lib.ptr(ids, _lib.C.c_int32),
            ),
            "plg_step_download",
        )
        return pos, vel, types, ids

    def set_tile(self, variant: int) -> None:
        self._c(self.lib.plg_set_tile(self.ctx, int(variant)), "plg_set_tile")

    def tile(self) -> int:
        v = _lib.C.c_int32()
        self._c(self.lib.plg_get_tile(self.ctx, _lib.C.byref(v)), "plg_get_tile")
        return v.value

    def autotune(self, steps: int = 5):
        """Times every force tile variant on the world as it is (the state is
        restored) and keeps the fastest; returns (variant, ms per step of
        each)."""
        chosen = _lib.C.c_int32()
        ms = np.zeros(_lib.PLG_TILE_VARIANTS, np.float64)
        self._c(self.lib.plg_autotune(self.ctx, int(steps), _lib.C.byref(chosen), _lib.ptr(ms, _lib.C.c_double)),
                "plg_autotune")
        return chosen.value, [float(x) for x in ms]

    def debug_step(self):
        """One step with the instrumented kernel: per-particle cell, pair
        count, pair hashes, FP32 accelerations (cell-sorted order)."""
        n = self.count()
        cell = np.empty(n, np.int32)
        pairs = np.empty(n, np.int32)
        hs = np.empty(n, np.uint64)
        hx = np.empty(n, np.uint64)
        acc = np.empty((n, self.dim), np.float32)
        cand = _lib.C.c_int64()
        self._c(
            self.lib.plg_debug_step(
                self.ctx,
                _lib.ptr(cell, _lib.C.c_int32),
                _lib.ptr(pairs, _lib.C.c_int32),
                _lib.ptr(hs, _lib.C.c_uint64),
                _lib.ptr(hx, _lib.C.c_uint64),
                _lib.ptr(acc, _lib.C.c_float),
                _lib.C.byref(cand),
            ),
            "plg_debug_step",
        )
        return dict(cell=cell, pairs=pairs, hsum=hs, hxor=hx, acc=acc, candidates=cand.value)

    def deferred(self) -> int:
        """Targets of the last step the force kernel recomputed in its deferred (global-memory) pass."""
        v = _lib.C.c_int64()
        self._c(self.lib.plg_step_stats(self.ctx, _lib.C.byref(v)), "plg_step_stats")
        return v.value

    # -- edits on the device (no re-upload) --

    def _cursor(self, x, y, z, size, shape):
        return _lib.plg_cursor(float(x), float(y), float(z), float(size), int(shape), 0)

    def cursor_count(self, x, y, z=0.0, size=0.1, shape=_lib.PLG_CURSOR_CIRCLE) -> int:
        v = _lib.C.c_int64()
        k = self._cursor(x, y, z, size, shape)
        self._c(self.lib.plg_cursor_count(self.ctx, _lib.C.byref(k), _lib.C.byref(v)), "plg_cursor_count")
        return v.value

    def cursor_move(self, x, y, z, size, shape, dx, dy, dz=0.0) -> int:
        v = _lib.C.c_int64()
        k = self._cursor(x, y, z, size, shape)
        self._c(self.lib.plg_cursor_move(self.ctx, _lib.C.byref(k), dx, dy, dz, _lib.C.byref(v)), "plg_cursor_move")
        return v.value

    def cursor_delete(self, x, y, z=0.0, size=0.1, shape=_lib.PLG_CURSOR_CIRCLE) -> int:
        v = _lib.C.c_int64()
        k = self._cursor(x, y, z, size, shape)
        self._c(self.lib.plg_cursor_delete(self.ctx, _lib.C.byref(k), _lib.C.byref(v)), "plg_cursor_delete")
        return v.value

    def append(self, pos: np.ndarray, vel: Optional[np.ndarray], types: np.ndarray) -> None:
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        velp = None
        if vel is not None:
            vel = np.ascontiguousarray(vel, dtype=np.float64).reshape(-1, 3)
            velp = _lib.ptr(vel, _lib.C.c_double)
        types = np.ascontiguousarray(types, dtype=np.int32)
        self._c(self.lib.plg_append(self.ctx, pos.shape[0], _lib.ptr(pos, _lib.C.c_double), velp,
                                    _lib.ptr(types, _lib.C.c_int32)), "plg_append")

    def permute(self, src: np.ndarray) -> None:
        src = np.ascontiguousarray(src, dtype=np.int32)
        self._c(self.lib.plg_permute(self.ctx, src.shape[0], _lib.ptr(src, _lib.C.c_int32)), "plg_permute")

    def set_types(self, types: np.ndarray) -> None:
        types = np.ascontiguousarray(types, dtype=np.int32)
        self._c(self.lib.plg_set_types(self.ctx, _lib.ptr(types, _lib.C.c_int32)), "plg_set_types")

    # -- initialisers on the device --

    def generate(self, n: int, position_setter: int = 0, type_setter: int = 0, seed: int = 0) -> None:
        self._c(self.lib.plg_generate(self.ctx, n, position_setter, type_setter, seed), "plg_generate")

    def apply_position_setter(self, setter: int, seed: int = 0) -> None:
        self._c(self.lib.plg_apply_position_setter(self.ctx, setter, seed), "plg_apply_position_setter")

    def apply_type_setter(self, setter: int, seed: int = 0) -> None:
        self._c(self.lib.plg_apply_type_setter(self.ctx, setter, seed), "plg_apply_type_setter")

    def render(self, width: int, height: int, palette: np.ndarray, cam=(0.5, 0.5, 1.0, 1.0), top_left=(0.0, 0.0),
               size: float = 0.015, wrap: bool = False) -> np.ndarray:
        """plg_render: (height, width, 4) uint8, rows bottom to top."""
        pal = np.ascontiguousarray(palette, dtype=np.float32).reshape(-1, 4)
        out = np.zeros((height, width, 4), np.uint8)
        rp = _lib.plg_render_params(width, height, cam[0], cam[1], cam[2], cam[3], top_left[0], top_left[1], size,
                                    1 if wrap else 0, 0)
        self._c(self.lib.plg_render(self.ctx, _lib.C.byref(rp), pal.shape[0], _lib.ptr(pal, _lib.C.c_float),
                                    out.ctypes.data_as(_lib.C.POINTER(_lib.C.c_uint8))), "plg_render")
        return out

    def request_stop(self) -> None:
        self._c(self.lib.plg_request_stop(self.ctx), "plg_request_stop")

    def stream(self) -> int:
        p = _lib.C.c_void_p()
        self._c(self.lib.plg_get_stream(self.ctx, _lib.C.byref(p)), "plg_get_stream")
        return p.value or 0


class Physics:
    """Mirror of com.particle_life.backend.Physics (Physics.java:9-512).

    ``dim`` = 3 selects the project's 3D extension (27-cell stencil); the
    reference itself is 2D.  Construction only touches the host: the GPU
    world is created on the first ``update()``.
    """

    DEFAULT_MATRIX_SIZE = 7

    def __init__(
        self,
        accelerator,
        position_setter=None,
        matrix_generator=None,
        type_setter=None,
        *,
        dim: int = 2,
        seed: int = 0,
        initial_count: int = 10000,
        capacity: Optional[int] = None,
        sync_policy: str = "every",
    ):
        self.rng = np.random.Generator(np.random.Philox(seed))
        self.dim = dim
        self.settings = PhysicsSettings()
        self.accelerator = accelerator
        self.position_setter = position_setter or DefaultPositionSetter(self.rng, dim)
        self.matrix_generator = matrix_generator or DefaultMatrixGenerator(self.rng)
        self.type_setter = type_setter or DefaultTypeSetter(self.rng)
        self.preferred_number_of_threads = 12  # kept for API parity; unused on the GPU
        self.sync_policy = sync_policy
        self.capacity = capacity
        self.positions = np.zeros((0, 3), np.float64)
        self.velocities = np.zeros((0, 3), np.float64)
        self.types = np.zeros(0, np.int32)
        self.ids = np.zeros(0, np.int32)
        self._world: Optional[GpuWorld] = None
        self._host_dirty = True
        self._device_newer = False
        self._pushed: Optional[tuple] = None
        self._pushed_matrix: Optional[np.ndarray] = None
        self.generate_matrix()
        self.set_particle_count(initial_count)

    # -- control (Physics.java:149-170) --

    def force_update_stop(self) -> None:
        if self._world is not None:
            self._world.request_stop()

    def kill(self) -> None:
        self.force_update_stop()

    def set_positions(self) -> None:
        self._sync_host()
        for i in range(len(self.types)):
            self._set_position(i)
        self._host_dirty = True

    def generate_matrix(self) -> None:
        prev = self.settings.matrix.size() if self.settings.matrix is not None else self.DEFAULT_MATRIX_SIZE
        self.settings.matrix = self.matrix_generator.make_matrix(prev)
        assert self.settings.matrix.size() == prev, "Matrix size should only change via setMatrixSize()"

    def set_particle_count(self, n: int) -> None:
        """Physics.java:190-223: shrink keeps a random subset, grow appends
        particles made by the type and position setters."""
        if n < 0:
            raise ValueError("n must be 0 or greater")
        self._sync_host()
        cur = len(self.types)
        if n < cur:
            order = self.rng.permutation(cur)
            keep = order[:n]
            self.positions = self.positions[keep].copy()
            self.velocities = self.velocities[keep].copy()
            self.types = self.types[keep].copy()
            self.ids = self.ids[keep].copy()
        elif n > cur:
            add = n - cur
            pos = np.zeros((add, 3), np.float64)
            vel = np.zeros((add, 3), np.float64)
            typ = np.zeros(add, np.int32)
            self.positions = np.concatenate([self.positions, pos])
            self.velocities = np.concatenate([self.velocities, vel])
            self.types = np.concatenate([self.types, typ])
            start = int(self.ids.max()) + 1 if len(self.ids) else 0
            self.ids = np.concatenate([self.ids, np.arange(start, start + add, dtype=np.int32)])
            for i in range(cur, n):
                self._set_type(i)
                self._set_position(i)
        self._host_dirty = True

    def set_matrix_size(self, new_size: int) -> None:
        """Physics.java:238-258."""
        prev = self.settings.matrix
        prev_size = prev.size()
        if new_size == prev_size:
            return
        self.settings.matrix = self.matrix_generator.make_matrix(new_size)
        assert self.settings.matrix.size() == new_size
        common = min(prev_size, new_size)
        for i in range(common):
            for j in range(common):
                self.settings.matrix.set(i, j, prev.get(i, j))
        if new_size < prev_size:
            self.ensure_types()

    def ensure_types(self) -> None:
        """Physics.java:266-272."""
        self._sync_host()
        n = self.settings.matrix.size()
        for i in np.nonzero(self.types >= n)[0]:
            self._set_type(int(i))
        self._host_dirty = True

    def set_types(self) -> None:
        """Physics.java:509-511."""
        self._sync_host()
        for i in range(len(self.types)):
            self._set_type(i)
        self._host_dirty = True

    # -- protected setters (Physics.java:297-307) --

    def _set_position(self, i: int) -> None:
        p = self.positions[i]
        self.position_setter.set(p, int(self.types[i]), self.settings.matrix.size())
        self.ensure_position(p)
        self.velocities[i] = 0.0

    def _set_type(self, i: int) -> None:
        self.types[i] = self.type_setter.get_type(
            self.positions[i].copy(), self.velocities[i].copy(), int(self.types[i]), self.settings.matrix.size()
        )

    # -- geometry helpers (Physics.java:460-505) --

    def connection(self, pos1, pos2) -> np.ndarray:
        delta = np.asarray(pos2, np.float64) - np.asarray(pos1, np.float64)
        if self.settings.wrap:
            for k in range(3):
                v = delta[k]
                delta[k] = v + 1 if v < -0.5 else (v - 1 if v >= 0.5 else v)
            if self.dim == 2:
                delta[2] = 0.0
        return delta

    def distance(self, pos1, pos2) -> float:
        d = self.connection(pos1, pos2)
        return math.sqrt(d[0] * d[0] + (d[1] * d[1] + d[2] * d[2]))

    def ensure_position(self, position: np.ndarray) -> None:
        dims = 3 if self.dim == 3 else 2
        for k in range(dims):
            v = float(position[k])
            if self.settings.wrap:
                if v < 0:
                    while True:
                        v += 1
                        if not v < 0:
                            break
                else:
                    while v >= 1:
                        v -= 1
            else:
                v = 0.0 if v < 0 else (1.0 if v > 1 else v)
            position[k] = v
        if self.dim == 2:
            position[2] = 0.0

    # -- the step (Physics.java:112-134) --

    @property
    def world(self) -> GpuWorld:
        if self._world is None:
            cap = max(self.capacity or 0, len(self.types), 1)
            self._world = GpuWorld(self.dim, cap)
        return self._world

    def _beta(self) -> float:
        if not isinstance(self.accelerator, ParticleLifeAccelerator):
            raise _lib.PlgError(
                _lib.PLG_E_UNSUPPORTED,
                "only ParticleLifeAccelerator has a GPU implementation; there is no CPU fallback",
            )
        return self.accelerator.beta

    def _push(self) -> None:
        w = self.world
        if len(self.types) > w.capacity:
            w.close()
            self._world = None
            self._pushed = None
            self._pushed_matrix = None
            w = self.world
        s = self.settings
        key = (s.wrap, s.rmax, s.friction, s.force, s.dt, self._beta())
        if key != self._pushed:
            w.set_settings(s.rmax, s.friction, s.force, s.dt, beta=key[5], wrap=s.wrap)
            self._pushed = key
        m = matrix_to_array(s.matrix)
        pm = self._pushed_matrix
        if pm is None or m.shape != pm.shape or not np.array_equal(m, pm):
            if pm is not None and m.shape != pm.shape:
                self._sync_host()
                self._host_dirty = True
            try:
                w.set_matrix(m)
            except _lib.PlgError as e:
                # A shrink below the uploaded types invalidates the device
                # state; the re-upload below validates the host types.
                if e.status != _lib.PLG_E_STATE:
                    raise
            self._pushed_matrix = m
        if self._host_dirty:
            w.upload(self.positions, self.velocities, self.types)
            self._device_ids = self.ids.copy()
            self._host_dirty = False

    def update(self) -> None:
        """One Physics.update() on the GPU.  With sync_policy 'every' the
        host arrays come back in the same call (plg_step_download: the step's
        force kernel writes them)."""
        self._push()
        if self.sync_policy == "every":
            self._take(*self.world.step_download(1))
        else:
            self.world.step(1)
            self._device_newer = True

    def _take(self, pos, vel, types, ids) -> None:
        self.positions, self.velocities, self.types = pos, vel, types
        self.ids = self._device_ids[ids]
        self._device_newer = False

    def _sync_host(self) -> None:
        if not self._device_newer or self._world is None:
            return
        self._take(*self._world.download())

    def sync_host(self) -> None:
        """Brings the host arrays up to date (for sync_policy='manual')."""
        self._sync_host()

    # -- saves (app/Main.java:1258-1348) --

    def thumbnail(self, palette, size: int = 256) -> np.ndarray:
        """Main.renderParticlesToImage (app/Main.java:1143-1188) on the GPU:
        the whole world (camera centre (0.5, 0.5), dimensions (1, 1)),
        particle size 0.015, no wrap, rows bottom to top.  `palette` holds
        one RGBA colour per type (the app uses its natural-rainbow palette
        sampled at the matrix size)."""
        self._push()
        return self.world.render(size, size, palette, cam=(0.5, 0.5, 1.0, 1.0), top_left=(0.0, 0.0), size=0.015,
                                 wrap=False)

    def save_state(self, path, image_png: Optional[bytes] = None, palette=None) -> None:
        """Main.saveState: particles, settings and matrix in the app's zip
        layout; with a palette (and no image given) the img.png thumbnail is
        rendered on the GPU."""
        from . import saves

        if image_png is None and palette is not None:
            image_png = saves.png_rgba(self.thumbnail(palette, saves.THUMBNAIL_SIZE))
        self._sync_host()
        s = self.settings
        saves.save_state(path, self.positions, self.velocities, self.types, wrap=s.wrap, rmax=s.rmax,
                         friction=s.friction, force=s.force, matrix=matrix_to_array(s.matrix), dim=self.dim,
                         image_png=image_png)

    def load_state(self, path) -> None:
        """Main.loadState: each entry present replaces that part of the state;
        a new matrix re-types particles outside it (ensureTypes)."""
        from . import saves

        st = saves.load_state(path)
        self._sync_host()
        if st.positions is not None:
            self.positions = st.positions.copy()
            self.velocities = st.velocities.copy()
            self.types = st.types.astype(np.int32)
            self.ids = np.arange(len(self.types), dtype=np.int32)
            for i in range(len(self.types)):
                self.ensure_position(self.positions[i])
        if st.rmax is not None:
            self.settings.wrap, self.settings.rmax = st.wrap, st.rmax
            self.settings.friction, self.settings.force = st.friction, st.force
        if st.matrix is not None:
            m = DefaultMatrix(st.matrix.shape[0])
            for i in range(st.matrix.shape[0]):
                for j in range(st.matrix.shape[0]):
                    m.set(i, j, float(st.matrix[i, j]))
            self.settings.matrix = m
            self.ensure_types()
        self._host_dirty = True

    def close(self) -> None:
        if self._world is not None:
            self._world.close()
            self._world = None
