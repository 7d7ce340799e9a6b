"""Batched worlds: many independent Physics worlds advanced by one step launch.

Thin owner of a ``plg_batch`` (include/plgpu.h).  Each world is described
like a single-world context (settings, matrix, initial particles) and keeps
an integer id across membership changes.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

from . import _lib


@dataclass
class WorldDesc:
    """One world: the arguments of plg_set_settings, plg_set_matrix and plg_upload."""

    pos: np.ndarray  # (n, 3) float64 in [0, 1]
    types: np.ndarray  # (n,) int32
    matrix: np.ndarray  # (t, t) float64
    rmax: float
    friction: float
    force: float = 1.0
    dt: float = 0.02
    beta: float = 0.3
    wrap: bool = True
    vel: Optional[np.ndarray] = None


def world_struct(w: WorldDesc, keep: list) -> "_lib.plg_world_desc":
    """The C description of a world; `keep` receives the arrays it points to."""
    pos = np.ascontiguousarray(w.pos, dtype=np.float64).reshape(-1, 3)
    types = np.ascontiguousarray(w.types, dtype=np.int32)
    m = np.ascontiguousarray(w.matrix, dtype=np.float64)
    vel = None if w.vel is None else np.ascontiguousarray(w.vel, dtype=np.float64).reshape(-1, 3)
    keep += [pos, types, m, vel]
    d = _lib.plg_world_desc()
    d.settings = _lib.plg_settings(w.rmax, w.friction, w.force, w.dt, w.beta, 1 if w.wrap else 0,
                                   _lib.PLG_ACCEL_PARTICLE_LIFE)
    d.ntypes = m.shape[0]
    d.matrix = _lib.ptr(m, _lib.C.c_double)
    d.n = pos.shape[0]
    d.pos = _lib.ptr(pos, _lib.C.c_double)
    d.vel = _lib.ptr(vel, _lib.C.c_double) if vel is not None else None
    d.type = _lib.ptr(types, _lib.C.c_int32)
    return d


def _check(status: int, b, what: str) -> None:
    if status != _lib.PLG_OK:
        lib = _lib.load()
        msg = lib.plg_batch_last_error(b).decode() if b else ""
        raise _lib.PlgError(status, f"{what}: {lib.plg_status_string(status).decode()}: {msg}")


class GpuBatch:
    def __init__(self, dim: int, particle_capacity: int, world_capacity: int, cell_capacity: int):
        self.lib = _lib.load()
        self.dim = dim
        h = _lib.C.c_void_p()
        _check(self.lib.plg_batch_create(dim, int(particle_capacity), int(world_capacity), int(cell_capacity),
                                         _lib.C.byref(h)), None, "plg_batch_create")
        self.b = h

    def close(self) -> None:
        if getattr(self, "b", None):
            self.lib.plg_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def update(self, remove: Sequence[int] = (), add: Sequence[WorldDesc] = ()) -> list[int]:
        """Removes worlds by id and adds new ones; returns the new ids."""
        keep: list = []
        descs = (_lib.plg_world_desc * max(len(add), 1))()
        for k, w in enumerate(add):
            descs[k] = world_struct(w, keep)
        rem = np.ascontiguousarray(list(remove), dtype=np.int32)
        ids = np.zeros(max(len(add), 1), np.int32)
        _check(self.lib.plg_batch_update(self.b, len(rem), _lib.ptr(rem, _lib.C.c_int32) if len(rem) else None,
                                         len(add), descs if len(add) else None, _lib.ptr(ids, _lib.C.c_int32)),
               self.b, "plg_batch_update")
        return [int(x) for x in ids[: len(add)]]

    def step(self, n: int = 1) -> None:
        _check(self.lib.plg_batch_step(self.b, n), self.b, "plg_batch_step")

    def step_async(self, n: int = 1) -> None:
        _check(self.lib.plg_batch_step_async(self.b, n), self.b, "plg_batch_step_async")

    def sync(self, timeout_s: float = 0.0) -> None:
        _check(self.lib.plg_batch_sync(self.b, timeout_s), self.b, "plg_batch_sync")

    def info(self, wid: int) -> tuple[int, int, int]:
        n, s, c = _lib.C.c_int64(), _lib.C.c_int64(), _lib.C.c_int64()
        _check(self.lib.plg_batch_world_info(self.b, wid, _lib.C.byref(n), _lib.C.byref(s), _lib.C.byref(c)),
               self.b, "plg_batch_world_info")
        return n.value, s.value, c.value

    def counts(self) -> tuple[int, int, int]:
        w, n, c = _lib.C.c_int32(), _lib.C.c_int64(), _lib.C.c_int64()
        _check(self.lib.plg_batch_counts(self.b, _lib.C.byref(w), _lib.C.byref(n), _lib.C.byref(c)), self.b,
               "plg_batch_counts")
        return w.value, n.value, c.value

    def download(self, wid: int):
        n = self.info(wid)[0]
        pos = np.empty((n, 3), np.float64)
        vel = np.empty((n, 3), np.float64)
        types = np.empty(n, np.int32)
        ids = np.empty(n, np.int32)
        _check(self.lib.plg_batch_download(self.b, wid, _lib.ptr(pos, _lib.C.c_double),
                                           _lib.ptr(vel, _lib.C.c_double), _lib.ptr(types, _lib.C.c_int32),
                                           _lib.ptr(ids, _lib.C.c_int32)), self.b, "plg_batch_download")
        return pos, vel, types, ids

    def debug_step(self):
        """One instrumented step of every world; arrays over all sorted slots."""
        n = self.counts()[1]
        cell = np.empty(n, np.int32)
        pairs = np.empty(n, np.int32)
        hs = np.empty(n, np.uint64)
        hx = np.empty(n, np.uint64)
        acc = np.empty((n, self.dim), np.float32)
        cand = _lib.C.c_int64()
        _check(self.lib.plg_batch_debug_step(self.b, _lib.ptr(cell, _lib.C.c_int32), _lib.ptr(pairs, _lib.C.c_int32),
                                             _lib.ptr(hs, _lib.C.c_uint64), _lib.ptr(hx, _lib.C.c_uint64),
                                             _lib.ptr(acc, _lib.C.c_float), _lib.C.byref(cand)),
               self.b, "plg_batch_debug_step")
        return dict(cell=cell, pairs=pairs, hsum=hs, hxor=hx, acc=acc, candidates=cand.value)

    def world_debug(self, dbg: dict, wid: int) -> dict:
        """The slice of a debug_step result that belongs to one world (local cells)."""
        n, s, c = self.info(wid)
        out = {k: v[s:s + n] for k, v in dbg.items() if isinstance(v, np.ndarray)}
        out["cell"] = out["cell"] - c
        return out

    def set_steps(self, wid: int, steps: int) -> None:
        """The world freezes after `steps` more batch steps (< 0: no limit)."""
        _check(self.lib.plg_batch_set_steps(self.b, wid, steps), self.b, "plg_batch_set_steps")

    def steps_left(self, wid: int) -> int:
        v = _lib.C.c_int32()
        _check(self.lib.plg_batch_steps_left(self.b, wid, _lib.C.byref(v)), self.b, "plg_batch_steps_left")
        return v.value

    def set_tile(self, variant: int) -> None:
        _check(self.lib.plg_batch_set_tile(self.b, variant), self.b, "plg_batch_set_tile")

    def tile(self) -> int:
        v = _lib.C.c_int32()
        _check(self.lib.plg_batch_get_tile(self.b, _lib.C.byref(v)), self.b, "plg_batch_get_tile")
        return v.value

    def autotune(self, steps: int = 3) -> tuple[int, list[float]]:
        """Times every tile variant on the current batch (state restored) and
        keeps the fastest; returns (variant, ms per step of each)."""
        chosen = _lib.C.c_int32()
        ms = (_lib.C.c_double * _lib.PLG_TILE_VARIANTS)()
        _check(self.lib.plg_batch_autotune(self.b, steps, _lib.C.byref(chosen), ms), self.b, "plg_batch_autotune")
        return chosen.value, list(ms)

    def world_ids(self) -> list[int]:
        """The worlds' ids in device order."""
        nw = self.counts()[0]
        ids = np.zeros(max(nw, 1), np.int32)
        _check(self.lib.plg_batch_world_ids(self.b, _lib.ptr(ids, _lib.C.c_int32)), self.b, "plg_batch_world_ids")
        return [int(x) for x in ids[:nw]]

    def set_world_tile(self, wid: int, variant: int) -> None:
        _check(self.lib.plg_batch_set_world_tile(self.b, wid, variant), self.b, "plg_batch_set_world_tile")

    def world_tile(self, wid: int) -> int:
        v = _lib.C.c_int32()
        _check(self.lib.plg_batch_get_world_tile(self.b, wid, _lib.C.byref(v)), self.b, "plg_batch_get_world_tile")
        return v.value

    def autotune_worlds(self, steps: int = 2) -> tuple[dict[int, int], list[float]]:
        """Gives every world its cheapest tile variant (measured per world;
        the mix kept only if it beats the best single variant); returns
        ({world id: variant}, ms per step of each variant alone and of the
        mix)."""
        nw = self.counts()[0]
        var = np.zeros(max(nw, 1), np.int32)
        ms = (_lib.C.c_double * (_lib.PLG_TILE_VARIANTS + 1))()
        _check(self.lib.plg_batch_autotune_worlds(self.b, steps, _lib.ptr(var, _lib.C.c_int32), ms), self.b,
               "plg_batch_autotune_worlds")
        return dict(zip(self.world_ids(), (int(x) for x in var[:nw]))), list(ms)

    def deferred(self) -> int:
        v = _lib.C.c_int64()
        _check(self.lib.plg_batch_step_stats(self.b, _lib.C.byref(v)), self.b, "plg_batch_step_stats")
        return v.value

    def stream(self) -> int:
        p = _lib.C.c_void_p()
        _check(self.lib.plg_batch_get_stream(self.b, _lib.C.byref(p)), self.b, "plg_batch_get_stream")
        return p.value or 0
