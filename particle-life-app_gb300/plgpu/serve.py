"""Serving: a native request loop over batched worlds (plg_server_*).

Requests (a world and a step count) are submitted from any thread; the
library's scheduler thread admits them under a device-memory budget, runs
them in continuously re-packed batches and keeps each final state until it
is collected.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import _lib
from .batch import WorldDesc, world_struct


@dataclass
class GeneratedWorld:
    """A world given by its generator (plg_world_gen): n particles made on the
    device at admission, exactly as GpuWorld.generate makes them."""

    n: int
    matrix: np.ndarray  # (t, t) float64
    rmax: float
    friction: float
    force: float = 1.0
    dt: float = 0.02
    beta: float = 0.3
    wrap: bool = True
    position_setter: int = 0  # PLG_POS_UNIFORM
    type_setter: int = 0  # PLG_TYPE_RANDOM
    seed: int = 0


def gen_struct(g: GeneratedWorld, keep: list) -> "_lib.plg_world_gen":
    m = np.ascontiguousarray(g.matrix, dtype=np.float64)
    keep.append(m)
    s = _lib.plg_world_gen()
    s.world.settings = _lib.plg_settings(g.rmax, g.friction, g.force, g.dt, g.beta, 1 if g.wrap else 0,
                                         _lib.PLG_ACCEL_PARTICLE_LIFE)
    s.world.ntypes = m.shape[0]
    s.world.matrix = _lib.ptr(m, _lib.C.c_double)
    s.world.n = int(g.n)
    s.position_setter = int(g.position_setter)
    s.type_setter = int(g.type_setter)
    s.seed = int(g.seed)
    return s


def _check(status: int, s, what: str) -> None:
    if status != _lib.PLG_OK:
        lib = _lib.load()
        msg = lib.plg_server_last_error(s).decode() if s else ""
        raise _lib.PlgError(status, f"{what}: {lib.plg_status_string(status).decode()}: {msg}")


class Server:
    def __init__(self, memory_budget_bytes: int, particle_capacity=(4_000_000, 4_000_000),
                 cell_capacity=(8_000_000, 8_000_000), max_worlds_per_batch: int = 512, max_chunk_steps: int = 16,
                 tile_variant: int = 0, autotune_interval_ms: int = 0):
        self.lib = _lib.load()
        cfg = _lib.plg_server_config()
        cfg.memory_budget_bytes = int(memory_budget_bytes)
        cfg.particle_capacity[0], cfg.particle_capacity[1] = (int(x) for x in particle_capacity)
        cfg.cell_capacity[0], cfg.cell_capacity[1] = (int(x) for x in cell_capacity)
        cfg.max_worlds_per_batch = max_worlds_per_batch
        cfg.max_chunk_steps = max_chunk_steps
        cfg.tile_variant = tile_variant
        cfg.autotune_interval_ms = autotune_interval_ms
        h = _lib.C.c_void_p()
        _check(self.lib.plg_server_create(_lib.C.byref(cfg), _lib.C.byref(h)), None, "plg_server_create")
        self.s = h
        self._n: dict[int, int] = {}

    def close(self) -> None:
        if getattr(self, "s", None):
            self.lib.plg_server_destroy(self.s)
            self.s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, dim: int, world: WorldDesc, steps: int) -> int:
        keep: list = []
        d = world_struct(world, keep)
        rid = _lib.C.c_int64()
        _check(self.lib.plg_server_submit(self.s, dim, _lib.C.byref(d), int(steps), _lib.C.byref(rid)), self.s,
               "plg_server_submit")
        self._n[rid.value] = int(d.n)
        return rid.value

    def submit_generated(self, dim: int, world: GeneratedWorld, steps: int) -> int:
        keep: list = []
        g = gen_struct(world, keep)
        rid = _lib.C.c_int64()
        _check(self.lib.plg_server_submit_generated(self.s, dim, _lib.C.byref(g), int(steps), _lib.C.byref(rid)),
               self.s, "plg_server_submit_generated")
        self._n[rid.value] = int(world.n)
        return rid.value

    def wait(self, rid: int, timeout_s: float = 0.0) -> int:
        st = _lib.C.c_int32()
        _check(self.lib.plg_server_wait(self.s, rid, timeout_s, _lib.C.byref(st)), self.s, "plg_server_wait")
        return st.value

    def wait_any(self, timeout_s: float = 0.0) -> Optional[int]:
        """The id of a request that finished (each is given once, in
        completion order), or None when none finished within timeout_s."""
        rid = _lib.C.c_int64()
        st = self.lib.plg_server_wait_any(self.s, timeout_s, _lib.C.byref(rid))
        if st == _lib.PLG_E_TIMEOUT:
            return None
        _check(st, self.s, "plg_server_wait_any")
        return rid.value

    def release(self, rid: int) -> float:
        """Drops a finished request's result; returns its latency in ms."""
        self._n.pop(rid, None)
        lat = _lib.C.c_double()
        _check(self.lib.plg_server_result(self.s, rid, None, None, None, None, None, _lib.C.byref(lat)), self.s,
               "plg_server_result")
        return lat.value

    def result(self, rid: int):
        """(pos, vel, types, ids, latency_ms) of a finished request."""
        n = self._n.pop(rid)
        pos = np.empty((n, 3))
        vel = np.empty((n, 3))
        types = np.empty(n, np.int32)
        ids = np.empty(n, np.int32)
        m = _lib.C.c_int64()
        lat = _lib.C.c_double()
        _check(self.lib.plg_server_result(self.s, rid, _lib.ptr(pos, _lib.C.c_double), _lib.ptr(vel, _lib.C.c_double),
                                          _lib.ptr(types, _lib.C.c_int32), _lib.ptr(ids, _lib.C.c_int32),
                                          _lib.C.byref(m), _lib.C.byref(lat)), self.s, "plg_server_result")
        return pos, vel, types, ids, lat.value

    def stats(self) -> dict:
        st = _lib.plg_server_stats_t()
        _check(self.lib.plg_server_stats(self.s, _lib.C.byref(st)), self.s, "plg_server_stats")
        out = {name: getattr(st, name) for name, _ in st._fields_}
        out["busy_dim_s"] = list(st.busy_dim_s)
        return out

    @staticmethod
    def device_bytes(dim: int, world: WorldDesc) -> int:
        keep: list = []
        d = world_struct(world, keep)
        return int(_lib.load().plg_world_device_bytes(dim, _lib.C.byref(d)))
