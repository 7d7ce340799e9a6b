"""Serving: a native request loop over batched worlds (plg_server_*).

Requests (a world and a step count) are submitted from any thread; the
library's scheduler thread admits them under a device-memory budget, runs
them in continuously re-packed batches and keeps each final state until it
is collected.
"""
from __future__ import annotations

from typing import Optional

import numpy as np

from . import _lib
from .batch import WorldDesc, world_struct


def _check(status: int, s, what: str) -> None:
    if status != _lib.PLG_OK:
        lib = _lib.load()
        msg = lib.plg_server_last_error(s).decode() if s else ""
        raise _lib.PlgError(status, f"{what}: {lib.plg_status_string(status).decode()}: {msg}")


class Server:
    def __init__(self, memory_budget_bytes: int, particle_capacity=(4_000_000, 4_000_000),
                 cell_capacity=(8_000_000, 8_000_000), max_worlds_per_batch: int = 512, max_chunk_steps: int = 16,
                 tile_variant: int = 0):
        self.lib = _lib.load()
        cfg = _lib.plg_server_config()
        cfg.memory_budget_bytes = int(memory_budget_bytes)
        cfg.particle_capacity[0], cfg.particle_capacity[1] = (int(x) for x in particle_capacity)
        cfg.cell_capacity[0], cfg.cell_capacity[1] = (int(x) for x in cell_capacity)
        cfg.max_worlds_per_batch = max_worlds_per_batch
        cfg.max_chunk_steps = max_chunk_steps
        cfg.tile_variant = tile_variant
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

    def wait(self, rid: int, timeout_s: float = 0.0) -> int:
        st = _lib.C.c_int32()
        _check(self.lib.plg_server_wait(self.s, rid, timeout_s, _lib.C.byref(st)), self.s, "plg_server_wait")
        return st.value

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
        return {name: getattr(st, name) for name, _ in st._fields_}

    @staticmethod
    def device_bytes(dim: int, world: WorldDesc) -> int:
        keep: list = []
        d = world_struct(world, keep)
        return int(_lib.load().plg_world_device_bytes(dim, _lib.C.byref(d)))
