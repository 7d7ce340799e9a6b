"""Serving loop (plg_server_*): requests that arrive while others run are
admitted at chunk boundaries under the memory budget, and every result is
bit for bit the same world run alone through a single-world context."""
import threading
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def alone(dim, w, steps):
    from plgpu.physics import GpuWorld

    g = GpuWorld(dim, max(w.pos.shape[0], 1))
    g.set_settings(w.rmax, w.friction, w.force, w.dt, beta=w.beta, wrap=w.wrap)
    g.set_matrix(w.matrix)
    g.upload(w.pos, w.vel, w.types)
    g.step(steps)
    out = g.download()
    g.close()
    return out


def requests(count, seed, n_hi=20_000, steps_hi=40):
    from plgpu import workloads

    rng = np.random.Generator(np.random.Philox(seed))
    return [workloads.serving_request(rng, n_lo=1_000, n_hi=n_hi, steps_lo=1, steps_hi=steps_hi)
            for _ in range(count)]


def test_results_equal_the_world_run_alone(gpu):
    from plgpu.serve import Server

    reqs = requests(10, seed=91)
    srv = Server(memory_budget_bytes=2 << 30, max_chunk_steps=8)
    ids = []

    def feed():  # arrivals spread over time, from another thread
        for dim, w, steps in reqs:
            ids.append(srv.submit(dim, w, steps))
            time.sleep(0.01)

    t = threading.Thread(target=feed)
    t.start()
    t.join()
    for rid in ids:
        srv.wait(rid, 60.0)
    results = [srv.result(rid) for rid in ids]
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(reqs) and st["latency_p99_ms"] >= st["latency_p50_ms"] > 0
    for (dim, w, steps), got in zip(reqs, results):
        ref = alone(dim, w, steps)
        for a, c in zip(ref, got[:4]):
            assert np.array_equal(a, c)


def test_admission_respects_the_memory_budget(gpu):
    from plgpu.serve import Server

    reqs = requests(8, seed=92, n_hi=8_000, steps_hi=20)
    sizes = [Server.device_bytes(dim, w) for dim, w, _ in reqs]
    budget = 2 * max(sizes)  # at most a few worlds resident at once
    srv = Server(memory_budget_bytes=budget, max_chunk_steps=4)
    ids = [srv.submit(dim, w, steps) for dim, w, steps in reqs]
    for rid in ids:
        srv.wait(rid, 60.0)
    st = srv.stats()
    for rid in ids:
        srv.result(rid)
    srv.close()
    assert st["completed"] == len(reqs)
    assert 0 < st["peak_resident_bytes"] <= budget
    assert st["resident_bytes"] == 0


def test_rejections_and_zero_steps(gpu):
    from plgpu import _lib, workloads
    from plgpu.serve import Server

    srv = Server(memory_budget_bytes=64 << 20)
    rng = np.random.Generator(np.random.Philox(93))
    big = workloads.random_world(rng, 2, 2_000_000, 4, 0.01, 0.8, 0.02)
    with pytest.raises(_lib.PlgError) as e:
        srv.submit(2, big, 10)
    assert e.value.status == _lib.PLG_E_CAPACITY
    bad = workloads.random_world(rng, 2, 100, 4, 0.6, 0.8, 0.02)  # nx = 1
    with pytest.raises(_lib.PlgError) as e:
        srv.submit(2, bad, 10)
    assert e.value.status == _lib.PLG_E_UNSUPPORTED
    w = workloads.random_world(rng, 3, 3_000, 5, 0.1, 0.8, 0.02)
    rid = srv.submit(3, w, 0)
    assert srv.wait(rid, 30.0) == _lib.PLG_REQ_DONE
    pos, vel, types, ids, _ = srv.result(rid)
    srv.close()
    assert np.array_equal(ids, np.arange(3_000))
    assert np.array_equal(pos, w.pos) and np.array_equal(types, w.types)


def alone_generated(dim, g, steps):
    from plgpu.physics import GpuWorld

    w = GpuWorld(dim, max(g.n, 1))
    w.set_settings(g.rmax, g.friction, g.force, g.dt, beta=g.beta, wrap=g.wrap)
    w.set_matrix(g.matrix)
    w.generate(g.n, g.position_setter, g.type_setter, g.seed)
    w.step(steps)
    out = w.download()
    w.close()
    return out


def test_large_worlds_equal_the_world_run_alone(gpu):
    """A 1M-particle 2D world (20 neighbours, uploaded) and a 3D world at 50
    neighbours (generated on the device), each served while small worlds
    arrive, finish and leave around them, end bit for bit where they end
    alone."""
    import math

    from plgpu import workloads
    from plgpu.serve import GeneratedWorld, Server

    rng = np.random.Generator(np.random.Philox(94))
    big2 = workloads.random_world(rng, 2, 1_000_000, 8, math.sqrt(20 / (math.pi * 1e6)), 0.7644, 0.01)
    m3 = np.asarray(2 * rng.random((12, 12)) - 1, np.float32).astype(np.float64)
    big3 = GeneratedWorld(n=300_000, matrix=m3, rmax=(3 * 50 / (4 * math.pi * 3e5)) ** (1 / 3), friction=0.7644,
                          dt=0.02, seed=5)
    small = requests(8, seed=95, n_hi=20_000, steps_hi=12)
    srv = Server(memory_budget_bytes=8 << 30, particle_capacity=(4_000_000, 2_000_000),
                 cell_capacity=(4_000_000, 4_000_000), max_chunk_steps=3)
    ids = [srv.submit(2, big2, 7), srv.submit_generated(3, big3, 5)]
    for dim, w, steps in small:
        ids.append(srv.submit(dim, w, steps))
        time.sleep(0.003)
    for rid in ids:
        srv.wait(rid, 120.0)
    results = [srv.result(rid) for rid in ids]
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(ids)
    refs = [alone(2, big2, 7), alone_generated(3, big3, 5)] + [alone(dim, w, steps) for dim, w, steps in small]
    for ref, got in zip(refs, results):
        for a, c in zip(ref, got[:4]):
            assert np.array_equal(a, c)


def test_generated_requests_and_compaction(gpu):
    """Generated worlds through a server whose batches hold only a few
    worlds and are re-tuned per world at almost every chunk boundary:
    finished worlds must be compacted away to admit the rest, and every
    result equals plg_generate + plg_step in a single-world context."""
    from plgpu import workloads
    from plgpu.serve import Server

    rng = np.random.Generator(np.random.Philox(96))
    reqs = [workloads.serving_request_generated(rng, n_lo=2_000, n_hi=30_000, steps_lo=1, steps_hi=20)
            for _ in range(14)]
    srv = Server(memory_budget_bytes=4 << 30, particle_capacity=(70_000, 70_000),
                 cell_capacity=(2_000_000, 2_000_000), max_chunk_steps=4, autotune_interval_ms=1)
    ids = []
    for dim, g, steps in reqs:
        ids.append(srv.submit_generated(dim, g, steps))
        time.sleep(0.002)
    seen = set()
    while len(seen) < len(ids):
        rid = srv.wait_any(60.0)
        assert rid is not None
        seen.add(rid)
    results = [srv.result(rid) for rid in ids]
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(ids) and st["compactions"] > 0 and st["autotunes"] > 0
    assert st["busy_s"] > 0 and st["resident_bytes"] == 0
    for (dim, g, steps), got in zip(reqs, results):
        ref = alone_generated(dim, g, steps)
        for a, c in zip(ref, got[:4]):
            assert np.array_equal(a, c)
