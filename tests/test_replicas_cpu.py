"""The multi-GPU form is replicas only (one world per rank, no collective on
the data path).  Its host logic runs here on CPU with two gloo ranks: the
timed region is the slowest rank's, the whole-job rate counts every rank's
units, only rank 0 is the leader that prints, and the reference arm runs on
rank 0 alone."""
import io
import os
import socket
import sys
from contextlib import redirect_stdout
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, queue):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, str(REPO))
    import bench

    reps = bench.Replicas("gloo")
    seconds = [1.0, 3.0][rank]
    queue.put((rank, reps.leader, reps.world_size, reps.max_over_ranks(seconds), reps.rate(100.0, seconds)))
    reps.barrier()
    reps.close()


def test_two_gloo_ranks_are_timed_by_the_slowest():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(k, 2, port, queue)) for k in range(2)]
    for p in procs:
        p.start()
    out = sorted(queue.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [True, False]  # rank 0 alone leads
    for _, _, world, slowest, rate in out:
        assert world == 2 and slowest == 3.0
        assert rate == pytest.approx(2 * 100.0 / 3.0)


def test_single_process_needs_no_group(monkeypatch):
    sys.path.insert(0, str(REPO))
    import bench

    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    reps = bench.Replicas("gloo")
    assert reps.leader and reps.world_size == 1 and reps.dist is None
    assert reps.rate(50.0, 2.0) == 25.0
    reps.close()


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    sys.path.insert(0, str(REPO))
    import bench

    monkeypatch.setenv("RANK", "1")
    buf = io.StringIO()
    with redirect_stdout(buf):
        assert bench.run_reference(bench.parse(["--impl", "reference"])) is None
    assert buf.getvalue() == ""
