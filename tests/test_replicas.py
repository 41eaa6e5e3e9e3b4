"""CPU: the replica form of bench.py (one process per GPU, the same
workload on each, no data-path collective) aggregates its ranks the way the
bench line reports them: the slowest rank's time and the accepted steps of
all ranks.  Two gloo ranks on 127.0.0.1 stand in for two GPUs."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        secs = [2.0, 3.5][rank]
        acc = [1000, 1200][rank]
        out.put((rank, bench.replica_totals(secs, acc, world, "cpu")))
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_slowest_time_and_all_steps():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got[0] == got[1] == (3.5, 2200.0)


def test_single_process_returns_its_own_figures():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.replica_totals(1.25, 77, 1, "cpu") == (1.25, 77)
