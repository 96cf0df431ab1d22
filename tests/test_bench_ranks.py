"""The replica aggregation of bench.py under torch.distributed with the gloo
backend on CPU, world size 2: every rank sees the slowest rank's time, and the
whole-job rate counts the units of all ranks over that time."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, times, out):
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        slow = bench.max_over_ranks(times[rank], dist, "cpu")
        rate = bench.whole_job_rate(1000, world, slow)
        out.put((rank, slow, rate))
    finally:
        dist.destroy_process_group()


def test_replica_aggregation_gloo_world2():
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    os.environ["PYTHONPATH"] = root + os.pathsep + os.environ.get("PYTHONPATH", "")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    times = [2.0, 5.0]
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, times, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[1] for g in got] == [5.0, 5.0]
    assert got[0][2] == pytest.approx(2 * 1000 / 5.0) and got[1][2] == got[0][2]


def test_single_process_aggregation():
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.whole_job_rate(10, 1, 2.0) == 5.0
