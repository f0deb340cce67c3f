"""The multi-rank bench path on the CPU: two gloo ranks (replicas, no data
collective) agree on the slowest rank's step time, the whole-job throughput
counts every rank's batch, and each rank draws its own phantoms."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    import torch.distributed as dist
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = 100.0 + 50.0 * rank  # rank 1 is the slow one
        slowest = bench.max_over_ranks(ms, dist)
        out.put((rank, slowest, bench.job_throughput(64, world, slowest), bench.rank_seed(rank)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_share_the_slowest_step():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [150.0, 150.0]
    assert res[0][2] == pytest.approx(2 * 64 / 0.150)
    assert res[0][3] != res[1][3]


def test_single_process_needs_no_group():
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.job_throughput(64, 1, 160.0) == pytest.approx(400.0)
