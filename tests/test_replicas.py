"""bench.py on N GPUs runs N independent replicas (the mobility path needs no
exchange between them): the whole-job rate is N x units per rank over the
slowest rank's time. The rank aggregation is exercised here with two gloo
ranks on the CPU."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist

    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        times = bench.max_over_ranks([1.0 + rank, 10.0 - rank, 0.5], world, "cpu")
        out.put((rank, times, bench.whole_job_rate(5, world, times[0])))
    finally:
        dist.destroy_process_group()


def test_max_over_two_gloo_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, times, rate in got:
        assert times == [2.0, 10.0, 0.5]  # every rank sees the slowest time
        assert rate == 2 * 5 / 2.0


def test_single_rank_passthrough():
    import bench

    assert bench.max_over_ranks([3.0, 4.0], 1, "cpu") == [3.0, 4.0]
    assert bench.whole_job_rate(10, 1, 2.0) == 5.0
