"""Replica bookkeeping over a two-rank gloo group on the CPU: slowest time, summed work."""
import os

import pytest


def _worker(rank, world, port, q):
    import torch.distributed as dist

    from accuratewigner_gb300.replicas import job_throughput

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sec, units, rate = job_throughput(1.0 + rank, 100.0 * (rank + 1))
        q.put((rank, sec, units, rate))
    finally:
        dist.destroy_process_group()


def test_two_ranks_gloo():
    import socket

    import torch.multiprocessing as mp

    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, sec, units, rate in out:
        assert sec == 2.0 and units == 300.0 and rate == pytest.approx(150.0)


def test_single_process_passthrough():
    from accuratewigner_gb300.replicas import job_throughput

    assert job_throughput(2.0, 10.0) == (2.0, 10.0, 5.0)
