"""The N>1 path of bench.py on CPU: two gloo ranks, each timing its own
replica; the job time is the maximum over ranks and the throughput counts
every rank's bodies (weak scaling, no data-path collective)."""
from __future__ import annotations

import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world_size, port, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world_size)
    import bench

    ms = 100.0 + 50.0 * rank          # rank 1 is the slow one
    job_ms, n = bench.reduce_over_ranks(ms, dist, "cpu")
    value = bench.job_throughput(n, 1000, 10, job_ms)
    dist.barrier()
    q.put((rank, job_ms, n, value))
    dist.destroy_process_group()


def test_two_rank_reduction_takes_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, job_ms, n, value in res:
        assert n == 2
        assert job_ms == 150.0
        assert value == pytest.approx(2 * 1000 * 10 / 0.150)


def test_reference_arm_runs_on_rank_zero_only():
    import bench

    class A:
        pass

    assert bench.run_reference(A(), 1) is None
