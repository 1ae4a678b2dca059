"""The multi-rank aggregation of bench.py (column shards, one per GPU): the
slowest rank's step time over a process group and the whole-job columns/s
(the globe's columns over that time), exercised with two gloo ranks on the
CPU."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as tdist

    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    tdist.init_process_group("gloo", rank=rank, world_size=world)
    ms, value = bench.job_rate(100.0 + 50.0 * rank, 1000, world, device="cpu")
    tdist.barrier()
    tdist.destroy_process_group()
    out.put((rank, ms, value))


def test_job_rate_takes_the_slowest_rank_over_gloo():
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
    for rank, ms, value in res:
        assert ms == 150.0  # the slower rank's step
        assert abs(value - 1000 / 0.150) < 1e-6


def test_job_rate_single_process():
    import bench
    ms, value = bench.job_rate(200.0, 500, 1)
    assert ms == 200.0 and abs(value - 2500.0) < 1e-9
