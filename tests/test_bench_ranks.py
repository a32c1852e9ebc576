"""The replica path of bench.py on CPU: two gloo ranks, each with its own
step time; the job time is the slower rank's and the whole-job throughput
counts both ranks' cells."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist

    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    local_ms = 100.0 if rank == 0 else 250.0
    q.put((rank, bench.job_throughput(local_ms, 1000, 10, dist, "cpu")))
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in (0, 1):
        max_ms, mlups = out[r]
        assert max_ms == 250.0
        assert mlups == pytest.approx(2 * 1000 * 10 / 0.25 / 1e6)


def test_single_process_needs_no_process_group():
    import bench

    assert bench.job_throughput(50.0, 2000, 5, None, "cpu") == (50.0, pytest.approx(2000 * 5 / 0.05 / 1e6))
