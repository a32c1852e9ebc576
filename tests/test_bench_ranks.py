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


def test_reference_arm_prints_its_line(monkeypatch, capsys):
    """`bench.py --impl reference` runs on the host alone: one JSON line with
    the keys the reference arm needs (a shortened CPU sample here)."""
    import json
    import sys

    import bench

    real = bench.cpu_baseline
    monkeypatch.setattr(bench, "cpu_baseline", lambda threads: real(min(threads, 2), budget_s=0.2))
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--steps", "2", "--warmup", "1"])
    bench.main()
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "MLUPS" and line["value"] > 0
    assert line["higher_is_better"] is True
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"] and cb["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
