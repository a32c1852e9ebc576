"""Independent domains over ranks (lbm_gb300.shard), on CPU.

* The contiguous shares of the 2048-cavity workload cover every cavity once,
  in order, and no rank carries more than 5 % above the mean cell count, for
  1 to 16 ranks.
* Two gloo ranks, each stepping its share of a set of small lid-driven
  cavities with the oracle, gather exactly the per-cavity results of one
  rank stepping them all.
"""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from lbm_gb300 import cases, shard

CAVITY_SIDES = [6, 9, 14, 7, 11, 20, 8, 12, 16, 10, 5, 13]
CAVITY_STEPS = 40


@pytest.mark.parametrize("world", [1, 2, 3, 4, 8, 16])
def test_cavity_shares_cover_every_domain_once_and_balance(world):
    c = cases.cavities()
    cells = c["sides"].astype(np.int64) ** 2
    ranges = shard.partition(cells, world)
    assert len(ranges) == world
    assert ranges[0][0] == 0 and ranges[-1][1] == len(cells)
    for (lo, hi), (lo2, _) in zip(ranges, ranges[1:]):
        assert lo < hi == lo2
    covered = np.concatenate([np.arange(lo, hi) for lo, hi in ranges])
    assert np.array_equal(covered, np.arange(len(cells)))
    assert shard.balance(cells, ranges) <= 0.05


def test_partition_edge_cases():
    assert shard.partition([5, 1, 1, 1], 3) == [(0, 1), (1, 2), (2, 4)]
    assert shard.partition([1, 1], 4) == [(0, 0), (0, 1), (1, 1), (1, 2)]
    assert shard.partition([], 2) == [(0, 0), (0, 0)]
    with pytest.raises(ValueError):
        shard.partition([1, 2], 0)


def _solve_cavities(lo, hi):
    """Per-cavity results of the oracle's FP64 cavity runs: mass, kinetic
    energy and the residual of the last step."""
    import oracle

    out = {"mass": [], "energy": [], "residual": []}
    for n in CAVITY_SIDES[lo:hi]:
        tau = 3.0 * 0.1 * n / 100.0 + 0.5
        wv = np.zeros((6, 3))
        wv[3, 0] = 0.1
        o = oracle.BoxOracle(2, (n, n, 1), 1.0 / tau, faces=("wall",) * 6, wall_velocity=wv, deviation=True)
        o.init_equilibrium()
        o.step(CAVITY_STEPS - 1)
        r0, u0 = o.moments()
        o.step(1)
        r1, u1 = o.moments()
        out["mass"].append(r1.sum())
        out["energy"].append(0.5 * float((r1 * (u1 ** 2).sum(axis=0)).sum()))
        out["residual"].append(np.abs(r1 - r0).sum() + np.abs(u1 - u0).sum())
    return {k: np.asarray(v, dtype=np.float64) for k, v in out.items()}


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    cells = [n * n for n in CAVITY_SIDES]
    lo, hi = shard.partition(cells, world)[rank]
    res = shard.run_sharded(cells, _solve_cavities, dist)
    q.put((rank, (lo, hi), {k: v.tolist() for k, v in res.items()}))
    dist.destroy_process_group()


def test_two_gloo_ranks_gather_the_one_rank_results():
    one = shard.run_sharded([n * n for n in CAVITY_SIDES], _solve_cavities, None)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    shares = sorted(r[1] for r in got)
    assert shares[0][0] == 0 and shares[0][1] == shares[1][0] and shares[1][1] == len(CAVITY_SIDES)
    assert shares[0][1] > shares[0][0] and shares[1][1] > shares[1][0]  # both ranks worked
    for _, _, res in got:
        for k, v in one.items():
            assert np.array_equal(np.asarray(res[k]), v), k
