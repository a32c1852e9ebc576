"""Independent domains shared out over ranks, one GPU per rank.

The batched lid-driven cavities and every parameter sweep (Reynolds number,
obstacle placement, Debye length) are sets of independent domains: no
population crosses from one domain to another, so the ranks need no device
collective at all.  Each rank takes one contiguous run of the domain list,
balanced by cell count (the work of a step is proportional to the cells),
steps it on its own GPU, and the host gathers the per-domain results on
every rank afterwards (one object gather over the process group: gloo on
CPU, NCCL between GPUs).

The reference has no counterpart: its grid generator and solver run on one
rank only (src/gridgenerator/gridGenerator.cpp:118-120, src/main.cpp:187-201).
"""
from __future__ import annotations

from typing import Callable, Dict, List, Sequence, Tuple

import numpy as np


def partition(cells: Sequence[int], world: int) -> List[Tuple[int, int]]:
    """Contiguous ranges [lo, hi) of the domain list, one per rank, whose cell
    counts are as close to total / world as a split between two domains
    allows: the k-th boundary is the domain edge nearest to k / world of the
    cumulative cell count.  Ranges are ordered by rank and cover every domain
    once; a rank gets an empty range only when there are fewer domains than
    ranks."""
    if world < 1:
        raise ValueError("world must be >= 1")
    w = np.asarray(cells, dtype=np.float64)
    n = int(w.size)
    if n == 0:
        return [(0, 0)] * world
    if np.any(w < 0):
        raise ValueError("cell counts must be non-negative")
    cum = np.concatenate([[0.0], np.cumsum(w)])
    total = cum[-1]
    bounds = [0]
    for k in range(1, world):
        target = total * k / world
        j = min(int(np.searchsorted(cum, target)), n)  # cum[j] = cells of domains [0, j)
        if j > 0 and abs(cum[j - 1] - target) <= abs(cum[j] - target):
            j -= 1  # the nearer of the two domain edges around the target
        if n >= world:  # ordered, and no rank without a domain
            j = min(max(j, bounds[-1] + 1), n - (world - k))
        else:
            j = min(max(j, bounds[-1]), n)
        bounds.append(j)
    bounds.append(n)
    return [(bounds[r], bounds[r + 1]) for r in range(world)]


def balance(cells: Sequence[int], ranges: List[Tuple[int, int]]) -> float:
    """Largest rank's cells over the mean per rank, minus 1."""
    w = np.asarray(cells, dtype=np.float64)
    loads = np.array([w[lo:hi].sum() for lo, hi in ranges])
    mean = loads.mean()
    return float(loads.max() / mean - 1.0) if mean > 0 else 0.0


def run_sharded(cells: Sequence[int], solve: Callable[[int, int], Dict[str, np.ndarray]], dist=None) -> Dict[str, np.ndarray]:
    """Run ``solve(lo, hi)`` on this rank's share of the domains and gather.

    ``solve`` steps domains [lo, hi) and returns per-domain arrays (first axis
    hi - lo) by name.  With ``dist`` an initialised torch.distributed module
    every rank receives the whole list's arrays, in domain order; without
    one (or with one rank) the call is ``solve(0, n)``."""
    world, rank = 1, 0
    if dist is not None and dist.is_initialized():
        world, rank = dist.get_world_size(), dist.get_rank()
    ranges = partition(cells, world)
    lo, hi = ranges[rank]
    local = {k: np.asarray(v) for k, v in solve(lo, hi).items()}
    for k, v in local.items():
        if v.shape[:1] != (hi - lo,):
            raise ValueError(f"solve: result {k!r} has {v.shape[:1]} rows for {hi - lo} domains")
    if world == 1:
        return local
    parts: List = [None] * world
    dist.all_gather_object(parts, local)
    return {k: np.concatenate([p[k] for p in parts], axis=0) for k in local}
