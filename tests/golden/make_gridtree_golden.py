"""Regenerate the multi-level grid fixtures from the reference's own grid
generator.

Run in a container that has the reference sources (the GPU hosts do not):

    oracle/build_ref.sh && python tests/golden/make_gridtree_golden.py

For every case below it runs oracle/_ref/ref_gridgen_harness (the
reference's GridGenerator, built from source) and stores in
tests/golden/gridtree_<case>.npz the config it ran (JSON text), the
generator's cell arrays (centres, levels, parents, global ids, children,
same-level neighbours, boundary property) and the points file the generator
wrote itself (<outputDir>/<gridFileName>.csv); for a few cases also the
smallest "maxNoCells" the generator accepts.  The configs are written here
in the reference's schema, or taken from the reference's own test configs
with the grid levels changed; the output block is set to the one format the
generator writes (ASCII points with the level and child-count columns).
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_gridgen_harness")
REF = subprocess.run([os.path.join(ROOT, "oracle", "build_ref.sh"), "--root"], capture_output=True, text=True,
                     check=True).stdout.strip()

OUTPUT = {"format": "ASCII", "cellFilter": "leafCells", "type": "points", "outputValues": ["level", "noChildren"]}
CHANNEL = {"cube": {"type": "box", "body": "flowregion", "A": [0.0, 0.0], "B": [10.0, 4.0]},
           "sphere": {"type": "sphere", "body": "flowregion", "subtract": True, "center": [3.1, 2.05], "radius": 0.8}}


HOLE = {"cube": {"type": "box", "body": "f", "A": [0.0, 0.0], "B": [3.0, 1.0]},
        "hole": {"type": "sphere", "body": "f", "subtract": True, "center": [1.1, 0.45], "radius": 0.2}}


def levels(p, u, m, cells=400000):
    return {"partitionLevel": p, "uniformLevel": u, "maxRfnmtLvl": m, "maxNoCells": cells}


# (fixture name, base config: ("own", dict) or ("ref", path), overrides)
CASES = [
    # channel with a subtracted cylinder: odd partitioning level (root at the
    # array's end), uniform then boundary refinement
    ("channel_p3u5m7", ("own", {"dim": 2, "geometry": CHANNEL}), levels(3, 5, 7)),
    # even partitioning level, boundary refinement straight from it
    ("channel_p2u2m6", ("own", {"dim": 2, "geometry": CHANNEL}), levels(2, 2, 6)),
    # uniform grid finer than its partitioning level (children in parent order)
    ("channel_p2u6", ("own", {"dim": 2, "geometry": CHANNEL}), levels(2, 6, 6)),
    # boundary refinement, then the finest level stretched onto the surface
    ("channel_p3u4m6_align", ("own", {"dim": 2, "geometry": CHANNEL, "alignNodesWithSurface": True}), levels(3, 4, 6)),
    # two disjoint discs: two regions for the flood fill, two bodies
    ("discs_p3u4m6", ("own", {"dim": 2, "geometry": {
        "a": {"type": "sphere", "center": [1.0, 1.0], "radius": 0.9},
        "b": {"type": "sphere", "center": [3.5, 1.3], "radius": 0.6}}}), levels(3, 4, 6)),
    # 1D line
    ("line_p2u4m7", ("own", {"dim": 1, "geometry": {"line": {"type": "box", "A": [0.0], "B": [3.3]}}}), levels(2, 4, 7)),
    # the reference's backward-facing step (one body of three boxes)
    ("step_p3u4m6", ("ref", "test/step/step_ns.json"), levels(3, 4, 6)),
    # the reference's 2D Poisson square with its alignNodesWithSurface
    ("poisson2D_p2u3m6", ("ref", "test/poisson/poisson2D.json"), levels(2, 3, 6)),
    ("poisson2D_l5", ("ref", "test/poisson/poisson2D.json"), levels(5, 5, 5)),
    # partitioning levels 0 and 1 (the root itself, or its children, in
    # curve order), and a uniform multi-level grid stretched by the alignment
    ("hole_p0u3m5", ("own", {"dim": 2, "geometry": HOLE}), levels(0, 3, 5)),
    ("hole_p1u1m4", ("own", {"dim": 2, "geometry": HOLE}), levels(1, 1, 4)),
    ("hole_p2u5_align", ("own", {"dim": 2, "geometry": HOLE, "alignNodesWithSurface": True}), levels(2, 5, 5)),
]


# cases whose smallest "maxNoCells" the generator accepts is recorded too
# (found by bisection; the generator stops with "Out of memory" below it)
MIN_CELLS_CASES = {"channel_p3u5m7", "channel_p2u6", "line_p2u4m7"}


def runs(cfg):
    """Whether the reference generator builds the config."""
    with tempfile.TemporaryDirectory() as tmp:
        os.makedirs(os.path.join(tmp, "out"))
        os.makedirs(os.path.join(tmp, "dump"))
        path = os.path.join(tmp, "cfg.json")
        with open(path, "w") as f:
            json.dump(cfg, f)
        r = subprocess.run([HARNESS, path, os.path.join(tmp, "dump")], cwd=tmp, capture_output=True, text=True)
        if r.returncode != 0 and "Out of memory" not in r.stdout + r.stderr:
            raise RuntimeError(f"harness failed for another reason\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
        return r.returncode == 0


def min_cells(cfg):
    lo, hi = 1, int(cfg["maxNoCells"])  # lo fails, hi builds
    assert runs(cfg) and not runs(dict(cfg, maxNoCells=lo))
    while hi - lo > 1:
        mid = (lo + hi) // 2
        if runs(dict(cfg, maxNoCells=mid)):
            hi = mid
        else:
            lo = mid
    return hi


def run_case(name, base, overrides):
    kind, src = base
    cfg = json.load(open(os.path.join(REF, src))) if kind == "ref" else dict(src)
    cfg.update(overrides)
    cfg.update({"outputDir": "out", "gridFileName": "grid", "output": OUTPUT})
    extra = {"min_cells": min_cells(cfg)} if name in MIN_CELLS_CASES else {}
    with tempfile.TemporaryDirectory() as tmp:
        os.makedirs(os.path.join(tmp, "out"))
        os.makedirs(os.path.join(tmp, "dump"))
        path = os.path.join(tmp, "cfg.json")
        with open(path, "w") as f:
            json.dump(cfg, f, indent=1)
        r = subprocess.run([HARNESS, path, os.path.join(tmp, "dump")], cwd=tmp, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"{name}: harness failed\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
        d = os.path.join(tmp, "dump")
        meta = json.load(open(os.path.join(d, "meta.json")))
        n, nd = meta["n"], meta["ndim"]
        arrays = {
            "centers": np.fromfile(os.path.join(d, "centers.f64")).reshape(n, nd),
            "level": np.fromfile(os.path.join(d, "level.i64"), np.int64),
            "parent": np.fromfile(os.path.join(d, "parent.i64"), np.int64),
            "global_id": np.fromfile(os.path.join(d, "global.i64"), np.int64),
            "children": np.fromfile(os.path.join(d, "children.i64"), np.int64).reshape(n, 1 << nd),
            "nghbr": np.fromfile(os.path.join(d, "nghbr.i64"), np.int64).reshape(n, 2 * nd),
            "bndry": np.fromfile(os.path.join(d, "bndry.u8"), np.uint8),
        }
        csv = open(os.path.join(tmp, "out", "grid.csv"), "rb").read()
    out = os.path.join(HERE, f"gridtree_{name}.npz")
    np.savez_compressed(out, config=np.array(json.dumps(cfg, sort_keys=True)),
                        partition_level=meta["partitionLvl"], highest_level=meta["currentHighestLvl"],
                        points_csv=np.frombuffer(csv, dtype=np.uint8), **arrays, **extra)
    print(f"{name}: {n} cells, levels {meta['partitionLvl']}-{meta['currentHighestLvl']} {extra} -> {os.path.basename(out)}")


def main(argv):
    if not os.path.exists(HARNESS):
        sys.exit("oracle/_ref/ref_gridgen_harness not built (run oracle/build_ref.sh)")
    want = set(argv[1:])
    for name, base, overrides in CASES:
        if not want or name in want:
            run_case(name, base, overrides)


if __name__ == "__main__":
    main(sys.argv)
