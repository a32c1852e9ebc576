"""Loading of the golden reference fixtures in tests/golden/*.npz.

Each fixture holds one run of the SFCMM/LBM reference's own CPU solver (built
from source by oracle/build_ref.sh and driven by oracle/ref_harness.cpp): the
grid tables the solver saw, its JSON ``solver`` block, the initial populations
and the populations / variables / residual after ``steps`` time steps.
tests/golden/make_golden.py writes them.
"""
from __future__ import annotations

import json
import os

import numpy as np

from lbm_gb300.refconfig import GridTables

HERE = os.path.dirname(os.path.abspath(__file__))


def fixture_path(name: str) -> str:
    return os.path.join(HERE, name + ".npz")


def list_fixtures():
    """The LBM fixtures (the particle solver's are lpt_*, the grid
    generator's gridtree_*)."""
    return sorted(f[:-4] for f in os.listdir(HERE) if f.endswith(".npz") and not f.startswith(("lpt_", "gridtree_")))


def list_lpt_fixtures():
    return sorted(f[:-4] for f in os.listdir(HERE) if f.endswith(".npz") and f.startswith("lpt_"))


def load_lpt(name: str):
    """meta, solver block, and the reference's particle state (m_vars layout,
    particles x (3*ndim+5)) before and after ``meta['steps']`` steps, and the
    start locations."""
    z = np.load(fixture_path(name), allow_pickle=False)
    meta = json.loads(str(z["meta"]))
    solver = json.loads(str(z["solver"]))
    nv = meta["nvars"]
    return meta, solver, z["vars0"].reshape(-1, nv), z["vars"].reshape(-1, nv), z["start"].reshape(-1, meta["ndim"])


def load(name: str):
    z = np.load(fixture_path(name), allow_pickle=False)
    meta = json.loads(str(z["meta"]))
    solver = json.loads(str(z["solver"]))
    ndim = meta["ndim"]
    surfaces = {}
    for k, v in meta["surfaces"].items():
        surfaces[k] = {"cells": np.asarray(v["cells"], dtype=np.int64),
                       "normals": np.asarray(v["normals"], dtype=np.float64).reshape(-1, ndim)}
    grid = GridTables(ndim=ndim, centers=z["centers"].reshape(-1, ndim), nghbr=z["nghbr"].reshape(meta["cells"], -1),
                      surfaces=surfaces, bbox=np.asarray(meta["bbox"], dtype=np.float64), cell_length=meta["cellLength"],
                      max_lvl=meta["maxLvl"])
    out = {k: z[k] for k in ("fold0", "fold", "vars", "varsold", "residual")}
    return meta, solver, grid, out
