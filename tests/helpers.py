"""Test helpers shared by the CPU and GPU suites."""
from __future__ import annotations

import numpy as np

import caseio
from lbm_gb300 import refconfig as rc


def load_case(name):
    meta, solver, grid, out = caseio.load(name)
    consts = rc.solver_constants(solver, grid)
    bnds = rc.boundary_list(solver, grid, consts)
    forcing = rc.forcing_desc(solver, grid)
    return meta, solver, grid, out, consts, bnds, forcing


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


def box_index(grid):
    """Map the reference's curve-ordered cells of a uniform 2D grid to (i, j)
    lattice coordinates (x fastest in the dense box)."""
    c = grid.centers
    h = grid.cell_length
    ij = np.rint((c - c.min(axis=0)) / h).astype(np.int64)
    shape = tuple(int(v) for v in ij.max(axis=0) + 1)
    return ij, shape


def channel_sphere_config(level=5, length=32.0, side=16.0, center=(10.0, 8.0, 8.0), radius=3.0):
    """The D3Q19 sphere-channel configuration in the reference's JSON schema:
    a box with a subtracted sphere, equilibrium inlet, zero-gradient outlet and
    free-slip sides (the last three are the box engine's boundary kinds)."""
    return {"dim": 3, "partitionLevel": level, "uniformLevel": level, "maxRfnmtLvl": level,
            "geometry": {"channel": {"type": "box", "A": [0.0, 0.0, 0.0], "B": [length, side, side], "body": "flow"},
                         "sphere": {"type": "sphere", "center": list(center), "radius": radius, "body": "flow", "subtract": True}},
            "solver": {"boundary": {"channel": {"-x": {"type": "inlet", "velocity": [0.05, 0.0, 0.0]}, "+x": {"type": "outlet"},
                                                "-y": {"type": "freeslip"}, "+y": {"type": "freeslip"},
                                                "-z": {"type": "freeslip"}, "+z": {"type": "freeslip"}},
                                    "sphere": {"all": {"type": "wall"}}}}}
