"""Solution output (the reference's binary VTK PolyData file).

* Round trip of the writer.
* Against the reference's own file for the same state: the fixture's final
  populations (cavity_small_100, poisson2d_helmholtz_small_100) go through the
  oracle's moment update (bitwise the reference's updateMacroscopicValues),
  the writer produces the file, and every array -- points, connectivity,
  offsets, U, V, rho / V -- equals the reference file's, with the same XML
  element sequence.
"""
import os
import re

import numpy as np
import pytest

import caseio
import oracle
from lbm_gb300 import refconfig as rc
from lbm_gb300.output import read_vtp, solution_arrays, write_vtp

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_writer_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    pts = rng.random((37, 2))
    a, b = rng.normal(size=37), rng.normal(size=37)
    path = write_vtp(str(tmp_path / "x"), pts, [("U", a), ("rho", b)], match_reference=False)
    p, arrs = read_vtp(path)
    assert np.array_equal(p[:, :2], pts.astype(np.float32)) and np.all(p[:, 2] == 0)
    assert np.array_equal(arrs["U"], a) and np.array_equal(arrs["rho"], b)
    assert np.array_equal(arrs["connectivity"], np.arange(37)) and arrs["offsets"][0] == 37


def test_reference_rounding_equals_the_text_round_trip():
    from lbm_gb300.output import reference_rounding

    rng = np.random.default_rng(1)
    v = np.concatenate([rng.normal(size=20000) * 10.0 ** rng.integers(-12, 1, size=20000), rng.uniform(-20, 20, 2000),
                        np.array([0.0, -0.0, 1.0, 0.5e-15, 1.5e-15, 2.5e-15, 7.999999999999999, 8.0])])
    text = np.char.mod("%.15f", v).astype(np.float64)
    assert np.array_equal(reference_rounding(v), text)


def _tags(text):
    return [re.sub(r"\s+", " ", t).strip() for t in re.findall(r"<[^>]+>", text)]


@pytest.mark.parametrize("name", ["cavity_small_100", "poisson2d_helmholtz_small_100", "cavity_p2u3m5_100"])
def test_matches_reference_vtk_output(name, tmp_path):
    """The solution file of the reference's output (src/lbm/solver.cpp:322-384)
    from the oracle's state: array for array, and tag for tag.  On the
    multi-level grid (cavity_p2u3m5) the file holds the leaf cells only, the
    solver's default "cellFilter" (GridTables.output_cells)."""
    import json

    from lbm_gb300 import gridgen

    meta, solver, grid, out = caseio.load(name)
    consts = rc.solver_constants(solver, grid)
    bnds = rc.boundary_list(solver, grid, consts)
    o = oracle.TableOracle(consts, grid, bnds, rc.forcing_desc(solver, grid) if "forcing" in solver else None)
    o.initial_condition()
    o.step(meta["steps"])
    o.update_moments()
    v = o.state()[2].reshape(grid.ncells, consts.nvar)
    if consts.equation == rc.EQ_NAVIER_STOKES:
        arrays = solution_arrays(grid.ndim, rho=v[:, grid.ndim], u=[v[:, d] for d in range(grid.ndim)])
    else:
        arrays = solution_arrays(grid.ndim, phi=v[:, 0])
    configs = json.load(open(os.path.join(GOLD, "grid_configs.json")))
    keep = gridgen.grid_tables(configs[name.rsplit("_", 1)[0]]).output_cells(solver)
    assert (keep.size < grid.ncells) == (name == "cavity_p2u3m5_100")
    arrays = [(k, a[keep]) for k, a in arrays]
    mine = write_vtp(str(tmp_path / "solution"), grid.centers.reshape(grid.ncells, grid.ndim)[keep], arrays)
    ref = os.path.join(GOLD, f"{name}_ref.vtp")
    p0, a0 = read_vtp(ref)
    p1, a1 = read_vtp(mine)
    assert np.array_equal(p0, p1)
    assert sorted(a0) == sorted(a1)
    for k in a0:
        assert np.array_equal(a0[k], a1[k]), k
    assert _tags(open(ref).read()) == _tags(open(mine).read())


# ---- line probes (the reference's post-processing line.csv) -----------------

LINES = [
    ("cavity_small", 100, "x0p53", [0.53125, 0.0], [0.53125, 1.0]),
    ("cavity_small", 100, "diag", [0.0, 0.0], [1.0, 1.0]),
    ("poisson2d_helmholtz_small", 100, "y0p41", [0.0, 0.40625], [1.0, 0.40625]),
    ("channel_mixed_small", 100, "x1p06", [1.0625, 0.0], [1.0625, 1.0]),
]


@pytest.mark.parametrize("name,steps,tag,a,b", LINES)
def test_line_probe_matches_reference_file(name, steps, tag, a, b, tmp_path):
    """Cell selection, order and formatting of the line probe against the
    reference's own line.csv for the same state: the fixture's vars after the
    steps (the reference's m_vars) through line_cells and write_line_csv give
    the reference's file byte for byte."""
    import json

    from lbm_gb300.output import line_cells, write_line_csv

    d = np.load(os.path.join(GOLD, f"{name}_{steps}.npz"))
    meta = json.loads(str(d["meta"]))
    centers = d["centers"].reshape(-1, meta["ndim"])
    v = d["vars"].reshape(-1, meta["nvar"])
    cells = line_cells(centers, 0.5 * meta["cellLength"], a, b)
    mine = write_line_csv(str(tmp_path / "line"), centers[cells], v[cells, 0])
    with open(mine) as fh, open(os.path.join(GOLD, f"{name}_{steps}_line_{tag}.csv")) as gh:
        assert fh.read() == gh.read()


def _brute_line(shape, h, a, b):
    from lbm_gb300.output import line_cells

    nx, ny, nz = (tuple(shape) + (1, 1))[:3]
    nd = 2 if nz == 1 else 3
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    cent = (np.stack([x.ravel(), y.ravel(), z.ravel()], 1)[:, :nd] + 0.5) * h
    return line_cells(cent, 0.5 * h, a, b)


def test_box_line_cells_match_a_scan_of_every_cell():
    """box_line_cells (a few cells per layer along the line) selects and
    orders exactly what testing every cell of the box selects."""
    from lbm_gb300.output import box_line_cells

    rng = np.random.default_rng(3)
    for trial in range(120):
        nd = 2 + trial % 2
        shape = tuple(int(v) for v in rng.integers(3, 12, size=nd)) + (1,) * (3 - nd)
        h = float(rng.choice([1.0, 0.25]))
        ext = np.array(shape[:nd]) * h
        a = rng.uniform(-0.5, 1.5, nd) * ext
        b = rng.uniform(-0.5, 1.5, nd) * ext
        if trial % 4 == 0:  # axis-parallel through cell centres
            a = (np.floor(a / h) + 0.5) * h
            b = a.copy()
            b[trial % nd] += 3 * h
        assert np.array_equal(box_line_cells(shape, h, a, b), _brute_line(shape, h, a, b)), (trial, shape, a, b)


def test_line_csv_format(tmp_path):
    """Header of coordinate names and 'u'; coordinates at precision 15 in the
    shortest form, values in fixed notation with 15 decimals."""
    from lbm_gb300.output import write_line_csv

    p = write_line_csv(str(tmp_path / "l"), np.array([[0.03125, 1.0 / 3.0], [2.5, 1e-7]]), np.array([-1.0 / 3.0, 5e-17]))
    with open(p) as fh:
        assert fh.read() == "x,y,u\n0.03125,0.333333333333333,-0.333333333333333\n2.5,1e-07,0.000000000000000\n"
