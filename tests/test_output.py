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


@pytest.mark.parametrize("name", ["cavity_small_100", "poisson2d_helmholtz_small_100"])
def test_matches_reference_vtk_output(name, tmp_path):
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
    mine = write_vtp(str(tmp_path / "solution"), grid.centers.reshape(grid.ncells, grid.ndim), arrays)
    ref = os.path.join(GOLD, f"{name}_ref.vtp")
    p0, a0 = read_vtp(ref)
    p1, a1 = read_vtp(mine)
    assert np.array_equal(p0, p1)
    assert sorted(a0) == sorted(a1)
    for k in a0:
        assert np.array_equal(a0[k], a1[k]), k
    assert _tags(open(ref).read()) == _tags(open(mine).read())
