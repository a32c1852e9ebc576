"""Host mirror of the reference's configuration step (no GPU)."""
import numpy as np
import pytest

from helpers import load_case
from lbm_gb300 import refconfig as rc


def test_boundary_order_is_sorted_json_order():
    _, solver, grid, _, consts, bnds, _ = load_case("poiseuille_bnd_pressure_neem2_50")
    assert [b.name for b in bnds] == ["cube_+x", "cube_+y", "cube_-x", "cube_-y"]
    assert [b.kind for b in bnds] == [rc.BND_PRESSURE_ABB, rc.BND_WALL_NEEM, rc.BND_PRESSURE_ABB, rc.BND_WALL_NEEM]


def test_dummy_periodic_boundaries_are_skipped():
    _, solver, grid, _, consts, bnds, forcing = load_case("poiseuille_1")
    assert [b.kind for b in bnds] == [rc.BND_WALL_BB, rc.BND_WALL_BB]
    assert forcing is not None and forcing.pressure_gradient == 8e-7


def test_reynolds_and_relaxation_are_exclusive():
    _, solver, grid, *_ = load_case("couette_1")
    bad = dict(solver)
    bad["relaxation"] = 0.8
    with pytest.raises(rc.ConfigError):
        rc.solver_constants(bad, grid)


def test_inlet_outlet_types_are_rejected_like_the_reference():
    _, solver, grid, _, consts, *_ = load_case("couette_1")
    bad = dict(solver)
    bad["boundary"] = {"cube": {"+y": {"type": "inlet", "pressure": 1.0}, "-y": {"type": "wall", "model": "bounceback"}}}
    with pytest.raises(rc.ConfigError, match="Broken"):
        rc.boundary_list(bad, grid, consts)


def test_expression_values_follow_the_cell_centres():
    _, solver, grid, _, consts, bnds, _ = load_case("poisson2d_helmholtz_small_100")
    b = [b for b in bnds if b.name == "line_-y"][0]
    x = grid.centers[b.cells][:, 0]
    assert np.allclose(b.values, np.cos(np.pi * x), rtol=0, atol=1e-15)
