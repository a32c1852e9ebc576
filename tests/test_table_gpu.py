"""Reference-table engine on the GPU against the reference's own CPU solver.

Every golden fixture (tests/golden/) is replayed through the C ABI: same grid
tables, same JSON, same number of steps.  The bar is relative L2 <= 1e-12 on
the populations (the engine is built to reproduce the reference bit for bit,
and the test also records whether it does), on the variables, and on the
residual, whose FP64 summation order differs from the reference's loop.
"""
import json
import os

import numpy as np
import pytest

import caseio
from helpers import load_case, rel_l2
from lbm_gb300.solver import LBMSolver, TableSolver
from lbm_gb300._lib import LBMError

pytestmark = pytest.mark.gpu
FIXTURES = caseio.list_fixtures()
TOL = 1e-12


@pytest.mark.parametrize("name", FIXTURES)
def test_table_engine_matches_reference(name):
    meta, solver, grid, out, consts, bnds, forcing = load_case(name)
    g = TableSolver(consts, grid, bnds, forcing)
    g.initial_condition()
    assert rel_l2(g.populations(), out["fold0"]) <= TOL
    g.step(meta["steps"])
    fold = g.populations()
    assert rel_l2(fold, out["fold"]) <= TOL
    assert rel_l2(g.vars(), out["vars"]) <= TOL
    assert rel_l2(g.varsold(), out["varsold"]) <= TOL
    r = g.residual()
    assert np.allclose(r, out["residual"], rtol=TOL, atol=1e-300)
    # the engine keeps the reference's operation order: populations are bitwise equal
    assert np.array_equal(fold, out["fold"]), f"max diff {np.abs(fold - out['fold']).max():.3e}"


GRID_CONFIGS = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "grid_configs.json")))


@pytest.mark.parametrize("name", FIXTURES)
def test_run_from_json_config_alone(name):
    """The reference's JSON config alone (grid keys, geometry, solver block):
    the native grid build (lbm_gb300.gridgen) feeds the GPU engine, and the
    populations after the fixture's steps equal the reference's bit for bit."""
    meta, solver, _, out = caseio.load(name)
    cfg = dict(GRID_CONFIGS[name.rsplit("_", 1)[0]])
    cfg["solver"] = solver
    s = LBMSolver.from_config(cfg)
    s.gpu.initial_condition()
    s.gpu.step(meta["steps"])
    assert np.array_equal(s.gpu.populations(), out["fold"])
    assert rel_l2(s.gpu.vars(), out["vars"]) <= TOL


def test_chunked_stepping_equals_one_call():
    meta, solver, grid, out, consts, bnds, forcing = load_case("poiseuille_50")
    a = TableSolver(consts, grid, bnds, forcing)
    b = TableSolver(consts, grid, bnds, forcing)
    a.initial_condition()
    b.initial_condition()
    a.step(50)
    for n in (1, 7, 2, 8, 16, 16):
        b.step(n)
    assert np.array_equal(a.populations(), b.populations())


def test_mass_momentum_reduction():
    meta, solver, grid, out, consts, bnds, forcing = load_case("couette_50")
    g = TableSolver(consts, grid, bnds, forcing)
    g.initial_condition()
    g.step(50)
    f = g.populations().reshape(grid.ncells, 9)
    c = np.array([[-1, 0], [1, 0], [0, -1], [0, 1], [1, 1], [1, -1], [-1, -1], [-1, 1], [0, 0]], dtype=np.float64)
    mm = g.mass_momentum()
    assert np.isclose(mm[0], f.sum(), rtol=1e-13)
    assert np.allclose(mm[1:], f @ c @ np.ones(1) if False else (f @ c).sum(axis=0), rtol=1e-10, atol=1e-14)


def test_bad_tables_fail_loudly():
    meta, solver, grid, out, consts, bnds, forcing = load_case("couette_1")
    g = TableSolver(consts, grid, [], None)
    bad = bnds[0]
    bad.cells = bad.cells.copy()
    bad.cells[0] = grid.ncells + 5
    with pytest.raises(LBMError) as ei:
        g.add_boundary(bad)
    assert ei.value.code == -3


ANALYTIC_SUITE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "analytic_suite.json")


def _analytic_cases():
    with open(ANALYTIC_SUITE) as fh:
        return json.load(fh)


@pytest.mark.parametrize("name", sorted(_analytic_cases()))
def test_reference_analytic_suite(name):
    """The reference's own analytic test suite (test/run.sh: every case whose
    config carries analyticalSolution): LBMSolver.run() on the GPU, on the grid
    built natively from the case's JSON config, stops after exactly the
    reference's number of steps (at convergence, or at maxSteps where the
    reference does not converge either), passes the reference's bounds
    (compareToAnalyticalResult, src/lbm/solver.cpp:387-482), and reports the
    reference's own max / L2 / GRE errors (the values the reference's run()
    printed, tests/golden/analytic_suite.json) to 1e-10 relative or 1e-14
    absolute."""
    from lbm_gb300.solver import LBMSolver

    e = _analytic_cases()[name]
    s = LBMSolver.from_config(e["config"])
    res = s.run()
    # the reference either reached its convergence criterion or ran to maxSteps
    assert res["converged"] == (e["converged_to"] is not None) and not res["diverged"], res
    assert res["steps"] == e["steps"], (res["steps"], e["steps"])
    cmp = s.compare_to_analytical()
    assert cmp["passed"], cmp
    # 1e-10 relative; where the errors themselves sit at the rounding level of
    # the velocities (the converged Couette cases, max error ~1e-12 on
    # velocities of ~0.1) the last bits of the analytic profile decide them,
    # and 1e-14 absolute is the bar
    for k in ("max", "l2", "gre"):
        ref = e[k]
        if ref is None:
            continue
        assert abs(cmp[k] - ref) <= max(1e-10 * abs(ref), 1e-14), (k, cmp[k], ref)


@pytest.mark.parametrize("name", ["cavity_small_100", "poisson2d_helmholtz_small_100"])
def test_solution_output_matches_reference_file(name, tmp_path):
    """LBMSolver.write_solution after the fixture's steps on the GPU writes
    the reference's own VTK file (same arrays, bit for bit, same layout)."""
    import os

    from lbm_gb300.output import read_vtp
    from lbm_gb300.solver import LBMSolver

    meta, solver, grid, out, consts, bnds, forcing = load_case(name)
    s = LBMSolver(solver, grid)
    s.gpu.initial_condition()
    s.gpu.step(meta["steps"])
    mine = s.write_solution(str(tmp_path / "solution"))
    ref = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", f"{name}_ref.vtp")
    p0, a0 = read_vtp(ref)
    p1, a1 = read_vtp(mine)
    assert np.array_equal(p0, p1) and sorted(a0) == sorted(a1)
    for k in a0:
        assert np.array_equal(a0[k], a1[k]), k


def test_multilevel_solution_output_matches_reference_file(tmp_path):
    """On a multi-level grid built from its JSON config (levels 2, 3 and
    boundary cells to 5), write_solution writes the leaf cells, the solver's
    default "cellFilter", as the reference's own file does."""
    import json
    import os

    from lbm_gb300.output import read_vtp
    from lbm_gb300.solver import LBMSolver

    here = os.path.dirname(os.path.abspath(__file__))
    cfg = json.load(open(os.path.join(here, "golden", "grid_configs.json")))["cavity_p2u3m5"]
    meta, solver, _, _, _, _, _ = load_case("cavity_p2u3m5_100")
    s = LBMSolver.from_config(dict(cfg, solver=solver))
    s.gpu.initial_condition()
    s.gpu.step(meta["steps"])
    mine = s.write_solution(str(tmp_path / "solution"))
    p0, a0 = read_vtp(os.path.join(here, "golden", "cavity_p2u3m5_100_ref.vtp"))
    p1, a1 = read_vtp(mine)
    assert p0.shape[0] < meta["cells"]
    assert np.array_equal(p0, p1) and sorted(a0) == sorted(a1)
    for k in a0:
        assert np.array_equal(a0[k], a1[k]), k


LINES = [
    ("cavity_small", 100, "x0p53", [0.53125, 0.0], [0.53125, 1.0]),
    ("cavity_small", 100, "diag", [0.0, 0.0], [1.0, 1.0]),
    ("poisson2d_helmholtz_small", 100, "y0p41", [0.0, 0.40625], [1.0, 0.40625]),
    ("channel_mixed_small", 100, "x1p06", [1.0625, 0.0], [1.0625, 1.0]),
]


@pytest.mark.parametrize("name,steps,tag,a,b", LINES)
def test_line_probe_matches_reference_file(name, steps, tag, a, b, tmp_path):
    """The reference's post-processing line probe after the fixture's steps on
    the GPU: LBMSolver.write_line writes the reference's own line.csv byte for
    byte.  run() with the line in the config's "postprocessing" (executed
    atEnd) writes it after the forced output of the last step has updated the
    variables (src/lbm/solver.cpp:194-199, 335-336), i.e. the probe of the
    updated variables."""
    import copy
    import os

    from lbm_gb300.solver import LBMSolver

    gold = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", f"{name}_{steps}_line_{tag}.csv")
    with open(gold) as fh:
        ref = fh.read()
    meta, solver, grid, out, consts, bnds, forcing = load_case(f"{name}_{steps}")
    s = LBMSolver(solver, grid)
    s.gpu.initial_condition()
    s.gpu.step(meta["steps"])
    with open(s.write_line(str(tmp_path / "line"), a, b)) as fh:
        assert fh.read() == ref
    cfg = copy.deepcopy(solver)
    cfg["postprocessing"] = {"line1": {"type": "line", "execute": "atEnd", "A": a, "B": b}}
    cfg["convergence"] = 0.0
    r = LBMSolver(cfg, grid)
    r.output_dir = str(tmp_path)
    res = r.run(max_steps=steps)
    assert res["steps"] == steps
    s.gpu.update_moments()
    with open(tmp_path / "line.csv") as fh, open(s.write_line(str(tmp_path / "updated"), a, b)) as gh:
        assert fh.read() == gh.read()
