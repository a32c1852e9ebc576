"""Error paths of the engines on the GPU, without a GPU fault.

* A NaN population written from the host surfaces as LBM_ERR_DIVERGED from
  the residual, as the reference flags a NaN residual
  (src/lbm/solver.cpp:254-259) and scans the state for NaN / Inf
  (src/lbm/solver.cpp:817-825); the context stays usable.
* A bounded device wait that runs out: the staged step kernels' pipeline
  waits are given a 1 ms limit and every CTA's first segment (row) is left
  unarmed (a barrier nothing completes), so the waits run out; the step call
  returns LBM_ERR_TIMEOUT and the context steps correctly afterwards.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from helpers import load_case, rel_l2
from lbm_gb300._lib import LBMError, load
from lbm_gb300.solver import BoxSolver, TableSolver
from test_box_gpu import make_pair

pytestmark = pytest.mark.gpu

DIVERGED, TIMEOUT = -5, -6


@pytest.mark.parametrize("case", ["poiseuille_50", "couette_bnd_NEEM_50", "poisson1D_reaction_50"])
def test_table_engine_nan_population_reports_divergence(case):
    meta, solver, grid, out, consts, bnds, forcing = load_case(case)
    g = TableSolver(consts, grid, bnds, forcing)
    g.initial_condition()
    g.step(5)
    f = g.populations().reshape(grid.ncells, g.q)
    f[grid.ncells // 2, 0] = np.nan
    g.set_populations(f.reshape(-1))
    g.step(2)
    with pytest.raises(LBMError) as e:
        g.residual()
    assert e.value.code == DIVERGED
    # the context is still usable
    g.initial_condition()
    g.step(3)
    assert np.all(np.isfinite(g.residual()))


@pytest.mark.parametrize("storage", ["f64", "f32", "f16dev"])
@pytest.mark.parametrize("value", [np.nan, np.inf])
def test_box_engine_nonfinite_population_reports_divergence(storage, value):
    g, _ = make_pair("d3q19_sphere_open", storage)
    g.initial_condition()
    g.step(4)
    f = g.populations()
    f[3, f.shape[1] // 2 + 5] = value
    g.set_populations(f)
    g.step(3)
    with pytest.raises(LBMError) as e:
        g.residual()
    assert e.value.code == DIVERGED
    g.initial_condition()
    g.step(3)
    assert np.all(np.isfinite(g.residual()))


@pytest.mark.parametrize("storage", ["f64", "f16dev"])
@pytest.mark.parametrize("kernel", ["staged", "rows"])
def test_staged_kernel_wait_timeout_reports_timeout(storage, kernel):
    g, o = make_pair("d3q19_long_rows", storage)
    try:
        g.kernel(kernel)
    except LBMError:
        pytest.skip(f"this box does not qualify for the {kernel} kernel in {storage}")
    lib = load()
    assert lib.lbm_gpu_box_test_wait(g.ctx, 1_000_000, 1) == 0  # 1 ms per wait, first segments never armed
    g.initial_condition()
    with pytest.raises(LBMError) as e:
        g.step(4)  # two plain steps, then the two halves of a residual step
    assert e.value.code == TIMEOUT
    # out-of-range settings are rejected
    assert lib.lbm_gpu_box_test_wait(g.ctx, 0, 0) == -1
    assert lib.lbm_gpu_box_test_wait(g.ctx, 1_000_000, 2) == -1
    # back to the defaults: the same context steps correctly
    assert lib.lbm_gpu_box_test_wait(g.ctx, 500_000_000, 0) == 0
    g.initial_condition()
    o.init_equilibrium(1.0, (0, 0, 0))
    g.step(45)
    o.step(45)
    if storage == "f64":
        assert rel_l2(g.populations(), o.populations()) <= 1e-12
    else:
        ref, _ = make_pair("d3q19_long_rows", storage)
        ref.kernel("thread")
        ref.initial_condition()
        ref.step(45)
        assert np.array_equal(g.populations(), ref.populations())


# A channel with pressure boundaries and an obstacle on a multi-level grid
# (partitioning level 2, uniform 3, boundary cells refined to 5): on the
# refined levels some -x / +x boundary cells have no second cell inside.
PRESSURE_MULTILEVEL = {
    "dim": 2, "partitionLevel": 2, "uniformLevel": 3, "maxRfnmtLvl": 5, "maxNoCells": 100000,
    "geometry": {"cube": {"type": "box", "body": "fluid", "A": [0.0, 0.0], "B": [4.0, 2.0]},
                 "obstacle": {"type": "sphere", "body": "fluid", "subtract": True, "center": [1.3, 1.05], "radius": 0.35}},
    "solver": {"type": "lbm", "relaxation": 0.8, "ma": 0.1, "maxSteps": 10,
               "boundary": {"cube": {"-x": {"type": "pressure", "pressure": 1.0000008}, "+x": {"type": "pressure", "pressure": 1.0},
                                     "-y": {"type": "wall", "model": "bounceback"}, "+y": {"type": "wall", "model": "bounceback"}},
                            "obstacle": {"all": {"type": "wall", "model": "bounceback"}}}}}


def test_multilevel_boundary_without_its_stencil_is_refused():
    """Boundary conditions whose stencil leaves the grid on a multi-level
    grid are refused when the table is uploaded (LBM_ERR_TABLE), before any
    kernel runs.  The reference does not check this for the pressure
    boundary: it reads the neighbour table at index -1 there
    (src/lbm/bnd/bnd_pressure.h:73-78)."""
    from lbm_gb300 import gridgen
    from lbm_gb300.solver import LBMSolver

    g = gridgen.grid_tables(PRESSURE_MULTILEVEL)
    cells = g.surfaces["cube_-x"]["cells"]
    inside = g.nghbr[cells, 1]
    assert np.any((inside < 0) | (g.nghbr[np.maximum(inside, 0), 1] < 0)), "the case must miss an inside cell"
    with pytest.raises(LBMError) as e:
        LBMSolver.from_config(PRESSURE_MULTILEVEL)
    assert e.value.code == -3
