"""Multi-level grids on the CPU: what the LBM tables and the oracle refuse,
and the solution output's cell filter.

The reference's solver steps every level of a multi-level array as a
lattice of its own.  Refinement can leave a boundary condition without the
cells its stencil reads: the pressure boundary reads two cells inside the
boundary cell (src/lbm/bnd/bnd_pressure.h:73-78; the reference does not
check, it reads its neighbour table at index -1), the Neumann boundary a
second extrapolation cell.  The oracle refuses such grids at set-up, as the
library's table upload does (LBM_ERR_TABLE, test_error_paths_gpu.py).
"""
import json
import os

import numpy as np
import pytest

import oracle
from lbm_gb300 import gridgen
from lbm_gb300 import refconfig as rc
from lbm_gb300.refconfig import ConfigError

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")

PRESSURE_MULTILEVEL = {
    "dim": 2, "partitionLevel": 2, "uniformLevel": 3, "maxRfnmtLvl": 5, "maxNoCells": 100000,
    "geometry": {"cube": {"type": "box", "body": "fluid", "A": [0.0, 0.0], "B": [4.0, 2.0]},
                 "obstacle": {"type": "sphere", "body": "fluid", "subtract": True, "center": [1.3, 1.05], "radius": 0.35}},
    "solver": {"type": "lbm", "relaxation": 0.8, "ma": 0.1, "maxSteps": 10,
               "boundary": {"cube": {"-x": {"type": "pressure", "pressure": 1.0000008}, "+x": {"type": "pressure", "pressure": 1.0},
                                     "-y": {"type": "wall", "model": "bounceback"}, "+y": {"type": "wall", "model": "bounceback"}},
                            "obstacle": {"all": {"type": "wall", "model": "bounceback"}}}}}


def oracle_for(cfg):
    grid = gridgen.grid_tables(cfg)
    consts = rc.solver_constants(cfg["solver"], grid)
    bnds = rc.boundary_list(cfg["solver"], grid, consts)
    return grid, oracle.TableOracle(consts, grid, bnds, rc.forcing_desc(cfg["solver"], grid))


def test_pressure_boundary_without_two_inside_cells_is_refused():
    grid = gridgen.grid_tables(PRESSURE_MULTILEVEL)
    cells = grid.surfaces["cube_-x"]["cells"]
    inside = grid.nghbr[cells, 1]
    assert np.any((inside < 0) | (grid.nghbr[np.maximum(inside, 0), 1] < 0))
    with pytest.raises(ValueError, match="rejected"):
        oracle_for(PRESSURE_MULTILEVEL)


def test_the_same_channel_on_one_level_is_accepted():
    cfg = dict(PRESSURE_MULTILEVEL, partitionLevel=5, uniformLevel=5, maxRfnmtLvl=5)
    grid, o = oracle_for(cfg)
    o.initial_condition()
    o.step(3)
    assert np.isfinite(o.state()[0]).all()


def test_neumann_boundary_without_its_second_cell_is_refused():
    """The own D2Q5 Poisson case with a Neumann face, refined (levels 2, 3,
    boundary cells to 5); the reference aborts on it with a corrupted heap."""
    cfg = json.load(open(os.path.join(GOLD, "cases", "poisson2d_d2q5_small.json")))
    cfg.update({"partitionLevel": 2, "uniformLevel": 3, "maxRfnmtLvl": 5})
    with pytest.raises(ValueError, match="rejected"):
        oracle_for(cfg)


def test_periodic_boundary_condition_on_a_multilevel_grid_is_refused():
    cfg = json.load(open(os.path.join(GOLD, "cases", "channel_mixed_small.json")))
    cfg.update({"partitionLevel": 2, "uniformLevel": 3, "maxRfnmtLvl": 5})
    with pytest.raises(ConfigError, match="generateBndry"):
        gridgen.grid_tables(cfg)


def test_output_cell_filters():
    configs = json.load(open(os.path.join(GOLD, "grid_configs.json")))
    g = gridgen.grid_tables(configs["cavity_p2u3m5"])
    lv = g.level.astype(int)
    assert (g.partition_lvl, g.highest_lvl) == (2, 5)
    leaf = g.output_cells({})
    assert np.array_equal(leaf, np.flatnonzero(g.nchildren == 0))
    assert np.array_equal(g.output_cells({"cellFilter": {"cellFilter": "highestLvl"}}), np.flatnonzero(lv == 5))
    assert np.array_equal(g.output_cells({"cellFilter": {"cellFilter": "partitionLvl"}}), np.flatnonzero(lv == 2))
    assert np.array_equal(g.output_cells({"cellFilter": {"cellFilter": "targetLvl", "outputLvl": 4}}), np.flatnonzero(lv == 4))
    with pytest.raises(ConfigError):
        g.output_cells({"cellFilter": {"cellFilter": "targetLvl", "outputLvl": 1}})
    with pytest.raises(ConfigError):
        g.output_cells({"cellFilter": {"cellFilter": "someLvl"}})
    # every cell of a uniform grid, whatever the filter
    u = gridgen.grid_tables(configs["cavity_small"])
    assert u.level is None and np.array_equal(u.output_cells({}), np.arange(u.ncells))
