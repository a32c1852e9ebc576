"""The native multi-level grid generator against the reference's own
GridGenerator.

Each tests/golden/gridtree_<case>.npz holds what the reference's generator
built for one config (make_gridtree_golden.py runs it from source): the whole
cell array (partitioning level in curve order, then each finer level), every
cell's centre, level, parent, global id, children, same-level neighbours and
boundary property, and the points file the generator wrote.
lbm_gb300.gridgen.grid_tree builds the tree from the config alone; it must be
equal bit for bit, and save_grid must write the same file byte for byte.
The cases cover partitioning levels 0 to 3 (odd and even), uniform
refinement finer than the partitioning level, boundary refinement,
alignNodesWithSurface on refined and on uniform multi-level grids, disjoint
regions, 1D, and two of the reference's own test geometries.  All host-only: no GPU.
"""
import glob
import json
import os

import numpy as np
import pytest

from lbm_gb300 import _lib, gridgen
from lbm_gb300.refconfig import ConfigError

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(os.path.basename(p)[len("gridtree_"):-len(".npz")]
                  for p in glob.glob(os.path.join(HERE, "golden", "gridtree_*.npz")))
FIELDS = ("centers", "parent", "global_id", "children", "nghbr", "bndry")


def load(name):
    z = np.load(os.path.join(HERE, "golden", f"gridtree_{name}.npz"))
    return json.loads(str(z["config"])), z


def test_fixtures_present():
    assert len(FIXTURES) >= 12


@pytest.mark.parametrize("name", FIXTURES)
def test_tree_equals_the_reference_generator(name):
    cfg, ref = load(name)
    t = gridgen.grid_tree(cfg)
    assert t.partition_level == int(ref["partition_level"])
    assert t.highest_level == int(ref["highest_level"])
    assert np.array_equal(t.level.astype(np.int64), ref["level"])
    for f in FIELDS:
        got, want = getattr(t, f), ref[f]
        assert got.shape == want.shape, f
        assert np.array_equal(got.astype(want.dtype), want), f
    # the child counts the generator's "noChildren" column reports
    assert np.array_equal(t.nchildren, (ref["children"] >= 0).sum(axis=1))


@pytest.mark.parametrize("name", FIXTURES)
def test_points_file_equals_the_reference_generator(name, tmp_path):
    cfg, ref = load(name)
    os.makedirs(tmp_path / cfg.get("outputDir", "out"))
    path = gridgen.save_grid(cfg, str(tmp_path))
    assert os.path.basename(path) == cfg["gridFileName"] + ".csv"
    assert open(path, "rb").read() == ref["points_csv"].tobytes()


def test_fixture_cases_exercise_what_they_name():
    """Sanity of the fixtures themselves: refinement, several levels, the
    alignment's cut of the array to the finest level's size."""
    _, z = load("channel_p3u5m7")
    assert set(z["level"].tolist()) == {3, 4, 5, 6, 7}
    lv = z["level"]
    # levels 6 and 7 refine only boundary cells: fewer than all children
    assert (lv == 6).sum() < 4 * (lv == 5).sum()
    _, z = load("channel_p3u4m6_align")
    # after alignNodesWithSurface the generator keeps as many cells as the
    # finest level holds, counted from the start of the array
    assert z["level"].max() < 6
    _, z = load("channel_p2u6")
    assert set(z["level"].tolist()) == {2, 3, 4, 5, 6}


def test_uniform_tree_matches_the_table_builder():
    """With partitionLevel == uniformLevel == maxRfnmtLvl the tree is one
    level: the cells grid_tables builds, in the same order."""
    cfg, _ = load("poisson2D_l5")
    t = gridgen.grid_tree(cfg)
    g = gridgen.grid_tables(dict(cfg, solver={"boundary": {}}))
    assert np.array_equal(t.centers, g.centers)
    assert np.array_equal(t.nghbr, g.nghbr[:, :4])


def sphere_3d(p, u, m, cells=2_000_000):
    return {"dim": 3, "partitionLevel": p, "uniformLevel": u, "maxRfnmtLvl": m, "maxNoCells": cells,
            "geometry": {"box": {"type": "box", "body": "fluid", "A": [0.0, 0.0, 0.0], "B": [4.0, 2.0, 2.0]},
                         "ball": {"type": "sphere", "body": "fluid", "subtract": True, "center": [1.3, 1.0, 1.05],
                                  "radius": 0.45}}}


def test_uniform_3d_tree_matches_the_table_builder():
    cfg = sphere_3d(5, 5, 5)
    t = gridgen.grid_tree(cfg)
    g = gridgen.grid_tables(dict(cfg, solver={"boundary": {}}))
    assert np.array_equal(t.centers, g.centers)
    assert np.array_equal(t.nghbr, g.nghbr[:, :6])


def check_tree(t, cfg):
    """Structural invariants of a generated tree."""
    D = t.centers.shape[1]
    nn = 2 * D
    h0 = None
    lv = t.level.astype(np.int64)
    # every child sits at its parent's centre plus or minus half its own length
    kids = np.argwhere(t.children >= 0)
    for c, k in kids:
        q = t.children[c, k]
        assert t.parent[q] == c and lv[q] == lv[c] + 1
        sign = np.where((k >> np.arange(D)) & 1, 1.0, -1.0)
        step = t.centers[q] - t.centers[c]
        assert np.all(np.sign(step) == sign)
        if h0 is None:
            h0 = np.abs(step[0]) * 2 ** (lv[q] + 1)
        assert np.allclose(np.abs(step), h0 / 2 ** (lv[q] + 1), rtol=1e-12)
    assert np.array_equal(t.nchildren, (t.children >= 0).sum(axis=1))
    # neighbours: symmetric, same level, one cell length along their axis
    for d in range(nn):
        c = np.flatnonzero(t.nghbr[:, d] >= 0)
        m = t.nghbr[c, d]
        assert np.array_equal(t.nghbr[m, d ^ 1], c)
        assert np.array_equal(lv[m], lv[c])
        delta = t.centers[m, d >> 1] - t.centers[c, d >> 1]
        assert np.all(np.sign(delta) == (1 if d & 1 else -1))
    # levels lie one after another; every cell above the partitioning level has a parent
    assert np.all(np.diff(lv) >= 0)
    assert np.all(t.parent[lv > t.partition_level] >= 0)
    assert np.all(t.parent[lv == t.partition_level] == -1)
    # boundary refinement: below the finest level, past uniformLevel, exactly
    # the boundary cells have children
    u = cfg["uniformLevel"]
    sel = (lv >= u) & (lv < t.highest_level)
    assert np.array_equal(t.nchildren[sel] > 0, t.bndry[sel] == 1)
    sel = lv < u
    assert np.all(t.nchildren[sel] > 0)


def test_refined_3d_tree_is_consistent():
    cfg = sphere_3d(2, 3, 6)
    t = gridgen.grid_tree(cfg)
    assert t.highest_level == 6 and (t.level == 6).sum() > 0
    check_tree(t, cfg)


@pytest.mark.parametrize("name", FIXTURES)
def test_reference_trees_pass_the_same_checks(name):
    cfg, _ = load(name)
    if cfg.get("alignNodesWithSurface"):
        pytest.skip("alignment moves the finest level off the refinement pattern")
    check_tree(gridgen.grid_tree(cfg), cfg)


@pytest.mark.parametrize("name", ["channel_p3u5m7", "channel_p2u6", "line_p2u4m7"])
def test_smallest_array_the_reference_accepts(name):
    """The generator's memory checks against maxNoCells: the smallest array
    the reference builds in builds here, into the same tree (the levels
    below the partitioning level, placed from the array's end, are not part
    of it), and one slot fewer is out of memory as in the reference."""
    cfg, z = load(name)
    need = int(z["min_cells"])
    t = gridgen.grid_tree(dict(cfg, maxNoCells=need))
    for f in FIELDS:
        assert np.array_equal(getattr(t, f).astype(z[f].dtype), z[f]), f
    with pytest.raises(_lib.LBMError) as e:
        gridgen.grid_tree(dict(cfg, maxNoCells=need - 1))
    assert e.value.code == -7


@pytest.mark.parametrize("levels", [(4, 3, 5), (3, 5, 4)])
def test_inconsistent_levels_are_rejected(levels):
    cfg, _ = load("channel_p3u5m7")
    p, u, m = levels
    with pytest.raises(ConfigError):
        gridgen.grid_tree(dict(cfg, partitionLevel=p, uniformLevel=u, maxRfnmtLvl=m))


def test_missing_keys_and_output_setup_are_rejected(tmp_path):
    cfg, _ = load("line_p2u4m7")
    bad = dict(cfg)
    del bad["maxNoCells"]
    with pytest.raises(ConfigError):
        gridgen.grid_tree(bad)
    with pytest.raises(ConfigError):  # the output directory must exist
        gridgen.save_grid(cfg, str(tmp_path))
    os.makedirs(tmp_path / "out")
    with pytest.raises(ConfigError):  # the reference's VTK point writers stop
        gridgen.save_grid(dict(cfg, output={"format": "VTKB"}), str(tmp_path))
