"""The native grid and table build against the reference's own grids.

Every golden fixture holds the grid tables the reference's LBMSolver saw: the
cell centres in curve order, the neighbour table after the periodic wiring and
the diagonal neighbours, and the named boundary surfaces with their normals.
lbm_gb300.gridgen builds them from the case's JSON config alone
(tests/golden/grid_configs.json, written by make_golden.py from the same
configs); they must be equal bit for bit.  The library call is host-only, so
these tests run without a GPU.
"""
import json
import os

import numpy as np
import pytest

import caseio
from helpers import channel_sphere_config
from lbm_gb300 import gridgen
from lbm_gb300.refconfig import ConfigError

HERE = os.path.dirname(os.path.abspath(__file__))
CONFIGS = json.load(open(os.path.join(HERE, "golden", "grid_configs.json")))
FIXTURES = caseio.list_fixtures()


def case_of(fixture):
    return fixture.rsplit("_", 1)[0]


def test_every_fixture_has_its_grid_config():
    assert {case_of(f) for f in FIXTURES} <= set(CONFIGS)


@pytest.mark.parametrize("name", FIXTURES)
def test_grid_tables_equal_the_reference(name):
    _, _, ref, _ = caseio.load(name)
    g = gridgen.grid_tables(CONFIGS[case_of(name)])
    assert g.ndim == ref.ndim
    assert np.array_equal(g.centers, ref.centers)
    assert np.array_equal(g.nghbr, ref.nghbr)
    assert g.cell_length == ref.cell_length
    assert np.array_equal(g.bbox, ref.bbox)
    assert g.max_lvl == ref.max_lvl
    assert sorted(g.surfaces) == sorted(ref.surfaces)
    for k, s in ref.surfaces.items():
        assert np.array_equal(g.surfaces[k]["cells"], s["cells"]), k
        assert np.array_equal(g.surfaces[k]["normals"], s["normals"]), k


def test_obstacle_surface_repeats_cells_with_their_last_normal():
    """The reference's circle surface lists a cell once per missing direction
    but keeps one normal per cell (the last)."""
    g = gridgen.grid_tables(CONFIGS["sphere_ns_l5"])
    s = g.surfaces["sphere"]
    cells = s["cells"].tolist()
    assert len(cells) > len(set(cells))
    for c in set(cells):
        rows = s["normals"][[i for i, x in enumerate(cells) if x == c]]
        assert (rows == rows[0]).all()


def _sphere_box_3d(level=5, r=0.2):
    return {"dim": 3, "partitionLevel": level, "uniformLevel": level, "maxRfnmtLvl": level,
            "geometry": {"box": {"type": "box", "A": [0.0, 0.0, 0.0], "B": [2.0, 1.0, 1.0], "body": "fluid"},
                         "ball": {"type": "sphere", "center": [0.6, 0.5, 0.45], "radius": r, "body": "fluid", "subtract": True}},
            "solver": {"boundary": {"box": {"-x": {"type": "periodic", "generateBndry": False, "connection": "box_+x"},
                                            "+x": {"type": "periodic", "generateBndry": False, "connection": "box_-x"},
                                            "-y": {"type": "wall"}, "+y": {"type": "wall"}, "-z": {"type": "wall"},
                                            "+z": {"type": "wall"}},
                                    "ball": {"all": {"type": "wall"}}}}}


def test_3d_box_with_a_sphere():
    """3D, which the reference cannot build: the cut layer around the box,
    the sphere's cells removed, periodic x wiring, symmetric links and edge
    neighbours consistent with two main steps."""
    level = 5
    g = gridgen.grid_tables(_sphere_box_3d(level))
    h = 2.0 / 2 ** level
    assert g.cell_length == h
    assert g.nghbr.shape[1] == 18
    c = g.centers
    # the box is [0,2]x[0,1]x[0,1]; along y and z the cut layer keeps one row
    # of centres half a cell outside each face (the reference's 2D rule, here
    # on six faces); along x, the longest axis, the root cell spans the box
    # exactly and the outermost centres lie half a cell inside
    for d in (1, 2):
        assert np.isclose(c[:, d].min(), -h / 2) and np.isclose(c[:, d].max(), 1 + h / 2)
    assert np.isclose(c[:, 0].min(), h / 2) and np.isclose(c[:, 0].max(), 2 - h / 2)
    # no centre deep inside the ball
    assert (np.linalg.norm(c - [0.6, 0.5, 0.45], axis=1) > 0.2 - h).all()
    # every cell is unique and sits on the level's lattice
    k = np.round((c + h / 2) / h).astype(np.int64)
    assert len({tuple(x) for x in k.tolist()}) == len(k)
    # main links are symmetric; the x links wrap
    n = g.ncells
    for d in range(6):
        nb = g.nghbr[:, d]
        has = nb >= 0
        assert (g.nghbr[nb[has], d ^ 1] == np.arange(n)[has]).all()
    east = g.nghbr[:, 1]
    wrap = (east >= 0) & (c[np.maximum(east, 0), 0] < c[:, 0])
    assert wrap.sum() > 0 and np.allclose(c[wrap, 0], 2 - h / 2)
    # edge neighbour (+x,+y) is the +y neighbour of the +x neighbour
    px = g.nghbr[:, 1]
    exp = np.where(px >= 0, g.nghbr[np.maximum(px, 0), 3], -1)
    assert np.array_equal(g.nghbr[:, 6 + 3], exp)
    # surfaces: walls on y and z, the ball on its own, periodic x faces
    assert {"box_-y", "box_+y", "box_-z", "box_+z", "box_-x", "box_+x", "ball"} == set(g.surfaces)
    assert len(g.surfaces["ball"]["cells"]) > 0
    assert (g.surfaces["box_+z"]["normals"] == [0, 0, 1]).all()


KAT = json.load(open(os.path.join(HERE, "golden", "hilbert_kat.json")))


def test_curve_index_known_answers():
    """Every known answer of the reference's own curve-index tests
    (UnitTest/test_hilbert.cpp, 2D to 4D)."""
    assert len(KAT) == 125
    for k in KAT:
        assert gridgen.curve_index(k["x"], k["level"]) == k["index"], k


def test_curve_order_is_the_reference_u_order():
    """The first cells of a 2D unit box follow the quadrant order (lo,lo),
    (lo,hi), (hi,hi), (hi,lo) of the reference's curve
    (UnitTest/test_hilbert.cpp pins hilbert::index)."""
    cfg = {"dim": 2, "partitionLevel": 3, "uniformLevel": 3, "maxRfnmtLvl": 3,
           "geometry": {"cube": {"type": "box", "A": [0.0, 0.0], "B": [1.0, 1.0]}}, "solver": {"boundary": {}}}
    g = gridgen.grid_tables(cfg)
    assert g.ncells == 64
    assert g.centers[:4].tolist() == [[0.0625, 0.0625], [0.0625, 0.1875], [0.1875, 0.1875], [0.1875, 0.0625]]


def test_config_errors():
    base = _sphere_box_3d(4)
    bad = dict(base, uniformLevel=5)
    with pytest.raises(ConfigError):
        gridgen.grid_tables(bad)
    bad = json.loads(json.dumps(base))
    bad["geometry"]["box"]["type"] = "stl"
    with pytest.raises(ConfigError):
        gridgen.grid_tables(bad)
    bad = json.loads(json.dumps(base))
    del bad["solver"]["boundary"]["box"]["+x"]
    with pytest.raises(ConfigError):
        gridgen.grid_tables(bad)


def test_box_case_of_a_3d_json_config():
    cfg = channel_sphere_config()
    g = gridgen.grid_tables(cfg)
    b = gridgen.box_case(g, cfg)
    # x: the longest axis, spanned exactly; y, z: the cut layer adds a row each side
    assert b["shape"] == (32, 18, 18)
    assert b["faces"] == ("open", "open", "freeslip", "freeslip", "freeslip", "freeslip")
    assert b["inlet"] == (0.05, 0.0, 0.0)
    assert len(np.unique(b["index"])) == g.ncells
    fl = b["flags"].reshape(18, 18, 32)
    assert (fl[:, :, 0] == gridgen.CELL_INLET).all() and (fl[:, :, -1] == gridgen.CELL_OUTLET).all()
    solid = np.argwhere(fl == gridgen.CELL_SOLID)
    # the solid cells are those the sphere covers whole: all eight vertices inside
    assert len(solid) > 0
    for z, y, x in solid:
        corners = np.array([[x + dx, y - 1 + dy, z - 1 + dz] for dx in (0, 1) for dy in (0, 1) for dz in (0, 1)], dtype=float)
        assert (np.linalg.norm(corners - [10.0, 8.0, 8.0], axis=1) <= 3.0).all()
    assert (fl != gridgen.CELL_SOLID).sum() == g.ncells
    with pytest.raises(ConfigError):
        bad = json.loads(json.dumps(cfg))
        bad["solver"]["boundary"]["channel"]["+y"] = {"type": "pressure"}
        gridgen.box_case(g, bad)


def test_box_case_of_a_2d_reference_config():
    """The reference's cavity config (walls on four sides of a unit box, level
    4): its grid is the 16 x 16 box itself (the longest axis spans the root
    cell), all fluid, every face a wall."""
    cfg = dict(CONFIGS["cavity_small"])
    cfg["solver"] = {"boundary": {"cube": {k: {"type": "wall", "model": "bounceback"} for k in ("-x", "+x", "-y", "+y")}}}
    g = gridgen.grid_tables(cfg)
    b = gridgen.box_case(g, cfg)
    assert b["shape"] == (16, 16, 1)
    assert (b["flags"] == gridgen.CELL_FLUID).all()
    assert b["faces"][:4] == ("wall",) * 4
    assert sorted(b["index"].tolist()) == list(range(256))


def test_particle_config_errors_need_no_gpu():
    from lbm_gb300.lpt import ParticleSolver

    for bad in ({"dt": 1e-3, "gravity": [0, 1], "model": "gravityOnly"},
                {"dt": 1e-3, "gravity": [0, 1], "integrationMethod": "RK4"},
                {"gravity": [0, 1]}):
        with pytest.raises(ConfigError):
            ParticleSolver.from_config(bad, 2)


def test_surface_call_takes_all_pairs_or_none():
    """Counting takes nothing; a buffer too small is refused and takes
    nothing either; a buffer of the counted size takes every pair once."""
    import ctypes as C

    from lbm_gb300._lib import LBM_OK

    cfg = CONFIGS["cavity_small"]
    lib = gridgen._grid_lib()
    descs, names = gridgen.geometry_objects(cfg["geometry"], 2)
    h = C.c_void_p()
    assert lib.lbm_grid_create(2, 4, C.cast(descs, C.c_void_p), len(names), None, C.byref(h)) == LBM_OK
    try:
        n = C.c_int64()
        assert lib.lbm_grid_add_surface(h, 0, 0, 4, None, None, 0, C.byref(n)) == LBM_OK
        total = n.value
        assert total == 4 * 16  # one row of 16 cells on each side of the box
        cells = np.empty(total, dtype=np.int64)
        dirs = np.empty(total, dtype=np.int8)
        assert lib.lbm_grid_add_surface(h, 0, 0, 4, cells.ctypes.data, dirs.ctypes.data, total - 1, C.byref(n)) == -1
        assert lib.lbm_grid_add_surface(h, 0, 0, 4, cells.ctypes.data, dirs.ctypes.data, total, C.byref(n)) == LBM_OK
        assert n.value == total and sorted(set(zip(cells.tolist(), dirs.tolist()))) == sorted(zip(cells.tolist(), dirs.tolist()))
        # now taken: a second surface over the same directions gets nothing
        assert lib.lbm_grid_add_surface(h, 0, 0, 4, None, None, 0, C.byref(n)) == LBM_OK and n.value == 0
    finally:
        lib.lbm_grid_destroy(h)


@pytest.mark.parametrize("threads", ["1", "3", "8"])
def test_host_build_is_independent_of_the_thread_count(threads, monkeypatch):
    """The host build splits positions, cells and neighbour rows over threads
    (LBM_GRID_THREADS forces the split): the tables must not change."""
    cfg = channel_sphere_config(level=6, radius=5.5)
    monkeypatch.setenv("LBM_GRID_THREADS", "1")
    one = gridgen.grid_tables(cfg)
    monkeypatch.setenv("LBM_GRID_THREADS", threads)
    many = gridgen.grid_tables(cfg)
    assert np.array_equal(one.centers, many.centers)
    assert np.array_equal(one.nghbr, many.nghbr)
    for k in one.surfaces:
        assert np.array_equal(one.surfaces[k]["cells"], many.surfaces[k]["cells"])
