"""Grid tables from the reference's JSON config, without its grid generator.

The SFCMM/LBM reference builds the LBM grid in two programs: the grid
generator (``src/gridgenerator/``) makes the cells, and ``CartesianGrid::
loadGridInplace`` (src/cartesiangrid.h:264-320) derives the boundary cells,
the named boundary surfaces, the periodic wiring and the diagonal neighbours.
:func:`grid_tables` does both for the uniform grids every reference LBM case
uses (``partitionLevel == uniformLevel == maxRfnmtLvl``), and for multi-level
grids, whose every level the reference's solver steps as a lattice of its
own, and returns the :class:`~lbm_gb300.refconfig.GridTables` the solvers
consume.  The per-cell
work runs in the native library (include/lbm_grid.h); this module walks the
config in the reference's order:

1. geometry objects in sorted key order (nlohmann::json iterates sorted),
   each with its body (``"body"``, default its own name) and ``"subtract"``;
2. the grid at the uniform level (``lbm_grid_create``), stretched onto the
   geometry's surface when ``"alignNodesWithSurface"`` is set
   (``lbm_grid_align``, along ``"alignDir"``, default 1);
3. surfaces (identifyBndrySurfaces, src/cartesiangrid.h:551-598): for each
   geometry of ``solver.boundary`` and each of its direction entries, both in
   sorted order, the surface ``<geometry>_<dir>`` (or ``<geometry>`` when it
   has one entry) takes the boundary cells without a neighbour in that
   direction that the geometry cuts, unless an earlier surface took the
   (cell, direction) pair.  A cell keeps the normal of the last direction it
   was added with (``Surface::addCell`` stores normals per cell,
   src/common/surface.h:52-55);
4. periodic surfaces with ``"generateBndry": false`` are wired across the
   period (setupPeriodicConnections, src/cartesiangrid.h:600-634);
5. the diagonal neighbours (addDiagonalNghbrs, src/cartesiangrid.h:450-487).

In 2D and 1D the tables equal the reference's bit for bit; 3D, which the
reference cannot build, follows the same rules (include/lbm_grid.h).

:func:`grid_tree` builds the generator's whole multi-level cell tree for any
``partitionLevel <= uniformLevel <= maxRfnmtLvl`` (``lbm_grid_tree_create``),
and :func:`save_grid` writes the generator's points file from it.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass
from typing import Dict, List, Optional

import numpy as np

from . import _lib
from .refconfig import ConfigError, GridTables

GEOM_BOX = 0
GEOM_SPHERE = 1
DIRS = {"-x": 0, "+x": 1, "-y": 2, "+y": 3, "-z": 4, "+z": 5}


class GeomDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("body", C.c_int32), ("subtract", C.c_int32), ("reserved", C.c_int32),
                ("a", C.c_double * 3), ("b", C.c_double * 3), ("center", C.c_double * 3), ("radius", C.c_double)]


_SIGS = {
    "lbm_grid_create": (C.c_int, [C.c_int32, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p, C.POINTER(C.c_void_p)]),
    "lbm_grid_create_device": (C.c_int, [C.c_int32, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p, C.c_int32,
                                         C.POINTER(C.c_void_p)]),
    "lbm_grid_align": (C.c_int, [C.c_void_p, C.c_int32]),
    "lbm_grid_curve_index": (C.c_int, [C.c_int32, C.c_int32, C.c_void_p, C.POINTER(C.c_uint64)]),
    "lbm_grid_ncells": (C.c_int64, [C.c_void_p]),
    "lbm_grid_nnghbr": (C.c_int32, [C.c_void_p]),
    "lbm_grid_info": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_double)]),
    "lbm_grid_centers": (C.c_int, [C.c_void_p, C.c_void_p]),
    "lbm_grid_boundary": (C.c_int, [C.c_void_p, C.c_void_p]),
    "lbm_grid_add_surface": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_int64,
                                       C.POINTER(C.c_int64)]),
    "lbm_grid_connect_periodic": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64]),
    "lbm_grid_neighbors": (C.c_int, [C.c_void_p, C.c_void_p]),
    "lbm_grid_destroy": (None, [C.c_void_p]),
    "lbm_grid_tree_create": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int64, C.c_void_p, C.c_int32, C.c_void_p,
                                       C.c_int32, C.POINTER(C.c_void_p)]),
    "lbm_grid_tree_ncells": (C.c_int64, [C.c_void_p]),
    "lbm_grid_tree_levels": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "lbm_grid_tree_cells": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "lbm_grid_tree_children": (C.c_int, [C.c_void_p, C.c_void_p]),
    "lbm_grid_tree_neighbors": (C.c_int, [C.c_void_p, C.c_void_p]),
    "lbm_grid_tree_write_points": (C.c_int, [C.c_void_p, C.c_char_p, C.c_void_p, C.c_int32]),
    "lbm_grid_tree_grid": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "lbm_grid_tree_destroy": (None, [C.c_void_p]),
}


def _grid_lib():
    lib = _lib.load()
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def _vec(values, ndim: int, what: str) -> List[float]:
    v = [float(x) for x in values]
    if len(v) != ndim:
        raise ConfigError(f"{what}: expected {ndim} values, got {len(v)}")
    return v + [0.0] * (3 - ndim)


def curve_index(x, level: int) -> int:
    """The reference's curve index (hilbert::index) of a point in the unit cube."""
    p = np.ascontiguousarray(x, dtype=np.float64)
    out = C.c_uint64()
    _lib.check(_grid_lib().lbm_grid_curve_index(len(p), level, p.ctypes.data, C.byref(out)), what="lbm_grid_curve_index")
    return int(out.value)


def geometry_objects(geometry: Dict, ndim: int):
    """GeomDesc array and names, in the reference's (sorted) order."""
    names = sorted(geometry)
    descs = (GeomDesc * max(1, len(names)))()
    bodies: Dict[str, int] = {}
    for i, name in enumerate(names):
        g = geometry[name]
        if "type" not in g:
            raise ConfigError(f'geometry "{name}": no "type" given')
        d = descs[i]
        if g["type"] == "box":
            d.kind = GEOM_BOX
            d.a[:] = _vec(g["A"], ndim, f"{name}.A")
            d.b[:] = _vec(g["B"], ndim, f"{name}.B")
        elif g["type"] == "sphere":
            d.kind = GEOM_SPHERE
            d.center[:] = _vec(g["center"], ndim, f"{name}.center")
            d.radius = float(g["radius"])
        else:
            raise ConfigError(f'geometry "{name}": type "{g["type"]}" is not supported (box, sphere)')
        body = g.get("body", "unique")
        body = name if body == "unique" else body
        d.body = bodies.setdefault(body, len(bodies))
        d.subtract = 1 if g.get("subtract", False) else 0
    return descs, names


def grid_tables(config: Dict, device: Optional[int] = None) -> GridTables:
    """The reference's LBM grid tables for a JSON config (the grid generator's
    keys plus ``solver.boundary``).  With ``device`` the cells of a uniform
    grid are enumerated on that GPU (``lbm_grid_create_device``, the same
    tables); a multi-level grid (levels not all equal) is built on the host
    from the generator's tree (``lbm_grid_tree_grid``) either way, and its
    tables carry each cell's level and child count (``GridTables.level``,
    ``nchildren``)."""
    ndim = int(config.get("dim", 0))
    if ndim not in (1, 2, 3):
        raise ConfigError(f"dim must be 1, 2 or 3, got {ndim}")
    levels = {k: int(config[k]) for k in ("partitionLevel", "uniformLevel", "maxRfnmtLvl") if k in config}
    level = levels.get("uniformLevel", levels.get("partitionLevel"))
    if level is None:
        raise ConfigError('"partitionLevel" and "uniformLevel" are required')
    multilevel = len(set(levels.values())) != 1
    geometry = config.get("geometry", {})
    descs, names = geometry_objects(geometry, ndim)
    bbox = None
    if not names or "boundingBox" in config:
        default = [0.0, 1.0] * ndim
        bbox = (C.c_double * (2 * ndim))(*[float(x) for x in config.get("boundingBox", default)])
    lib = _grid_lib()
    h = C.c_void_p()
    pb = C.cast(bbox, C.c_void_p) if bbox else None
    if multilevel:
        # every level of the generator's array, as the reference's solver
        # loads and steps it (src/lbm/solver.cpp:525: each level a lattice
        # of its own); built on the host
        p, u, level, cap = _tree_levels(config)
        for gname, entries in config.get("solver", {}).get("boundary", {}).items():
            for e in entries.values():
                if isinstance(e, dict) and e.get("type") == "periodic" and e.get("generateBndry", True):
                    # its mapping steps one cell length of the mapped cell's
                    # level; the engine maps with one length
                    raise ConfigError(f'periodic boundary condition "{gname}" (generateBndry) on a multi-level grid is not '
                                      "supported")
        align = int(config.get("alignDir", 1)) if config.get("alignNodesWithSurface", False) else -1
        t = C.c_void_p()
        _lib.check(lib.lbm_grid_tree_create(ndim, p, u, level, cap, C.cast(descs, C.c_void_p), len(names), pb, align, C.byref(t)),
                   what="lbm_grid_tree_create")
        try:
            nt = int(lib.lbm_grid_tree_ncells(t))
            pl, hl = C.c_int32(), C.c_int32()
            _lib.check(lib.lbm_grid_tree_levels(t, C.byref(pl), C.byref(hl)), what="lbm_grid_tree_levels")
            tree_level = np.empty(nt, dtype=np.int8)
            tree_nchildren = np.empty(nt, dtype=np.int32)
            _lib.check(lib.lbm_grid_tree_cells(t, None, tree_level.ctypes.data, None, None, tree_nchildren.ctypes.data, None),
                       what="lbm_grid_tree_cells")
            _lib.check(lib.lbm_grid_tree_grid(t, C.byref(h)), what="lbm_grid_tree_grid")
        finally:
            lib.lbm_grid_tree_destroy(t)
    else:
        if device is None:
            rc = lib.lbm_grid_create(ndim, level, C.cast(descs, C.c_void_p), len(names), pb, C.byref(h))
        else:
            rc = lib.lbm_grid_create_device(ndim, level, C.cast(descs, C.c_void_p), len(names), pb, int(device), C.byref(h))
        _lib.check(rc, what="lbm_grid_create")
    try:
        if config.get("alignNodesWithSurface", False) and not multilevel:
            _lib.check(lib.lbm_grid_align(h, int(config.get("alignDir", 1))), what="lbm_grid_align")
        n = int(lib.lbm_grid_ncells(h))
        centers = np.empty((n, ndim), dtype=np.float64)
        _lib.check(lib.lbm_grid_centers(h, centers.ctypes.data), what="lbm_grid_centers")
        box = np.empty(2 * ndim, dtype=np.float64)
        cl = C.c_double()
        _lib.check(lib.lbm_grid_info(h, box.ctypes.data, C.byref(cl)), what="lbm_grid_info")

        surfaces: Dict[str, dict] = {}
        periodic = {}
        boundary = config.get("solver", {}).get("boundary", {})
        for gname in sorted(boundary):
            entries = boundary[gname]
            for dname in sorted(entries):
                sname = f"{gname}_{dname}" if len(entries) > 1 else gname
                if dname == "all":
                    d0, d1 = 0, 2 * ndim
                elif dname in DIRS and DIRS[dname] < 2 * ndim:
                    d0 = DIRS[dname]
                    d1 = d0 + 1
                else:
                    raise ConfigError(f'boundary "{gname}": invalid direction "{dname}"')
                got = C.c_int64()
                m = 0
                if gname in names:
                    obj = names.index(gname)
                    _lib.check(lib.lbm_grid_add_surface(h, obj, d0, d1, None, None, 0, C.byref(got)), what="lbm_grid_add_surface")
                    m = int(got.value)
                cells = np.empty(m, dtype=np.int64)
                dirs = np.empty(m, dtype=np.int8)
                if m:
                    _lib.check(lib.lbm_grid_add_surface(h, obj, d0, d1, cells.ctypes.data, dirs.ctypes.data, m, C.byref(got)),
                               what="lbm_grid_add_surface")
                lst = cells
                # Surface::addCell keeps one normal per cell: that of its last entry
                last = {c: d for c, d in zip(lst.tolist(), dirs[:m].tolist())}
                dl = np.array([last[c] for c in lst.tolist()], dtype=np.int64)
                normals = np.zeros((m, ndim), dtype=np.float64)
                normals[np.arange(m), dl // 2] = np.where(dl & 1, 1.0, -1.0)
                surfaces[sname] = {"cells": lst, "normals": normals}
                e = entries[dname]
                if isinstance(e, dict) and e.get("type") == "periodic" and not e.get("generateBndry", True):
                    if "connection" not in e:
                        raise ConfigError(f'periodic boundary "{gname}_{dname}" without "connection"')
                    periodic[f"{gname}_{dname}"] = e["connection"]
        # wire each connected pair once (the pairing is symmetric)
        done = set()
        for a in sorted(periodic):
            b = periodic[a]
            if a in done:
                continue
            if periodic.get(b) is None:
                raise ConfigError("Invalid periodic setup!")
            done.update((a, b))
            for s in (a, b):
                if s not in surfaces:
                    raise ConfigError(f'periodic connection to unknown surface "{s}"')
            ca, cb = surfaces[a]["cells"], surfaces[b]["cells"]
            _lib.check(lib.lbm_grid_connect_periodic(h, ca.ctypes.data, len(ca), cb.ctypes.data, len(cb)),
                       what="lbm_grid_connect_periodic")
        w = int(lib.lbm_grid_nnghbr(h))
        nghbr = np.empty((n, w), dtype=np.int64)
        _lib.check(lib.lbm_grid_neighbors(h, nghbr.ctypes.data), what="lbm_grid_neighbors")
    finally:
        lib.lbm_grid_destroy(h)
    extra = dict(level=tree_level, nchildren=tree_nchildren, partition_lvl=int(pl.value), highest_lvl=int(hl.value)) if multilevel else {}
    return GridTables(ndim=ndim, centers=centers, nghbr=nghbr, surfaces=surfaces, bbox=box, cell_length=float(cl.value),
                      max_lvl=level, **extra)


@dataclass
class GridTree:
    """The reference grid generator's cell array (all levels, its order)."""
    ndim: int
    partition_level: int
    highest_level: int
    centers: np.ndarray    # (n, ndim)
    level: np.ndarray      # (n,) int8
    parent: np.ndarray     # (n,) int64, -1: none
    global_id: np.ndarray  # (n,) int64
    nchildren: np.ndarray  # (n,) int32
    bndry: np.ndarray      # (n,) uint8
    children: np.ndarray   # (n, 2**ndim) int64, -1: none
    nghbr: np.ndarray      # (n, 2*ndim) int64, -1: none

    def leaves(self) -> np.ndarray:
        """Cells without children (the reference's "leafCells" filter)."""
        return np.flatnonzero(self.nchildren == 0)


# GridGenerator's "outputValues" (src/gridgenerator/cartesiangrid_generation.h:224-240)
TREE_COLUMNS = {"level": 0, "noChildren": 1}


def _tree_levels(config: Dict):
    """partitionLevel, uniformLevel, maxRfnmtLvl and maxNoCells with the
    generator's checks (src/gridgenerator/gridGenerator.cpp:245-255, 130-133)."""
    for key in ("partitionLevel", "uniformLevel", "maxNoCells"):
        if key not in config:
            raise ConfigError(f'"{key}" is required')
    p, u = int(config["partitionLevel"]), int(config["uniformLevel"])
    m = int(config.get("maxRfnmtLvl", u))
    if p > u:
        raise ConfigError("Invalid definition of grid level partitionLevel >= uniformLevel")
    if m < u:
        raise ConfigError("Invalid definition of grid level uniformLevel >= maxRfnmtLvl")
    return p, u, m, int(config["maxNoCells"])


def grid_tree(config: Dict, points_file: Optional[str] = None) -> GridTree:
    """The reference grid generator's whole cell tree for a JSON config (its
    keys: ``dim``, ``partitionLevel``, ``uniformLevel``, ``maxRfnmtLvl``,
    ``maxNoCells``, ``geometry``, ``boundingBox``, ``alignNodesWithSurface``,
    ``alignDir``), built natively (``lbm_grid_tree_create``).  With
    ``points_file`` the generator's points file is written there too, with
    the columns of ``output.outputValues`` (default ``["level"]``)."""
    ndim = int(config.get("dim", 0))
    if ndim not in (1, 2, 3):
        raise ConfigError(f"dim must be 1, 2 or 3, got {ndim}")
    p, u, m, cap = _tree_levels(config)
    descs, names = geometry_objects(config.get("geometry", {}), ndim)
    bbox = None
    if not names or "boundingBox" in config:
        bbox = (C.c_double * (2 * ndim))(*[float(x) for x in config.get("boundingBox", [0.0, 1.0] * ndim)])
    align = int(config.get("alignDir", 1)) if config.get("alignNodesWithSurface", False) else -1
    lib = _grid_lib()
    h = C.c_void_p()
    _lib.check(lib.lbm_grid_tree_create(ndim, p, u, m, cap, C.cast(descs, C.c_void_p), len(names),
                                        C.cast(bbox, C.c_void_p) if bbox else None, align, C.byref(h)),
               what="lbm_grid_tree_create")
    try:
        n = int(lib.lbm_grid_tree_ncells(h))
        pl, hl = C.c_int32(), C.c_int32()
        _lib.check(lib.lbm_grid_tree_levels(h, C.byref(pl), C.byref(hl)), what="lbm_grid_tree_levels")
        t = GridTree(ndim=ndim, partition_level=int(pl.value), highest_level=int(hl.value),
                     centers=np.empty((n, ndim)), level=np.empty(n, np.int8), parent=np.empty(n, np.int64),
                     global_id=np.empty(n, np.int64), nchildren=np.empty(n, np.int32), bndry=np.empty(n, np.uint8),
                     children=np.empty((n, 1 << ndim), np.int64), nghbr=np.empty((n, 2 * ndim), np.int64))
        _lib.check(lib.lbm_grid_tree_cells(h, t.centers.ctypes.data, t.level.ctypes.data, t.parent.ctypes.data,
                                           t.global_id.ctypes.data, t.nchildren.ctypes.data, t.bndry.ctypes.data),
                   what="lbm_grid_tree_cells")
        _lib.check(lib.lbm_grid_tree_children(h, t.children.ctypes.data), what="lbm_grid_tree_children")
        _lib.check(lib.lbm_grid_tree_neighbors(h, t.nghbr.ctypes.data), what="lbm_grid_tree_neighbors")
        if points_file is not None:
            values = config.get("output", {}).get("outputValues", ["level"])
            cols = [TREE_COLUMNS[v] for v in values if v in TREE_COLUMNS]  # the reference skips unknown values
            arr = (C.c_int32 * max(1, len(cols)))(*cols)
            _lib.check(lib.lbm_grid_tree_write_points(h, os.fsencode(points_file), C.cast(arr, C.c_void_p), len(cols)),
                       what="lbm_grid_tree_write_points")
    finally:
        lib.lbm_grid_tree_destroy(h)
    return t


def save_grid(config: Dict, workdir: str = ".") -> str:
    """GridGenerator::run's output: the tree's points file at
    ``<workdir>/<outputDir>/<gridFileName>.csv`` (defaults ``out`` and
    ``grid``; the directory must exist, as the reference requires).  Only the
    ASCII format is written; the reference's VTK point writers stop with
    "Work in progress" (src/common/IO.h:219).  Every cell is written whatever
    ``cellFilter`` says: the generator builds its filter without the grid, so
    it passes all cells (src/gridgenerator/cartesiangrid_generation.h:220,
    src/cell_filter.h:62)."""
    out = config.get("output", {"format": "ASCII"})
    if out.get("format", "ASCII") != "ASCII":
        raise ConfigError(f'grid output format "{out.get("format")}" is not written (the reference stops on it too)')
    outdir = os.path.join(workdir, config.get("outputDir", "out"))
    if not os.path.isdir(outdir):
        raise ConfigError(f"Is not a valid output directory! {outdir}")
    path = os.path.join(outdir, config.get("gridFileName", "grid") + ".csv")
    grid_tree(config, points_file=path)
    return path


# box-engine face kinds for the reference's boundary types, plus the kinds the
# box engine adds for the 3D configurations (the reference has no free-slip,
# velocity-inlet or zero-gradient-outlet condition)
BOX_FACES = {"wall": "wall", "periodic": "periodic", "freeslip": "freeslip", "inlet": "open", "outlet": "open"}
CELL_FLUID, CELL_SOLID, CELL_INLET, CELL_OUTLET = 0, 1, 2, 3


def box_case(grid: GridTables, config: Dict) -> Dict:
    """The dense-box form of a grid built from a config whose domain is one
    box (objects subtracted from it become solid cells): shape, per-cell flags
    (x fastest), face kinds, inlet velocity, and for each grid cell its index
    in the box.  The box spans every cell of the grid, cut layer included, so
    a "wall" face bounces back half a cell beyond the outermost cells, where
    the reference's halfway bounce-back at its wet boundary rows puts the
    wall; a removed cell is solid and bounces back the same way.

    Face entries of the domain box in ``solver.boundary``: ``"wall"`` (no
    moving-wall value), ``"periodic"``, and the box engine's ``"freeslip"``,
    ``"inlet"`` (``"velocity"``: equilibrium inflow, -x face) and
    ``"outlet"`` (zero gradient, +x face)."""
    ndim = grid.ndim
    if ndim < 2:
        raise ConfigError("the box engine needs a 2D or 3D grid")
    geometry = config.get("geometry", {})
    domains = [n for n in sorted(geometry) if geometry[n]["type"] == "box" and not geometry[n].get("subtract", False)]
    if len(domains) != 1:
        raise ConfigError(f"one domain box expected, found {domains}")
    dom = domains[0]
    h = grid.cell_length
    c = grid.centers
    rel = (c - c.min(axis=0)) / h
    k = np.rint(rel).astype(np.int64)
    if np.abs(rel - k).max() > 1e-6:
        raise ConfigError("cell centres are not on one uniform lattice")
    ext = k.max(axis=0) + 1
    shape = (int(ext[0]), int(ext[1]), int(ext[2]) if ndim == 3 else 1)
    kz = k[:, 2] if ndim == 3 else np.zeros(len(k), dtype=np.int64)
    index = k[:, 0] + shape[0] * (k[:, 1] + shape[1] * kz)
    flags = np.full(shape[0] * shape[1] * shape[2], CELL_SOLID, dtype=np.uint8)
    flags[index] = CELL_FLUID
    entries = config.get("solver", {}).get("boundary", {}).get(dom, {})
    faces, inlet = [], (0.0, 0.0, 0.0)
    for d, name in enumerate(("-x", "+x", "-y", "+y", "-z", "+z")):
        if d >= 2 * ndim:
            faces.append("wall")  # a 2D lattice has no z links
            continue
        e = entries.get(name, entries.get("all"))
        if e is None:
            raise ConfigError(f'domain box "{dom}": no boundary for face {name}')
        kind = e.get("type")
        if kind not in BOX_FACES:
            raise ConfigError(f'domain box "{dom}", face {name}: type "{kind}" has no box-engine form')
        if kind == "wall" and any(key in e for key in ("value", "velocity", "tangentialVelocity")):
            raise ConfigError(f'domain box "{dom}", face {name}: moving walls are set through wall_velocity')
        if kind == "inlet":
            if name != "-x":
                raise ConfigError("the inlet is the -x face")
            v = [float(x) for x in e.get("velocity", [0.0] * ndim)]
            inlet = tuple(v + [0.0] * (3 - len(v)))
            plane = flags.reshape(shape[2], shape[1], shape[0])[:, :, 0]
            plane[plane == CELL_FLUID] = CELL_INLET
        if kind == "outlet":
            if name != "+x":
                raise ConfigError("the outlet is the +x face")
            plane = flags.reshape(shape[2], shape[1], shape[0])[:, :, -1]
            plane[plane == CELL_FLUID] = CELL_OUTLET
        faces.append(BOX_FACES[kind])
    return {"shape": shape, "flags": flags, "faces": tuple(faces), "inlet": inlet, "index": index}
