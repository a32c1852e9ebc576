"""Host-side mirror of the reference solver's configuration step.

The SFCMM/LBM reference turns its JSON ``solver{}`` block into relaxation
constants in ``LBMSolver::loadConfiguration`` (src/lbm/solver.cpp:70-163) and
into an ordered list of boundary-condition objects in
``LBMBndManager::setupBndryCnds`` (src/lbm/bnd/bnd.h:71-279).  This module does
the same translation, with the same keys, defaults and error behaviour, and
produces plain descriptors that the C-ABI (include/lbm_gpu.h) consumes:

* :func:`solver_constants` -- omega, tau, nu, dt and the Poisson source
  coefficient, computed with the reference's expressions;
* :func:`boundary_list` -- one :class:`BndDesc` per BC object, in the order the
  reference applies them (nlohmann::json iterates object keys sorted, so
  geometries and then surface ids are visited in lexicographic order);
* :func:`forcing_desc` -- the inlet/outlet pairing of the pressure "forcing"
  (src/lbm/solver.cpp:625-696).

The grid side (cell list, neighbour table, named surfaces with per-cell
normals) is passed in as a :class:`GridTables`, i.e. exactly what
``CartesianGrid`` holds after ``loadGridInplace`` (src/cartesiangrid.h:264-320).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

# lattice ids and BC kinds: the values of include/lbm_gpu.h
LATTICES = {"D1Q3": 0, "D2Q5": 1, "D2Q9": 2, "D3Q7": 3, "D3Q19": 4}
LATTICE_Q = {0: 3, 1: 5, 2: 9, 3: 7, 4: 19}
LATTICE_DIM = {0: 1, 1: 2, 2: 2, 3: 3, 4: 3}
EQ_NAVIER_STOKES = 0
EQ_POISSON = 1

BND_PERIODIC = 1
BND_WALL_BB = 2
BND_WALL_BB_TANGENTIAL = 3
BND_DIRICHLET_BB = 4
BND_WALL_EQ = 5
BND_WALL_NEEM = 6
BND_WALL_NEBB = 7
BND_PRESSURE_ABB = 8
BND_DIRICHLET_NEEM = 9
BND_NEUMANN_NEEM = 10

BND_NAMES = {
    BND_PERIODIC: "periodic",
    BND_WALL_BB: "wall_bb",
    BND_WALL_BB_TANGENTIAL: "wall_bb_tangential",
    BND_DIRICHLET_BB: "dirichlet_bb",
    BND_WALL_EQ: "wall_eq",
    BND_WALL_NEEM: "wall_neem",
    BND_WALL_NEBB: "wall_nebb",
    BND_PRESSURE_ABB: "pressure_abb",
    BND_DIRICHLET_NEEM: "dirichlet_neem",
    BND_NEUMANN_NEEM: "neumann_neem",
}

GDOUBLE_EPS = float(np.finfo(np.float64).eps)
# lbm_cs = 1/sqrt(3) (src/lbm/constants.h:26)
LBM_CS = 1.0 / math.sqrt(3.0)


class ConfigError(ValueError):
    """Raised where the reference would stop with TERMM."""


@dataclass
class GridTables:
    """The reference grid as the solver sees it after ``loadGridInplace``."""

    ndim: int
    centers: np.ndarray  # (N, ndim) float64, curve order
    nghbr: np.ndarray  # (N, nnghbr) int64, -1 = missing
    surfaces: Dict[str, dict]  # name -> {"cells": int64[n], "normals": float64[n, ndim]}
    bbox: np.ndarray  # (2*ndim,) min0,max0,min1,max1,...
    cell_length: float
    max_lvl: int
    # multi-level grids (every level of the generator's array): each cell's
    # level and number of children; None for a uniform grid
    level: Optional[np.ndarray] = None
    nchildren: Optional[np.ndarray] = None
    partition_lvl: Optional[int] = None
    highest_lvl: Optional[int] = None

    @property
    def ncells(self) -> int:
        return int(self.centers.shape[0])

    def output_cells(self, solver: Optional[dict] = None) -> np.ndarray:
        """The cells the solution output writes: the solver's "cellFilter"
        (default "leafCells"; CellFilterManager, src/cell_filter.h:57-110:
        "leafCells", "highestLvl", "lowestLvl" / "partitionLvl", "targetLvl"
        with "outputLvl"), in cell order.  Every cell of a uniform grid."""
        if self.level is None:
            return np.arange(self.ncells)
        conf = (solver or {}).get("cellFilter", {"cellFilter": "leafCells"})
        kind = conf.get("cellFilter") if isinstance(conf, dict) else None
        lv = self.level.astype(np.int64)
        if kind == "leafCells":
            keep = self.nchildren == 0
        elif kind == "highestLvl":
            keep = lv == int(self.highest_lvl)
        elif kind in ("lowestLvl", "partitionLvl"):
            keep = lv == int(self.partition_lvl)
        elif kind == "targetLvl":
            if "outputLvl" not in conf:
                raise ConfigError('"targetLvl" needs "outputLvl"')
            if int(conf["outputLvl"]) < int(self.partition_lvl):
                raise ConfigError("Outputting a lvl below the partition lvl is not possible!")
            keep = lv == int(conf["outputLvl"])
        else:
            raise ConfigError(f"Unknown output filter {kind}")
        return np.flatnonzero(keep)


@dataclass
class BndDesc:
    kind: int
    name: str
    cells: np.ndarray
    normals: np.ndarray
    values: Optional[np.ndarray] = None
    vec: np.ndarray = field(default_factory=lambda: np.zeros(3))
    has_vec: bool = False
    scalar: float = 0.0
    has_pressure: bool = False
    conn_cells: Optional[np.ndarray] = None
    conn_normals: Optional[np.ndarray] = None


@dataclass
class SolverConstants:
    lattice: int
    equation: int
    omega: float
    relax_time: float
    nu: float
    dt: float
    poisson_k: float
    nvar: int


def _opt(cfg: dict, key: str, default):
    return cfg[key] if key in cfg else default


def solver_constants(solver: dict, grid: GridTables) -> SolverConstants:
    """``LBMSolverExecutor::init`` + ``loadConfiguration`` (src/lbm/solverExe.h:17-93,
    src/lbm/solver.cpp:70-136) and the Poisson source coefficient of
    ``collisionStep`` (src/lbm/solver.cpp:589-599)."""
    model = _opt(solver, "model", "D2Q9")
    equation = _opt(solver, "equation", "navierstokes")
    if model not in LATTICES:
        raise ConfigError("Invalid model configuration!")
    if equation not in ("navierstokes", "poisson"):
        raise ConfigError("Invalid equation configuration!")
    lattice = LATTICES[model]
    eq = EQ_NAVIER_STOKES if equation == "navierstokes" else EQ_POISSON
    supported = {(2, EQ_NAVIER_STOKES), (2, EQ_POISSON), (1, EQ_POISSON), (0, EQ_POISSON)}
    if (lattice, eq) not in supported:
        raise ConfigError("Unsupported model")
    if LATTICE_DIM[lattice] != grid.ndim:
        raise ConfigError("Invalid configuration the grid dimensionality is not matching!")
    method = _opt(solver, "method", "bgk")
    if method != "bgk":
        raise ConfigError("Invalid equation configuration!")

    ref_length = float(_opt(solver, "refLength", 1.0))
    spacing = 1.0 / (math.pow(grid.ncells, 1.0 / grid.ndim) - 1)
    if eq == EQ_NAVIER_STOKES:
        if "reynoldsnumber" in solver and "relaxation" in solver:
            raise ConfigError("Only set either reynoldsnumber or relaxation")
        ma = float(solver["ma"])
        if "relaxation" in solver:
            relax = float(solver["relaxation"])
            omega = 1.0 / relax
            nu = (2 * relax - 1) / 6.0
        else:
            re = float(solver["reynoldsnumber"])
            nu = ma / re * ref_length
            omega = 2.0 / (1.0 + 2.0 * nu * math.pow(2.0, grid.max_lvl))
            relax = 1.0 / omega
        dt = spacing * ma * LBM_CS / ref_length
        poisson_k = 0.0
        nvar = grid.ndim + 1
    else:
        relax = float(solver["relaxation"])
        ma = 1.0 / LBM_CS
        omega = 1.0 / relax
        nu = (2.0 * relax - 1) / 6.0
        dt = spacing * ma * LBM_CS / ref_length
        app = _opt(solver, "equation_application", "debye_huckel")
        if app == "simple_diff_reaction":
            poisson_k = float(solver["equation_th"])
        elif app == "debye_huckel":
            poisson_k = 27.79
        else:
            raise ConfigError("Invalid model configuration!")
        nvar = 1
    return SolverConstants(lattice, eq, omega, relax, nu, dt, poisson_k, nvar)


def _eval_expression(expr: str, center: np.ndarray) -> float:
    """A math expression value at a cell centre (the reference evaluates these with
    exprtk in ``MathExpression``, src/common/mathexpr.h:7-47): variables x, y, z,
    the constant pi and the usual functions; ``^`` is the power operator."""
    env = {
        "sin": math.sin, "cos": math.cos, "tan": math.tan, "sinh": math.sinh, "cosh": math.cosh,
        "tanh": math.tanh, "exp": math.exp, "log": math.log, "sqrt": math.sqrt, "abs": abs,
        "pi": math.pi, "__builtins__": {},
    }
    for i, name in enumerate("xyz"[: center.shape[0]]):
        env[name] = float(center[i])
    return float(eval(expr.replace("^", "**"), env))  # noqa: S307 - trusted solver config


def boundary_list(solver: dict, grid: GridTables, consts: SolverConstants) -> List[BndDesc]:
    """Mirror of ``LBMBndManager::setupBndryCnds`` (src/lbm/bnd/bnd.h:71-142)."""
    out: List[BndDesc] = []
    cfg = solver.get("boundary")
    if cfg is None:
        raise ConfigError("required config value boundary missing")
    ndim = grid.ndim
    for geometry in sorted(cfg.keys()):
        geom_cfg = cfg[geometry]
        nbnds = len(geom_cfg)
        for surf_id in sorted(geom_cfg.keys()):
            bc = geom_cfg[surf_id]
            name = f"{geometry}_{surf_id}" if nbnds > 1 else geometry
            if name not in grid.surfaces:
                raise ConfigError(f'Invalid bndryId "{name}"')
            srf = grid.surfaces[name]
            cells = np.asarray(srf["cells"], dtype=np.int64)
            normals = np.asarray(srf["normals"], dtype=np.float64).reshape(-1, ndim)
            if cells.size == 0:
                continue  # "WARNING: Skipping ... no valid cells!"
            btype = bc["type"]
            generate = bool(_opt(bc, "generateBndry", True))

            def desc(kind, **kw):
                return BndDesc(kind=kind, name=name, cells=cells, normals=normals, **kw)

            if btype == "periodic":
                conn = grid.surfaces[bc["connection"]]
                if not generate:
                    continue  # dummy: periodicity lives in the neighbour table
                d = desc(BND_PERIODIC, conn_cells=np.asarray(conn["cells"], dtype=np.int64),
                         conn_normals=np.asarray(conn["normals"], dtype=np.float64).reshape(-1, ndim))
                if "pressure" in bc:
                    d.has_pressure = True
                    d.scalar = float(bc["pressure"])
                out.append(d)
            elif btype == "wall":
                if not generate:
                    continue
                model = bc["model"]
                if model == "bounceback":
                    tv = float(_opt(bc, "tangentialVelocity", 0.0))
                    if abs(tv) > GDOUBLE_EPS:
                        out.append(desc(BND_WALL_BB_TANGENTIAL, scalar=tv))
                    else:
                        out.append(desc(BND_WALL_BB))
                elif model in ("equilibrium", "neem", "nebb"):
                    kind = {"equilibrium": BND_WALL_EQ, "neem": BND_WALL_NEEM, "nebb": BND_WALL_NEBB}[model]
                    if kind == BND_WALL_NEBB and consts.lattice != LATTICES["D2Q9"]:
                        raise ConfigError("Not implemented for this distribution!")
                    d = desc(kind)
                    if "velocity" in bc:
                        v = np.zeros(3)
                        v[:ndim] = np.asarray(bc["velocity"], dtype=np.float64)[:ndim]
                        d.vec = v
                        d.has_vec = True
                    out.append(d)
                else:
                    raise ConfigError("Invalid wall boundary model: " + model)
            elif btype == "pressure":
                if not generate:
                    continue
                out.append(desc(BND_PRESSURE_ABB, scalar=float(bc["pressure"])))
            elif btype in ("inlet", "outlet"):
                raise ConfigError("Broken")
            elif btype == "dirichlet":
                if not generate:
                    continue
                model = bc["model"]
                if model == "bounceback":
                    if consts.equation == EQ_POISSON:
                        raise ConfigError("this is incorrect!")
                    v = np.zeros(3)
                    val = np.atleast_1d(np.asarray(bc["value"], dtype=np.float64))
                    v[: min(ndim, val.size)] = val[:ndim]
                    out.append(desc(BND_DIRICHLET_BB, vec=v))
                elif model == "neem":
                    if consts.equation != EQ_POISSON:
                        raise ConfigError("FIX ME")
                    value = bc["value"]
                    centers = grid.centers[cells]
                    if isinstance(value, str):
                        vals = np.array([_eval_expression(value, c) for c in centers])
                    elif isinstance(value, list) and value and isinstance(value[0], str):
                        raise ConfigError("Impl")
                    else:
                        vals = np.full(cells.size, float(np.atleast_1d(value)[0]))
                    out.append(desc(BND_DIRICHLET_NEEM, values=vals))
                # any other model: the reference silently adds nothing
            elif btype == "neumann":
                if not generate:
                    continue
                if bc["model"] == "neem":
                    if consts.equation != EQ_POISSON:
                        raise ConfigError("Not implemented")
                    value = bc["value"]
                    vals = np.full(cells.size, float(np.atleast_1d(value)[0])) if not isinstance(value, str) else None
                    out.append(desc(BND_NEUMANN_NEEM, values=vals))
            else:
                raise ConfigError("Invalid bndCndType: " + btype)
    return out


@dataclass
class ForcingDesc:
    pressure_gradient: float
    inlet_cells: np.ndarray
    outlet_cells: np.ndarray


def forcing_desc(solver: dict, grid: GridTables) -> Optional[ForcingDesc]:
    """The pressure "forcing" of src/lbm/solver.cpp:625-696 (hard-coded surfaces
    cube_-x and cube_+x)."""
    if not _opt(solver, "forcing", ""):
        return None
    dp = float(solver["poiseuillePressureGradient"])
    inlet = np.asarray(grid.surfaces["cube_-x"]["cells"], dtype=np.int64)
    outlet = np.asarray(grid.surfaces["cube_+x"]["cells"], dtype=np.int64)
    return ForcingDesc(dp, inlet, outlet)
