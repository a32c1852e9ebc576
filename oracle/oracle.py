"""ctypes binding of the C oracle (oracle/lbm_oracle.c, oracle/lbm_oracle_box.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and
the CPU-baseline legs of bench.py.  The product package never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import List, Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liblbm_oracle.so")
SOURCES = [os.path.join(HERE, "lbm_oracle.c"), os.path.join(HERE, "lbm_oracle_box.c")]


def build(force: bool = False) -> str:
    """Compile the oracle with gcc.  -ffp-contract=off keeps every multiply and
    add separately rounded (GCC on aarch64 would otherwise fuse them), so the
    oracle gives the same bits on x86-64 and on the Arm GPU hosts."""
    os.makedirs(BUILD, exist_ok=True)
    newest = max(os.path.getmtime(s) for s in SOURCES + [os.path.join(HERE, "lbm_oracle.h")])
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    cmd = ["gcc", "-std=c11", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
           "-o", LIB + ".tmp"] + SOURCES + ["-lm"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        vp, i64, dbl, i32 = C.c_void_p, C.c_int64, C.c_double, C.c_int
        L.ora_create.restype = vp
        L.ora_create.argtypes = [i32, i32, i64, dbl, dbl, dbl, dbl, vp, i32, vp, vp, dbl]
        L.ora_destroy.argtypes = [vp]
        L.ora_add_bnd.restype = i32
        L.ora_add_bnd.argtypes = [vp, i32, i64, vp, vp, vp, vp, i32, dbl, i32, i64, vp, vp]
        L.ora_set_forcing.argtypes = [vp, dbl, i64, vp, i64, vp]
        L.ora_initial_condition.argtypes = [vp]
        L.ora_step.argtypes = [vp, i64]
        L.ora_update_moments.argtypes = [vp]
        L.ora_residual.argtypes = [vp, vp]
        L.ora_get.argtypes = [vp, vp, vp, vp, vp]
        L.ora_set_state.argtypes = [vp, vp, vp]
        L.ora_nvar.argtypes = [vp]
        L.ora_nvar.restype = i32
        L.ora_ndist.argtypes = [vp]
        L.ora_ndist.restype = i32
        L.ora_box_create.restype = vp
        L.ora_box_create.argtypes = [i32, i32, i32, i32, i32, dbl, vp, vp, vp, vp, vp, dbl]
        L.ora_box_destroy.argtypes = [vp]
        L.ora_box_set_poisson.argtypes = [vp, dbl, i32, vp]
        L.ora_box_set_poisson.restype = i32
        L.ora_box_set_slice_kappa.argtypes = [vp, vp]
        L.ora_box_set_slice_kappa.restype = i32
        L.ora_box_init_equilibrium.argtypes = [vp, dbl, vp]
        L.ora_box_step.argtypes = [vp, i64, i32]
        L.ora_box_get.argtypes = [vp, vp, vp, vp]
        L.ora_box_set.argtypes = [vp, vp]
        L.ora_box_set_deviation.argtypes = [vp, i32]
        L.ora_box_set_deviation.restype = i32
        _lib = L
    return _lib


def _p(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data


class TableOracle:
    """The reference step restated in C on the reference's own tables."""

    def __init__(self, consts, grid, bnds: List, forcing=None):
        L = lib()
        self._keep = []
        nghbr = np.ascontiguousarray(grid.nghbr, dtype=np.int64)
        centers = np.ascontiguousarray(grid.centers, dtype=np.float64)
        bbox = np.ascontiguousarray(grid.bbox, dtype=np.float64)
        self.n = grid.ncells
        self.h = L.ora_create(consts.lattice, consts.equation, self.n, consts.omega, consts.relax_time, consts.dt,
                              consts.poisson_k, _p(nghbr), nghbr.shape[1], _p(centers), _p(bbox), grid.cell_length)
        if not self.h:
            raise ValueError("oracle: unsupported lattice")
        self.q = L.ora_ndist(self.h)
        self.nvar = L.ora_nvar(self.h)
        for b in bnds:
            cells = np.ascontiguousarray(b.cells, dtype=np.int64)
            normals = np.ascontiguousarray(b.normals, dtype=np.float64)
            values = None if b.values is None else np.ascontiguousarray(b.values, dtype=np.float64)
            vec = np.ascontiguousarray(b.vec, dtype=np.float64)
            conn = None if b.conn_cells is None else np.ascontiguousarray(b.conn_cells, dtype=np.int64)
            connn = None if b.conn_normals is None else np.ascontiguousarray(b.conn_normals, dtype=np.float64)
            self._keep += [cells, normals, values, vec, conn, connn]
            rc = L.ora_add_bnd(self.h, b.kind, cells.size, _p(cells), _p(normals), _p(values), _p(vec), int(b.has_vec),
                               float(b.scalar), int(b.has_pressure), 0 if conn is None else conn.size, _p(conn), _p(connn))
            if rc != 0:
                raise ValueError(f"oracle: boundary {b.name} rejected ({rc})")
        if forcing is not None:
            i = np.ascontiguousarray(forcing.inlet_cells, dtype=np.int64)
            o = np.ascontiguousarray(forcing.outlet_cells, dtype=np.int64)
            self._keep += [i, o]
            L.ora_set_forcing(self.h, forcing.pressure_gradient, i.size, _p(i), o.size, _p(o))

    def __del__(self):
        if getattr(self, "h", None):
            lib().ora_destroy(self.h)
            self.h = None

    def initial_condition(self):
        lib().ora_initial_condition(self.h)

    def step(self, n: int):
        lib().ora_step(self.h, int(n))

    def update_moments(self):
        lib().ora_update_moments(self.h)

    def residual(self) -> np.ndarray:
        r = np.zeros(self.nvar)
        lib().ora_residual(self.h, _p(r))
        return r

    def state(self):
        fold = np.zeros(self.n * self.q)
        f = np.zeros(self.n * self.q)
        v = np.zeros(self.n * self.nvar)
        vo = np.zeros(self.n * self.nvar)
        lib().ora_get(self.h, _p(fold), _p(f), _p(v), _p(vo))
        return fold, f, v, vo


class BoxOracle:
    """Dense-box engine of the oracle (same arguments as the GPU BoxSolver)."""

    FACE = {"wall": 0, "periodic": 1, "freeslip": 2, "open": 3}

    def __init__(self, lattice, shape, omega, faces=("wall",) * 6, flags=None, wall_velocity=None, body_force=(0, 0, 0),
                 inlet_velocity=(0, 0, 0), inlet_density=1.0, equation=0, kappa_sq=0.0, pb_nonlinear=True, dirichlet=None,
                 deviation=False):
        L = lib()
        nx, ny, nz = (tuple(shape) + (1, 1))[:3]
        self.shape = (nx, ny, nz)
        self.ncells = nx * ny * nz
        self.q = {0: 3, 1: 5, 2: 9, 3: 7, 4: 19}[lattice]
        self.ndim = 2 if lattice == 2 else 3
        self.equation = equation
        face = np.array([self.FACE[f] if isinstance(f, str) else int(f) for f in faces], dtype=np.int32)
        wv = np.zeros((6, 3)) if wall_velocity is None else np.asarray(wall_velocity, dtype=np.float64).reshape(6, 3)
        fl = None if flags is None else np.ascontiguousarray(flags, dtype=np.uint8).reshape(-1)
        bf = np.asarray(body_force, dtype=np.float64)
        iv = np.asarray(inlet_velocity, dtype=np.float64)
        wv = np.ascontiguousarray(wv)
        self._keep = [face, wv, fl, bf, iv]
        self.h = L.ora_box_create(lattice, equation, nx, ny, nz, omega, _p(fl), _p(face), _p(wv), _p(bf), _p(iv),
                                  inlet_density)
        if not self.h:
            raise ValueError("oracle: unsupported box")
        if deviation:
            L.ora_box_set_deviation(self.h, 1)
        if equation == 1:
            di = None if dirichlet is None else np.ascontiguousarray(dirichlet, dtype=np.float64).reshape(-1)
            self._keep.append(di)
            L.ora_box_set_poisson(self.h, kappa_sq, int(pb_nonlinear), _p(di))

    def __del__(self):
        if getattr(self, "h", None):
            lib().ora_box_destroy(self.h)
            self.h = None

    def set_slice_kappa(self, kappa_sq):
        """One kappa^2 per z-slice (Poisson-Boltzmann; None: the box's single
        kappa^2), as lbm_gpu_box_set_slice_kappa."""
        k = None if kappa_sq is None else np.ascontiguousarray(kappa_sq, dtype=np.float64)
        lib().ora_box_set_slice_kappa(self.h, _p(k))

    def init_equilibrium(self, rho=1.0, u=(0, 0, 0)):
        uu = np.asarray(u, dtype=np.float64)
        lib().ora_box_init_equilibrium(self.h, rho, _p(uu))

    def step(self, n, threads=1):
        lib().ora_box_step(self.h, int(n), int(threads))

    def populations(self):
        f = np.zeros(self.q * self.ncells)
        lib().ora_box_get(self.h, _p(f), None, None)
        return f.reshape(self.q, self.ncells)

    def set_populations(self, f):
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(-1)
        lib().ora_box_set(self.h, _p(f))

    def moments(self):
        rho = np.zeros(self.ncells)
        u = np.zeros(3 * self.ncells)
        lib().ora_box_get(self.h, None, _p(rho), _p(u))
        return rho, u.reshape(3, self.ncells)[: self.ndim]
