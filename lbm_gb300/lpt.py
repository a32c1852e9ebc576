"""Lagrangian particles on the GPU (include/lbm_lpt.h).

:class:`ParticleSolver` mirrors the reference's ``LPTSolver`` for one step
call at a time: :meth:`from_config` reads its ``solver`` block with the
reference's keys and defaults (src/lpt/solver.cpp:94-228), the particle
array has the reference's ``m_vars`` layout (src/lpt/particle.h:11-36), and
:meth:`step` runs ``timeStep()`` (src/lpt/solver.cpp:335-347) n times on the
GPU.  :meth:`couple` takes the ambient velocity from a dense-box LBM solver
instead of the constant ``v_infty``.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence

import numpy as np

from . import _lib
from .refconfig import ConfigError

MODELS = ["constDensityRatioGrav", "constDensityRatioGravStokesDrag", "constDensityRatioGravNlinDrag", "constDensityRatioGravBuo",
          "constDensityRatioGravBuoStokesDrag", "constDensityRatioGravBuoNlinDrag", "constDensityaGravBuo",
          "constDensityaGravBuoStokesDrag", "constDensityaGravBuoNlinDrag"]
INTEGRATORS = ["ForwardEuler", "ImplicitEuler"]


class LptDesc(C.Structure):
    _fields_ = [("ndim", C.c_int32), ("model", C.c_int32), ("integration", C.c_int32), ("device", C.c_int32),
                ("capacity", C.c_int64), ("dt", C.c_double), ("gravity", C.c_double * 3), ("rho_ambient", C.c_double),
                ("nu_ambient", C.c_double), ("v_ambient", C.c_double * 3)]


_SIGS = {
    "lbm_lpt_create": (C.c_int, [C.POINTER(LptDesc), C.POINTER(C.c_void_p)]),
    "lbm_lpt_set_particles": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p]),
    "lbm_lpt_get_particles": (C.c_int, [C.c_void_p, C.c_void_p]),
    "lbm_lpt_count": (C.c_int64, [C.c_void_p]),
    "lbm_lpt_step": (C.c_int, [C.c_void_p, C.c_int64]),
    "lbm_lpt_couple_box": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_double]),
    "lbm_lpt_last_error": (C.c_char_p, [C.c_void_p]),
    "lbm_lpt_destroy": (None, [C.c_void_p]),
}


def _lpt_lib():
    lib = _lib.load()
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


class ParticleSolver:
    def __init__(self, ndim: int, model: int, implicit: bool, dt: float, gravity: Sequence[float], rho_ambient: float = 1.205,
                 nu_ambient: float = 1.82e-5, v_ambient: Optional[Sequence[float]] = None, capacity: int = 1024, device: int = 0):
        self._lib = _lpt_lib()
        self.ndim = ndim
        self.nvars = 3 * ndim + 5
        d = LptDesc()
        d.ndim, d.model, d.integration, d.device, d.capacity, d.dt = ndim, model, 1 if implicit else 0, device, capacity, dt
        d.gravity[:] = list(gravity) + [0.0] * (3 - len(gravity))
        d.rho_ambient, d.nu_ambient = rho_ambient, nu_ambient
        va = list(v_ambient) if v_ambient is not None else [0.0] * ndim
        d.v_ambient[:] = va + [0.0] * (3 - len(va))
        self.ctx = C.c_void_p()
        self._box = None
        self._check(self._lib.lbm_lpt_create(C.byref(d), C.byref(self.ctx)), "lbm_lpt_create")

    @classmethod
    def from_config(cls, solver: dict, ndim: int, capacity: int = 1024, device: int = 0) -> "ParticleSolver":
        """The reference's LPT ``solver`` block (keys and defaults of
        src/lpt/solver.cpp:94-228 and src/lpt/solver.h:231-240)."""
        model = solver.get("model", "constDensityRatioGravBuoStokesDrag")
        integ = solver.get("integrationMethod", "ForwardEuler")
        if model not in MODELS:
            raise ConfigError(f"Invalid model configuration! ({model})")
        if integ not in INTEGRATORS:
            raise ConfigError(f"Invalid integration method: {integ}")
        if "gravity" not in solver or "dt" not in solver:
            raise ConfigError('"gravity" and "dt" are required')
        return cls(ndim, MODELS.index(model), integ == "ImplicitEuler", float(solver["dt"]), [float(g) for g in solver["gravity"]],
                   float(solver.get("rho_infty", 1.205)), float(solver.get("nu_infty", 1.82e-5)),
                   [float(v) for v in solver.get("v_infty", [0.0] * ndim)], capacity=capacity, device=device)

    def _check(self, rc: int, what: str):
        if rc != _lib.LBM_OK:
            msg = self._lib.lbm_lpt_last_error(self.ctx) if self.ctx else None
            raise _lib.LBMError(rc, f"{what}: {msg.decode() if msg else ''}")

    def set_particles(self, vars_: np.ndarray):
        """particles x (3*ndim+5) doubles, the reference's m_vars layout"""
        a = np.ascontiguousarray(vars_, dtype=np.float64)
        if a.ndim != 2 or a.shape[1] != self.nvars:
            raise ValueError(f"expected (n, {self.nvars}) particle variables")
        self._check(self._lib.lbm_lpt_set_particles(self.ctx, a.shape[0], a.ctypes.data), "set_particles")

    def particles(self) -> np.ndarray:
        n = int(self._lib.lbm_lpt_count(self.ctx))
        out = np.empty((n, self.nvars), dtype=np.float64)
        self._check(self._lib.lbm_lpt_get_particles(self.ctx, out.ctypes.data), "get_particles")
        return out

    def step(self, n: int = 1):
        self._check(self._lib.lbm_lpt_step(self.ctx, int(n)), "step")

    def couple(self, box, origin: Sequence[float] = (0.0, 0.0, 0.0), cell_length: float = 1.0, velocity_scale: float = 1.0):
        """Ambient velocity from a :class:`~lbm_gb300.solver.BoxSolver` (its last
        step call's velocity at the particle's cell); ``None`` uncouples."""
        o = (C.c_double * 3)(*(list(origin) + [0.0] * (3 - len(origin))))
        self._check(self._lib.lbm_lpt_couple_box(self.ctx, box.ctx if box is not None else None, o, cell_length, velocity_scale),
                    "couple")
        self._box = box  # keep the box alive while coupled

    def close(self):
        if self.ctx:
            self._lib.lbm_lpt_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
