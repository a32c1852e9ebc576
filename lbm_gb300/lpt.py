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
import math
import struct
from collections import deque
from typing import List, Optional, Sequence

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
        self.dt = dt
        self._injectors: list = []
        self._prng = None
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
        gen = solver.get("generation_method", "none")
        if gen not in ("none", "injection"):
            raise ConfigError(f'generation method "{gen}" is not built')
        injectors = [Injector(solver.get("injection_model", {}))] if gen == "injection" else []
        ps = cls(ndim, MODELS.index(model), integ == "ImplicitEuler", float(solver["dt"]), [float(g) for g in solver["gravity"]],
                 float(solver.get("rho_infty", 1.205)), float(solver.get("nu_infty", 1.82e-5)),
                 [float(v) for v in solver.get("v_infty", [0.0] * ndim)], capacity=capacity, device=device)
        if injectors:
            ps._injectors = injectors
            ps._prng = RandXor(1223)  # the solver-wide generator of LPTSolver::injection
        return ps

    def advance(self, n: int = 1):
        """n time steps as LPTSolver::timeStep: with injection, each step first
        appends the step's new particles (generated on the host), then steps
        all particles on the GPU; without, one call of :meth:`step`."""
        if not self._injectors:
            self.step(n)
            return
        for _ in range(int(n)):
            new = injection_step(self._injectors, self._prng, self.dt)
            if len(new):
                self.set_particles(np.concatenate([self.particles(), new]))
            self.step(1)

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


# ---- particle injection (host side) -------------------------------------------
# The reference generates particles on the host before each step
# (LPTSolver::injection, src/lpt/solver.cpp:526-555; Injector,
# src/lpt/injection.h).  Restated here; the new particles are appended to the
# GPU state before the step kernel runs.  Elementary functions come from the C
# library, where the reference evaluates gcem's constexpr series, so sizes and
# directions can differ from the reference's in the last bits.

_M64 = (1 << 64) - 1


class RandXor:
    """The reference's pseudo-random generator (include/common/randxor.h):
    xoshiro256+ seeded with four outputs of splitmix64, both as published by
    Blackman and Vigna; doubles in [0, 1) from the top 52 bits."""

    def __init__(self, seed: int):
        self._sm = seed & _M64
        self.s = [self._splitmix() for _ in range(4)]

    def _splitmix(self) -> int:
        self._sm = (self._sm + 0x9E3779B97F4A7C15) & _M64
        z = self._sm
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _M64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _M64
        return z ^ (z >> 31)

    def next(self) -> int:
        s = self.s
        result = (s[0] + s[3]) & _M64
        t = (s[1] << 17) & _M64
        s[2] ^= s[0]
        s[3] ^= s[1]
        s[1] ^= s[2]
        s[0] ^= s[3]
        s[2] ^= t
        s[3] = ((s[3] << 45) | (s[3] >> 19)) & _M64
        return result

    def double(self, lo: Optional[float] = None, hi: Optional[float] = None) -> float:
        v = struct.unpack("<d", struct.pack("<Q", (self.next() >> 12) | (0x3FF << 52)))[0] - 1.0
        return v if lo is None else (v * (hi - lo)) + lo


def _cube(x: float) -> float:
    return x * x * x


def _pow(a: float, b: float) -> float:
    return math.exp(b * math.log(a))


def _normalized(v):
    n = math.sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2])
    return [v[0] / n, v[1] / n, v[2] / n] if n > 0 else list(v)


def _cross(a, b):
    return [a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]]


def _basis(normal):
    """Two unit vectors orthogonal to `normal`, built as the reference builds
    them (src/common/geometry/circle.h:15-48, random_special.h:20-88)."""
    c = _normalized(normal)
    v1 = [0.0, 0.0, 0.0]
    if abs(c[0]) > 0.0:
        v1[0] = 1.0 / c[0]
    elif abs(c[1]) > 0.0:
        v1[1] = 1.0 / c[1]
    else:
        v1[2] = 1.0 / c[2]
    eps = np.finfo(np.float64).eps
    if abs(normal[0]) < eps:
        v1[0] = 1.0
    elif abs(normal[1]) < eps:
        v1[1] = 1.0
    elif abs(normal[2]) < eps:
        v1[2] = 1.0
    v1 = _cross(v1, c)
    v2 = _cross(v1, c)
    return c, _normalized(v1), _normalized(v2)


class Injector:
    """One entry of ``injection_model`` (src/lpt/injection.h): mass inflow at
    ``mass_rate``, Rosin-Rammler droplet sizes around the hole diameter."""

    def __init__(self, cfg: dict):
        try:
            self.location = [float(x) for x in cfg["injector_location"]]
            self.orientation = [float(x) for x in cfg["injector_orientation"]]
            self.opening_angle = float(cfg["injector_opening_angle"])
            self.hole = float(cfg["injector_hole_diameter"])
            self.mass_rate = float(cfg["mass_rate"])
            self.density = float(cfg["injected_density"])
            self.velocity = float(cfg["injection_velocity"])
        except KeyError as exc:
            raise ConfigError(f"injection_model: missing {exc}") from None
        if len(self.location) != 3 or len(self.orientation) != 3:
            raise ConfigError("injection is 3D only (as in the reference)")
        self.mass = 0.0
        self.sizes: deque = deque()
        self.prng = RandXor(123342896)

    def _rosin_rammler(self) -> float:
        mean = self.hole
        rr_max, rr_min = 3.0 * mean, 0.3 * mean
        k = 1.0 - math.exp(-_cube((rr_max - rr_min) / mean))
        x = self.prng.double()
        return rr_min + mean * _pow(-math.log(1.0 - x * k), 1.0 / 3)

    def time_step(self, dt: float) -> int:
        """Injector::timeStep: the number of droplets this step, their sizes
        queued (a droplet larger than the mass left waits for the next step)."""
        self.mass += self.mass_rate * dt
        min_mass = 0.3 * self.density * 1.0 / 6.0 * math.pi * _cube(0.3 * self.hole)
        last = self.sizes[0] if self.sizes else math.nan
        self.sizes.clear()
        n = 0
        while self.mass > min_mass:
            d = self._rosin_rammler() if math.isnan(last) else last
            m = self.density * (1.0 / 6.0 * math.pi * _cube(d))
            last = math.nan
            self.sizes.append(d)
            if m > self.mass:
                return n
            self.mass -= m
            n += 1
        return n


def injection_step(injectors: List[Injector], prng: RandXor, dt: float) -> np.ndarray:
    """New particles of one step (LPTSolver::injection), in the particle
    layout (3D, 14 variables; acceleration, temperature and DC not set)."""
    rows = []
    for inj in injectors:
        n = inj.time_step(dt)
        c, v1, v2 = _basis(inj.orientation)
        cone = inj.opening_angle * 0.5 / 180.0 * math.pi
        for _ in range(n):
            # position: uniform angle and radius on the hole (randomPoint_inCircle)
            phi = prng.double(0.0, 2.0 * math.pi)
            dia = prng.double() * inj.hole
            cp, sp = math.cos(phi), math.sin(phi)
            pos = [inj.location[k] + (0.5 * dia) * (cp * v1[k] + sp * v2[k]) for k in range(3)]
            # direction within the cone (randomNormalizedDirection_inCone)
            phi = prng.double(0.0, 2.0 * math.pi)
            om = math.acos(prng.double(math.cos(cone), 1.0))
            so, co, cp, sp = math.sin(om), math.cos(om), math.cos(phi), math.sin(phi)
            d = _normalized([so * (cp * v1[k] + sp * v2[k]) + co * c[k] for k in range(3)])
            r = 0.5 * inj.sizes.popleft()
            row = [math.nan] * 14
            row[0:3] = pos
            row[3:6] = [inj.velocity * d[k] for k in range(3)]
            row[9], row[10] = r, inj.density
            row[12] = 4.0 / 3.0 * math.pi * _cube(r)
            rows.append(row)
    return np.array(rows, dtype=np.float64).reshape(-1, 14)

