"""CPU restatement of the reference's particle step (TEST INFRASTRUCTURE).

Only tests/ and bench.py's CPU-baseline leg use this module, as the checker.
It restates LPTSolver::calcA and LPTSolver::timeIntegration
(src/lpt/solver.cpp:356-496) for the "Normal" particle type, with the force
models of src/lpt/forces.h, in the reference's operation order on IEEE
doubles, so that it reproduces the reference's particle state bit for bit
(pinned against the reference's own solver: tests/golden/lpt_*.npz, made by
tests/golden/make_golden.py through oracle/ref_lpt_harness.cpp).  The one
exception is the Putnam drag factor 1 + Re^(2/3)/6 for 0.1 < Re <= 1000: the
reference evaluates the power with gcem's constexpr series, this module with
the C library's pow, which differ in the last bits.

Particle layout (the reference's m_vars, src/lpt/particle.h:11-36):
center[D], velocity[D], a[D], radius, density, temperature, volume, DC.
"""
from __future__ import annotations

import math

import numpy as np

MODELS = ["constDensityRatioGrav", "constDensityRatioGravStokesDrag", "constDensityRatioGravNlinDrag", "constDensityRatioGravBuo",
          "constDensityRatioGravBuoStokesDrag", "constDensityRatioGravBuoNlinDrag", "constDensityaGravBuo",
          "constDensityaGravBuoStokesDrag", "constDensityaGravBuoNlinDrag"]
INTEGRATORS = ["ForwardEuler", "ImplicitEuler"]
DRAG = {1, 2, 4, 5, 7, 8}
NLIN = {2, 5, 8}
BUOYANT = {3, 4, 5, 6, 7, 8}
OWN_DENSITY = {6, 7, 8}  # the other models use particle 0's density for all


def putnam(re: float) -> float:
    """force::dragCoefficient<Putnam61> (src/lpt/forces.h)."""
    if re > 1000:
        return 0.424 * re / 24.0
    if re <= 0.1:
        return 1.0
    return 1.0 + math.pow(re, 2.0 / 3.0) / 6.0


def step(vars_: np.ndarray, ndim: int, model: int, implicit: bool, dt: float, gravity, rho_a: float, nu_a: float, v_a,
         nsteps: int = 1) -> np.ndarray:
    """nsteps particle steps on a copy of vars_ (particles x (3*ndim+5))."""
    D = ndim
    out = vars_.copy()
    R, RHO, DCI = 3 * D, 3 * D + 1, 3 * D + 4
    for _ in range(nsteps if out.shape[0] else 0):
        rho_p0 = out[0, RHO]
        for p in range(out.shape[0]):
            row = out[p]
            rho_p = row[RHO] if model in OWN_DENSITY else rho_p0
            r_p = row[R]
            vel = [row[D + d] for d in range(D)]
            # calcA
            if model in BUOYANT:
                fac = 1.0 - rho_a / rho_p
                a = [gravity[d] * fac for d in range(D)]
            else:
                a = [gravity[d] for d in range(D)]
            if model in DRAG:
                dc = 18.0 * nu_a / (4.0 * r_p * r_p * rho_p)
                if model in NLIN:
                    s = 0.0
                    for d in range(D):
                        s = vel[d] * vel[d] if d == 0 else s + vel[d] * vel[d]
                    re = rho_a * math.sqrt(s) * 2.0 * r_p / nu_a
                    dc *= putnam(re)
                if not implicit:
                    a = [a[d] + dc * (v_a[d] - vel[d]) for d in range(D)]
            else:
                dc = 0.0
            row[DCI] = dc
            # timeIntegration
            if not implicit:
                for d in range(D):
                    v = vel[d] + a[d] * dt
                    row[D + d] = v
                    row[d] = row[d] + v * dt
                    row[2 * D + d] = a[d]
            else:
                den = 1.0 + dc * dt
                for d in range(D):
                    v = (vel[d] + a[d] * dt + dc * v_a[d] * dt) / den
                    row[D + d] = v
                    row[2 * D + d] = (vel[d] - v) / dt
                    row[d] = row[d] + 0.5 * (v + vel[d]) * dt
    return out


def config_params(solver: dict, ndim: int):
    """model id, implicit flag and constants of a solver block, with the
    reference's defaults (src/lpt/solver.cpp:94-228, solver.h:231-240)."""
    model = MODELS.index(solver.get("model", "constDensityRatioGravBuoStokesDrag"))
    implicit = INTEGRATORS.index(solver.get("integrationMethod", "ForwardEuler")) == 1
    return dict(model=model, implicit=implicit, dt=float(solver["dt"]), gravity=[float(g) for g in solver["gravity"]],
                rho_a=float(solver.get("rho_infty", 1.205)), nu_a=float(solver.get("nu_infty", 1.82e-5)),
                v_a=[float(v) for v in solver.get("v_infty", [0.0] * ndim)])
