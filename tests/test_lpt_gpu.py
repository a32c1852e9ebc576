"""The GPU particle step (include/lbm_lpt.h) against the reference's own LPT
solver, and its coupling to the dense-box LBM engine.

* Every fixture (the reference's LPTSolver, 2000 steps): the GPU state equals
  the reference's bit for bit.  The nonlinear-drag models differ only where
  the reference's gcem power and CUDA's pow round differently: relative
  1e-12 there.
* Step calls of any length give the same bits (each call keeps the particle
  state in registers for all its steps).
* Coupled to a box: a uniform flow gives the oracle's answer with that
  ambient velocity; a shear field is sampled at the particle's own cell.
"""
import numpy as np
import pytest

import caseio
import lpt_oracle as lo
from lbm_gb300.lpt import ParticleSolver
from lbm_gb300.solver import BoxSolver

pytestmark = pytest.mark.gpu
FIXTURES = [f for f in caseio.list_lpt_fixtures() if "injection" not in f]
NLIN = {2, 5, 8}


def close_or_same(a, b, model):
    a = np.nan_to_num(a, nan=-7.25)
    b = np.nan_to_num(b, nan=-7.25)
    if model in NLIN:
        return np.allclose(a, b, rtol=1e-12, atol=0)
    return np.array_equal(a, b)


def solver_for(name, capacity=64):
    meta, solver, v0, v1, _ = caseio.load_lpt(name)
    ps = ParticleSolver.from_config(solver, meta["ndim"], capacity=capacity)
    ps.set_particles(v0)
    return meta, solver, ps, v0, v1


@pytest.mark.parametrize("name", FIXTURES)
def test_gpu_matches_reference(name):
    meta, solver, ps, v0, v1 = solver_for(name)
    assert np.array_equal(np.nan_to_num(ps.particles(), nan=1), np.nan_to_num(v0, nan=1))
    ps.step(meta["steps"])
    model = lo.config_params(solver, meta["ndim"])["model"]
    assert close_or_same(ps.particles(), v1, model)


@pytest.mark.parametrize("name", ["lpt_falling_2000", "lpt_falling3d_2000", "lpt_constDensityRatioGravBuoNlinDrag_3d_2000"])
def test_chunked_calls_equal_one_call(name):
    meta, _, a, _, _ = solver_for(name)
    _, _, b, _, _ = solver_for(name)
    a.step(meta["steps"])
    for n in (1, 999, meta["steps"] - 1000):
        b.step(n)
    assert np.array_equal(np.nan_to_num(a.particles(), nan=1), np.nan_to_num(b.particles(), nan=1))


def _particles(n, ndim, rng, lo_, hi_, radius=0.01, density=50.0):
    v = np.full((n, 3 * ndim + 5), np.nan)
    v[:, :ndim] = rng.uniform(lo_, hi_, (n, ndim))
    v[:, ndim:2 * ndim] = 0.0
    v[:, 3 * ndim] = radius
    v[:, 3 * ndim + 1] = density
    v[:, 3 * ndim + 3] = 4.0 / 3.0 * np.pi * radius ** 3
    return v


def test_coupled_uniform_flow_matches_oracle():
    """A periodic D2Q9 box at rest in a uniform flow keeps it; particles with
    Stokes drag and no gravity follow the oracle with that ambient velocity."""
    u0 = (0.05, -0.02)
    box = BoxSolver(2, (16, 16, 1), 1 / 0.8, "f64", faces=("periodic",) * 4 + ("wall", "wall"), init_velocity=u0 + (0.0,))
    box.initial_condition()
    box.step(2)
    _, u = box.moments()
    assert np.allclose(u[0], u0[0], rtol=1e-13) and np.allclose(u[1], u0[1], rtol=1e-13)
    rng = np.random.default_rng(3)
    v0 = _particles(40, 2, rng, 0.0, 16.0, radius=1.0)
    # drag coefficient 18 nu / (4 r^2 rho_p) = 0.0045: forward Euler is stable
    ps = ParticleSolver(2, 7, False, 0.5, (0.0, 0.0), rho_ambient=1.0, nu_ambient=0.05, capacity=64)
    ps.set_particles(v0)
    ps.couple(box, (0.0, 0.0), 1.0, 1.0)
    ps.step(300)
    ref = lo.step(v0, 2, 7, False, 0.5, [0.0, 0.0], 1.0, 0.05, list(u0), nsteps=300)
    got = ps.particles()
    assert np.allclose(got[:, :6], ref[:, :6], rtol=1e-12, atol=1e-15)


def test_coupled_field_is_read_at_the_particle_cell():
    """A shear field u = (U sin(2 pi y / ny), U sin(2 pi x / nx)); with a huge
    drag and implicit Euler one particle step takes the ambient velocity of
    the particle's cell, which must be that cell's (not a neighbour's)."""
    nx, ny, U = 48, 40, 0.04
    x = np.arange(nx) + 0.5
    y = np.arange(ny) + 0.5
    X, Y = np.meshgrid(x, y)  # (ny, nx), x fastest when flattened
    ux = U * np.sin(2 * np.pi * Y / ny)
    uy = U * np.sin(2 * np.pi * X / nx)
    c = np.array([[-1, 0], [1, 0], [0, -1], [0, 1], [1, 1], [1, -1], [-1, -1], [-1, 1], [0, 0]], dtype=float)
    w = np.array([1 / 9] * 4 + [1 / 36] * 4 + [4 / 9])
    usq = ux ** 2 + uy ** 2
    f = np.stack([w[q] * (1 + 3 * (c[q, 0] * ux + c[q, 1] * uy) + 4.5 * (c[q, 0] * ux + c[q, 1] * uy) ** 2 - 1.5 * usq)
                  for q in range(9)]).reshape(9, -1)
    box = BoxSolver(2, (nx, ny, 1), 1 / 0.9, "f64", faces=("periodic",) * 4 + ("wall", "wall"))
    box.set_populations(f)
    box.step(1)  # records the moments of the state it started from: the field above
    u = (ux.ravel(), uy.ravel())
    rng = np.random.default_rng(8)
    v0 = _particles(200, 2, rng, 0.0, [nx, ny])
    # drag coefficient 18 nu / (4 r^2 rho_p) * dt >> 1: v1 = (v0 + DC va dt) / (1 + DC dt) ~ va
    ps = ParticleSolver(2, 7, True, 1.0, (0.0, 0.0), rho_ambient=1.0, nu_ambient=1e4, capacity=256)
    ps.set_particles(v0)
    ps.couple(box, (0.0, 0.0), 1.0, 1.0)
    ps.step(1)
    got = ps.particles()[:, 2:4]
    cell = np.floor(v0[:, 0]).astype(int) + nx * np.floor(v0[:, 1]).astype(int)
    expect = np.stack([u[0][cell], u[1][cell]], axis=1)
    # v1 = va DC dt / (1 + DC dt): within 1e-7 relative of the cell's velocity
    assert np.allclose(got, expect, rtol=1e-6, atol=1e-12)
    neighbour = np.stack([u[0][(cell + nx) % (nx * ny)], u[1][(cell + 1) % (nx * ny)]], axis=1)
    assert np.abs(got - neighbour).max() > 1e-3


def test_uncoupled_again_and_errors():
    from lbm_gb300._lib import LBMError

    ps = ParticleSolver(2, 4, False, 1e-3, (0.0, -9.81), capacity=4)
    with pytest.raises(LBMError):
        ps.set_particles(np.zeros((5, 11)))
    box = BoxSolver(2, (8, 8, 1), 1.2, "f64", faces=("periodic",) * 4 + ("wall", "wall"))
    box.initial_condition()
    ps.set_particles(_particles(3, 2, np.random.default_rng(1), 1.0, 7.0))
    ps.couple(box, (0.0, 0.0), 1.0, 1.0)
    with pytest.raises(LBMError):
        ps.step(1)  # the box has not stepped: no velocity field yet
    ps.couple(None)
    ps.step(3)


def test_injection_through_advance_matches_reference():
    """The reference's 3D injection test (100 steps) through
    ParticleSolver.advance on the GPU: each step appends the host-generated
    new particles, then steps every particle on the device.  Same particle
    count as the reference's, values up to the last bits of the elementary
    functions (gcem's series in the reference, the C library and CUDA here)."""
    meta, solver, v0, v1, _ = caseio.load_lpt("lpt_injection_100")
    assert v0.shape[0] == 0 and v1.shape[0] > 500
    ps = ParticleSolver.from_config(solver, meta["ndim"], capacity=2 * v1.shape[0])
    ps.advance(meta["steps"])
    got = ps.particles()
    assert got.shape == v1.shape
    a, b = np.nan_to_num(got, nan=-7.25), np.nan_to_num(v1, nan=-7.25)
    assert np.allclose(a, b, rtol=1e-12, atol=1e-18)
