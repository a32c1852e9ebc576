"""Physics checks of the oracle's box engine where the reference has no
implementation to pin against (CPU).

The reference runs no 3D case, and it has no Guo forcing, free slip,
velocity inlet, zero-gradient outlet or D3Q7 lattice.  For those, the GPU
engine is checked against this oracle (tests/test_box_gpu.py,
test_configs_gpu.py), and the oracle itself is checked here against
solutions known in closed form:

* D3Q19 Guo-forced channel between halfway bounce-back walls: the parabola.
* Free-slip walls take no momentum: under a body force the total momentum
  grows by the force on every cell, every step.
* Equilibrium inlet, zero-gradient outlet and free-slip walls hold a uniform
  flow exactly.
* D3Q7 Poisson in its linear limit in a slab: sinh(kappa (L - x)) / sinh(kappa L).
"""
import numpy as np

import oracle

D2Q9, D3Q7, D3Q19 = 2, 3, 4


def test_d3q19_guo_channel_relaxes_to_the_parabola():
    ny, g, tau = 16, 1e-6, 0.8
    o = oracle.BoxOracle(D3Q19, (4, ny, 4), 1.0 / tau, faces=("periodic", "periodic", "wall", "wall", "periodic", "periodic"),
                         body_force=(g, 0.0, 0.0))
    o.init_equilibrium()
    o.step(20000, threads=4)
    _, u = o.moments()
    ux = u[0].reshape(4, ny, 4).mean(axis=(0, 2))
    nu = (tau - 0.5) / 3.0
    y = np.arange(ny) + 0.5  # distance of the cell centre from the wall half a cell below row 0
    exact = g / (2.0 * nu) * y * (ny - y)
    assert np.abs(ux - exact).max() / exact.max() < 1e-2
    assert np.abs(u[1]).max() < 1e-12 and np.abs(u[2]).max() < 1e-12  # rounding noise only


def test_free_slip_walls_take_no_momentum():
    shape, F = (6, 5, 4), 2e-6
    o = oracle.BoxOracle(D3Q19, shape, 1.0 / 0.7, faces=("periodic", "periodic") + ("freeslip",) * 4, body_force=(F, 0.0, 0.0))
    o.init_equilibrium()
    n = shape[0] * shape[1] * shape[2]

    def momentum():
        rho, u = o.moments()
        return (rho * u).sum(axis=1)

    o.step(10)
    p0 = momentum()
    o.step(300)
    p1 = momentum()
    assert abs((p1[0] - p0[0]) - 300 * F * n) <= 1e-9 * 300 * F * n
    assert np.abs(p1[1:]).max() < 1e-14


def test_inlet_outlet_and_free_slip_hold_a_uniform_flow():
    nx, u0 = 24, 0.05
    flags = np.zeros((6, 6, nx), dtype=np.uint8)
    flags[:, :, 0] = 2
    flags[:, :, -1] = 3
    o = oracle.BoxOracle(D3Q19, (nx, 6, 6), 1.0 / 0.6, faces=("open", "open") + ("freeslip",) * 4, flags=flags.reshape(-1),
                         inlet_velocity=(u0, 0.0, 0.0))
    o.init_equilibrium(1.0, (u0, 0.0, 0.0))
    o.step(500)
    rho, u = o.moments()
    assert np.abs(u[0] - u0).max() < 1e-13
    assert np.abs(u[1:]).max() < 1e-13
    assert np.abs(rho - 1.0).max() < 1e-13


def test_d3q7_debye_hueckel_slab():
    n, kappa = 48, 1.0 / 6.0
    flags = np.zeros((3, 3, n), dtype=np.uint8)
    phi = np.zeros((3, 3, n))
    flags[:, :, 0] = flags[:, :, -1] = 4  # Dirichlet cells
    phi[:, :, 0] = 1.0
    o = oracle.BoxOracle(D3Q7, (n, 3, 3), 1.0, faces=("wall", "wall") + ("periodic",) * 4, flags=flags.reshape(-1), equation=1,
                         kappa_sq=kappa * kappa, pb_nonlinear=False, dirichlet=phi.reshape(-1))
    o.init_equilibrium(0.0)
    o.step(8000, threads=4)
    p, _ = o.moments()
    prof = p.reshape(3, 3, n)[1, 1]
    x = np.arange(n, dtype=np.float64)
    L = n - 1
    exact = np.sinh(kappa * (L - x)) / np.sinh(kappa * L)
    assert np.abs(prof - exact).max() < 2e-2
