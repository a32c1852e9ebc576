"""The oracle's box engine (CPU) against the reference's own fixtures.

The box restatement covers features the reference lacks (D3Q19, D3Q7, Guo
forcing, inlet/outlet, free slip); its 2D bounce-back limit is tied to the
reference here, on the Couette fixtures, in both of its arithmetic forms:

* plain form (populations f): relative L2 <= 1e-12 against the reference's
  populations, and
* deviation form (f - w_q, the form the GPU engine stores): the same bound,
  and within 1e-13 of the plain form.
"""
import numpy as np
import pytest

import oracle
from helpers import box_index, load_case, rel_l2
from lbm_gb300 import cases
from lbm_gb300 import refconfig as rc


def couette_oracle(name, deviation):
    meta, solver, grid, out, consts, bnds, forcing = load_case(name)
    ij, (nx, ny) = box_index(grid)
    tv = [b for b in bnds if b.kind == rc.BND_WALL_BB_TANGENTIAL][0].scalar
    wv = np.zeros((6, 3))
    wv[3, 0] = tv
    o = oracle.BoxOracle(rc.LATTICES["D2Q9"], (nx, ny, 1), consts.omega, faces=("periodic", "periodic", "wall", "wall", "wall", "wall"),
                         wall_velocity=wv, deviation=deviation)
    o.init_equilibrium()
    o.step(meta["steps"])
    idx = ij[:, 0] + nx * ij[:, 1]
    return o.populations()[:, idx].T, out["fold"].reshape(grid.ncells, 9)


@pytest.mark.parametrize("name", ["couette_1", "couette_50", "couette_1000"])
@pytest.mark.parametrize("deviation", [False, True])
def test_box_oracle_matches_reference_couette(name, deviation):
    f, ref = couette_oracle(name, deviation)
    assert rel_l2(f, ref) <= 1e-12


def test_deviation_form_tracks_plain_form():
    plain, _ = couette_oracle("couette_50", False)
    dev, _ = couette_oracle("couette_50", True)
    assert rel_l2(dev, plain) <= 1e-13


def test_deviation_form_on_a_forced_channel():
    c = cases.poiseuille_guo(nx=32, ny=16)
    kw = cases.box_kwargs(c)
    a = oracle.BoxOracle(c["lattice"], c["shape"], c["omega"], **kw)
    b = oracle.BoxOracle(c["lattice"], c["shape"], c["omega"], deviation=True, **kw)
    a.init_equilibrium()
    b.init_equilibrium()
    a.step(500)
    b.step(500)
    assert rel_l2(b.populations(), a.populations()) <= 1e-13
    ra, ua = a.moments()
    rb, ub = b.moments()
    assert np.abs(ra - rb).max() <= 1e-13


def _one_and_two_step_change(nx):
    c = cases.forced_channel(100000, nx, 32, re=40.0)
    st = cases.stacked_forced([c])
    o = oracle.BoxOracle(st["lattice"], st["shape"], st["omega"], deviation=True, **cases.box_kwargs(st))
    o.init_equilibrium()
    o.step(20000, threads=8)
    a = o.moments()[1][0].copy()
    o.step(1, threads=8)
    b = o.moments()[1][0].copy()
    o.step(1, threads=8)
    c2 = o.moments()[1][0].copy()
    return np.abs(b - a).sum(), np.abs(c2 - a).sum()


def test_even_periodic_channel_can_keep_a_period_two_mode():
    """Forced periodic channel, BGK + halfway bounce-back: for this geometry an
    even periodic length keeps an undamped period-2 (staggered) oscillation, so
    the one-step residual stalls near 1e-4 while the two-step change is at
    round-off; an odd length (127) has no such mode.  This is why the warm-start
    channels are 511 cells long."""
    one, two = _one_and_two_step_change(128)
    assert one > 1e-5 and two < 1e-10
    one_odd, _ = _one_and_two_step_change(127)
    assert one_odd < 1e-7


def test_debye_sweep_boxes_are_independent():
    """A Debye-length sweep as the engine runs it (lbm_gpu_box_set_slice_kappa):
    charged-sphere boxes of different Debye lengths, each closed by Dirichlet
    planes, stacked along z with a kappa^2 per z-slice.  In the oracle each
    stacked box steps bit for bit as a box of its own: the Dirichlet planes
    emit their own equilibrium whatever they receive, so nothing crosses."""
    from lbm_gb300 import cases

    units = [cases.pb_spheres(n=16, seed=s, count=1) for s in (3, 5, 9)]
    assert len({u["kappa_sq"] for u in units}) == 3
    st = cases.stacked_debye(units)
    o = oracle.BoxOracle(st["lattice"], st["shape"], st["omega"], pb_nonlinear=True, **cases.box_kwargs(st))
    o.set_slice_kappa(st["slice_kappa_sq"])
    o.init_equilibrium()
    o.step(30)
    f = o.populations()
    n3 = 16 ** 3
    for k, u in enumerate(units):
        one = oracle.BoxOracle(u["lattice"], u["shape"], u["omega"], pb_nonlinear=True, **cases.box_kwargs(u))
        one.init_equilibrium()
        one.step(30)
        assert np.array_equal(f[:, k * n3:(k + 1) * n3], one.populations()), k
    # one kappa^2 for every slice again: the stack differs from the sweep
    o.set_slice_kappa(None)
    o.init_equilibrium()
    o.step(30)
    assert not np.array_equal(o.populations()[:, n3:2 * n3], f[:, n3:2 * n3])
