"""Batched D2Q9 lid-driven cavities (one persistent launch per step) against
the oracle's box engine, one cavity at a time.

Each cavity is an n x n box with halfway bounce-back walls and the +y wall
moving in x (the reference's moving-wall bounce-back with rho_w = 1).  The
oracle runs the same cavity alone in its deviation form; FP64 populations
agree within relative L2 1e-12 at both parities of the AA pattern, per-cavity
residuals agree with the oracle's moment differences, and converged cavities
freeze at the step count where they met the tolerance while the rest go on.
"""
import numpy as np
import pytest

import oracle
from helpers import rel_l2
from lbm_gb300._lib import LBMError
from lbm_gb300.solver import BatchSolver

pytestmark = pytest.mark.gpu
LID = 0.1
SIDES = [3, 7, 31, 32, 33, 50]
OMEGAS = [1.0, 1.9, 1.2, 0.7, 1.6, 1.75]


def cavity_oracle(n, omega, lid=LID):
    wv = np.zeros((6, 3))
    wv[3, 0] = lid
    o = oracle.BoxOracle(2, (n, n, 1), omega, faces=("wall",) * 6, wall_velocity=wv, deviation=True)
    o.init_equilibrium()
    return o


def moments_vec(o):
    rho, u = o.moments()
    return np.stack([rho, u[0], u[1]])


@pytest.mark.parametrize("storage", ["f64"])
def test_batch_fp64_matches_oracle_per_cavity(storage):
    b = BatchSolver(SIDES, OMEGAS, LID, storage)
    b.initial_condition()
    ors = [cavity_oracle(n, om) for n, om in zip(SIDES, OMEGAS)]
    done = 0
    for target in (1, 2, 37, 60):
        b.step(target - done)
        for o in ors:
            o.step(target - done)
        done = target
        for d, o in enumerate(ors):
            err = rel_l2(b.domain_populations(d), o.populations())
            assert err <= 1e-12, (target, SIDES[d], err)


def test_batch_residuals_match_oracle_moment_change():
    b = BatchSolver(SIDES, OMEGAS, LID, "f64")
    b.initial_condition()
    b.step(12)
    res = b.residuals()
    for d, (n, om) in enumerate(zip(SIDES, OMEGAS)):
        o = cavity_oracle(n, om)
        o.step(10)
        m10 = moments_vec(o)
        o.step(1)
        m11 = moments_vec(o)
        want = np.abs(m11 - m10).sum(axis=1)
        np.testing.assert_allclose(res[d], want, rtol=1e-9, atol=1e-300)


def test_batch_residuals_need_two_steps():
    b = BatchSolver([8, 9], [1.0, 1.0], LID, "f64")
    b.initial_condition()
    b.step(1)
    with pytest.raises(LBMError):
        b.residuals()


def test_batch_run_freezes_converged_cavities():
    sides = [8, 12, 24, 40]
    omegas = [1.0, 1.3, 1.5, 1.8]
    b = BatchSolver(sides, omegas, LID, "f64")
    b.initial_condition()
    tol = 1e-7
    steps = b.run(max_steps=3000, check_interval=50, tol=tol)
    assert steps.min() < steps.max(), steps  # small viscous cavities stop first
    assert steps.max() <= 3000
    for d, (n, om) in enumerate(zip(sides, omegas)):
        o = cavity_oracle(n, om)
        o.step(int(steps[d]) - 2)
        m0 = moments_vec(o)
        o.step(1)
        m1 = moments_vec(o)
        o.step(1)
        assert rel_l2(b.domain_populations(d), o.populations()) <= 1e-12
        r = np.abs(m1 - m0).sum(axis=1).max()
        if steps[d] < 3000:
            assert r < tol, (n, steps[d], r)
        else:
            assert r >= tol * 0.999, (n, steps[d], r)


@pytest.mark.parametrize("storage,bound", [("f32", 1e-5), ("f16dev", 5e-3), ("bf16dev", 5e-2)])
def test_batch_reduced_precision_against_fp64(storage, bound):
    b = BatchSolver(SIDES, OMEGAS, LID, storage)
    b.initial_condition()
    b.step(200)
    for d, (n, om) in enumerate(zip(SIDES, OMEGAS)):
        o = cavity_oracle(n, om)
        o.step(200)
        assert rel_l2(b.domain_populations(d), o.populations()) <= bound, (storage, n)


def test_batch_rejects_bad_descriptions():
    with pytest.raises(LBMError):
        BatchSolver([2, 8], [1.0, 1.0], LID, "f32")
    with pytest.raises(LBMError):
        BatchSolver([8, 8], [1.0, 2.0], LID, "f32")


def test_batch_run_reports_diverged_cavities():
    # BGK at tau 0.512 on a 40-cell cavity at Re ~1000 blows up (the FP64
    # oracle turns non-finite within 800 steps); the stable cavity goes on
    sides, omegas = [40, 16], [1.0 / 0.5120358287428449, 1.0]
    b = BatchSolver(sides, omegas, LID, "f64")
    b.initial_condition()
    steps = b.run(max_steps=3000, check_interval=50, tol=0.0, raise_on_divergence=False)
    assert list(b.status()) == [b.DIVERGED, b.ACTIVE]
    assert steps[0] < steps[1] == 3000
    b.initial_condition()
    assert list(b.status()) == [b.ACTIVE, b.ACTIVE]
    with pytest.raises(LBMError, match="diverged"):
        b.run(max_steps=3000, check_interval=50, tol=0.0)
