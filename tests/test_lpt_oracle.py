"""The particle oracle against the reference's own LPT solver.

tests/golden/lpt_*.npz hold the reference's LPTSolver state (m_vars) before
and after 2000 steps (oracle/ref_lpt_harness.cpp through make_golden.py): its
freefall tests and every force model with both integrators.  The oracle
(oracle/lpt_oracle.py) restates calcA and timeIntegration in the reference's
operation order and must reproduce them bit for bit.
"""
import numpy as np
import pytest

import caseio
import lpt_oracle as lo

FIXTURES = [f for f in caseio.list_lpt_fixtures() if "injection" not in f]  # injection: its own test below


def same(a, b):
    return np.array_equal(np.nan_to_num(a, nan=-7.25), np.nan_to_num(b, nan=-7.25))


@pytest.mark.parametrize("name", FIXTURES)
def test_oracle_matches_reference_bitwise(name):
    meta, solver, v0, v1, _ = caseio.load_lpt(name)
    prm = lo.config_params(solver, meta["ndim"])
    assert prm["dt"] == meta["dt"] and prm["rho_a"] == meta["rho_infty"] and prm["nu_a"] == meta["nu_infty"]
    out = lo.step(v0, meta["ndim"], nsteps=meta["steps"], **prm)
    assert same(out, v1)


def test_fixtures_cover_every_model_and_integrator():
    seen = set()
    for name in FIXTURES:
        meta, solver, *_ = caseio.load_lpt(name)
        prm = lo.config_params(solver, meta["ndim"])
        seen.add((prm["model"], prm["implicit"]))
        assert meta["particles"] == 10
    assert {m for m, _ in seen} == set(range(9))
    assert {i for _, i in seen} == {False, True}


def test_oracle_detects_a_planted_error():
    meta, solver, v0, v1, _ = caseio.load_lpt("lpt_falling_2000")
    prm = lo.config_params(solver, meta["ndim"])
    bad = v0.copy()
    bad[3, 0] += 1e-12
    assert not same(lo.step(bad, meta["ndim"], nsteps=meta["steps"], **prm), v1)


def test_injection_matches_reference():
    """Particle injection (the reference's 3D injection test, 100 steps): the
    host-side generator (lbm_gb300.lpt) with the oracle's step gives the
    reference's particles: the same number, and the same values up to the last
    bits of the elementary functions (gcem's series in the reference, the C
    library here)."""
    from lbm_gb300.lpt import Injector, RandXor, injection_step

    meta, solver, v0, v1, _ = caseio.load_lpt("lpt_injection_100")
    assert v0.shape[0] == 0 and v1.shape[0] > 500
    injectors = [Injector(solver["injection_model"])]
    prng = RandXor(1223)
    prm = lo.config_params(solver, 3)
    state = v0
    for _ in range(meta["steps"]):
        state = np.concatenate([state, injection_step(injectors, prng, prm["dt"])])
        state = lo.step(state, 3, nsteps=1, **prm)
    assert state.shape == v1.shape
    a, b = np.nan_to_num(state, nan=-7.25), np.nan_to_num(v1, nan=-7.25)
    assert np.allclose(a, b, rtol=1e-12, atol=1e-18)


def test_random_generator_known_answers():
    """xoshiro256+ seeded by splitmix64: the state is the first four outputs
    of splitmix64 for seed 0, the published test values."""
    from lbm_gb300.lpt import RandXor

    r = RandXor(0)
    assert r.s == [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F, 0xF88BB8A8724C81EC]
    assert r.next() == (0xE220A8397B1DCDAF + 0xF88BB8A8724C81EC) & ((1 << 64) - 1)  # xoshiro256+: s0 + s3
    assert 0.0 <= r.double() < 1.0
