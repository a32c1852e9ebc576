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

FIXTURES = caseio.list_lpt_fixtures()


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
