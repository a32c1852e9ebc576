"""The C oracle against the reference's own CPU solver (golden fixtures).

The fixtures in tests/golden/ were produced by the reference built from its
own sources (oracle/build_ref.sh, tests/golden/make_golden.py).  The oracle
restates the reference's step in C in the same operation order; it must give
the same doubles, bit for bit, for every boundary-condition class, the
pressure forcing and the Poisson lattices.
"""
import numpy as np
import pytest

import caseio
import oracle
from helpers import load_case

FIXTURES = caseio.list_fixtures()


@pytest.mark.parametrize("name", FIXTURES)
def test_oracle_matches_reference_bitwise(name):
    meta, solver, grid, out, consts, bnds, forcing = load_case(name)
    # the host mirror of loadConfiguration reproduces the reference constants
    assert consts.omega == meta["omega"]
    assert consts.relax_time == meta["relaxTime"]
    assert consts.dt == meta["dt"]
    o = oracle.TableOracle(consts, grid, bnds, forcing)
    o.initial_condition()
    fold0 = o.state()[0]
    assert np.array_equal(fold0, out["fold0"])
    o.step(meta["steps"])
    fold, _, v, vo = o.state()
    assert np.array_equal(fold, out["fold"])
    assert np.array_equal(v, out["vars"])
    assert np.array_equal(vo, out["varsold"])
    assert np.array_equal(o.residual(), out["residual"])


def test_fixture_inventory_covers_every_boundary_kind():
    from lbm_gb300 import refconfig as rc
    kinds = set()
    forcing = False
    lattices = set()
    for name in FIXTURES:
        _, _, _, _, consts, bnds, f = load_case(name)
        kinds.update(b.kind for b in bnds)
        forcing |= f is not None
        lattices.add((consts.lattice, consts.equation))
    assert kinds == set(rc.BND_NAMES), sorted(set(rc.BND_NAMES) - kinds)
    assert forcing
    assert lattices == {(2, 0), (2, 1), (1, 1), (0, 1)}


def test_oracle_detects_a_planted_error():
    """A perturbed population in the oracle is visible in the comparison."""
    meta, solver, grid, out, consts, bnds, forcing = load_case("couette_1")
    o = oracle.TableOracle(consts, grid, bnds, forcing)
    o.initial_condition()
    fold0 = o.state()[0].copy()
    fold0[5] += 1e-12
    oracle.lib().ora_set_state(o.h, fold0.ctypes.data, None)
    o.step(1)
    assert not np.array_equal(o.state()[0], out["fold"])
