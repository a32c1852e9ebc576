"""Host parts of the learned warm start (lbm_gb300.warmstart), on CPU, with
the oracle's box engine standing in for the GPU solver where a state is
needed."""
import numpy as np
import pytest

import oracle
from lbm_gb300 import cases
from lbm_gb300 import warmstart as ws


def test_aitken_recovers_the_limit_of_an_exponential_relaxation():
    t = np.array([2500.0, 4500.0, 6500.0])
    p_inf = np.array([120.0, 80.0, 95.0])
    amp = np.array([-60.0, 30.0, -5.0])
    T = np.array([5000.0, 2000.0, 8000.0])
    pa, pb, pc = (p_inf + amp * np.exp(-tt / T) for tt in t)
    s = ws.aitken_scales(pa, pb, pc)
    assert np.allclose(s * pc, p_inf, rtol=1e-12)
    # not contracting (growing, or oscillating): left alone
    assert np.all(ws.aitken_scales([1.0, 1.0], [2.0, 0.5], [4.0, 0.8]) == 1.0)


@pytest.mark.parametrize("s", [1.0, 1.7, 0.6])
def test_rescale_flow_scales_the_guo_velocity(s):
    """A developed forced channel (oracle): rescaling by s multiplies every
    fluid cell's Guo velocity by s (to the size of the body force) and leaves
    the solid cells' populations as they were."""
    chans = [ws.cases.forced_channel(seed, 48, 16, re=30.0) for seed in (1, 2)]
    st = cases.stacked_forced(chans)
    o = oracle.BoxOracle(st["lattice"], st["shape"], st["omega"], **cases.box_kwargs(st))
    o.init_equilibrium()
    o.step(3000, threads=4)
    f0 = o.populations().copy()
    _, u0 = o.moments()
    ws.rescale_flow(o, chans, np.array([s, s]))
    f1 = o.populations()
    _, u1 = o.moments()
    fluid = np.concatenate([(c["flags"] != cases.SOLID).reshape(-1) for c in chans])
    g = max(c["g"] for c in chans)
    for d in range(2):
        assert np.allclose(u1[d][fluid], s * u0[d][fluid], rtol=0, atol=abs(1 - s) * g + 1e-15)
    assert np.array_equal(f1[:, ~fluid], f0[:, ~fluid])
