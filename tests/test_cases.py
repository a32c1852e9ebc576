"""Workload builders (lbm_gb300.cases), on CPU."""
import numpy as np
import pytest

from lbm_gb300 import cases


def test_stacked_sweep_keeps_each_channel_and_its_rate():
    chans = [cases.cylinder_channel(s, nx=96, ny=32) for s in (3, 5, 8)]
    st = cases.stacked_sweep(chans)
    assert st["shape"] == (96, 32, 3)
    flags = st["flags"].reshape(3, 32, 96)
    for k, c in enumerate(chans):
        assert np.array_equal(flags[k], c["flags"])
        assert st["slice_omega"][k] == 1.0 / c["tau"]
        # Re = u_in ny / nu, nu = (tau - 1/2) / 3
        assert abs(c["u_in"] * 32 / ((c["tau"] - 0.5) / 3.0) - c["re"]) < 1e-9 * c["re"]
    assert st["inlet_velocity"] == (chans[0]["u_in"], 0.0, 0.0)


def test_stacked_sweep_rejects_mixed_shapes():
    with pytest.raises(ValueError):
        cases.stacked_sweep([cases.cylinder_channel(1, nx=96, ny=32), cases.cylinder_channel(2, nx=64, ny=32)])
