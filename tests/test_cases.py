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


def test_stacked_debye_keeps_each_box_and_its_kappa():
    units = [cases.pb_spheres(n=20, seed=s, count=2) for s in (3, 5)]
    st = cases.stacked_debye(units)
    assert st["shape"] == (20, 20, 40)
    assert st["z0"] == [0, 20]
    assert st["slice_kappa_sq"] == [units[0]["kappa_sq"]] * 20 + [units[1]["kappa_sq"]] * 20
    flags = st["flags"].reshape(40, 20, 20)
    phi = st["dirichlet"].reshape(40, 20, 20)
    for k, u in enumerate(units):
        assert np.array_equal(flags[20 * k:20 * (k + 1)].reshape(-1), u["flags"])
        assert np.array_equal(phi[20 * k:20 * (k + 1)].reshape(-1), u["dirichlet"])
        # closed by Dirichlet planes at potential 0: nothing crosses between boxes
        assert np.all(flags[20 * k] == cases.DIRICHLET) and np.all(flags[20 * k + 19] == cases.DIRICHLET)


def test_stacked_debye_rejects_open_or_mismatched_boxes():
    a = cases.pb_spheres(n=20, seed=3, count=1)
    with pytest.raises(ValueError):
        cases.stacked_debye([a, cases.pb_spheres(n=16, seed=4, count=1)])
    b = dict(a, flags=a["flags"].copy())
    b["flags"].reshape(20, 20, 20)[0, 5, 5] = cases.FLUID
    with pytest.raises(ValueError):
        cases.stacked_debye([a, b])
