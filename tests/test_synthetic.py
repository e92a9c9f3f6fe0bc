"""The synthetic-state builder against the reference's grid and topography code."""

import numpy as np

from conftest import load_golden
from veros_gb300 import synthetic


def test_grid_and_topo_match_reference():
    g = load_golden("grid_topo")
    grid = synthetic.calc_grid(g["in_dxt"], g["in_dyt"], g["in_dzt"], 0.0, -60.0)
    for name in ("dxt", "dxu", "xt", "xu", "dyt", "dyu", "yt", "yu", "dzt", "dzw", "zt", "zw", "cost", "cosu"):
        np.testing.assert_allclose(grid[name], g[f"out_{name}"], rtol=1e-14, atol=1e-9, err_msg=name)
    kbot, mT, mU, mV, mW = synthetic.calc_topo(g["in_kbot"], int(g["nz"]))
    for name, arr in (("kbot", kbot), ("maskT", mT), ("maskU", mU), ("maskV", mV), ("maskW", mW)):
        assert np.array_equal(arr, g[f"out_{name}"]), name


def test_small_state_properties():
    st = synthetic.small_linear_state(seed=0)
    assert st.temp.shape == (68, 52, 20, 3)
    assert st.Ai_ez.shape == (68, 52, 20, 2, 2)
    assert st.kbot.dtype == np.int32 and st.maskT.dtype == np.bool_
    assert 0.10 < st.meta["land_fraction_realised"] < 0.20
    # tracers vanish on land and are identical on all time levels
    assert np.all(st.temp[~st.maskT] == 0)
    assert np.array_equal(st.temp[..., 0], st.temp[..., 2])
    # the rim is closed
    assert np.all(st.kbot[:2] == 0) and np.all(st.kbot[:, -2:] == 0)


def test_seed_determinism():
    a = synthetic.make_state(10, 8, 5, seed=3)
    b = synthetic.make_state(10, 8, 5, seed=3)
    c = synthetic.make_state(10, 8, 5, seed=4)
    assert np.array_equal(a.temp, b.temp) and np.array_equal(a.kbot, b.kbot)
    assert not np.array_equal(a.temp, c.temp)
