"""The oracle against golden vectors produced by the reference NumPy backend."""

import numpy as np
import pytest

from conftest import load_golden
from oracle import isoneutral_oracle as orc

ISO_CASES = ["iso_random_energy", "iso_random_noenergy", "iso_synth_eq1", "iso_synth_eq2", "iso_synth_eq3",
             "iso_synth_eq4"]


def _state_and_settings(g):
    arrays = {k[3:]: v.copy() for k, v in g.items() if k.startswith("in_")}
    settings = {k[8:]: v.item() for k, v in g.items() if k.startswith("setting_")}
    vs = orc.OracleState(arrays, tau=int(g["tau"]), taup1=int(g["taup1"]), taum1=int(g["taum1"]))
    return vs, settings


def _close(a, b, name):
    # the oracle restates the same NumPy expressions, so agreement is to rounding
    scale = max(np.max(np.abs(b)), 1e-300)
    err = np.max(np.abs(a - b)) / scale if a.size else 0.0
    assert err <= 1e-13, f"{name}: relative max-norm error {err:.3e}"


@pytest.mark.parametrize("case", ISO_CASES)
def test_pre_matches_reference(case):
    g = load_golden(case)
    vs, s = _state_and_settings(g)
    out = orc.isoneutral_diffusion_pre(vs, s)
    for k, v in out.items():
        _close(v, g[f"pre_{k}"], k)


@pytest.mark.parametrize("case", ISO_CASES)
def test_diffusion_chain_matches_reference(case):
    g = load_golden(case)
    vs, s = _state_and_settings(g)
    vs.__dict__.update(orc.isoneutral_diffusion_pre(vs, s))
    vs.__dict__.update(orc.isoneutral_diffusion(vs, s, True))
    for k in ("temp", "dtemp_iso", "P_diss_iso"):
        _close(getattr(vs, k), g[f"diffT_{k}"], f"T:{k}")
    vs.__dict__.update(orc.isoneutral_diffusion(vs, s, False))
    for k in ("salt", "dsalt_iso", "P_diss_iso"):
        _close(getattr(vs, k), g[f"diffS_{k}"], f"S:{k}")
    if f"skewT_temp" in g:
        vs.__dict__.update(orc.isoneutral_diffusion(vs, s, True, iso=False))
        for k in ("temp", "dtemp_iso", "P_diss_skew"):
            _close(getattr(vs, k), g[f"skewT_{k}"], f"skew:{k}")


def test_tridiag_matches_reference():
    g = load_golden("tridiag")
    out = orc.solve_tridiagonal(g["a"], g["b"], g["c"], g["d"], g["water_mask"], g["edge_mask"])
    np.testing.assert_allclose(out, g["out_random"], rtol=1e-13, atol=0)
    out = orc.solve_implicit(g["ad"], g["bd"], g["cd"], g["d"], g["water_mask"], g["edge_mask"],
                             b_edge=g["b_edge"], d_edge=g["d_edge"])
    np.testing.assert_allclose(out, g["out_dd"], rtol=1e-13, atol=0)


def test_water_masks_match_reference_semantics():
    g = load_golden("tridiag")
    _, wm, em = orc.create_water_masks(g["kbot"], g["a"].shape[-1])
    assert np.array_equal(wm, g["water_mask"])
    assert np.array_equal(em, g["edge_mask"])


def test_vertmix_and_streamfunction_match_reference():
    g = load_golden("vertmix_random")
    vs, s = _state_and_settings(g)
    out = orc.vertmix_tempsalt(vs, s)
    for k in ("temp", "salt", "dtemp_vmix", "dsalt_vmix"):
        assert np.array_equal(out[k], g[f"vmix_{k}"]), k
    out = orc.isoneutral_diag_streamfunction(vs)
    for k in ("B1_gm", "B2_gm"):
        _close(out[k], g[f"sf_{k}"], k)


def test_thermodynamics_sequence_matches_reference():
    """thermodynamics.py:425-441 (pre, diffusion and skew diffusion of both
    tracers, vertical mixing with the cyclic boundary exchange) on the
    reference's random state with enable_cyclic_x."""
    g = load_golden("thermo_cyclic")
    vs, s = _state_and_settings(g)
    assert s["enable_cyclic_x"]
    vs.P_diss_iso = np.zeros_like(vs.P_diss_iso)
    vs.dtemp_iso = np.zeros_like(vs.dtemp_iso)
    vs.dsalt_iso = np.zeros_like(vs.dsalt_iso)
    vs.__dict__.update(orc.isoneutral_diffusion_pre(vs, s))
    vs.__dict__.update(orc.isoneutral_diffusion(vs, s, True))
    vs.__dict__.update(orc.isoneutral_diffusion(vs, s, False))
    vs.P_diss_skew = np.zeros_like(vs.P_diss_skew)
    vs.__dict__.update(orc.isoneutral_diffusion(vs, s, True, iso=False))
    vs.__dict__.update(orc.isoneutral_diffusion(vs, s, False, iso=False))
    vs.__dict__.update(orc.vertmix_tempsalt(vs, s))
    for k in ("temp", "salt", "dtemp_iso", "dsalt_iso", "P_diss_iso", "P_diss_skew", "dtemp_vmix", "dsalt_vmix",
              "Ai_ez", "Ai_nz", "Ai_bx", "Ai_by", "K_11", "K_22", "K_33"):
        _close(getattr(vs, k), g[f"out_{k}"], k)


def test_enforce_boundaries_is_the_periodic_halo_copy():
    arr = np.arange(9 * 4 * 2, dtype=float).reshape(9, 4, 2)
    out = orc.enforce_boundaries(arr, True)
    assert np.array_equal(out[-2:], arr[2:4]) and np.array_equal(out[:2], arr[-4:-2])
    assert np.array_equal(out[2:-2], arr[2:-2])
    assert np.array_equal(orc.enforce_boundaries(arr, False), arr)


def test_float32_tridiag_matches_reference():
    """float32 systems: dgtsv in float64, the solution rounded to float32
    (veros/core/operators.py:64, :75-76), bit for bit."""
    g = load_golden("tridiag_f32")
    out = orc.solve_implicit(g["a"], g["b"], g["c"], g["d"], g["water_mask"], g["edge_mask"],
                             b_edge=g["b_edge"], d_edge=g["d_edge"])
    assert out.dtype == np.float32 and np.array_equal(out, g["out_dd"])
    out = orc.solve_tridiagonal(g["ra"], g["rb"], g["rc"], g["rd"], g["water_mask"], g["edge_mask"])
    assert out.dtype == np.float32 and np.array_equal(out, g["out_random"])
