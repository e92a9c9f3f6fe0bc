"""Generate the golden vectors that pin the oracle and the synthetic-state builder.

Runs the Veros reference NumPy backend in this process, so it only works
where a checkout of the reference exists; the ``.npz`` files it writes are
committed and the tests read only those. Usage::

    python tests/golden/make_golden.py /path/to/veros/checkout [case ...]

(or with the checkout in the ``REF_ROOT`` environment variable).

``loguru`` is not installed here, so a no-op stand-in module is registered
before Veros is imported (Veros only logs through it).

Cases (all float64, reference layout):

* ``iso_random_*``: the reference's own random-state fixture
  (veros/pyom_compat.py:487-526, seeded like test/conftest.py:31-35) at a small
  size with the settings of test/pyom_consistency/isoneutral_test.py:9-19;
  every variable, including the outputs' untouched cells, starts random.
  Runs pre, diffusion of temp and salt (energy branch on) and skew diffusion.
* ``iso_synth_eq1`` / ``iso_synth_eq3``: ``veros_gb300.synthetic.make_state``
  states run through the reference pre + diffusion(temp) + diffusion(salt).
* ``tridiag_random``: the reference's tridiagonal test form
  (test/pyom_consistency/tridiag_test.py:40-67) at a small size.
* ``grid_topo``: reference ``numerics.calc_grid`` / ``calc_topo`` outputs for the
  spacings and ``kbot`` the synthetic builder uses.
* ``vertmix_random``: ``vertmix_tempsalt`` (veros/core/thermodynamics.py:248-300)
  and ``isoneutral_diag_streamfunction_kernel`` (veros/core/isoneutral/isoneutral.py:232-254)
  on the random-state fixture, with a non-negative vertical diffusivity.
* ``thermo_cyclic``: the tracer part of ``thermodynamics`` as Veros calls it
  (veros/core/thermodynamics.py:425-441: zeroed tendencies, pre, diffusion of
  temp and salt, skew diffusion of both, vertical mixing with its closing
  boundary exchange) on a random state with ``enable_cyclic_x``.
* ``tridiag_f32``: the reference's NumPy solve on float32 systems (its float64
  LAPACK call and float32 output, veros/core/operators.py:60-77).
"""

import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def _import_reference(path):
    class _NoLog:
        def patch(self, *a, **k):
            return self

        def opt(self, *a, **k):
            return self

        def __getattr__(self, name):
            return lambda *a, **k: None

    mod = types.ModuleType("loguru")
    mod.logger = _NoLog()
    sys.modules.setdefault("loguru", mod)
    sys.path.insert(0, path)
    os.environ["VEROS_BACKEND"] = "numpy"
    import veros  # noqa: F401


PRE_FIELDS = ("Ai_ez", "Ai_nz", "Ai_bx", "Ai_by", "K_11", "K_22", "K_33")
INPUT_FIELDS = (
    "dxt", "dxu", "dyt", "dyu", "cost", "cosu", "dzt", "dzw", "zt", "kbot",
    "maskT", "maskU", "maskV", "maskW", "temp", "salt", "K_iso", "K_gm",
    "int_drhodT", "int_drhodS", "dtemp_iso", "dsalt_iso", "P_diss_iso", "P_diss_skew",
) + PRE_FIELDS
SETTING_KEYS = ("iso_slopec", "iso_dslope", "K_iso_steep", "dt_tracer", "grav", "rho_0",
                "eq_of_state_type", "enable_conserve_energy")


def _snapshot(vs, names):
    return {n: np.array(getattr(vs, n)).copy() for n in names}


def _settings_blob(settings):
    return {f"setting_{k}": np.array(getattr(settings, k)) for k in SETTING_KEYS}


def _run_iso_chain(state, with_skew):
    from veros.core import isoneutral

    vs = state.variables
    out = {}
    vs.update(isoneutral.isoneutral_diffusion_pre(state))
    out.update({f"pre_{k}": np.array(getattr(vs, k)).copy() for k in PRE_FIELDS})
    isoneutral.isoneutral_diffusion(state, vs.temp, True)
    for k in ("temp", "dtemp_iso", "P_diss_iso"):
        out[f"diffT_{k}"] = np.array(getattr(vs, k)).copy()
    isoneutral.isoneutral_diffusion(state, vs.salt, False)
    for k in ("salt", "dsalt_iso", "P_diss_iso"):
        out[f"diffS_{k}"] = np.array(getattr(vs, k)).copy()
    if with_skew:
        isoneutral.isoneutral_skew_diffusion(state, vs.temp, True)
        for k in ("temp", "dtemp_iso", "P_diss_skew"):
            out[f"skewT_{k}"] = np.array(getattr(vs, k)).copy()
    return out


def make_random_case(nx, ny, nz, conserve_energy):
    from veros.pyom_compat import get_random_state

    np.random.seed(17)
    settings = dict(nx=nx, ny=ny, nz=nz, dt_tracer=3600, dt_mom=3600, enable_neutral_diffusion=True,
                    enable_skew_diffusion=True, enable_TEM_friction=True, K_iso_steep=1,
                    enable_conserve_energy=conserve_energy)
    state = get_random_state(extra_settings=settings)
    vs = state.variables
    blob = {f"in_{k}": v for k, v in _snapshot(vs, INPUT_FIELDS).items()}
    blob.update(_settings_blob(state.settings))
    blob.update(tau=np.array(vs.tau), taup1=np.array(vs.taup1), taum1=np.array(vs.taum1))
    blob.update(_run_iso_chain(state, with_skew=True))
    return blob


def _reference_state_from_host(host):
    from veros.state import get_default_state

    state = get_default_state()
    s = host.settings
    with state.settings.unlock():
        state.settings.update(
            nx=host.nx, ny=host.ny, nz=host.nz, enable_neutral_diffusion=True, coord_degree=True,
            **{k: s[k] for k in SETTING_KEYS},
        )
    state.initialize_variables()
    state.variables.__locked__ = False
    vs = state.variables
    for name in INPUT_FIELDS:
        setattr(vs, name, host.arrays[name])
    return state


def make_synth_case(seed, eq_type, conserve_energy, sigma):
    sys.path.insert(0, REPO)
    from veros_gb300.synthetic import make_state

    host = make_state(16, 12, 10, seed=seed, y_origin=-60.0, dz_top=10.0, dz_bottom=400.0,
                      land_fraction=0.2, eq_of_state_type=eq_type, k_iso_lognormal_sigma=sigma,
                      settings=dict(enable_conserve_energy=conserve_energy))
    state = _reference_state_from_host(host)
    vs = state.variables
    blob = {f"in_{k}": v for k, v in _snapshot(vs, INPUT_FIELDS).items()}
    blob.update(_settings_blob(state.settings))
    blob.update(tau=np.array(vs.tau), taup1=np.array(vs.taup1), taum1=np.array(vs.taum1))
    blob.update(_run_iso_chain(state, with_skew=False))
    return blob


def make_vertmix_case(nx, ny, nz, seed):
    """vertmix_tempsalt and isoneutral_diag_streamfunction on the reference's random state."""
    from veros.core.isoneutral.isoneutral import isoneutral_diag_streamfunction_kernel
    from veros.core.thermodynamics import vertmix_tempsalt
    from veros.pyom_compat import get_random_state

    np.random.seed(seed)
    settings = dict(nx=nx, ny=ny, nz=nz, dt_tracer=3600, dt_mom=3600, enable_neutral_diffusion=True,
                    enable_skew_diffusion=True)
    state = get_random_state(extra_settings=settings)
    vs = state.variables
    # a physical (non-negative) vertical diffusivity, as the TKE/IDEMIX closures produce
    vs.kappaH = np.abs(np.asarray(vs.kappaH)) * 1e-2
    names = ("dxt", "dxu", "dyt", "dyu", "cost", "cosu", "dzt", "dzw", "zt", "kbot", "maskT", "maskU", "maskV",
             "maskW", "temp", "salt", "kappaH", "forc_temp_surface", "forc_salt_surface", "dtemp_vmix",
             "dsalt_vmix", "K_gm", "Ai_ez", "Ai_nz", "B1_gm", "B2_gm")
    blob = {f"in_{k}": v for k, v in _snapshot(vs, names).items()}
    blob.update(_settings_blob(state.settings))
    blob.update(tau=np.array(vs.tau), taup1=np.array(vs.taup1), taum1=np.array(vs.taum1))
    out = vertmix_tempsalt(state)
    for k in ("temp", "salt", "dtemp_vmix", "dsalt_vmix"):
        blob[f"vmix_{k}"] = np.array(getattr(out, k)).copy()
    out = isoneutral_diag_streamfunction_kernel(state)
    blob["sf_B1_gm"] = np.array(out.B1_gm).copy()
    blob["sf_B2_gm"] = np.array(out.B2_gm).copy()
    return blob


THERMO_FIELDS = ("dxt", "dxu", "dyt", "dyu", "cost", "cosu", "dzt", "dzw", "zt", "kbot", "maskT", "maskU",
                 "maskV", "maskW", "temp", "salt", "K_iso", "K_gm", "int_drhodT", "int_drhodS", "dtemp_iso",
                 "dsalt_iso", "P_diss_iso", "P_diss_skew", "kappaH", "forc_temp_surface", "forc_salt_surface",
                 "dtemp_vmix", "dsalt_vmix") + PRE_FIELDS
THERMO_OUT = ("temp", "salt", "dtemp_iso", "dsalt_iso", "P_diss_iso", "P_diss_skew", "dtemp_vmix",
              "dsalt_vmix") + PRE_FIELDS
THERMO_SETTINGS = SETTING_KEYS + ("enable_cyclic_x", "enable_neutral_diffusion", "enable_skew_diffusion")


def make_thermo_case(nx, ny, nz, seed):
    """thermodynamics.py:425-441 on the random-state fixture with a cyclic x boundary."""
    from veros.core import isoneutral
    from veros.core.thermodynamics import vertmix_tempsalt
    from veros.core.operators import update, at
    from veros.pyom_compat import get_random_state

    np.random.seed(seed)
    settings = dict(nx=nx, ny=ny, nz=nz, dt_tracer=3600, dt_mom=3600, enable_neutral_diffusion=True,
                    enable_skew_diffusion=True, enable_conserve_energy=True, enable_cyclic_x=True, K_iso_steep=1)
    state = get_random_state(extra_settings=settings)
    vs = state.variables
    vs.kappaH = np.abs(np.asarray(vs.kappaH)) * 1e-2  # non-negative, as the mixing closures produce
    blob = {f"in_{k}": v for k, v in _snapshot(vs, THERMO_FIELDS).items()}
    blob.update({f"setting_{k}": np.array(getattr(state.settings, k)) for k in THERMO_SETTINGS})
    blob.update(nx=np.array(nx), ny=np.array(ny), nz=np.array(nz))
    blob.update(tau=np.array(vs.tau), taup1=np.array(vs.taup1), taum1=np.array(vs.taum1))
    # veros/core/thermodynamics.py:425-441, the enable_neutral_diffusion branch and vertical mixing
    vs.P_diss_iso = update(vs.P_diss_iso, at[...], 0.0)
    vs.dtemp_iso = update(vs.dtemp_iso, at[...], 0.0)
    vs.dsalt_iso = update(vs.dsalt_iso, at[...], 0.0)
    vs.update(isoneutral.isoneutral_diffusion_pre(state))
    vs.update(isoneutral.isoneutral_diffusion(state, tr=vs.temp, istemp=True))
    vs.update(isoneutral.isoneutral_diffusion(state, tr=vs.salt, istemp=False))
    vs.P_diss_skew = update(vs.P_diss_skew, at[...], 0.0)
    vs.update(isoneutral.isoneutral_skew_diffusion(state, tr=vs.temp, istemp=True))
    vs.update(isoneutral.isoneutral_skew_diffusion(state, tr=vs.salt, istemp=False))
    vs.update(vertmix_tempsalt(state))
    blob.update({f"out_{k}": np.array(getattr(vs, k)).copy() for k in THERMO_OUT})
    return blob


def make_tridiag_f32_case():
    from veros.core.utilities import create_water_masks, solve_implicit

    rng = np.random.default_rng(23)
    nx, ny, nz = 12, 10, 16
    kbot = rng.integers(0, nz, size=(nx, ny))
    _, water_mask, edge_mask = create_water_masks(kbot, nz)
    delta = (np.abs(rng.standard_normal((nx, ny, nz))) * 3.0).astype(np.float32)
    a = -delta
    c = -np.roll(delta, -1, axis=-1)
    b = np.float32(1.0) + delta + np.roll(delta, -1, axis=-1)
    d = rng.standard_normal((nx, ny, nz)).astype(np.float32)
    b_edge = (1.0 + np.abs(rng.standard_normal((nx, ny, nz)))).astype(np.float32)
    d_edge = rng.standard_normal((nx, ny, nz)).astype(np.float32)
    # general (non-dominant) float32 systems: pivot interchanges in dgtsv
    ra, rb, rc, rd = (rng.standard_normal((nx, ny, nz)).astype(np.float32) for _ in range(4))
    out_dd = solve_implicit(a.copy(), b, c.copy(), d, water_mask, edge_mask, b_edge=b_edge, d_edge=d_edge)
    out_random = solve_implicit(ra.copy(), rb, rc.copy(), rd, water_mask, edge_mask)
    assert out_dd.dtype == np.float32 and out_random.dtype == np.float32
    return dict(a=a, b=b, c=c, d=d, b_edge=b_edge, d_edge=d_edge, kbot=kbot, water_mask=water_mask,
                edge_mask=edge_mask, out_dd=out_dd, ra=ra, rb=rb, rc=rc, rd=rd, out_random=out_random)


def make_tridiag_case():
    from veros.core.operators import solve_tridiagonal_numpy
    from veros.core.utilities import create_water_masks, solve_implicit

    np.random.seed(17)
    nx, ny, nz = 12, 10, 16
    a, b, c, d = (np.random.randn(nx, ny, nz) for _ in range(4))
    kbot = np.random.randint(0, nz, size=(nx, ny))
    _, water_mask, edge_mask = create_water_masks(kbot, nz)
    out_random = solve_tridiagonal_numpy(a, b, c, d, water_mask, edge_mask)
    # diagonally dominant systems of the implicit-mixing form, with b_edge/d_edge substitution
    delta = np.abs(np.random.randn(nx, ny, nz)) * 3.0
    ad = -delta
    cd = -np.roll(delta, -1, axis=-1)
    bd = 1.0 + delta + np.roll(delta, -1, axis=-1)
    b_edge = 1.0 + np.abs(np.random.randn(nx, ny, nz))
    d_edge = np.random.randn(nx, ny, nz)
    out_dd = solve_implicit(ad, bd, cd, d, water_mask, edge_mask, b_edge=b_edge, d_edge=d_edge)
    return dict(a=a, b=b, c=c, d=d, kbot=kbot, water_mask=water_mask, edge_mask=edge_mask, out_random=out_random,
                ad=ad, bd=bd, cd=cd, b_edge=b_edge, d_edge=d_edge, out_dd=out_dd)


def make_grid_case():
    sys.path.insert(0, REPO)
    from veros.core import numerics
    from veros.state import get_default_state
    from veros_gb300.synthetic import geometric_dz

    nx, ny, nz = 14, 11, 9
    rng = np.random.default_rng(5)
    dxt = np.full(nx + 4, 1.0) * (1 + 0.01 * rng.standard_normal(nx + 4))
    dyt = np.full(ny + 4, 1.0) * (1 + 0.01 * rng.standard_normal(ny + 4))
    dzt = geometric_dz(nz, 10.0, 400.0)
    kbot = np.zeros((nx + 4, ny + 4), dtype=np.int32)
    kbot[1:-1, 1:-1] = rng.integers(0, nz + 1, size=(nx + 2, ny + 2))

    state = get_default_state()
    with state.settings.unlock():
        state.settings.update(nx=nx, ny=ny, nz=nz, coord_degree=True, x_origin=0.0, y_origin=-60.0)
    state.initialize_variables()
    state.variables.__locked__ = False
    vs = state.variables
    vs.dxt, vs.dyt, vs.dzt, vs.kbot = dxt, dyt, dzt, kbot
    numerics.calc_grid(state)
    numerics.calc_topo(state)
    names = ("dxt", "dxu", "xt", "xu", "dyt", "dyu", "yt", "yu", "dzt", "dzw", "zt", "zw", "cost", "cosu",
             "kbot", "maskT", "maskU", "maskV", "maskW")
    blob = {f"out_{n}": np.array(getattr(vs, n)).copy() for n in names}
    blob.update(in_dxt=dxt, in_dyt=dyt, in_dzt=dzt, in_kbot=kbot, nx=np.array(nx), ny=np.array(ny), nz=np.array(nz))
    return blob


def main():
    """make_golden.py reference_root [case ...]: writes the named cases (all by default)."""
    args = sys.argv[1:]
    ref = args.pop(0) if args and os.path.isdir(os.path.join(args[0], "veros")) else os.environ.get("REF_ROOT")
    if not ref or not os.path.isdir(os.path.join(ref, "veros")):
        sys.exit("usage: make_golden.py <reference checkout> [case ...]  (or set REF_ROOT)")
    only = set(args)
    _import_reference(ref)
    makers = {
        "iso_random_energy": lambda: make_random_case(12, 10, 8, True),
        "iso_random_noenergy": lambda: make_random_case(10, 9, 7, False),
        "iso_synth_eq1": lambda: make_synth_case(0, 1, False, None),
        "iso_synth_eq2": lambda: make_synth_case(2, 2, True, None),
        "iso_synth_eq3": lambda: make_synth_case(1, 3, True, 0.3),
        "iso_synth_eq4": lambda: make_synth_case(3, 4, False, 0.3),
        "tridiag": make_tridiag_case,
        "vertmix_random": lambda: make_vertmix_case(12, 10, 9, 17),
        "thermo_cyclic": lambda: make_thermo_case(16, 12, 8, 29),
        "tridiag_f32": make_tridiag_f32_case,
        "grid_topo": make_grid_case,
    }
    cases = {name: make() for name, make in makers.items() if not only or name in only}
    for name, blob in cases.items():
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **blob)
        print(f"wrote {path} ({os.path.getsize(path) / 1024:.0f} KiB)")


if __name__ == "__main__":
    main()
