"""The drop-ins as an installed Veros calls them, on the GPU.

``plugin.install()`` rebinds the names veros/core/thermodynamics.py looks up
at call time; a NumPy-backend Veros then hands its ``VerosState`` (host
arrays) to them. These tests run the tracer part of ``thermodynamics``
(thermodynamics.py:425-441: zeroed tendencies, pre, diffusion of temp and
salt, skew diffusion, vertical mixing) through the installed functions on a
stand-in of that state, and compare with the reference's own outputs of the
same sequence (``tests/golden/thermo_cyclic.npz``, a random state with a
cyclic x boundary, written by the reference NumPy backend). The same chain on
a device-resident state, and the float32 tridiagonal solve, are checked
against their goldens too.

Tolerance: FP64 relative max-norm 1e-12 per field, with the differencing
floors of the tendencies and of ``P_diss_iso`` (tests/conftest.py); the
cyclic halo columns and every cell the reference leaves alone are compared
like all others (the whole arrays).
"""

import numpy as np
import pytest

from conftest import assert_field_close, load_golden, p_diss_floor
from veros_like import plugin_call_sites, state_from_golden

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

OUT_FIELDS = ("temp", "salt", "dtemp_iso", "dsalt_iso", "P_diss_iso", "P_diss_skew", "dtemp_vmix", "dsalt_vmix",
              "Ai_ez", "Ai_nz", "Ai_bx", "Ai_by", "K_11", "K_22", "K_33")


def _check_thermo_outputs(g, get):
    """Compare every output field of the thermo_cyclic sequence; ``get(name)``
    returns this library's array in the reference layout."""
    dt = float(g["setting_dt_tracer"])
    settings = {k[8:]: v.item() for k, v in g.items() if k.startswith("setting_")}
    arrays = {k[3:]: v for k, v in g.items() if k.startswith("in_")}
    # P_diss_iso's floor: K_33 times 4 ulp of the new tracers (before vertical mixing, whose
    # output is what the golden holds: the same magnitude)
    arrays.update(K_33=g["out_K_33"], temp=g["out_temp"], salt=g["out_salt"])
    pfloor = p_diss_floor(arrays, settings, int(g["tau"]))
    for name in OUT_FIELDS:
        ref = g[f"out_{name}"]
        tracer = None
        if name in ("dtemp_iso", "dtemp_vmix"):
            tracer = g["out_temp"]
        elif name in ("dsalt_iso", "dsalt_vmix"):
            tracer = g["out_salt"]
        tol_name = {"dtemp_vmix": "dtemp_iso", "dsalt_vmix": "dsalt_iso"}.get(name, name)
        assert_field_close(tol_name, get(name), ref, tracer=tracer, dt=dt,
                           floor=pfloor if name == "P_diss_iso" else 0.0)
    # the closing boundary exchange of vertical mixing: periodic x halo of the new level
    tp1 = int(g["taup1"])
    for name in ("temp", "salt"):
        got = get(name)[..., tp1]
        assert np.array_equal(got[-2:], got[2:4]), name
        assert np.array_equal(got[:2], got[-4:-2]), name


def test_thermodynamics_sequence_through_installed_dropins(monkeypatch):
    """thermodynamics.py:425-441 verbatim, on a NumPy state, through plugin.install()."""
    g = load_golden("thermo_cyclic")
    mods, handle = plugin_call_sites(monkeypatch)
    try:
        isoneutral = mods["veros.core.isoneutral"]
        thermodynamics = mods["veros.core.thermodynamics"]
        state = state_from_golden(g)
        vs = state.variables
        settings = state.settings
        assert settings.enable_cyclic_x and settings.enable_neutral_diffusion and settings.enable_skew_diffusion

        vs.P_diss_iso = np.zeros_like(vs.P_diss_iso)
        vs.dtemp_iso = np.zeros_like(vs.dtemp_iso)
        vs.dsalt_iso = np.zeros_like(vs.dsalt_iso)

        vs.update(isoneutral.isoneutral_diffusion_pre(state))
        vs.update(isoneutral.isoneutral_diffusion(state, tr=vs.temp, istemp=True))
        vs.update(isoneutral.isoneutral_diffusion(state, tr=vs.salt, istemp=False))

        if settings.enable_skew_diffusion:
            vs.P_diss_skew = np.zeros_like(vs.P_diss_skew)
            vs.update(isoneutral.isoneutral_skew_diffusion(state, tr=vs.temp, istemp=True))
            vs.update(isoneutral.isoneutral_skew_diffusion(state, tr=vs.salt, istemp=False))

        vs.update(thermodynamics.vertmix_tempsalt(state))
    finally:
        handle.uninstall()
    _check_thermo_outputs(g, lambda n: getattr(vs, n))
    for name in OUT_FIELDS:  # results are host arrays of the reference's dtype and shape
        arr = getattr(vs, name)
        assert isinstance(arr, np.ndarray) and arr.dtype == np.float64 and arr.shape == g[f"out_{name}"].shape


def test_thermodynamics_sequence_on_float32_state(monkeypatch):
    """A float32 run (runtime_settings.float_type = "float32", veros/runtime.py:93):
    the installed functions compute in FP64 from the state's float32 arrays and
    vs.update stores their results as float32, so every output is float32 and
    stays within float32 rounding (1e-6 relative) of the same sequence on a
    float64 state holding the same (float32-rounded) inputs."""
    g = load_golden("thermo_cyclic")
    g32 = {k: (v.astype(np.float32).astype(np.float64) if k.startswith("in_") and v.dtype == np.float64 else v)
           for k, v in g.items()}
    mods, handle = plugin_call_sites(monkeypatch)
    try:
        s32 = state_from_golden(g32, float_type=np.float32)
        s64 = state_from_golden(g32)
        iso, thermo = mods["veros.core.isoneutral"], mods["veros.core.thermodynamics"]
        _thermo_sequence(iso, thermo, s32)
        from veros_gb300.state import release_host_mirrors

        release_host_mirrors()
        _thermo_sequence(iso, thermo, s64)
    finally:
        handle.uninstall()
    for name in OUT_FIELDS:
        got, ref = getattr(s32.variables, name), getattr(s64.variables, name)
        assert isinstance(got, np.ndarray) and got.dtype == np.float32 and got.shape == ref.shape, name
        scale = float(np.max(np.abs(ref)))
        err = float(np.max(np.abs(got.astype(np.float64) - ref))) / scale if scale else 0.0
        assert err <= 1e-6, (name, err)  # measured <= 8e-8: a few float32 ulps


def test_thermodynamics_sequence_on_device_state():
    """The same sequence with the fields resident on the GPU (DeviceState)."""
    from veros_gb300 import isoneutral, thermodynamics
    from veros_gb300.state import DeviceState
    from veros_gb300.synthetic import HostState

    g = load_golden("thermo_cyclic")
    arrays = {k[3:]: v for k, v in g.items() if k.startswith("in_")}
    settings = {k[8:]: v.item() for k, v in g.items() if k.startswith("setting_")}
    X, Y, Z = arrays["temp"].shape[:3]
    host = HostState(X - 4, Y - 4, Z, settings, arrays, tau=int(g["tau"]), taup1=int(g["taup1"]),
                     taum1=int(g["taum1"]))
    dev = DeviceState.from_host(host, device="cuda")
    v = dev.variables
    for n in ("P_diss_iso", "dtemp_iso", "dsalt_iso", "P_diss_skew"):
        getattr(v, n).zero_()
    v.update(isoneutral.isoneutral_diffusion_pre(dev))
    isoneutral.isoneutral_diffusion(dev, tr=v.temp, istemp=True)
    isoneutral.isoneutral_diffusion(dev, tr=v.salt, istemp=False)
    isoneutral.isoneutral_skew_diffusion(dev, tr=v.temp, istemp=True)
    isoneutral.isoneutral_skew_diffusion(dev, tr=v.salt, istemp=False)
    v.update(thermodynamics.vertmix_tempsalt(dev))
    torch.cuda.synchronize()
    _check_thermo_outputs(g, dev.download)


def test_vertmix_cyclic_flag_controls_the_halo():
    """enable_cyclic_x off: the halo columns of the new level keep their
    values (the reference's non-cyclic single-process exchange is a no-op);
    on: they are copies of the periodic interior columns, bit for bit."""
    from veros_gb300 import thermodynamics
    from veros_gb300.state import DeviceState
    from veros_gb300.synthetic import HostState

    g = load_golden("vertmix_random")
    arrays = {k[3:]: v for k, v in g.items() if k.startswith("in_")}
    settings = {k[8:]: v.item() for k, v in g.items() if k.startswith("setting_")}
    X, Y, Z = arrays["temp"].shape[:3]
    tp1 = int(g["taup1"])
    for cyclic in (False, True):
        settings["enable_cyclic_x"] = cyclic
        host = HostState(X - 4, Y - 4, Z, settings, arrays, tau=int(g["tau"]), taup1=int(g["taup1"]),
                         taum1=int(g["taum1"]))
        dev = DeviceState.from_host(host, device="cuda")
        thermodynamics.vertmix_tempsalt(dev)
        torch.cuda.synchronize()
        for n in ("temp", "salt"):
            got = dev.download(n)[..., tp1]
            assert_field_close(n, got[2:-2], g[f"vmix_{n}"][2:-2, ..., tp1])
            if cyclic:
                assert np.array_equal(got[-2:], got[2:4]) and np.array_equal(got[:2], got[-4:-2]), n
            else:
                before = arrays[n][..., tp1]
                assert np.array_equal(got[:2], before[:2]) and np.array_equal(got[-2:], before[-2:]), n


def test_enforce_boundaries_entry_point_matches_numpy():
    """vg_enforce_boundaries_f64 on one field against NumPy's assignments
    (veros/core/utilities.py:14-15), including the narrowest domain (X = 5),
    where sources and destinations overlap."""
    from veros_gb300 import _capi
    from veros_gb300.state import canonical_empty, pitch_for

    lib = _capi.load()
    rng = np.random.default_rng(4)
    for X, Y, Z in ((5, 6, 3), (6, 5, 2), (23, 9, 4)):
        arr = rng.standard_normal((X, Y, Z))
        t = canonical_empty(X, Y, Z, device="cuda")
        t.copy_(torch.from_numpy(arr))
        P = pitch_for(X)
        dom = _capi.VgDomain(X, Y, Z, P, P * Y)
        for flag in (0, 1):
            st = lib.vg_enforce_boundaries_f64(dom, t.data_ptr(), flag, torch.cuda.current_stream().cuda_stream)
            _capi.check(st, "vg_enforce_boundaries_f64")
            if flag:
                arr[-2:, ...] = arr[2:4, ...]
                arr[:2, ...] = arr[-4:-2, ...]
            torch.cuda.synchronize()
            assert np.array_equal(t.cpu().numpy(), arr), (X, Y, Z, flag)


def test_solve_implicit_float32_vs_reference_golden():
    """float32 systems: the reference's NumPy solve (dgtsv in float64, float32
    output) bit for bit, on diagonally dominant systems with edge
    substitution and on random ones with pivot interchanges; NumPy and device
    inputs."""
    from veros_gb300.utilities import solve_implicit, solve_tridiagonal

    g = load_golden("tridiag_f32")
    wm, em = g["water_mask"], g["edge_mask"]
    out = solve_implicit(g["a"], g["b"], g["c"], g["d"], wm, em, b_edge=g["b_edge"], d_edge=g["d_edge"])
    assert out.dtype == np.float32
    assert np.array_equal(out, g["out_dd"])
    out = solve_tridiagonal(g["ra"], g["rb"], g["rc"], g["rd"], wm, em)
    assert out.dtype == np.float32
    assert np.array_equal(out, g["out_random"])
    dev = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()  # noqa: E731
    bad = torch.zeros(1, dtype=torch.int32, device="cuda")
    out = solve_implicit(dev(g["a"]), dev(g["b"]), dev(g["c"]), dev(g["d"]), dev(wm), dev(em),
                         b_edge=dev(g["b_edge"]), d_edge=dev(g["d_edge"]), bad_columns=bad)
    assert out.dtype == torch.float32
    assert np.array_equal(out.cpu().numpy(), g["out_dd"])
    assert int(bad.item()) == 0
    # a float64 operand among float32 ones: dgtsv's float64 arithmetic, output in a's dtype
    out = solve_implicit(g["a"], g["b"], g["c"], g["d"].astype(np.float64), wm, em, b_edge=g["b_edge"],
                         d_edge=g["d_edge"])
    assert out.dtype == np.float32
    assert np.array_equal(out, g["out_dd"])


def _thermo_sequence(isoneutral, thermodynamics, state):
    """thermodynamics.py:425-441 on a NumPy state, as the first test runs it."""
    vs = state.variables
    vs.P_diss_iso = np.zeros_like(vs.P_diss_iso)
    vs.dtemp_iso = np.zeros_like(vs.dtemp_iso)
    vs.dsalt_iso = np.zeros_like(vs.dsalt_iso)
    vs.update(isoneutral.isoneutral_diffusion_pre(state))
    vs.update(isoneutral.isoneutral_diffusion(state, tr=vs.temp, istemp=True))
    vs.update(isoneutral.isoneutral_diffusion(state, tr=vs.salt, istemp=False))
    vs.P_diss_skew = np.zeros_like(vs.P_diss_skew)
    vs.update(isoneutral.isoneutral_skew_diffusion(state, tr=vs.temp, istemp=True))
    vs.update(isoneutral.isoneutral_skew_diffusion(state, tr=vs.salt, istemp=False))
    vs.update(thermodynamics.vertmix_tempsalt(state))
    vs.taum1, vs.tau, vs.taup1 = vs.tau, vs.taup1, vs.taum1


def test_host_mirror_uploads_only_changed_fields_and_changes_no_result(monkeypatch):
    """Two steps of the installed sequence with the device mirror kept between
    calls against the same steps with the mirror dropped before every call:
    identical arrays; the second step uploads less than a full state; the
    arrays the drop-ins return are read-only, as the NumPy backend's own."""
    from veros_gb300.state import DeviceState, release_host_mirrors

    g = load_golden("thermo_cyclic")
    mods, handle = plugin_call_sites(monkeypatch)
    try:
        iso, thermo = mods["veros.core.isoneutral"], mods["veros.core.thermodynamics"]
        kept, fresh = state_from_golden(g), state_from_golden(g)
        release_host_mirrors()
        uploads = []
        for _ in range(2):
            b0 = DeviceState.transfer_bytes["h2d"]
            _thermo_sequence(iso, thermo, kept)
            uploads.append(DeviceState.transfer_bytes["h2d"] - b0)
        for _ in range(2):
            # dropping the mirror before each call forces every field to be uploaded
            class Releasing:
                def __getattr__(self, n):
                    fn = getattr(iso if hasattr(iso, n) else thermo, n)

                    def call(*a, **k):
                        release_host_mirrors()
                        return fn(*a, **k)
                    return call
            r = Releasing()
            _thermo_sequence(r, r, fresh)
    finally:
        handle.uninstall()
        release_host_mirrors()
    for n in OUT_FIELDS:
        a, b = getattr(kept.variables, n), getattr(fresh.variables, n)
        assert np.array_equal(a, b), n
        assert not a.flags.writeable, n
    assert uploads[1] < 0.5 * uploads[0], uploads
