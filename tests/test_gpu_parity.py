"""GPU parity: the CUDA path against the reference's golden outputs and the oracle.

Tolerance (FP64): relative max-norm ``max|gpu - ref| / max|ref| <= 1e-12`` per
field. Cells the reference leaves untouched must keep their previous contents
bit for bit, and masked (land) cells must be exactly zero where the reference
multiplies by a mask.
"""

import numpy as np
import pytest

from conftest import assert_field_close, load_golden, p_diss_floor

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

TOL = 1e-12


def _rel(got, ref):
    scale = np.max(np.abs(ref)) if ref.size else 0.0
    if scale == 0.0:
        return float(np.max(np.abs(got))) if got.size else 0.0
    return float(np.max(np.abs(got - ref)) / scale)


def _golden_device_state(g):
    from veros_gb300.state import DeviceState
    from veros_gb300.synthetic import HostState

    arrays = {k[3:]: v for k, v in g.items() if k.startswith("in_")}
    settings = {k[8:]: v.item() for k, v in g.items() if k.startswith("setting_")}
    X, Y, Z = arrays["temp"].shape[:3]
    host = HostState(X - 4, Y - 4, Z, settings, arrays, tau=int(g["tau"]), taup1=int(g["taup1"]),
                     taum1=int(g["taum1"]))
    return DeviceState.from_host(host, device="cuda")


# output sub-ranges written by isoneutral_diffusion_pre (isoneutral.py:130-225)
def _written(name, shape):
    X, Y, Z = shape[:3]
    w = np.zeros(shape, dtype=bool)
    if name == "K_11":
        w[1:-2, 2:-2, :] = True
    elif name == "K_22":
        w[2:-2, 1:-2, :] = True
    elif name == "K_33":
        w[2:-2, 2:-2, :-1] = True
        w[:, :, -1] = True
    elif name == "Ai_ez":
        w[1:-2, 2:-2, 1:, :, 0] = True
        w[1:-2, 2:-2, :, :, 1] = True
    elif name == "Ai_nz":
        w[2:-2, 1:-2, 1:, :, 0] = True
        w[2:-2, 1:-2, :, :, 1] = True
    elif name in ("Ai_bx", "Ai_by"):
        w[2:-2, 2:-2, :-1] = True
    return w


@pytest.mark.parametrize("case", ["iso_random_energy", "iso_random_noenergy", "iso_synth_eq1", "iso_synth_eq2",
                                  "iso_synth_eq3", "iso_synth_eq4"])
def test_pre_vs_reference_golden(case):
    from veros_gb300.isoneutral import run_pre

    g = load_golden(case)
    dev = _golden_device_state(g)
    run_pre(dev)
    torch.cuda.synchronize()
    for name in ("Ai_ez", "Ai_nz", "Ai_bx", "Ai_by", "K_11", "K_22", "K_33"):
        got, ref, before = dev.download(name), g[f"pre_{name}"], g[f"in_{name}"]
        assert _rel(got, ref) <= TOL, f"{name}: {_rel(got, ref):.3e}"
        untouched = ~_written(name, got.shape)
        assert np.array_equal(got[untouched], before[untouched]), f"{name}: untouched cells changed"


@pytest.mark.parametrize("case", ["iso_random_energy", "iso_random_noenergy", "iso_synth_eq1", "iso_synth_eq2",
                                  "iso_synth_eq3", "iso_synth_eq4"])
def test_diffusion_chain_vs_reference_golden(case):
    from veros_gb300.isoneutral import run_diffusion, run_pre

    g = load_golden(case)
    dev = _golden_device_state(g)
    run_pre(dev)
    run_diffusion(dev, istemp=True)
    torch.cuda.synchronize()
    dt = float(g["setting_dt_tracer"])
    settings = {k[8:]: v.item() for k, v in g.items() if k.startswith("setting_")}
    arrays = {k[3:]: v for k, v in g.items() if k.startswith("in_")}
    arrays.update(K_33=g["pre_K_33"], temp=g["diffT_temp"], salt=g["diffS_salt"])
    pfloor = p_diss_floor(arrays, settings, int(g["tau"]))
    for name in ("temp", "dtemp_iso", "P_diss_iso"):
        assert_field_close(name, dev.download(name), g[f"diffT_{name}"], tracer=g["diffT_temp"], dt=dt,
                           floor=pfloor if name == "P_diss_iso" else 0.0)
    run_diffusion(dev, istemp=False)
    torch.cuda.synchronize()
    for name in ("salt", "dsalt_iso", "P_diss_iso"):
        assert_field_close(name, dev.download(name), g[f"diffS_{name}"], tracer=g["diffS_salt"], dt=dt,
                           floor=pfloor if name == "P_diss_iso" else 0.0)
    if "skewT_temp" in g:
        run_diffusion(dev, istemp=True, skew=True)
        torch.cuda.synchronize()
        for name in ("temp", "dtemp_iso", "P_diss_skew"):
            assert_field_close(name, dev.download(name), g[f"skewT_{name}"], tracer=g["skewT_temp"], dt=dt)


def test_tridiag_vs_reference_golden():
    from veros_gb300.utilities import solve_implicit, solve_tridiagonal

    g = load_golden("tridiag")
    # the reference's own random-matrix test form and tolerance (tridiag_test.py:40-67)
    out = solve_tridiagonal(g["a"], g["b"], g["c"], g["d"], g["water_mask"], g["edge_mask"])
    np.testing.assert_allclose(out, g["out_random"], rtol=1e-7)
    assert np.all(out[~g["water_mask"]] == 0.0)
    # dgtsv's operation order without contraction: identical bits, interchanges included
    assert np.array_equal(out, g["out_random"])
    out = solve_implicit(g["ad"], g["bd"], g["cd"], g["d"], g["water_mask"], g["edge_mask"],
                         b_edge=g["b_edge"], d_edge=g["d_edge"])
    assert _rel(out, g["out_dd"]) <= TOL
    assert np.array_equal(out, g["out_dd"])


def test_tridiag_device_tensors_and_bad_masks():
    from veros_gb300.utilities import solve_tridiagonal, create_water_masks

    rng = np.random.default_rng(1)
    nx, ny, nz = 30, 20, 15
    kbot = rng.integers(0, nz + 1, size=(nx, ny))
    _, wm, em = create_water_masks(kbot, nz)
    a, c = -rng.random((2, nx, ny, nz))
    b = 2.5 + rng.random((nx, ny, nz))
    d = rng.standard_normal((nx, ny, nz))
    out_host = solve_tridiagonal(a, b, c, d, wm, em)
    dev = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()  # noqa: E731
    out_dev = solve_tridiagonal(dev(a), dev(b), dev(c), dev(d), dev(wm), dev(em))
    assert np.array_equal(out_dev.cpu().numpy(), out_host)
    from oracle.isoneutral_oracle import solve_tridiagonal as ref

    assert _rel(out_host, ref(a, b, c, d, wm, em)) <= TOL
    bad = wm.copy()
    bad[0, 0, :] = False
    bad[0, 0, nz - 1] = True
    bad[0, 0, 0] = True
    with pytest.raises(ValueError):
        solve_tridiagonal(a, b, c, d, bad, em)


@pytest.mark.parametrize("dtype", ["double", "float"])
def test_xla_tdma_entry_point(dtype):
    """The XLA custom-call target against scipy's banded solver. Systems
    scaled by 1e-300 and 1e300 (same solution) have pivots outside the FP32
    range, where the double kernel's reciprocal falls back to the IEEE
    quotient."""
    import ctypes

    from scipy.linalg import solve_banded

    from veros_gb300 import _capi

    rng = np.random.default_rng(2)
    nsys, depth = 1000, 40
    a = -rng.random((depth, nsys))
    c = -rng.random((depth, nsys))
    b = 3.0 + rng.random((depth, nsys))
    d = rng.standard_normal((depth, nsys))
    scale = np.ones(nsys)
    if dtype == "double":
        scale[1::3] = 1e-300
        scale[2::3] = 1e300
    a, b, c, d = (x * scale for x in (a, b, c, d))
    tdt, ndt, tol = (torch.float64, np.float64, 1e-13) if dtype == "double" else (torch.float32, np.float32, 1e-5)
    bufs = [torch.from_numpy(x.astype(ndt)).cuda() for x in (a, b, c, d)]
    bufs += [torch.empty((depth, nsys), dtype=tdt, device="cuda")] * 2
    ptrs = (ctypes.c_void_p * 6)(*(t.data_ptr() for t in bufs))
    desc = np.array([nsys, depth], dtype=np.int32).tobytes()
    lib = _capi.load()
    getattr(lib, f"vg_tdma_cuda_{dtype}")(ctypes.c_void_p(torch.cuda.current_stream().cuda_stream), ptrs, desc,
                                          len(desc))
    torch.cuda.synchronize()
    assert _capi.last_error() == ""
    out = bufs[4].cpu().numpy().astype(np.float64)
    for s in list(range(0, nsys, 97)) + [1, 2, 4, 5]:
        ab = np.zeros((3, depth))
        ab[0, 1:] = c[:-1, s]
        ab[1] = b[:, s]
        ab[2, :-1] = a[1:, s]
        ref = solve_banded((1, 1), ab, d[:, s])
        assert _rel(out[:, s], ref) <= tol, s


@pytest.mark.parametrize("dtype", ["double", "float"])
def test_xla_tdma_matches_reference_cuda_kernel(dtype):
    """vg_tdma_cuda_* against the reference's own CUDA kernel (TridiagKernel,
    veros/core/special/cuda_tdma_kernels.cu:19-63, built from its source for
    sm_103a) on the same buffers: the same Thomas recurrence, with a
    reciprocal within an ulp of the reference's quotient in double."""
    import ctypes

    from oracle import ref_tdma
    from veros_gb300 import _capi

    if not ref_tdma.available():
        pytest.skip("reference TDMA kernel not built (oracle/_ref)")
    ref = ref_tdma.ReferenceTdma()
    rng = np.random.default_rng(7)
    nsys, depth = 5000, 60
    tdt, ndt, tol = (torch.float64, np.float64, 1e-13) if dtype == "double" else (torch.float32, np.float32, 1e-5)
    a = -rng.random((depth, nsys))
    c = -rng.random((depth, nsys))
    b = 2.2 + rng.random((depth, nsys))
    d = rng.standard_normal((depth, nsys))
    ins = [torch.from_numpy(x.astype(ndt)).cuda() for x in (a, b, c, d)]
    outs = {}
    for who in ("ours", "reference"):
        out, ws = torch.empty((depth, nsys), dtype=tdt, device="cuda"), torch.empty((depth, nsys), dtype=tdt,
                                                                                    device="cuda")
        ptrs = [t.data_ptr() for t in ins] + [out.data_ptr(), ws.data_ptr()]
        stream = torch.cuda.current_stream().cuda_stream
        if who == "ours":
            desc = np.array([nsys, depth], dtype=np.int32).tobytes()
            getattr(_capi.load(), f"vg_tdma_cuda_{dtype}")(ctypes.c_void_p(stream), (ctypes.c_void_p * 6)(*ptrs),
                                                          desc, len(desc))
        else:
            ref(stream, ptrs, nsys, depth, dtype == "double")
        torch.cuda.synchronize()
        outs[who] = out.cpu().numpy().astype(np.float64)
    assert _capi.last_error() == ""
    scale = np.abs(outs["reference"]).max(axis=0)
    assert np.all(np.abs(outs["ours"] - outs["reference"]).max(axis=0) <= tol * scale)


def _oracle_steps(host, n):
    from oracle import isoneutral_oracle as orc

    vs = orc.OracleState({k: v.copy() for k, v in host.arrays.items()})
    for _ in range(n):
        orc.isoneutral_step(vs, host.settings)
    return vs


def _check_state(dev, vs, names, settings, tau_in):
    """Compare every named field; tendencies and P_diss_iso get their differencing floors."""
    arrays = vs.__dict__
    for name in names:
        tracer = None
        floor = 0.0
        if name == "dtemp_iso":
            tracer = vs.temp
        elif name == "dsalt_iso":
            tracer = vs.salt
        elif name == "P_diss_iso":
            floor = p_diss_floor(arrays, settings, tau_in)
        assert_field_close(name, dev.download(name), getattr(vs, name), tracer=tracer, dt=settings["dt_tracer"],
                           floor=floor)


STEP_FIELDS = ("temp", "salt", "dtemp_iso", "dsalt_iso", "K_11", "K_22", "K_33", "Ai_ez", "Ai_nz", "Ai_bx", "Ai_by")


def _teacher_forced_rollout(host, nsteps, stages=False):
    """Every step of a GPU rollout against one oracle step from the GPU's own previous state.

    A free-running comparison would mix the per-step parity with the
    rollout's own amplification of last-bit differences (slopes divide by
    near-zero vertical density gradients); this checks each step at the FP64
    bar and returns the GPU state.
    """
    from oracle import isoneutral_oracle as orc
    from veros_gb300.state import DeviceState
    from veros_gb300.step import IsoneutralStepper

    dev = DeviceState.from_host(host)
    st = IsoneutralStepper(dev)
    fields = STEP_FIELDS + (("P_diss_iso",) if host.settings["enable_conserve_energy"] else ())
    for n in range(nsteps):
        v = dev.variables
        arrays = dict(host.arrays)
        arrays.update(dev.to_host_dict([f for f in host.arrays if f in v.fields()]))
        vs = orc.OracleState({k: np.array(a, copy=True) for k, a in arrays.items()}, tau=v.tau, taup1=v.taup1,
                             taum1=v.taum1)
        tau_in = vs.tau
        orc.isoneutral_step(vs, host.settings)
        if stages and n % 2 == 0:
            st.step_stages()
        else:
            st.step(1)
        torch.cuda.synchronize()
        assert dev.variables.tau == vs.tau
        _check_state(dev, vs, fields, host.settings, tau_in)
    return dev


@pytest.mark.parametrize("energy", [False, True])
def test_small_linear_rollout_vs_oracle(energy):
    """64 x 48 x 20, linear EOS: 5 steps, each against the oracle."""
    from veros_gb300 import synthetic

    host = synthetic.small_linear_state(seed=0)
    host.settings["enable_conserve_energy"] = energy
    _teacher_forced_rollout(host, 5)


def test_rollout_drift_is_bounded():
    """Free-running: 5 GPU steps against 5 oracle steps from the same start stay within 1e-9."""
    from veros_gb300 import synthetic
    from veros_gb300.state import DeviceState
    from veros_gb300.step import IsoneutralStepper

    host = synthetic.small_linear_state(seed=1)
    dev = DeviceState.from_host(host)
    IsoneutralStepper(dev).step(5)
    torch.cuda.synchronize()
    vs = _oracle_steps(host, 5)
    for name in ("temp", "salt", "K_11", "K_33", "Ai_bx"):
        assert _rel(dev.download(name), getattr(vs, name)) <= 1e-9, name


@pytest.mark.parametrize("energy", [False, True])
def test_global_1deg_step_vs_oracle(energy):
    """The benchmark workload (360 x 180 x 60, nonlinear EOS): 2 steps, staged
    and fused C calls; with the energy branch (the reference's default) the
    energy kernel walks the columns in chunks of levels."""
    from veros_gb300 import synthetic

    host = synthetic.global_1deg_state(seed=0)
    host.settings["enable_conserve_energy"] = energy
    dev = _teacher_forced_rollout(host, 2, stages=True)
    # masks and kbot indexing: land cells of the tracers stay exactly zero
    land = ~host.maskT
    assert np.all(dev.download("temp")[land] == 0.0)


def test_quarter_degree_step_vs_oracle():
    """The 0.25-degree workload (1440 x 720 x 60, 62 M cells, nonlinear EOS):
    one FP64 step against one oracle step from the same state. The oracle
    step takes about a minute of one host core at this size; it reads the
    host state without a copy (the step copies what it writes)."""
    from oracle import isoneutral_oracle as orc
    from veros_gb300 import synthetic
    from veros_gb300.state import DeviceState
    from veros_gb300.step import IsoneutralStepper

    host = synthetic.global_quarter_deg_state(seed=0)
    dev = DeviceState.from_host(host)
    IsoneutralStepper(dev).step(1)
    torch.cuda.synchronize()
    vs = orc.OracleState(host.arrays, tau=host.tau, taup1=host.taup1, taum1=host.taum1)
    tau_in = vs.tau
    orc.isoneutral_step(vs, host.settings)
    assert dev.variables.tau == vs.tau
    _check_state(dev, vs, STEP_FIELDS, host.settings, tau_in)


def test_column_order_gives_identical_results():
    """The implicit solve over columns sorted by depth equals the natural order bit for bit."""
    from veros_gb300 import _capi, synthetic
    from veros_gb300.state import DeviceState
    from veros_gb300.step import IsoneutralStepper

    host = synthetic.make_state(40, 30, 16, seed=4, eq_of_state_type=3, land_fraction=0.3)
    a = DeviceState.from_host(host)
    b = DeviceState.from_host(host)
    IsoneutralStepper(a).step_stages()  # ordered pair call
    st = IsoneutralStepper(b)
    lib, f = st.lib, st._fields()
    stream = torch.cuda.current_stream().cuda_stream
    dom, grid, sett = b.domain(), b.grid(), b.settings.to_struct()
    _capi.check(lib.vg_isoneutral_step_prepare_f64(dom, f, stream), "prepare")
    _capi.check(lib.vg_isoneutral_pre_f64(dom, grid, sett, f.temp_tau, f.salt_tau, f.K_iso, f.mask_bits, f.ten,
                                          stream), "pre")
    trT = _capi.VgTracerArgs(f.temp_tau, f.temp_taup1, f.dtemp_iso, None, None)
    trS = _capi.VgTracerArgs(f.salt_tau, f.salt_taup1, f.dsalt_iso, None, None)
    _capi.check(lib.vg_isoneutral_diffusion_pair_f64(dom, grid, sett, f.ten, f.K_iso, f.mask_bits, f.kbot, trT, trS,
                                                     st.scratch.data_ptr(), st.scratch.numel() * 8, stream), "pair")
    st._rotate()
    torch.cuda.synchronize()
    for name in ("temp", "salt", "dtemp_iso", "dsalt_iso"):
        np.testing.assert_array_equal(a.download(name), b.download(name))
    order = a.column_order().cpu().numpy()
    assert np.array_equal(np.sort(order), np.arange((a.X - 4) * (a.Y - 4)))


@pytest.mark.parametrize("precision", ["f64", "f32split"])
@pytest.mark.parametrize("energy", [False, True])
def test_fused_preparation_matches_separate_pass(precision, energy):
    """The step with the preparation fused into the flux kernel (rim kernel,
    pre, fused diffusion) equals a separate preparation of every cell, pre and
    the unfused diffusion, bit for bit, over two steps, land and coast
    columns included."""
    from veros_gb300 import synthetic
    from veros_gb300.state import DeviceState
    from veros_gb300.step import IsoneutralStepper

    host = synthetic.make_state(37, 26, 14, seed=9, eq_of_state_type=3, land_fraction=0.3,
                                settings=dict(enable_conserve_energy=energy))
    a = IsoneutralStepper(DeviceState.from_host(host, precision=precision))
    b = IsoneutralStepper(DeviceState.from_host(host, precision=precision))
    for _ in range(2):
        a.step(1)
        b.step_unfused()
    torch.cuda.synchronize()
    names = ("temp", "salt", "dtemp_iso", "dsalt_iso") + (("P_diss_iso",) if energy else ())
    for n in names:
        np.testing.assert_array_equal(a.dev.download(n), b.dev.download(n), err_msg=n)


@pytest.mark.parametrize("precision", ["f64", "f32split"])
def test_weighted_shares_change_no_result(precision):
    """The pre and flux kernels' CTAs take shares of the tile-levels weighted
    by their water (vg_isoneutral_step_shares): the starts cover the
    tile-levels in order, and two steps give the fields of equal shares, bit
    for bit."""
    from veros_gb300 import synthetic
    from veros_gb300.state import DeviceState
    from veros_gb300.step import IsoneutralStepper

    host = synthetic.global_1deg_state(seed=2, nz=20)
    a = IsoneutralStepper(DeviceState.from_host(host, precision=precision))
    b = IsoneutralStepper(DeviceState.from_host(host, precision=precision))
    pre, flux = a.dev.step_shares()
    assert pre is not None and (flux is not None) == (precision == "f64")  # the split flux kernel: equal counts
    X, Y, Z = a.dev.X, a.dev.Y, a.dev.Z
    ty = 8 if precision == "f64" else 4  # the kernels' tile rows (32 columns wide)
    ntiles = {"pre": -(-(X - 3) // 32) * -(-(Y - 3) // ty), "flux": -(-(X - 4) // 32) * -(-(Y - 4) // ty)}
    for name, starts in (("pre", pre), ("flux", flux)):
        if starts is None:
            continue
        s = starts.cpu().numpy()
        # every tile-level once, in order: CTA c takes [s[c], s[c+1])
        assert s[0] == 0 and np.all(np.diff(s) >= 0) and s[-1] == ntiles[name] * Z, name
    b.dev.step_shares = lambda stream=None: (None, None)
    a.step(2)
    b.step(2)
    torch.cuda.synchronize()
    for n in ("temp", "salt", "dtemp_iso", "dsalt_iso", "K_11", "K_33", "Ai_ez", "Ai_by"):
        np.testing.assert_array_equal(a.dev.download(n), b.dev.download(n), err_msg=n)


def test_drop_in_signatures_on_device_state():
    import veros_gb300 as vg
    from veros_gb300 import synthetic
    from veros_gb300.state import DeviceState
    from oracle import isoneutral_oracle as orc

    host = synthetic.make_state(24, 20, 12, seed=5, eq_of_state_type=3, settings=dict(enable_conserve_energy=True))
    dev = DeviceState.from_host(host)
    out = vg.isoneutral_diffusion_pre(dev)
    assert out._fields == ("Ai_ez", "Ai_nz", "Ai_bx", "Ai_by", "K_11", "K_22", "K_33")
    dev.variables.update(out)
    assert vg.isoneutral_diffusion(dev, tr=dev.variables.temp, istemp=True) is None
    assert vg.isoneutral_diffusion(dev, dev.variables.salt, False) is None
    torch.cuda.synchronize()
    vs = orc.OracleState({k: v.copy() for k, v in host.arrays.items()})
    vs.__dict__.update(orc.isoneutral_diffusion_pre(vs, host.settings))
    vs.__dict__.update(orc.isoneutral_diffusion(vs, host.settings, True))
    vs.__dict__.update(orc.isoneutral_diffusion(vs, host.settings, False))
    _check_state(dev, vs, ("temp", "salt", "dtemp_iso", "dsalt_iso", "P_diss_iso", "K_33"), host.settings, vs.tau)


def test_deep_columns_step_and_drop_in_vs_oracle():
    """200 levels (the implicit solves then take fewer columns per CTA to fit
    their shared memory): one fused step and the per-tracer drop-in calls
    against the oracle."""
    import veros_gb300 as vg
    from oracle import isoneutral_oracle as orc
    from veros_gb300 import synthetic
    from veros_gb300.state import DeviceState

    host = synthetic.make_state(24, 20, 200, seed=4, eq_of_state_type=3, dz_bottom=100.0)
    _teacher_forced_rollout(host, 1)
    dev = DeviceState.from_host(host)
    v = dev.variables
    v.temp[..., v.taup1] = v.temp[..., v.tau] * v.maskT
    v.salt[..., v.taup1] = v.salt[..., v.tau] * v.maskT
    v.update(vg.isoneutral_diffusion_pre(dev))
    vg.isoneutral_diffusion(dev, v.temp, True)
    vg.isoneutral_diffusion(dev, v.salt, False)
    torch.cuda.synchronize()
    vs = orc.OracleState({k: a.copy() for k, a in host.arrays.items()})
    for name in ("temp", "salt"):
        tr = getattr(vs, name)
        tr[..., vs.taup1] = tr[..., vs.tau] * vs.maskT
    vs.__dict__.update(orc.isoneutral_diffusion_pre(vs, host.settings))
    vs.__dict__.update(orc.isoneutral_diffusion(vs, host.settings, True))
    vs.__dict__.update(orc.isoneutral_diffusion(vs, host.settings, False))
    _check_state(dev, vs, ("temp", "salt", "dtemp_iso", "dsalt_iso", "K_33"), host.settings, vs.tau)


@pytest.mark.parametrize("precision", ["f64", "f32split"])
def test_energy_branch_per_tracer_calls_match_fused_step(precision):
    """P_diss_iso from the per-tracer drop-in calls (one energy launch each)
    equals the fused step's (one launch for temp and salt) bit for bit."""
    import veros_gb300 as vg
    from veros_gb300 import synthetic
    from veros_gb300.state import DeviceState
    from veros_gb300.step import IsoneutralStepper

    host = synthetic.make_state(40, 28, 16, seed=12, eq_of_state_type=3, settings=dict(enable_conserve_energy=True))
    a = DeviceState.from_host(host, precision=precision)
    b = DeviceState.from_host(host, precision=precision)
    v = a.variables
    v.temp[..., v.taup1] = v.temp[..., v.tau] * v.maskT
    v.salt[..., v.taup1] = v.salt[..., v.tau] * v.maskT
    v.update(vg.isoneutral_diffusion_pre(a))
    vg.isoneutral_diffusion(a, v.temp, True)
    vg.isoneutral_diffusion(a, v.salt, False)
    IsoneutralStepper(b).step(1)
    torch.cuda.synchronize()
    for n in ("temp", "salt", "P_diss_iso"):
        np.testing.assert_array_equal(a.download(n), b.download(n), err_msg=n)
    assert np.any(a.download("P_diss_iso") != 0.0)


@pytest.mark.parametrize("precision", ["f64", "f32split"])
def test_host_buffer_step_matches_device_step(precision):
    """step_host (reference-layout host buffers, layout conversion on the
    device) gives the device step's fields bit for bit, on a domain whose X
    and Z are not multiples of the 32-wide conversion tiles and whose Y (25)
    leaves a partial group of the conversion's four rows per CTA."""
    from veros_gb300 import synthetic
    from veros_gb300.state import DeviceState
    from veros_gb300.step import IsoneutralStepper

    host = synthetic.make_state(45, 21, 13, seed=2, eq_of_state_type=3)
    a = DeviceState.from_host(host, precision=precision)
    b = DeviceState.from_host(host, precision=precision)
    IsoneutralStepper(a).step(1)
    X, Y, Z = b.X, b.Y, b.Z
    hT = torch.from_numpy(np.ascontiguousarray(host.temp[..., host.tau])).pin_memory()
    hS = torch.from_numpy(np.ascontiguousarray(host.salt[..., host.tau])).pin_memory()
    outs = [torch.empty((X, Y, Z), dtype=torch.float64).pin_memory() for _ in range(4)]
    IsoneutralStepper(b).step_host(hT, hS, *outs)
    v = a.variables
    assert np.array_equal(outs[0].numpy(), a.download("temp")[..., v.tau])
    assert np.array_equal(outs[1].numpy(), a.download("salt")[..., v.tau])
    assert np.array_equal(outs[2].numpy(), a.download("dtemp_iso").astype(np.float64))
    assert np.array_equal(outs[3].numpy(), a.download("dsalt_iso").astype(np.float64))


def test_host_pipeline_matches_serial_host_steps():
    """Independent batches through the overlapped-copy pipeline equal lone step_host calls."""
    from veros_gb300 import synthetic
    from veros_gb300.state import DeviceState
    from veros_gb300.step import IsoneutralStepper

    host = synthetic.make_state(30, 20, 12, seed=6, eq_of_state_type=3, land_fraction=0.3)
    a = IsoneutralStepper(DeviceState.from_host(host))
    b = IsoneutralStepper(DeviceState.from_host(host))
    X, Y, Z = a.dev.X, a.dev.Y, a.dev.Z
    rng = np.random.default_rng(3)
    pin = lambda x: torch.from_numpy(np.ascontiguousarray(x)).pin_memory()  # noqa: E731
    batches = []
    for _ in range(4):
        dT = rng.normal(0.0, 0.05, (X, Y, Z)) * host.maskT
        batches.append((pin(host.temp[..., host.tau] + dT), pin(host.salt[..., host.tau])))
    serial = []
    for hT, hS in batches:
        outs = [torch.empty((X, Y, Z), dtype=torch.float64).pin_memory() for _ in range(4)]
        a.step_host(hT, hS, *outs)
        serial.append([o.numpy().copy() for o in outs])
    pipe = b.pipeline()
    piped = []
    for hT, hS in batches:
        outs = [torch.empty((X, Y, Z), dtype=torch.float64).pin_memory() for _ in range(4)]
        pipe.submit(hT, hS, *outs)
        piped.append(outs)
    pipe.finish()
    for want, got in zip(serial, piped):
        for w, g in zip(want, got):
            np.testing.assert_array_equal(g.numpy(), w)


def test_vertmix_and_streamfunction_vs_reference_golden():
    """vertmix_tempsalt and the GM streamfunction diagnostics against the reference's outputs."""
    from veros_gb300.isoneutral import isoneutral_diag_streamfunction_kernel
    from veros_gb300.thermodynamics import vertmix_tempsalt

    g = load_golden("vertmix_random")
    dev = _golden_device_state(g)
    for n in ("kappaH", "forc_temp_surface", "forc_salt_surface", "dtemp_vmix", "dsalt_vmix", "B1_gm", "B2_gm"):
        dev.upload(n, g[f"in_{n}"])
    out = vertmix_tempsalt(dev)
    assert out._fields == ("dtemp_vmix", "temp", "dsalt_vmix", "salt")
    torch.cuda.synchronize()
    dt = float(g["setting_dt_tracer"])
    for n, tr in (("temp", None), ("salt", None), ("dtemp_vmix", "temp"), ("dsalt_vmix", "salt")):
        name = {"dtemp_vmix": "dtemp_iso", "dsalt_vmix": "dsalt_iso"}.get(n, n)  # same differencing floor
        assert_field_close(name, dev.download(n), g[f"vmix_{n}"], tracer=None if tr is None else g[f"vmix_{tr}"],
                           dt=dt)
    out = isoneutral_diag_streamfunction_kernel(dev)
    torch.cuda.synchronize()
    for n in ("B1_gm", "B2_gm"):
        got, ref = dev.download(n), g[f"sf_{n}"]
        assert _rel(got, ref) <= TOL, n
    # untouched cells keep their contents
    before = g["in_B2_gm"]
    w = np.zeros(before.shape, dtype=bool)
    w[1:-2, 2:-2] = True
    assert np.array_equal(dev.download("B2_gm")[~w], before[~w])


def test_vertmix_on_synthetic_state_vs_oracle():
    from oracle import isoneutral_oracle as orc
    from veros_gb300 import synthetic
    from veros_gb300.state import DeviceState
    from veros_gb300.thermodynamics import vertmix_tempsalt

    host = synthetic.make_state(70, 50, 30, seed=8, eq_of_state_type=3, dz_bottom=250.0)
    dev = DeviceState.from_host(host)
    vertmix_tempsalt(dev)
    torch.cuda.synchronize()
    vs = orc.OracleState({k: v.copy() for k, v in host.arrays.items()})
    out = orc.vertmix_tempsalt(vs, host.settings)
    dt = host.settings["dt_tracer"]
    for n, tr in (("temp", None), ("salt", None), ("dtemp_vmix", "temp"), ("dsalt_vmix", "salt")):
        name = {"dtemp_vmix": "dtemp_iso", "dsalt_vmix": "dsalt_iso"}.get(n, n)
        assert_field_close(name, dev.download(n), out[n], tracer=None if tr is None else out[tr], dt=dt)


@pytest.mark.parametrize("case", ["iso_random_energy", "iso_random_noenergy"])
def test_diffusion_with_tensors_not_written_by_pre(case):
    """The diffusion on the reference's random state without pre first: the
    tensor fields are random on every face, dry ones included, as a caller
    may pass them. The flux kernel orders its columns by their first wet level
    and skips the FP64 work of dry faces only where their coefficients are
    zero, so fluxes through dry faces with non-zero coefficients must still
    enter the neighbouring wet cells as in the reference (which multiplies the
    divergence by maskT, not the fluxes by the face masks)."""
    from oracle import isoneutral_oracle as orc
    from veros_gb300.isoneutral import run_diffusion

    g = load_golden(case)
    dev = _golden_device_state(g)
    arrays = {k[3:]: v.copy() for k, v in g.items() if k.startswith("in_")}
    settings = {k[8:]: v.item() for k, v in g.items() if k.startswith("setting_")}
    vs = orc.OracleState(arrays, tau=int(g["tau"]), taup1=int(g["taup1"]), taum1=int(g["taum1"]))
    # dry faces really carry non-zero coefficients here
    dry_u = ~arrays["maskU"][1:-2, 2:-2]
    assert np.any(arrays["Ai_ez"][1:-2, 2:-2][dry_u] != 0.0)
    dt = float(settings["dt_tracer"])
    for istemp, name in ((True, "temp"), (False, "salt")):
        run_diffusion(dev, istemp)
        torch.cuda.synchronize()
        out = orc.isoneutral_diffusion(vs, settings, istemp)
        vs.__dict__.update(out)
        dname = "dtemp_iso" if istemp else "dsalt_iso"
        for n in (name, dname):
            assert_field_close(n, dev.download(n), out[n], tracer=out[name], dt=dt)
        if "P_diss_iso" in out:
            pf = p_diss_floor({**arrays, "temp": vs.temp, "salt": vs.salt}, settings, int(g["tau"]))
            assert_field_close("P_diss_iso", dev.download("P_diss_iso"), out["P_diss_iso"], floor=pf)
