"""GPU parity: the CUDA path against the reference's golden outputs and the oracle.

Tolerance (FP64): relative max-norm ``max|gpu - ref| / max|ref| <= 1e-12`` per
field. Cells the reference leaves untouched must keep their previous contents
bit for bit, and masked (land) cells must be exactly zero where the reference
multiplies by a mask.
"""

import numpy as np
import pytest

from conftest import load_golden

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


@pytest.mark.parametrize("case", ["iso_random_energy", "iso_random_noenergy", "iso_synth_eq1", "iso_synth_eq3"])
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


@pytest.mark.parametrize("case", ["iso_random_energy", "iso_random_noenergy", "iso_synth_eq1", "iso_synth_eq3"])
def test_diffusion_chain_vs_reference_golden(case):
    from veros_gb300.isoneutral import run_diffusion, run_pre

    g = load_golden(case)
    dev = _golden_device_state(g)
    run_pre(dev)
    run_diffusion(dev, istemp=True)
    torch.cuda.synchronize()
    for name in ("temp", "dtemp_iso", "P_diss_iso"):
        got, ref = dev.download(name), g[f"diffT_{name}"]
        assert _rel(got, ref) <= TOL, f"T {name}: {_rel(got, ref):.3e}"
    run_diffusion(dev, istemp=False)
    torch.cuda.synchronize()
    for name in ("salt", "dsalt_iso", "P_diss_iso"):
        got, ref = dev.download(name), g[f"diffS_{name}"]
        assert _rel(got, ref) <= TOL, f"S {name}: {_rel(got, ref):.3e}"
    if "skewT_temp" in g:
        run_diffusion(dev, istemp=True, skew=True)
        torch.cuda.synchronize()
        for name in ("temp", "dtemp_iso", "P_diss_skew"):
            got, ref = dev.download(name), g[f"skewT_{name}"]
            assert _rel(got, ref) <= TOL, f"skew {name}: {_rel(got, ref):.3e}"


def test_tridiag_vs_reference_golden():
    from veros_gb300.utilities import solve_implicit, solve_tridiagonal

    g = load_golden("tridiag")
    # the reference's own random-matrix test form and tolerance (tridiag_test.py:40-67)
    out = solve_tridiagonal(g["a"], g["b"], g["c"], g["d"], g["water_mask"], g["edge_mask"])
    np.testing.assert_allclose(out, g["out_random"], rtol=1e-7)
    assert np.all(out[~g["water_mask"]] == 0.0)
    out = solve_implicit(g["ad"], g["bd"], g["cd"], g["d"], g["water_mask"], g["edge_mask"],
                         b_edge=g["b_edge"], d_edge=g["d_edge"])
    assert _rel(out, g["out_dd"]) <= TOL


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


def test_xla_tdma_entry_point():
    import ctypes

    from veros_gb300 import _capi

    rng = np.random.default_rng(2)
    nsys, depth = 1000, 40
    a = -rng.random((depth, nsys))
    c = -rng.random((depth, nsys))
    b = 3.0 + rng.random((depth, nsys))
    d = rng.standard_normal((depth, nsys))
    bufs = [torch.from_numpy(x).cuda() for x in (a, b, c, d)] + [torch.empty((depth, nsys), dtype=torch.float64,
                                                                              device="cuda")] * 2
    ptrs = (ctypes.c_void_p * 6)(*(t.data_ptr() for t in bufs))
    desc = np.array([nsys, depth], dtype=np.int32).tobytes()
    lib = _capi.load()
    lib.vg_tdma_cuda_double(ctypes.c_void_p(torch.cuda.current_stream().cuda_stream), ptrs, desc, len(desc))
    torch.cuda.synchronize()
    assert _capi.last_error() == ""
    out = bufs[4].cpu().numpy()
    from scipy.linalg import solve_banded

    for s in range(0, nsys, 97):
        ab = np.zeros((3, depth))
        ab[0, 1:] = c[:-1, s]
        ab[1] = b[:, s]
        ab[2, :-1] = a[1:, s]
        ref = solve_banded((1, 1), ab, d[:, s])
        assert _rel(out[:, s], ref) <= 1e-13


def _oracle_steps(host, n):
    from oracle import isoneutral_oracle as orc

    vs = orc.OracleState({k: v.copy() for k, v in host.arrays.items()})
    for _ in range(n):
        orc.isoneutral_step(vs, host.settings)
    return vs


STEP_FIELDS = ("temp", "salt", "dtemp_iso", "dsalt_iso", "K_11", "K_22", "K_33", "Ai_ez", "Ai_nz", "Ai_bx", "Ai_by")


@pytest.mark.parametrize("energy", [False, True])
def test_small_linear_rollout_vs_oracle(energy):
    """64 x 48 x 20, linear EOS: 5 steps of the GPU stepper against 5 oracle steps."""
    from veros_gb300 import synthetic
    from veros_gb300.state import DeviceState
    from veros_gb300.step import IsoneutralStepper

    host = synthetic.small_linear_state(seed=0)
    host.settings["enable_conserve_energy"] = energy
    dev = DeviceState.from_host(host)
    IsoneutralStepper(dev).step(5)
    torch.cuda.synchronize()
    vs = _oracle_steps(host, 5)
    assert dev.variables.tau == vs.tau
    fields = STEP_FIELDS + (("P_diss_iso",) if energy else ())
    for name in fields:
        err = _rel(dev.download(name), getattr(vs, name))
        assert err <= TOL, f"{name}: {err:.3e}"


def test_global_1deg_step_vs_oracle():
    """The benchmark workload (360 x 180 x 60, nonlinear EOS): 2 steps, stages driven one by one."""
    from veros_gb300 import synthetic
    from veros_gb300.state import DeviceState
    from veros_gb300.step import IsoneutralStepper

    host = synthetic.global_1deg_state(seed=0)
    dev = DeviceState.from_host(host)
    st = IsoneutralStepper(dev)
    st.step_stages()
    st.step(1)
    torch.cuda.synchronize()
    vs = _oracle_steps(host, 2)
    for name in STEP_FIELDS:
        err = _rel(dev.download(name), getattr(vs, name))
        assert err <= TOL, f"{name}: {err:.3e}"
    # masks and kbot indexing: land cells of the tracers stay exactly zero
    land = ~host.maskT
    assert np.all(dev.download("temp")[land] == 0.0)


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
    for name in ("temp", "salt", "dtemp_iso", "dsalt_iso", "P_diss_iso", "K_33"):
        assert _rel(dev.download(name), getattr(vs, name)) <= TOL, name


def test_host_buffer_step_matches_device_step():
    from veros_gb300 import synthetic
    from veros_gb300.state import DeviceState
    from veros_gb300.step import IsoneutralStepper

    host = synthetic.small_linear_state(seed=2)
    a = DeviceState.from_host(host)
    b = DeviceState.from_host(host)
    IsoneutralStepper(a).step(1)
    X, Y, Z = b.X, b.Y, b.Z
    hT = torch.from_numpy(np.ascontiguousarray(host.temp[..., host.tau])).pin_memory()
    hS = torch.from_numpy(np.ascontiguousarray(host.salt[..., host.tau])).pin_memory()
    outs = [torch.empty((X, Y, Z), dtype=torch.float64).pin_memory() for _ in range(4)]
    IsoneutralStepper(b).step_host(hT, hS, *outs)
    v = a.variables
    assert np.array_equal(outs[0].numpy(), a.download("temp")[..., v.tau])
    assert np.array_equal(outs[3].numpy(), a.download("dsalt_iso"))
