"""The FP32/FP64-split form against the FP64 path.

Split form: tracers, tracer differences, the clamped slope denominators and
the implicit solve in FP64; slopes, taper, diffusivities, tensors, fluxes,
tendencies and dissipation in FP32. Error budget (relative max-norm against
the FP64 result of the same state, per output field): tracers <= 1e-6;
tensors, tendencies and dissipation <= 1e-4. The tests print the measured
figures.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

TRACER_TOL = 1e-6
FIELD_TOL = 1e-4
FIELDS = ("temp", "salt", "dtemp_iso", "dsalt_iso", "K_11", "K_22", "K_33", "Ai_ez", "Ai_nz", "Ai_bx", "Ai_by")


def _errors(split, ref, names):
    out = {}
    for n in names:
        a = split.download(n).astype(np.float64)
        b = ref.download(n) if hasattr(ref, "download") else getattr(ref, n)
        scale = float(np.max(np.abs(b))) or 1.0
        d = np.abs(a - b)
        out[n] = (float(d.max() / scale), float(np.sqrt(np.mean(d ** 2)) / scale))
    return out


def _check(errs):
    for n, (mx, rms) in errs.items():
        print(f"  {n:10s} max {mx:.2e} rms {rms:.2e}")
        tol = TRACER_TOL if n in ("temp", "salt") else FIELD_TOL
        assert mx <= tol, f"{n}: relative max-norm error {mx:.3e} > {tol:.0e}"


@pytest.mark.parametrize("energy", [False, True])
def test_split_step_against_oracle(energy):
    from oracle import isoneutral_oracle as orc
    from veros_gb300 import synthetic
    from veros_gb300.state import DeviceState
    from veros_gb300.step import IsoneutralStepper

    host = synthetic.make_state(64, 48, 20, seed=4, eq_of_state_type=3, dz_bottom=250.0,
                                settings=dict(enable_conserve_energy=energy))
    dev = DeviceState.from_host(host, precision="f32split")
    assert dev.variables.temp.dtype == torch.float64 and dev.variables.K_11.dtype == torch.float32
    IsoneutralStepper(dev).step(1)
    torch.cuda.synchronize()
    vs = orc.OracleState({k: v.copy() for k, v in host.arrays.items()})
    orc.isoneutral_step(vs, host.settings)
    names = FIELDS + (("P_diss_iso",) if energy else ())
    _check(_errors(dev, vs, names))


def test_split_rollout_on_benchmark_grid():
    """360 x 180 x 60, nonlinear EOS: 10 split steps against 10 FP64 GPU steps from the same state."""
    from veros_gb300 import synthetic
    from veros_gb300.state import DeviceState
    from veros_gb300.step import IsoneutralStepper

    host = synthetic.global_1deg_state(seed=0)
    ref = DeviceState.from_host(host)
    split = DeviceState.from_host(host, precision="f32split")
    IsoneutralStepper(ref).step(10)
    IsoneutralStepper(split).step(10)
    torch.cuda.synchronize()
    errs = _errors(split, ref, ("temp", "salt"))
    _check(errs)


def test_split_drop_in_calls_match_step():
    """The per-call drop-ins in split precision give the same fields as the fused split step."""
    import veros_gb300 as vg
    from veros_gb300 import synthetic
    from veros_gb300.state import DeviceState
    from veros_gb300.step import IsoneutralStepper

    host = synthetic.make_state(30, 20, 12, seed=9, eq_of_state_type=3)
    a = DeviceState.from_host(host, precision="f32split")
    b = DeviceState.from_host(host, precision="f32split")
    v = a.variables
    v.temp[..., v.taup1] = v.temp[..., v.tau] * v.maskT
    v.salt[..., v.taup1] = v.salt[..., v.tau] * v.maskT
    v.update(vg.isoneutral_diffusion_pre(a))
    vg.isoneutral_diffusion(a, v.temp, True)
    vg.isoneutral_diffusion(a, v.salt, False)
    IsoneutralStepper(b).step(1)
    torch.cuda.synchronize()
    # the step shares one implicit factorisation between the tracers: same arithmetic
    for n in ("temp", "salt", "K_33", "Ai_bx"):
        np.testing.assert_array_equal(a.download(n), b.download(n))
