"""The CUDA adjoint (vg_isoneutral_step_adjoint_f64 behind torch.autograd)
against the NumPy adjoint oracle and central differences of the forward.

Loss of the adjoint workload: sum over wet interior cells of
(temp after n steps - target)^2, gradients with respect to the initial
temperature, the initial salinity and a 3-D K_iso.

* Small grids (12 x 10 x 8, 3 steps): the CUDA gradients equal the NumPy
  adjoint to rounding, and agree with central differences of the forward
  oracle (the reference algorithm) within 1e-6 along 16 seeded random unit
  directions (the kink-aware protocol of ``oracle.isoneutral_adjoint``).
* The 1-degree adjoint workload (360 x 180 x 30, 8 steps, lognormal K_iso):
  the CUDA adjoint equals the NumPy adjoint run on the same checkpoints,
  per step and over the rollout. Central differences are only a coarse check
  there: the gradient norm is ~1e13-1e14, carried by a few cells whose
  vertical density gradient is nearly zero while their slope lies in the
  taper's transition (ds/dT ~ s/G), so FP64 rounding of the forward itself
  limits a difference quotient to ~1e-4 relative at any step size, and steps
  above ~1e-10 cross thousands of slope sign changes (the taper's kink).
"""

import numpy as np
import pytest
import torch

from oracle import isoneutral_adjoint as A
from veros_gb300 import synthetic
from veros_gb300.state import DeviceState

pytestmark = pytest.mark.gpu

RTOL_FD = 1e-6
EPS = {"T": 1e-6, "S": 1e-6, "K": 1e-4}
NDIR = {"T": 6, "S": 5, "K": 5}  # 16 directions


def _model(host):
    from veros_gb300.adjoint import IsoneutralAdjoint

    return IsoneutralAdjoint(DeviceState.from_host(host, device="cuda"))


def _small(eq, seed=3):
    host = synthetic.make_state(12, 10, 8, seed=seed, eq_of_state_type=eq, k_iso_lognormal_sigma=0.3,
                                land_fraction=0.3)
    return _inputs(host, np.random.default_rng(100 + seed))


def _workload():
    host = synthetic.global_1deg_state(seed=0, nz=30, k_iso_lognormal_sigma=0.3)
    return _inputs(host, np.random.default_rng(4))


def _inputs(host, rng):
    T0 = host.arrays["temp"][..., 1].copy()
    S0 = host.arrays["salt"][..., 1].copy()
    K = host.arrays["K_iso"].copy()
    wet = A.wet_interior(host)
    target = T0 + rng.normal(0.0, 0.05, T0.shape) * wet
    return host, T0, S0, K, target, wet, rng


def _gpu_rollout_grad(model, T0, S0, K, target, wet, n):
    leaves = [model.field(x).requires_grad_() for x in (T0, S0, K)]
    T, _ = model.rollout(*leaves, n)
    loss = ((T - model.field(target)) ** 2 * model.field(wet)).sum()
    loss.backward()
    return (loss.item(),) + tuple(leaf.grad.cpu().numpy() for leaf in leaves)


def _close(a, b, max_rel, cell_rel):
    """max-norm relative error, and per-cell error against |b| + median|b|."""
    scale = np.abs(b).max()
    med = np.median(np.abs(b[b != 0]))
    err = np.abs(a - b)
    assert err.max() <= max_rel * scale, (err.max() / scale, max_rel)
    assert np.max(err / (np.abs(b) + med)) <= cell_rel


@pytest.mark.parametrize("eq", [1, 3])
def test_adjoint_matches_numpy_adjoint(eq):
    host, T0, S0, K, target, wet, _ = _small(eq)
    model = _model(host)
    Lg, gT, gS, gK = _gpu_rollout_grad(model, T0, S0, K, target, wet, 3)
    L, nT, nS, nK = A.rollout_grad(host, T0, S0, K, target, 3)
    assert Lg == pytest.approx(L, rel=1e-12)
    for a, b in ((gT, nT), (gS, nS), (gK, nK)):
        _close(a, b, 1e-11, 1e-9)


@pytest.mark.parametrize("eq", [1, 3])
def test_adjoint_central_differences_of_the_oracle(eq):
    host, T0, S0, K, target, wet, rng = _small(eq)
    model = _model(host)
    _, gT, gS, gK = _gpu_rollout_grad(model, T0, S0, K, target, wet, 3)

    def loss_of(T, S, K):
        Ts, _ = A.rollout(host, T, S, K, 3)
        return A.loss(Ts[-1], target, wet)

    def signs_of(T, S, K):
        return A.rollout_slope_signs(host, T, S, K, 3)

    checks = A.directional_checks(loss_of, signs_of, dict(T=T0, S=S0, K=K), dict(T=gT, S=gS, K=gK), EPS, NDIR, rng)
    n = 0
    for which, fd, ad, scale in checks:
        assert abs(fd - ad) <= RTOL_FD * scale, (which, fd, ad)
        n += 1
    assert n == 16


def test_adjoint_step_equals_numpy_adjoint_at_workload_size():
    host, T0, S0, K, target, wet, rng = _workload()
    model = _model(host)
    Td, Sd, Kd = model.field(T0), model.field(S0), model.field(K)
    with torch.no_grad():
        T1, S1 = model.forward_step(Td, Sd, Kd)
    lT = rng.standard_normal(T0.shape)
    lS = rng.standard_normal(T0.shape)
    gK = model.empty().zero_()
    gT, gS = model.backward_step(Td, Sd, Kd, T1, S1, model.field(lT), model.field(lS), gK)
    nT, nS, nK = A.step_adjoint(host, T0, S0, K, lT, lS, T1.cpu().numpy(), S1.cpu().numpy())
    for a, b in ((gT, nT), (gS, nS), (gK, nK)):
        _close(a.cpu().numpy(), b, 1e-11, 1e-8)


def test_adjoint_rollout_equals_numpy_adjoint_at_workload_size():
    """8 steps; the NumPy adjoint runs on the CUDA forward's checkpoints."""
    host, T0, S0, K, target, wet, _ = _workload()
    model = _model(host)
    Kd = model.field(K)
    Ts, Ss = [model.field(T0)], [model.field(S0)]
    with torch.no_grad():
        for _ in range(8):
            T, S = model.forward_step(Ts[-1], Ss[-1], Kd)
            Ts.append(T)
            Ss.append(S)
    Tn = [x.cpu().numpy() for x in Ts]
    Sn = [x.cpu().numpy() for x in Ss]
    Lg, gT, gS, gK = _gpu_rollout_grad(model, T0, S0, K, target, wet, 8)
    assert Lg == pytest.approx(A.loss(Tn[-1], target, wet), rel=1e-13)
    lam_T = 2.0 * wet * (Tn[-1] - target)
    lam_S = np.zeros_like(lam_T)
    nK = np.zeros_like(K)
    for n in range(7, -1, -1):
        lam_T, lam_S, k = A.step_adjoint(host, Tn[n], Sn[n], K, lam_T, lam_S, Tn[n + 1], Sn[n + 1])
        nK += k
    for a, b in ((gT, lam_T), (gS, lam_S), (gK, nK)):
        _close(a, b, 1e-9, 1e-7)


def test_adjoint_central_differences_at_workload_size():
    """Coarse: central differences of the CUDA forward at steps below the
    kink spacing (temperature/salinity 1e-11, K_iso 1e-7) agree within 1e-2;
    measured 2e-5..7e-4 (T, S) and 1e-4..5e-3 (K)."""
    host, T0, S0, K, target, wet, rng = _workload()
    model = _model(host)
    _, gT, gS, gK = _gpu_rollout_grad(model, T0, S0, K, target, wet, 8)
    tgt, w = model.field(target), model.field(wet)

    def loss_of(T, S, KK):
        T, S, KK = model.field(T), model.field(S), model.field(KK)
        with torch.no_grad():
            for _ in range(8):
                T, S = model.forward_step(T, S, KK)
            return float(((T - tgt) ** 2 * w).sum())

    base = dict(T=T0, S=S0, K=K)
    for which, eps, g in (("T", 1e-11, gT), ("S", 1e-11, gS), ("K", 1e-7, gK)):
        for _ in range(2):
            u = rng.standard_normal(K.shape)
            u /= np.linalg.norm(u)
            h = eps * np.linalg.norm(base[which])
            plus = {n: v + (h * u if n == which else 0.0) for n, v in base.items()}
            minus = {n: v - (h * u if n == which else 0.0) for n, v in base.items()}
            fd = (loss_of(plus["T"], plus["S"], plus["K"]) - loss_of(minus["T"], minus["S"], minus["K"])) / (2 * h)
            ad = float(np.sum(g * u))
            scale = max(abs(ad), np.linalg.norm(g) / np.sqrt(g.size))
            assert abs(fd - ad) <= 1e-2 * scale, (which, fd, ad)


def test_checkpoint_memory_is_two_fields_per_step():
    host, T0, S0, K, target, wet, _ = _workload()
    model = _model(host)
    field = model.dev.plane * model.dev.Z * 8
    peaks = {}
    for n in (4, 8):
        torch.cuda.synchronize()
        torch.cuda.reset_peak_memory_stats()
        base = torch.cuda.memory_allocated()
        _gpu_rollout_grad(model, T0, S0, K, target, wet, n)
        torch.cuda.synchronize()
        peaks[n] = torch.cuda.max_memory_allocated() - base
    per_step = (peaks[8] - peaks[4]) / 4
    assert 1.5 * field <= per_step <= 2.5 * field, per_step / field


def test_adjoint_is_linear_and_deterministic():
    host, T0, S0, K, target, wet, rng = _small(3, seed=8)
    model = _model(host)
    Td, Sd, Kd = model.field(T0), model.field(S0), model.field(K)
    with torch.no_grad():
        T1, S1 = model.forward_step(Td, Sd, Kd)
    l1 = [model.field(rng.standard_normal(T0.shape)) for _ in range(2)]
    l2 = [model.field(rng.standard_normal(T0.shape)) for _ in range(2)]
    outs = []
    for lam in (l1, l2, [model.field(a + b) for a, b in zip(l1, l2)], l1):
        gK = model.empty().zero_()
        gT, gS = model.backward_step(Td, Sd, Kd, T1, S1, lam[0], lam[1], gK)
        outs.append([x.cpu().numpy() for x in (gT, gS, gK)])
    for a, b, c, d in zip(*outs):
        np.testing.assert_array_equal(a, d)  # bit-identical rerun
        np.testing.assert_allclose(c, a + b, rtol=1e-12, atol=1e-12 * np.abs(c).max())
