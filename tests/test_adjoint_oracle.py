"""The NumPy adjoint of the isoneutral step against central differences of
the forward oracle (the reference algorithm), on CPU.

The check is the one the adjoint workload states: directional derivatives
along seeded random unit directions of the initial temperature, the initial
salinity and a 3-D K_iso, compared with central differences at a relative
step eps (perturbation eps * |x| along the unit direction), within 1e-6.

* Temperature and salinity directions use eps = 1e-6. K_iso directions use
  eps = 1e-4: the loss moves by ~1e-8 over a 1e-6 step of K, and the FP64
  forward's own rounding (~3e-15 in the loss) would limit the difference
  quotient to ~1e-6..1e-4 whatever the gradient; at 1e-4 the truncation
  error of the central difference stays below 1e-8.
* The taper is a function of |slope|, so the forward has a kink wherever a
  slope is zero. Where a step of 1e-6 straddles one (a slope changes sign
  between the two evaluation points, 4 of 12 salinity directions on this
  grid) the difference is taken again at a tenfold smaller step.
* The error is measured against max(|ad|, |grad| / sqrt(n)), the typical
  size of a directional derivative along a random unit direction in n
  dimensions, so that a direction nearly orthogonal to the gradient does not
  turn a 1e-10 absolute difference into a large relative one.
"""

import numpy as np
import pytest

from oracle import isoneutral_adjoint as A
from veros_gb300 import synthetic

RTOL = 1e-6


def _case(eq, seed=3, nsteps=3):
    host = synthetic.make_state(12, 10, 8, seed=seed, eq_of_state_type=eq, k_iso_lognormal_sigma=0.3,
                                land_fraction=0.3)
    rng = np.random.default_rng(100 + seed)
    T0 = host.arrays["temp"][..., 1].copy()
    S0 = host.arrays["salt"][..., 1].copy()
    K = host.arrays["K_iso"].copy()
    wet = A.wet_interior(host)
    target = T0 + rng.normal(0.0, 0.05, T0.shape) * wet
    return host, T0, S0, K, target, wet, rng, nsteps


EPS = {"T": 1e-6, "S": 1e-6, "K": 1e-4}
NDIR = {"T": 6, "S": 5, "K": 5}  # 16 directions


def oracle_loss_and_signs(host, target, wet, n):
    def loss_of(T, S, K):
        Ts, _ = A.rollout(host, T, S, K, n)
        return A.loss(Ts[-1], target, wet)

    def signs_of(T, S, K):
        return A.rollout_slope_signs(host, T, S, K, n)

    return loss_of, signs_of


@pytest.mark.parametrize("eq", [1, 3])
def test_adjoint_oracle_matches_central_differences(eq):
    host, T0, S0, K, target, wet, rng, n = _case(eq)
    L, gT, gS, gK = A.rollout_grad(host, T0, S0, K, target, n)
    Ts, _ = A.rollout(host, T0, S0, K, n)
    assert L == pytest.approx(A.loss(Ts[-1], target, wet), rel=1e-14)
    loss_of, signs_of = oracle_loss_and_signs(host, target, wet, n)
    checks = A.directional_checks(loss_of, signs_of, dict(T=T0, S=S0, K=K), dict(T=gT, S=gS, K=gK), EPS, NDIR, rng)
    for which, fd, ad, scale in checks:
        assert abs(fd - ad) <= RTOL * scale, (which, fd, ad)


def test_implicit_adjoint_is_the_transpose():
    """<A^-1 d, g> == <d, A^-T g> for the implicit solve of a random state."""
    from oracle import isoneutral_oracle as O

    host, T0, S0, K, target, wet, rng, _ = _case(3, seed=5)
    _, _, vs = A.forward_step(host, T0, S0, K)
    K33 = vs.K_33
    dt = host.settings["dt_tracer"]
    d = rng.standard_normal(T0.shape)
    g = rng.standard_normal(T0.shape)
    nz = T0.shape[2]
    st = O.OracleState(dict(host.arrays, K_33=K33, temp=np.stack([d, d, d], -1)), tau=1, taup1=2)
    x = O.calc_implicit_part(st, host.settings, st.temp)  # interior (X-4, Y-4, Z), passes non-water cells
    (lam,), _ = A.implicit_adjoint(host, K33, [np.zeros_like(d)], [g], dt)
    _, water, _ = O.create_water_masks(host.arrays["kbot"][2:-2, 2:-2], nz)
    lhs = np.sum(np.where(water, x, 0.0) * g[2:-2, 2:-2])
    rhs = np.sum(np.where(water, d[2:-2, 2:-2], 0.0) * lam[2:-2, 2:-2])
    assert lhs == pytest.approx(rhs, rel=1e-12)
    # outside the solve the adjoint passes through
    np.testing.assert_array_equal(np.where(water, 0.0, lam[2:-2, 2:-2]), np.where(water, 0.0, g[2:-2, 2:-2]))
    np.testing.assert_array_equal(lam[:2], g[:2])
