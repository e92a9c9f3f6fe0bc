"""NumPy adjoint of the isoneutral step. TEST INFRASTRUCTURE ONLY.

Only ``tests/`` and ``__graft_entry__.smoke()`` may import this module.

The reference has no derivative of this path: Veros defines no custom VJP and
its TDMA primitive has no transpose rule. The gradient oracle is therefore the
central finite difference of the forward oracle
(``isoneutral_oracle.isoneutral_step``, the restatement of
veros/core/thermodynamics.py:226-241 and :425-432); this module restates the
hand-derived adjoint of that step in NumPy, in the same per-slope formulation
as the CUDA kernels, and ``tests/test_adjoint_oracle.py`` checks it against
those differences.

Per-slope formulation. Every slope of isoneutral.py:100-224 is attached to a
T point P, one of its four horizontal faces h (east, west, north, south) and
one of its two vertical faces v (below, above):
``s(P,h,v) = -(drdT(P) dT/dh + drdS(P) dS/dh) / (min(0, drdT(P) dT/dz(v) +
drdS(P) dS/dz(v)) - epsln)``. Each slope enters two terms with the same
value: the term of face h (Ai_ez/Ai_nz and K_11/K_22, isoneutral.py:100-168)
and the term of face v (Ai_bx/Ai_by and K_33, :173-224). The adjoint
therefore visits the eight slopes of each point once.
"""

import numpy as np

from . import isoneutral_oracle as O


def _g(base, name):
    return np.asarray(base.arrays[name])


def forward_step(base, T, S, K):
    """One step of the forward oracle from tracers ``T``, ``S`` ((X, Y, Z)) and
    diffusivity ``K``; returns ``(T_new, S_new, vs)`` where ``vs`` carries the
    step's diffusion tensor."""
    a = dict(base.arrays)
    a.update(temp=np.stack([T, T, T], axis=-1), salt=np.stack([S, S, S], axis=-1), K_iso=K)
    vs = O.OracleState(a, tau=1, taup1=2, taum1=0)
    O.isoneutral_step(vs, base.settings)
    return vs.temp[..., vs.tau].copy(), vs.salt[..., vs.tau].copy(), vs


def rollout(base, T0, S0, K, nsteps):
    """Tracer checkpoints ``[T_0 .. T_n]``, ``[S_0 .. S_n]`` of an n-step rollout."""
    Ts, Ss = [T0], [S0]
    for _ in range(nsteps):
        T, S, _ = forward_step(base, Ts[-1], Ss[-1], K)
        Ts.append(T)
        Ss.append(S)
    return Ts, Ss


def rollout_slope_signs(base, T0, S0, K, nsteps):
    """Signs of every slope of every step of a rollout (the taper depends on
    |slope|, so the forward is not differentiable where a slope is zero)."""
    T, S = T0, S0
    out = []
    for _ in range(nsteps):
        T, S, vs = forward_step(base, T, S, K)
        out.append(np.concatenate([np.sign(getattr(vs, n)).ravel() for n in ("Ai_ez", "Ai_nz", "Ai_bx", "Ai_by")]))
    return np.concatenate(out)


def central_difference(loss_of, signs_of, x, u, eps, shrink=2):
    """Central difference of ``loss_of`` at ``x`` along ``u`` with step
    ``eps * |x|``. Where the two evaluation points lie on different sides of
    a kink (``signs_of`` differs between them) the step shrinks tenfold, at
    most ``shrink`` times. Returns ``(derivative, eps used)``."""
    for _ in range(shrink + 1):
        h = eps * np.linalg.norm(x)
        if np.array_equal(signs_of(x + h * u), signs_of(x - h * u)):
            break
        eps *= 0.1
    return (loss_of(x + h * u) - loss_of(x - h * u)) / (2 * h), eps


def directional_checks(loss_of, signs_of, inputs, grads, eps0, ndir, rng):
    """Directional derivatives of ``loss_of(**inputs)`` along seeded random
    unit directions of one input at a time, as central differences
    (``central_difference``) and from the gradients ``grads``.

    ``ndir`` maps input names to direction counts and ``eps0`` to relative
    steps. Yields ``(name, fd, ad, scale)`` with ``scale = max(|ad|,
    |grad| / sqrt(n))``, the typical size of a directional derivative along a
    random unit direction in n dimensions.
    """
    for which, count in ndir.items():
        def with_(x, which=which):
            a = dict(inputs)
            a[which] = x
            return a

        for _ in range(count):
            x = inputs[which]
            u = rng.standard_normal(x.shape)
            u /= np.linalg.norm(u)
            fd, _ = central_difference(lambda y: loss_of(**with_(y)), lambda y: signs_of(**with_(y)), x, u,
                                       eps0[which])
            g = np.asarray(grads[which])
            ad = float(np.sum(g * u))
            yield which, fd, ad, max(abs(ad), float(np.linalg.norm(g)) / np.sqrt(g.size))


def wet_interior(base):
    m = _g(base, "maskT").astype(np.float64)
    w = np.zeros_like(m)
    w[2:-2, 2:-2] = m[2:-2, 2:-2]
    return w


def loss(T_final, target, wet):
    """Sum over wet cells of (temp - target)^2."""
    return float(np.sum(wet * (T_final - target) ** 2))


def _drdT_dT(eq_type):
    """d(drho/dT)/dT of veros/core/density/get_rho.py:93-111."""
    if eq_type == 1:
        return 0.0
    if eq_type == 3:
        return -O.BETA_TS_EQ3 * O.RHO0
    if eq_type in (2, 4):
        return -2.0 * O.BETA_TS_EQ24 * O.RHO0
    raise ValueError(f"unsupported eq_of_state_type {eq_type}")


def _shift_x(F):
    """Value of the x-face west of each point (face i-1), zero at i = 0."""
    out = np.zeros_like(F)
    out[1:] = F[:-1]
    return out


def _shift_y(F):
    out = np.zeros_like(F)
    out[:, 1:] = F[:, :-1]
    return out


def _shift_z(F):
    """Value of the z-face below each point (face k-1), zero at k = 0."""
    out = np.zeros_like(F)
    out[:, :, 1:] = F[:, :, :-1]
    return out


def implicit_adjoint(base, K33, x_new, g_new, dt):
    """Adjoint of the implicit vertical solve (diffusion.py:142-169) for the
    tracers ``x_new`` (list of solutions) with incoming adjoints ``g_new``.

    The matrix is A = tridiag(a, b, c) with a_k = -delta_{k-1}/dzt_k,
    c_k = -delta_k/dzt_k, b_k = 1 + (delta_k + delta_{k-1})/dzt_k (no
    delta_{k-1} on the bottom row), delta_k = dt K_33/dzw_k. For x = A^-1 d:
    lambda_d = A^-T lambda_x, and
    dL/ddelta_k = (x_{k+1} - x_k) (lambda_d_k/dzt_k - lambda_d_{k+1}/dzt_{k+1}).
    Returns the adjoints of the right-hand sides (full arrays; cells outside
    the solve pass the adjoint through) and dL/dK_33.
    """
    dzt, dzw = _g(base, "dzt"), _g(base, "dzw")
    kbot = _g(base, "kbot")
    Z = dzt.shape[0]
    ks = kbot[2:-2, 2:-2].astype(np.int64) - 1
    _, water, edge = O.create_water_masks(kbot[2:-2, 2:-2], Z)
    delta = np.zeros(K33[2:-2, 2:-2].shape)
    delta[..., :-1] = dt / dzw[:-1] * K33[2:-2, 2:-2, :-1]
    a = np.zeros_like(delta)
    a[..., 1:] = -delta[..., :-1] / dzt[1:]
    c = np.zeros_like(delta)
    c[..., :-1] = -delta[..., :-1] / dzt[:-1]
    b = np.ones_like(delta)
    b[..., 1:] = 1 + (delta[..., 1:] + delta[..., :-1]) / dzt[1:]
    b = np.where(edge, 1 + delta / dzt, b)

    outs = []
    ys = []
    for g in g_new:
        rhs = g[2:-2, 2:-2]
        cp = np.zeros_like(delta)
        dp = np.zeros_like(delta)
        with np.errstate(divide="ignore", invalid="ignore"):
            for k in range(Z):
                act = water[..., k]
                first = edge[..., k]
                sub = np.where(first | (k == 0), 0.0, c[..., k - 1] if k > 0 else 0.0)
                prev_cp = cp[..., k - 1] if k > 0 else 0.0
                prev_dp = dp[..., k - 1] if k > 0 else 0.0
                den = b[..., k] - sub * prev_cp
                sup = a[..., k + 1] if k < Z - 1 else 0.0
                cp[..., k] = np.where(act, sup / den, 0.0)
                dp[..., k] = np.where(act, (rhs[..., k] - sub * prev_dp) / den, 0.0)
        y = np.zeros_like(delta)
        y[..., Z - 1] = dp[..., Z - 1]
        for k in range(Z - 2, -1, -1):
            y[..., k] = dp[..., k] - cp[..., k] * y[..., k + 1]
        y = np.where(water, y, 0.0)
        out = g.copy()
        out[2:-2, 2:-2] = np.where(water, y, rhs)
        outs.append(out)
        ys.append(y)

    ldelta = np.zeros_like(delta)
    for x, y in zip(x_new, ys):
        xi = x[2:-2, 2:-2]
        term = (xi[..., 1:] - xi[..., :-1]) * (y[..., :-1] / dzt[:-1] - y[..., 1:] / dzt[1:])
        ldelta[..., :-1] += np.where(water[..., :-1], term, 0.0)
    gK33 = np.zeros(K33.shape)
    gK33[2:-2, 2:-2, :-1] = ldelta[..., :-1] * dt / dzw[:-1]
    return outs, gK33


def step_adjoint(base, T, S, K, gT_new, gS_new, T_new=None, S_new=None):
    """Adjoint of one step: from dL/dT_new, dL/dS_new to dL/dT, dL/dS and dL/dK."""
    st = base.settings
    if T_new is None or S_new is None:
        T_new, S_new, vs = forward_step(base, T, S, K)
    else:
        a = dict(base.arrays)
        a.update(temp=np.stack([T, T, T], axis=-1), salt=np.stack([S, S, S], axis=-1), K_iso=K)
        vs = O.OracleState(a, tau=1, taup1=2, taum1=0)
        vs.__dict__.update(O.isoneutral_diffusion_pre(vs, st))
    K11, K22, K33 = vs.K_11, vs.K_22, vs.K_33
    X, Y, Z = T.shape
    dt = float(st["dt_tracer"])
    slopec, dslope, ksteep = float(st["iso_slopec"]), float(st["iso_dslope"]), float(st["K_iso_steep"])
    eq = int(st["eq_of_state_type"])
    mT, mU, mV, mW = (_g(base, n).astype(np.float64) for n in ("maskT", "maskU", "maskV", "maskW"))
    dxt, dxu, dyt, dyu = (_g(base, n) for n in ("dxt", "dxu", "dyt", "dyu"))
    cost, cosu, dzt, dzw, zt = (_g(base, n) for n in ("cost", "cosu", "dzt", "dzw", "zt"))
    X3 = lambda v: v[:, None, None]  # noqa: E731
    Y3 = lambda v: v[None, :, None]  # noqa: E731
    Z3 = lambda v: v[None, None, :]  # noqa: E731
    zeros = lambda: np.zeros((X, Y, Z))  # noqa: E731

    # ---- implicit part ----------------------------------------------------------------------
    (gTp, gSp), gK33 = implicit_adjoint(base, K33, [T_new, S_new], [gT_new, gS_new], dt)

    # ---- explicit part: adjoints of the face fluxes -----------------------------------------
    interior = np.zeros((X, Y, 1))
    interior[2:-2, 2:-2] = 1.0
    tr = {"T": T, "S": S}
    lfe, lfn, lft = {}, {}, {}
    inv_cdxt = 1.0 / (Y3(cost) * X3(dxt))
    inv_cdyt = 1.0 / (Y3(cost) * Y3(dyt))
    for n, gp in (("T", gTp), ("S", gSp)):
        mu = dt * mT * gp * interior
        e = zeros()
        e[:-1] = mu[:-1] * inv_cdxt[:-1] - mu[1:] * inv_cdxt[1:]
        e[0] = 0.0
        e[X - 2:] = 0.0
        e[:, :2] = 0.0
        e[:, Y - 2:] = 0.0
        lfe[n] = e
        f = zeros()
        f[:, :-1] = Y3(cosu[:-1]) * (mu[:, :-1] * inv_cdyt[:, :-1] - mu[:, 1:] * inv_cdyt[:, 1:])
        f[:, 0] = 0.0
        f[:, Y - 2:] = 0.0
        f[:2] = 0.0
        f[X - 2:] = 0.0
        lfn[n] = f
        t = zeros()
        t[..., :-1] = mu[..., :-1] / dzt[:-1] - mu[..., 1:] / dzt[1:]
        lft[n] = t

    # ---- point and face quantities ----------------------------------------------------------
    rT = mT * O.get_drhodT(eq, T, np.abs(Z3(zt)))
    rS = mT * O.get_drhodS(eq, T, np.abs(Z3(zt)))
    drT = mT * _drdT_dT(eq)
    gx, gy, gz, hdx, hdy, vd = {}, {}, {}, {}, {}, {}
    for n, q in tr.items():
        a = zeros()
        a[:-1] = mU[:-1] * (q[1:] - q[:-1]) / (X3(dxu[:-1]) * Y3(cost))
        gx[n] = a
        b = zeros()
        b[:, :-1] = mV[:, :-1] * (q[:, 1:] - q[:, :-1]) / Y3(dyu[:-1])
        gy[n] = b
        c = zeros()
        c[..., :-1] = mW[..., :-1] * (q[..., 1:] - q[..., :-1]) / Z3(dzw[:-1])
        gz[n] = c
        h = zeros()
        h[:-1] = q[1:] - q[:-1]
        hdx[n] = h
        h = zeros()
        h[:, :-1] = q[:, 1:] - q[:, :-1]
        hdy[n] = h
        v1 = zeros()
        v1[..., :-1] = q[..., 1:] - q[..., :-1]
        vd[n] = (_shift_z(v1), v1)  # below, above
    G = [rT * _shift_z(gz["T"]) + rS * _shift_z(gz["S"]), rT * gz["T"] + rS * gz["S"]]
    R = [1.0 / (np.minimum(0.0, g) - O.EPSLN) for g in G]

    dlx = zeros()
    dlx[:-1, :, 1:] = 0.25 * (K[:-1, :, 1:] + K[:-1, :, :-1] + K[1:, :, 1:] + K[1:, :, :-1])
    dlx[:-1, :, 0] = 0.5 * (K[:-1, :, 0] + K[1:, :, 0])
    dly = zeros()
    dly[:, :-1, 1:] = 0.25 * (K[:, :-1, 1:] + K[:, :-1, :-1] + K[:, 1:, 1:] + K[:, 1:, :-1])
    dly[:, :-1, 0] = 0.5 * (K[:, :-1, 0] + K[:, 1:, 0])
    gK11 = (lfe["T"] * hdx["T"] + lfe["S"] * hdx["S"]) / (X3(dxu) * Y3(cost))
    gK22 = (lfn["T"] * hdy["T"] + lfn["S"] * hdy["S"]) / Y3(dyu)

    ii = np.arange(X)[:, None, None]
    jj = np.arange(Y)[None, :, None]
    kk = np.arange(Z)[None, None, :]
    int_ij = (ii >= 2) & (ii < X - 2) & (jj >= 2) & (jj < Y - 2)
    q4dzt = 1.0 / (4.0 * Z3(dzt))
    dzw_v = [_shift_z(np.broadcast_to(Z3(dzw), (X, Y, Z)).copy()), np.broadcast_to(Z3(dzw), (X, Y, Z))]

    # faces: (kind, shift, E-range, face mask, dl, adjoint flux, K11/K22 adjoint, T-term factors)
    def face(h):
        if h in (0, 1):  # x-faces
            sh = (lambda F: F) if h == 0 else _shift_x
            fi = ii if h == 0 else ii - 1
            rngE = (fi >= 1) & (fi < X - 2) & (jj >= 2) & (jj < Y - 2)
            fidx = np.clip(fi, 0, X - 1)[:, 0, 0]
            c_h = X3(dxu[fidx]) / (4.0 * X3(dxt))
            cp_h = 1.0 / (Y3(cost) * 4.0 * X3(dxt))
            return sh, rngE, sh(mU), sh(dlx), {n: sh(lfe[n]) for n in tr}, sh(gK11), c_h, cp_h, \
                {n: sh(gx[n]) for n in tr}, {n: sh(hdx[n]) for n in tr}, "x"
        sh = (lambda F: F) if h == 2 else _shift_y
        fj = jj if h == 2 else jj - 1
        rngE = (fj >= 1) & (fj < Y - 2) & (ii >= 2) & (ii < X - 2)
        fjdx = np.clip(fj, 0, Y - 1)[0, :, 0]
        c_h = Y3(cosu[fjdx] * dyu[fjdx]) / (4.0 * Y3(dyt) * Y3(cost))
        cp_h = Y3(cosu[fjdx]) / (4.0 * Y3(dyt) * Y3(cost))
        return sh, rngE, sh(mV), sh(dly), {n: sh(lfn[n]) for n in tr}, sh(gK22), c_h, cp_h, \
            {n: sh(gy[n]) for n in tr}, {n: sh(hdy[n]) for n in tr}, "y"

    lrT = zeros()
    lG = [zeros(), zeros()]
    lgx = {n: zeros() for n in tr}
    lgy = {n: zeros() for n in tr}
    lhdx = {n: zeros() for n in tr}
    lhdy = {n: zeros() for n in tr}
    lvd = {n: [zeros(), zeros()] for n in tr}
    ldlx, ldly = zeros(), zeros()
    lK = zeros()

    def scatter(dst, val, h):
        """Add a per-point value onto the point's face h."""
        if h in (0, 2):
            dst += val
        elif h == 1:
            dst[:-1] += val[1:]
        else:
            dst[:, :-1] += val[:, 1:]

    for h in range(4):
        sh, rngE, mH, dl, lf, gKh, c_h, cp_h, gxh, hdh, kind = face(h)
        for v in range(2):
            s = -(rT * gxh["T"] + rS * gxh["S"]) * R[v]
            x = (slopec - np.abs(s)) / dslope
            t = 0.5 * (1.0 + np.tanh(x))
            tp = -2.0 * np.sign(s) * t * (1.0 - t) / dslope
            # term of face h
            vE = rngE & ((v == 1) | (kk >= 1))
            Ef = np.where(vE, mH, 0.0)
            lfv = lf["T"] * vd["T"][v] + lf["S"] * vd["S"][v]
            gAiE = lfv * dl * q4dzt
            sw = (dl * t > ksteep).astype(np.float64)
            gs = Ef * (gAiE * (t + s * tp) + gKh * dzw_v[v] * q4dzt * sw * dl * tp)
            scatter(ldlx if kind == "x" else ldly, Ef * (gKh * dzw_v[v] * q4dzt * sw * t + lfv * t * s * q4dzt), h)
            for n in tr:
                lvd[n][v] += Ef * lf[n] * dl * t * s * q4dzt
            # term of face v
            kw = kk - 1 + v
            vT = int_ij & (kw >= 0) & (kw <= Z - 2)
            if v == 1:
                mWv, KW, lK33 = mW, K, gK33
                lftv = {n: lft[n] for n in tr}
            else:
                mWv, KW, lK33 = _shift_z(mW), _shift_z(K), _shift_z(gK33)
                lftv = {n: _shift_z(lft[n]) for n in tr}
            Tf = np.where(vT, mWv, 0.0)
            lfh = lftv["T"] * hdh["T"] + lftv["S"] * hdh["S"]
            gAiT = lfh * KW * cp_h
            gs = gs + Tf * (gAiT * (t + s * tp) + lK33 * KW * c_h * (tp * s * s + 2.0 * t * s))
            lKv = Tf * (lK33 * c_h * t * s * s + lfh * t * s * cp_h)
            if v == 1:
                lK += lKv
            else:
                lK[:, :, :-1] += lKv[:, :, 1:]
            for n in tr:
                scatter(lhdx[n] if kind == "x" else lhdy[n], Tf * lftv[n] * KW * t * s * cp_h, h)
            # the slope itself
            lN = -gs * R[v]
            lG[v] += np.where(G[v] < 0.0, -gs * s * R[v], 0.0)
            lrT += lN * gxh["T"]
            scatter(lgx["T"] if kind == "x" else lgy["T"], lN * rT, h)
            scatter(lgx["S"] if kind == "x" else lgy["S"], lN * rS, h)

    lgz = {n: zeros() for n in tr}
    for n, r in (("T", rT), ("S", rS)):
        lgz[n] += lG[1] * r
        lgz[n][..., :-1] += (lG[0] * r)[..., 1:]
    lrT += lG[1] * gz["T"] + lG[0] * _shift_z(gz["T"])
    for n in tr:
        lhdx[n] += lfe[n] * K11 / (X3(dxu) * Y3(cost))
        lhdy[n] += lfn[n] * K22 / Y3(dyu)

    # ---- back to the tracers and to K_iso ----------------------------------------------------
    out = {}
    for n, gp in (("T", gTp), ("S", gSp)):
        g = mT * gp
        if n == "T":
            g = g + drT * lrT
        w = lgx[n] * mU / (X3(dxu) * Y3(cost)) + lhdx[n]
        g[1:] += w[:-1]
        g[:-1] -= w[:-1]
        w = lgy[n] * mV / Y3(dyu) + lhdy[n]
        g[:, 1:] += w[:, :-1]
        g[:, :-1] -= w[:, :-1]
        w = lgz[n] * mW / Z3(dzw)
        g[..., 1:] += w[..., :-1]
        g[..., :-1] -= w[..., :-1]
        w = lvd[n][1]
        g[..., 1:] += w[..., :-1]
        g[..., :-1] -= w[..., :-1]
        w = lvd[n][0]
        g[..., 1:] += w[..., 1:]
        g[..., :-1] -= w[..., 1:]
        out[n] = g
    gK = lK.copy()
    for dl, ax in ((ldlx, 0), (ldly, 1)):
        w = np.moveaxis(dl, ax, 0)
        gk = np.moveaxis(gK, ax, 0)
        gk[:-1, :, 1:] += 0.25 * w[:-1, :, 1:]
        gk[:-1, :, :-1] += 0.25 * w[:-1, :, 1:]
        gk[1:, :, 1:] += 0.25 * w[:-1, :, 1:]
        gk[1:, :, :-1] += 0.25 * w[:-1, :, 1:]
        gk[:-1, :, 0] += 0.5 * w[:-1, :, 0]
        gk[1:, :, 0] += 0.5 * w[:-1, :, 0]
    return out["T"], out["S"], gK


def rollout_grad(base, T0, S0, K, target, nsteps):
    """Loss of an n-step rollout and its gradients with respect to T0, S0, K."""
    Ts, Ss = rollout(base, T0, S0, K, nsteps)
    wet = wet_interior(base)
    L = loss(Ts[-1], target, wet)
    gT = 2.0 * wet * (Ts[-1] - target)
    gS = np.zeros_like(gT)
    gK = np.zeros_like(K)
    for n in range(nsteps - 1, -1, -1):
        gT, gS, gKn = step_adjoint(base, Ts[n], Ss[n], K, gT, gS, Ts[n + 1], Ss[n + 1])
        gK += gKn
    return L, gT, gS, gK
