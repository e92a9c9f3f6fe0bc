"""CPU oracle for the isoneutral mixing path. TEST INFRASTRUCTURE ONLY.

This module is the checker: only ``tests/``, ``__graft_entry__.smoke()`` and
the CPU-baseline legs of ``bench.py`` may import it. The product path
(``veros_gb300``) never calls it and fails loudly without its CUDA library.

It restates, in vectorised NumPy on reference-layout float64 arrays
(``(X, Y, Z)`` fields, tracers with a trailing time axis, ``Ai_*`` with a
trailing ``(ip|jp, kr)`` pair), the Veros NumPy-backend algorithm for:

* ``isoneutral_diffusion_pre``      veros/core/isoneutral/isoneutral.py:18-229
* ``dm_taper``                      veros/core/isoneutral/isoneutral.py:10-15
* ``get_drhodT / get_drhodS``       veros/core/density/get_rho.py:93-132
* ``_calc_tracer_fluxes``           veros/core/isoneutral/diffusion.py:9-113
* ``_calc_explicit_part``           veros/core/isoneutral/diffusion.py:116-139
* ``_calc_implicit_part``           veros/core/isoneutral/diffusion.py:142-169
* ``isoneutral_diffusion_tracer``   veros/core/isoneutral/diffusion.py:172-207
* ``isoneutral_diffusion_kernel``   veros/core/isoneutral/diffusion.py:210-283
* ``compute_dissipation``           veros/core/diffusion.py:9-36
* ``dissipation_on_wgrid``          veros/core/diffusion.py:39-62
* ``pad_z_edges / create_water_masks / solve_implicit``
                                    veros/core/utilities.py:24-59
* ``solve_tridiagonal_numpy``       veros/core/operators.py:60-77
* ``vertmix_tempsalt``              veros/core/thermodynamics.py:248-300
* ``enforce_boundaries`` (one process)
                                    veros/core/utilities.py:7-16
* ``isoneutral_diag_streamfunction_kernel``
                                    veros/core/isoneutral/isoneutral.py:232-254

The tridiagonal solve is LAPACK ``dgtsv`` (the routine the reference calls
through ``scipy.linalg.lapack``), restated column-parallel in ``dgtsv_columns``
for masks of the ``create_water_masks`` form and called through SciPy for any
other form, as the reference does.

Pinning: ``tests/golden/make_golden.py`` runs the reference NumPy backend on
seeded states and stores inputs and outputs; ``tests/test_oracle_golden.py``
checks this module against them.
"""

import numpy as np

EPSLN = 1e-20

# equation-of-state constants (veros/core/density/linear_eq.py:10-16,
# nonlinear_eq1.py:10-17, nonlinear_eq2.py:11-20, nonlinear_eq3.py:10-17)
RHO0 = 1024.0
THETA0 = 283.0 - 273.15
BETA_T = 1.67e-4
BETA_S = 0.78e-3
BETA_TS_EQ3 = 1e-5
BETA_TS_EQ24 = 1e-5 / 2.0
GAMMAS = 1.1e-8
GRAV_EOS = 9.81


class OracleState:
    """Attribute view of a dict of reference-layout arrays plus time indices."""

    def __init__(self, arrays, tau=1, taup1=2, taum1=0):
        self.__dict__.update(arrays)
        self.tau, self.taup1, self.taum1 = tau, taup1, taum1


def _settings_get(settings, name):
    return settings[name] if isinstance(settings, dict) else getattr(settings, name)


def get_drhodT(eq_type, temp, p):
    """veros/core/density/get_rho.py:93-111 for eq types 1-4."""
    if eq_type == 1:
        return -BETA_T * RHO0  # linear_eq.py:36-38
    if eq_type in (2, 4):
        return -(BETA_T + 2 * BETA_TS_EQ24 * (temp - THETA0)) * RHO0  # nonlinear_eq1.py:39-42
    if eq_type == 3:
        zz = -p - 0.0
        thetas = temp - THETA0
        return -(BETA_TS_EQ3 * thetas + BETA_T * (1 - GAMMAS * GRAV_EOS * zz * RHO0)) * RHO0  # nonlinear_eq2.py:57-61
    raise ValueError(f"unsupported eq_of_state_type {eq_type}")


def get_drhodS(eq_type, temp, p):
    """veros/core/density/get_rho.py:114-132 for eq types 1-4."""
    if eq_type in (1, 2, 3):
        return BETA_S * RHO0
    if eq_type == 4:
        return 0 * RHO0
    raise ValueError(f"unsupported eq_of_state_type {eq_type}")


def dm_taper(sx, iso_slopec, iso_dslope):
    """veros/core/isoneutral/isoneutral.py:10-15."""
    return 0.5 * (1.0 + np.tanh((-np.abs(sx) + iso_slopec) / iso_dslope))


def isoneutral_diffusion_pre(vs, settings):
    """Slopes and diffusion tensor (veros/core/isoneutral/isoneutral.py:18-229).

    Returns a dict with new ``Ai_ez, Ai_nz, Ai_bx, Ai_by, K_11, K_22, K_33``;
    cells the reference does not write keep the values of ``vs``.
    """
    S = lambda n: _settings_get(settings, n)  # noqa: E731
    tau = vs.tau
    T = vs.temp[:, :, :, tau]
    Sa = vs.salt[:, :, :, tau]
    shape = T.shape
    p = np.abs(vs.zt)

    drdT = vs.maskT * get_drhodT(S("eq_of_state_type"), T, p)
    drdS = vs.maskT * get_drhodS(S("eq_of_state_type"), T, p)

    # face gradients (:46-95)
    dTdz = np.zeros(shape)
    dSdz = np.zeros(shape)
    dTdx = np.zeros(shape)
    dSdx = np.zeros(shape)
    dTdy = np.zeros(shape)
    dSdy = np.zeros(shape)
    dTdz[:, :, :-1] = vs.maskW[:, :, :-1] * (T[:, :, 1:] - T[:, :, :-1]) / vs.dzw[None, None, :-1]
    dSdz[:, :, :-1] = vs.maskW[:, :, :-1] * (Sa[:, :, 1:] - Sa[:, :, :-1]) / vs.dzw[None, None, :-1]
    facx = vs.dxu[:-1, None, None] * vs.cost[None, :, None]
    dTdx[:-1] = vs.maskU[:-1] * (T[1:] - T[:-1]) / facx
    dSdx[:-1] = vs.maskU[:-1] * (Sa[1:] - Sa[:-1]) / facx
    dTdy[:, :-1] = vs.maskV[:, :-1] * (T[:, 1:] - T[:, :-1]) / vs.dyu[None, :-1, None]
    dSdy[:, :-1] = vs.maskV[:, :-1] * (Sa[:, 1:] - Sa[:, :-1]) / vs.dyu[None, :-1, None]

    slopec, dslope, ksteep = S("iso_slopec"), S("iso_dslope"), S("K_iso_steep")
    K_iso = vs.K_iso
    Ai_ez = vs.Ai_ez.copy()
    Ai_nz = vs.Ai_nz.copy()
    Ai_bx = vs.Ai_bx.copy()
    Ai_by = vs.Ai_by.copy()
    K_11 = vs.K_11.copy()
    K_22 = vs.K_22.copy()
    K_33 = vs.K_33.copy()

    # east face (:100-132)
    diffloc = np.zeros(shape)
    diffloc[1:-2, 2:-2, 1:] = 0.25 * (K_iso[1:-2, 2:-2, 1:] + K_iso[1:-2, 2:-2, :-1]
                                      + K_iso[2:-1, 2:-2, 1:] + K_iso[2:-1, 2:-2, :-1])
    diffloc[1:-2, 2:-2, 0] = 0.5 * (K_iso[1:-2, 2:-2, 0] + K_iso[2:-1, 2:-2, 0])
    sumz = np.zeros(shape)[1:-2, 2:-2]
    for kr in range(2):
        ki = 0 if kr == 1 else 1
        zsl = slice(None, -1 + kr or None)
        for ip in range(2):
            xs = slice(1 + ip, -2 + ip or None)
            drodxe = drdT[xs, 2:-2, ki:] * dTdx[1:-2, 2:-2, ki:] + drdS[xs, 2:-2, ki:] * dSdx[1:-2, 2:-2, ki:]
            drodze = drdT[xs, 2:-2, ki:] * dTdz[xs, 2:-2, zsl] + drdS[xs, 2:-2, ki:] * dSdz[xs, 2:-2, zsl]
            sxe = -drodxe / (np.minimum(0.0, drodze) - EPSLN)
            taper = dm_taper(sxe, slopec, dslope)
            sumz[:, :, ki:] += (vs.dzw[None, None, zsl] * vs.maskU[1:-2, 2:-2, ki:]
                                * np.maximum(ksteep, diffloc[1:-2, 2:-2, ki:] * taper))
            Ai_ez[1:-2, 2:-2, ki:, ip, kr] = taper * sxe * vs.maskU[1:-2, 2:-2, ki:]
    K_11[1:-2, 2:-2, :] = sumz / (4.0 * vs.dzt[None, None, :])

    # north face (:137-168)
    diffloc = np.zeros(shape)
    diffloc[2:-2, 1:-2, 1:] = 0.25 * (K_iso[2:-2, 1:-2, 1:] + K_iso[2:-2, 1:-2, :-1]
                                      + K_iso[2:-2, 2:-1, 1:] + K_iso[2:-2, 2:-1, :-1])
    diffloc[2:-2, 1:-2, 0] = 0.5 * (K_iso[2:-2, 1:-2, 0] + K_iso[2:-2, 2:-1, 0])
    sumz = np.zeros(shape)[2:-2, 1:-2]
    for kr in range(2):
        ki = 0 if kr == 1 else 1
        zsl = slice(None, -1 + kr or None)
        for jp in range(2):
            ys = slice(1 + jp, -2 + jp or None)
            drodyn = drdT[2:-2, ys, ki:] * dTdy[2:-2, 1:-2, ki:] + drdS[2:-2, ys, ki:] * dSdy[2:-2, 1:-2, ki:]
            drodzn = drdT[2:-2, ys, ki:] * dTdz[2:-2, ys, zsl] + drdS[2:-2, ys, ki:] * dSdz[2:-2, ys, zsl]
            syn = -drodyn / (np.minimum(0.0, drodzn) - EPSLN)
            taper = dm_taper(syn, slopec, dslope)
            sumz[:, :, ki:] += (vs.dzw[None, None, zsl] * vs.maskV[2:-2, 1:-2, ki:]
                                * np.maximum(ksteep, diffloc[2:-2, 1:-2, ki:] * taper))
            Ai_nz[2:-2, 1:-2, ki:, jp, kr] = taper * syn * vs.maskV[2:-2, 1:-2, ki:]
    K_22[2:-2, 1:-2, :] = sumz / (4.0 * vs.dzt[None, None, :])

    # bottom face of the cell above / top face of this one (:173-225)
    sumx = np.zeros(shape)[2:-2, 2:-2, :-1]
    sumy = np.zeros(shape)[2:-2, 2:-2, :-1]
    for kr in range(2):
        ks = slice(kr, -1 + kr or None)
        drodzb = drdT[2:-2, 2:-2, ks] * dTdz[2:-2, 2:-2, :-1] + drdS[2:-2, 2:-2, ks] * dSdz[2:-2, 2:-2, :-1]
        for ip in range(2):
            xs = slice(1 + ip, -3 + ip)
            drodxb = drdT[2:-2, 2:-2, ks] * dTdx[xs, 2:-2, ks] + drdS[2:-2, 2:-2, ks] * dSdx[xs, 2:-2, ks]
            sxb = -drodxb / (np.minimum(0.0, drodzb) - EPSLN)
            taper = dm_taper(sxb, slopec, dslope)
            sumx = sumx + (vs.dxu[xs, None, None] * K_iso[2:-2, 2:-2, :-1] * taper * sxb**2
                           * vs.maskW[2:-2, 2:-2, :-1])
            Ai_bx[2:-2, 2:-2, :-1, ip, kr] = taper * sxb * vs.maskW[2:-2, 2:-2, :-1]
        for jp in range(2):
            ys = slice(1 + jp, -3 + jp)
            facty = vs.cosu[ys] * vs.dyu[ys]
            drodyb = drdT[2:-2, 2:-2, ks] * dTdy[2:-2, ys, ks] + drdS[2:-2, 2:-2, ks] * dSdy[2:-2, ys, ks]
            syb = -drodyb / (np.minimum(0.0, drodzb) - EPSLN)
            taper = dm_taper(syb, slopec, dslope)
            sumy = sumy + (facty[None, :, None] * K_iso[2:-2, 2:-2, :-1] * taper * syb**2
                           * vs.maskW[2:-2, 2:-2, :-1])
            Ai_by[2:-2, 2:-2, :-1, jp, kr] = taper * syb * vs.maskW[2:-2, 2:-2, :-1]
    K_33[2:-2, 2:-2, :-1] = (sumx / (4 * vs.dxt[2:-2, None, None])
                             + sumy / (4 * vs.dyt[None, 2:-2, None] * vs.cost[None, 2:-2, None]))
    K_33[..., -1] = 0.0
    return dict(Ai_ez=Ai_ez, Ai_nz=Ai_nz, Ai_bx=Ai_bx, Ai_by=Ai_by, K_11=K_11, K_22=K_22, K_33=K_33)


def pad_z_edges(array):
    """veros/core/utilities.py:24-35."""
    if array.ndim == 1:
        return np.pad(array, 1, mode="edge")
    return np.pad(array, ((0, 0), (0, 0), (1, 1)), mode="edge")


def create_water_masks(ks, nz):
    """veros/core/utilities.py:38-48."""
    ks = ks - 1
    land_mask = ks >= 0
    kk = np.arange(nz)[None, None, :]
    water_mask = land_mask[:, :, None] & (kk >= ks[:, :, None])
    edge_mask = land_mask[:, :, None] & (kk == ks[:, :, None])
    return land_mask, water_mask, edge_mask


def _kbot_form(water_mask, edge_mask):
    """True if every column is water from its first wet level to the top with the edge there."""
    nz = water_mask.shape[-1]
    wm = water_mask.reshape(-1, nz)
    em = edge_mask.reshape(-1, nz)
    has = wm.any(axis=1)
    ks = np.where(has, wm.argmax(axis=1), nz)
    kk = np.arange(nz)[None, :]
    return np.array_equal(wm, kk >= ks[:, None]) and np.array_equal(em, (kk == ks[:, None]) & has[:, None])


def dgtsv_columns(dl, d, du, b, ks):
    """LAPACK ``dgtsv`` (Gaussian elimination with partial pivoting, NRHS = 1)
    restated column-parallel in NumPy.

    LAPACK 3.x ``dgtsv`` is the third-party routine the reference calls
    (veros/core/operators.py:75, through scipy.linalg.lapack; scipy 1.18.1 with
    OpenBLAS 0.3.x). Its published algorithm, for rows i = 0..n-2: if
    ``|d[i]| >= |dl[i]|`` eliminate without interchange (``fact = dl/d``,
    ``d[i+1] -= fact*du[i]``, ``b[i+1] -= fact*b[i]``, second super-diagonal 0);
    otherwise interchange rows i and i+1 (``fact = d/dl``; the second
    super-diagonal takes ``du[i+1]`` except on the last step). Back
    substitution ``x[i] = (b[i] - du[i] x[i+1] - du2[i] x[i+2]) / d[i]``.

    Arrays are (ncols, nz); column ``s`` is the system of rows ``ks[s]..nz-1``
    (``dl[:, k]`` is the entry left of the diagonal in row k). Every operation
    is a single IEEE-rounded NumPy ufunc, so results do not depend on the
    platform's floating-point contraction.
    """
    ncols, nz = d.shape
    D = d.copy()
    DU = du.copy()
    DU2 = np.zeros_like(d)
    B = b.copy()
    kk = np.arange(nz)
    with np.errstate(divide="ignore", invalid="ignore"):
        for k in range(nz - 1):
            act = k >= ks
            if not act.any():
                continue
            l = dl[:, k + 1]
            dk, dk1, duk, bk, bk1 = D[:, k], D[:, k + 1], DU[:, k], B[:, k], B[:, k + 1]
            du1 = DU[:, k + 1]
            keep = np.abs(dk) >= np.abs(l)
            f_keep = l / dk
            f_swap = dk / l
            n_dk = np.where(keep, dk, l)
            n_dk1 = np.where(keep, dk1 - f_keep * duk, duk - f_swap * dk1)
            n_duk = np.where(keep, duk, dk1)
            n_bk = np.where(keep, bk, bk1)
            n_bk1 = np.where(keep, bk1 - f_keep * bk, bk - f_swap * bk1)
            if k < nz - 2:
                n_du2 = np.where(keep, 0.0, du1)
                n_du1 = np.where(keep, du1, -f_swap * du1)
            else:
                n_du2 = np.zeros(ncols)
                n_du1 = du1
            D[:, k] = np.where(act, n_dk, dk)
            D[:, k + 1] = np.where(act, n_dk1, dk1)
            DU[:, k] = np.where(act, n_duk, duk)
            DU[:, k + 1] = np.where(act, n_du1, du1)
            DU2[:, k] = np.where(act, n_du2, 0.0)
            B[:, k] = np.where(act, n_bk, bk)
            B[:, k + 1] = np.where(act, n_bk1, bk1)
        X = np.zeros_like(d)
        X[:, nz - 1] = B[:, nz - 1] / D[:, nz - 1]
        if nz > 1:
            X[:, nz - 2] = (B[:, nz - 2] - DU[:, nz - 2] * X[:, nz - 1]) / D[:, nz - 2]
        for k in range(nz - 3, -1, -1):
            X[:, k] = (B[:, k] - DU[:, k] * X[:, k + 1] - DU2[:, k] * X[:, k + 2]) / D[:, k]
    return np.where(kk[None, :] >= ks[:, None], X, 0.0)


def solve_tridiagonal(a, b, c, d, water_mask, edge_mask):
    """veros/core/operators.py:60-77: one ``dgtsv`` over all wet cells, couplings cut.

    With masks of the ``create_water_masks`` form the cut couplings make the
    concatenated system block-diagonal, one block per column, so the
    column-parallel restatement ``dgtsv_columns`` gives the same result;
    masks of any other form go to LAPACK exactly as the reference does.
    """
    out = np.zeros(a.shape, dtype=a.dtype)
    if not np.any(water_mask):
        return out
    a = a.copy()
    c = c.copy()
    a[edge_mask] = 0
    c[..., -1] = 0
    if _kbot_form(water_mask, edge_mask):
        # dgtsv works in float64 on whatever the reference hands it; the
        # solution is stored in an array of a's dtype (float32 runs round it).
        # Wider types (np.longdouble, for extended-precision checks of this
        # oracle) keep their precision.
        nz = a.shape[-1]
        shape = a.shape
        wm = water_mask.reshape(-1, nz)
        has = wm.any(axis=1)
        ks = np.where(has, wm.argmax(axis=1), nz)
        wt = np.result_type(a, b, c, d, np.float64)
        f64 = lambda x: np.asarray(x, dtype=wt).reshape(-1, nz)  # noqa: E731
        sol = dgtsv_columns(f64(a), f64(b), f64(c), f64(d), ks)
        return sol.reshape(shape).astype(out.dtype, copy=False)
    from scipy.linalg import lapack

    sol = lapack.dgtsv(a[water_mask][1:], b[water_mask], c[water_mask][:-1], d[water_mask])[3]
    out[water_mask] = sol
    return out


def solve_implicit(a, b, c, d, water_mask, edge_mask, b_edge=None, d_edge=None):
    """veros/core/utilities.py:51-59."""
    if b_edge is not None:
        b = np.where(edge_mask, b_edge, b)
    if d_edge is not None:
        d = np.where(edge_mask, d_edge, d)
    return solve_tridiagonal(a, b, c, d, water_mask, edge_mask)


def calc_tracer_fluxes(vs, tr, K_iso, K_skew):
    """veros/core/isoneutral/diffusion.py:9-113."""
    tau = vs.tau
    trt = tr[..., tau]
    tr_pad = pad_z_edges(trt)
    K1 = K_iso - K_skew
    K2 = K_iso + K_skew
    shape = trt.shape
    flux_east = np.zeros(shape)
    flux_north = np.zeros(shape)
    flux_top = np.zeros(shape)

    diffloc = np.zeros(shape)[1:-2, 2:-2]
    diffloc[:, :, 1:] = 0.25 * (K1[1:-2, 2:-2, 1:] + K1[1:-2, 2:-2, :-1] + K1[2:-1, 2:-2, 1:] + K1[2:-1, 2:-2, :-1])
    diffloc[:, :, 0] = 0.5 * (K1[1:-2, 2:-2, 0] + K1[2:-1, 2:-2, 0])
    sumz = 0.0
    for kr in range(2):
        for ip in range(2):
            xs = slice(1 + ip, -2 + ip or None)
            sumz = sumz + diffloc * vs.Ai_ez[1:-2, 2:-2, :, ip, kr] * (
                tr_pad[xs, 2:-2, 1 + kr:-1 + kr or None] - tr_pad[xs, 2:-2, kr:-2 + kr])
    flux_east[1:-2, 2:-2, :] = (sumz / (4.0 * vs.dzt[None, None, :])
                                + (trt[2:-1, 2:-2, :] - trt[1:-2, 2:-2, :])
                                / (vs.cost[None, 2:-2, None] * vs.dxu[1:-2, None, None]) * vs.K_11[1:-2, 2:-2, :])

    diffloc = np.zeros(shape)[2:-2, 1:-2]
    diffloc[:, :, 1:] = 0.25 * (K1[2:-2, 1:-2, 1:] + K1[2:-2, 1:-2, :-1] + K1[2:-2, 2:-1, 1:] + K1[2:-2, 2:-1, :-1])
    diffloc[:, :, 0] = 0.5 * (K1[2:-2, 1:-2, 0] + K1[2:-2, 2:-1, 0])
    sumz = 0.0
    for kr in range(2):
        for jp in range(2):
            ys = slice(1 + jp, -2 + jp or None)
            sumz = sumz + diffloc * vs.Ai_nz[2:-2, 1:-2, :, jp, kr] * (
                tr_pad[2:-2, ys, 1 + kr:-1 + kr or None] - tr_pad[2:-2, ys, kr:-2 + kr])
    flux_north[2:-2, 1:-2, :] = vs.cosu[None, 1:-2, None] * (
        sumz / (4.0 * vs.dzt[None, None, :])
        + (trt[2:-2, 2:-1, :] - trt[2:-2, 1:-2, :]) / vs.dyu[None, 1:-2, None] * vs.K_22[2:-2, 1:-2, :])

    diffloc = K2[2:-2, 2:-2, :-1]
    sumx = 0.0
    for ip in range(2):
        for kr in range(2):
            ks = slice(kr, -1 + kr or None)
            sumx = sumx + diffloc * vs.Ai_bx[2:-2, 2:-2, :-1, ip, kr] / vs.cost[None, 2:-2, None] * (
                trt[2 + ip:-2 + ip or None, 2:-2, ks] - trt[1 + ip:-3 + ip, 2:-2, ks])
    sumy = 0.0
    for jp in range(2):
        for kr in range(2):
            ks = slice(kr, -1 + kr or None)
            sumy = sumy + diffloc * vs.Ai_by[2:-2, 2:-2, :-1, jp, kr] * vs.cosu[None, 1 + jp:-3 + jp, None] * (
                trt[2:-2, 2 + jp:-2 + jp or None, ks] - trt[2:-2, 1 + jp:-3 + jp, ks])
    flux_top[2:-2, 2:-2, :-1] = (sumx / (4 * vs.dxt[2:-2, None, None])
                                 + sumy / (4 * vs.dyt[None, 2:-2, None] * vs.cost[None, 2:-2, None]))
    flux_top[:, :, -1] = 0.0
    return flux_east, flux_north, flux_top


def calc_explicit_part(vs, flux_east, flux_north, flux_top):
    """veros/core/isoneutral/diffusion.py:116-139."""
    ep = np.zeros(flux_east.shape)
    ep[2:-2, 2:-2, :] = vs.maskT[2:-2, 2:-2, :] * (
        (flux_east[2:-2, 2:-2, :] - flux_east[1:-3, 2:-2, :])
        / (vs.cost[None, 2:-2, None] * vs.dxt[2:-2, None, None])
        + (flux_north[2:-2, 2:-2, :] - flux_north[2:-2, 1:-3, :])
        / (vs.cost[None, 2:-2, None] * vs.dyt[None, 2:-2, None]))
    ep[:, :, 0] += vs.maskT[:, :, 0] * flux_top[:, :, 0] / vs.dzt[0]
    ep[:, :, 1:] += vs.maskT[:, :, 1:] * (flux_top[:, :, 1:] - flux_top[:, :, :-1]) / vs.dzt[None, None, 1:]
    return ep


def calc_implicit_part(vs, settings, tr):
    """veros/core/isoneutral/diffusion.py:142-169."""
    dt = _settings_get(settings, "dt_tracer")
    nz = vs.dzt.shape[0]
    _, water_mask, edge_mask = create_water_masks(vs.kbot[2:-2, 2:-2], nz)
    shape = vs.K_33[2:-2, 2:-2].shape
    a_tri = np.zeros(shape)
    b_tri = np.zeros(shape)
    c_tri = np.zeros(shape)
    delta = np.zeros(shape)
    delta[:, :, :-1] = dt / vs.dzw[None, None, :-1] * vs.K_33[2:-2, 2:-2, :-1]
    delta[:, :, -1] = 0.0
    a_tri[:, :, 1:] = -delta[:, :, :-1] / vs.dzt[None, None, 1:]
    b_tri[:, :, 1:-1] = 1 + (delta[:, :, 1:-1] + delta[:, :, :-2]) / vs.dzt[None, None, 1:-1]
    b_tri[:, :, -1] = 1 + delta[:, :, -2] / vs.dzt[None, None, -1]
    b_tri_edge = 1 + (delta[:, :, :] / vs.dzt[None, None, :])
    c_tri[:, :, :-1] = -delta[:, :, :-1] / vs.dzt[None, None, :-1]
    d = tr[2:-2, 2:-2, :, vs.taup1]
    sol = solve_implicit(a_tri, b_tri, c_tri, d, water_mask, edge_mask, b_edge=b_tri_edge)
    return np.where(water_mask, sol, d)


def isoneutral_diffusion_tracer(vs, settings, tr, dtracer_iso, iso=True, skew=False):
    """veros/core/isoneutral/diffusion.py:172-207."""
    dt = _settings_get(settings, "dt_tracer")
    K_iso = vs.K_iso if iso else 0.0
    K_skew = vs.K_gm if skew else 0.0
    flux_east, flux_north, flux_top = calc_tracer_fluxes(vs, tr, K_iso, K_skew)
    dtr = calc_explicit_part(vs, flux_east, flux_north, flux_top)
    dtracer_iso = dtracer_iso + dtr
    tr = tr.copy()
    tr[2:-2, 2:-2, :, vs.taup1] += dt * dtr[2:-2, 2:-2, :]
    if iso:
        new_tr = tr.copy()
        new_tr[2:-2, 2:-2, :, vs.taup1] = calc_implicit_part(vs, settings, tr)
        dtracer_iso = dtracer_iso + (new_tr[:, :, :, vs.taup1] - tr[:, :, :, vs.taup1]) / dt
        tr = new_tr
    return tr, dtracer_iso, flux_east, flux_north, flux_top


def compute_dissipation(vs, settings, int_drhodX, flux_east, flux_north):
    """veros/core/diffusion.py:9-36."""
    g, rho0 = _settings_get(settings, "grav"), _settings_get(settings, "rho_0")
    diss = np.zeros(flux_east.shape)
    diss[1:-1, 1:-1, :] = (
        0.5 * g / rho0 * ((int_drhodX[2:, 1:-1, :] - int_drhodX[1:-1, 1:-1, :]) * flux_east[1:-1, 1:-1, :]
                          + (int_drhodX[1:-1, 1:-1, :] - int_drhodX[:-2, 1:-1, :]) * flux_east[:-2, 1:-1, :])
        / (vs.dxt[1:-1, None, None] * vs.cost[None, 1:-1, None])
        + 0.5 * g / rho0 * ((int_drhodX[1:-1, 2:, :] - int_drhodX[1:-1, 1:-1, :]) * flux_north[1:-1, 1:-1, :]
                            + (int_drhodX[1:-1, 1:-1, :] - int_drhodX[1:-1, :-2, :]) * flux_north[1:-1, :-2, :])
        / (vs.dyt[None, 1:-1, None] * vs.cost[None, 1:-1, None]))
    return diss


def dissipation_on_wgrid(vs, diss, ks):
    """veros/core/diffusion.py:39-62."""
    nz = vs.dzt.shape[0]
    land_mask, water_mask, edge_mask = create_water_masks(ks, nz)
    water_mask = water_mask & ~edge_mask
    dzw_pad = pad_z_edges(vs.dzw)
    diss_w = np.zeros(diss.shape)
    diss_w[:, :, :-1] = (
        (0.5 * (diss[:, :, :-1] + diss[:, :, 1:])
         + 0.5 * (diss[:, :, :-1] * dzw_pad[None, None, :-3] / vs.dzw[None, None, :-1]))
        * edge_mask[:, :, :-1]
        + 0.5 * (diss[:, :, :-1] + diss[:, :, 1:]) * water_mask[:, :, :-1])
    diss_w[:, :, -1] = diss[:, :, -1] * land_mask
    return diss_w


def isoneutral_diffusion(vs, settings, istemp, iso=True):
    """``isoneutral_diffusion_kernel`` (veros/core/isoneutral/diffusion.py:210-283).

    Returns a dict of the updated fields (``temp``/``salt``, ``dtemp_iso``/``dsalt_iso``
    and, when ``enable_conserve_energy``, ``P_diss_iso`` or ``P_diss_skew``).
    """
    tr = vs.temp if istemp else vs.salt
    dtracer_iso = vs.dtemp_iso if istemp else vs.dsalt_iso
    tr, dtracer_iso, flux_east, flux_north, flux_top = isoneutral_diffusion_tracer(
        vs, settings, tr, dtracer_iso, iso=iso, skew=not iso)
    out = {}
    if istemp:
        out.update(temp=tr, dtemp_iso=dtracer_iso)
    else:
        out.update(salt=tr, dsalt_iso=dtracer_iso)

    if _settings_get(settings, "enable_conserve_energy"):
        g, rho0 = _settings_get(settings, "grav"), _settings_get(settings, "rho_0")
        int_drhodX = (vs.int_drhodT if istemp else vs.int_drhodS)[:, :, :, vs.tau]
        diss = compute_dissipation(vs, settings, int_drhodX, flux_east, flux_north)
        diss_wgrid = dissipation_on_wgrid(vs, diss, vs.kbot)
        fxa = (-int_drhodX[2:-2, 2:-2, 1:] + int_drhodX[2:-2, 2:-2, :-1]) / vs.dzw[None, None, :-1]
        if not iso:
            P = vs.P_diss_skew + diss_wgrid
            P[2:-2, 2:-2, :-1] += -g / rho0 * fxa * flux_top[2:-2, 2:-2, :-1] * vs.maskW[2:-2, 2:-2, :-1]
            out["P_diss_skew"] = P
        else:
            P = vs.P_diss_iso + diss_wgrid
            P[2:-2, 2:-2, :-1] += -g / rho0 * fxa * (
                flux_top[2:-2, 2:-2, :-1] * vs.maskW[2:-2, 2:-2, :-1]
                + vs.K_33[2:-2, 2:-2, :-1] * (tr[2:-2, 2:-2, 1:, vs.taup1] - tr[2:-2, 2:-2, :-1, vs.taup1])
                / vs.dzw[None, None, :-1] * vs.maskW[2:-2, 2:-2, :-1])
            out["P_diss_iso"] = P
    return out


def isoneutral_step(vs, settings):
    """One isoneutral step of a rollout, in place on ``vs``.

    Mirrors the caller veros/core/thermodynamics.py:226-241 and :425-432 with
    zero advection tendencies, then the time-level rotation of
    veros/veros.py:321-322:

    1. ``tr[..., taup1] = tr[..., tau] * maskT`` for temp and salt
    2. zero ``dtemp_iso``, ``dsalt_iso`` (and ``P_diss_iso``)
    3. ``isoneutral_diffusion_pre``
    4. ``isoneutral_diffusion`` for temp, then for salt
    5. rotate ``(taum1, tau, taup1)``
    """
    vs.temp = vs.temp.copy()
    vs.salt = vs.salt.copy()
    vs.temp[..., vs.taup1] = vs.temp[..., vs.tau] * vs.maskT
    vs.salt[..., vs.taup1] = vs.salt[..., vs.tau] * vs.maskT
    vs.dtemp_iso = np.zeros_like(vs.dtemp_iso)
    vs.dsalt_iso = np.zeros_like(vs.dsalt_iso)
    vs.P_diss_iso = np.zeros_like(vs.P_diss_iso)
    vs.__dict__.update(isoneutral_diffusion_pre(vs, settings))
    vs.__dict__.update(isoneutral_diffusion(vs, settings, True))
    vs.__dict__.update(isoneutral_diffusion(vs, settings, False))
    vs.taum1, vs.tau, vs.taup1 = vs.tau, vs.taup1, vs.taum1


def enforce_boundaries(arr, enable_cyclic_x):
    """``enforce_boundaries`` (veros/core/utilities.py:7-16) on one process:
    with a cyclic x boundary the two halo columns on each side take the
    periodic interior columns; otherwise nothing changes."""
    arr = arr.copy()
    if enable_cyclic_x:
        arr[-2:, ...] = arr[2:4, ...]
        arr[:2, ...] = arr[-4:-2, ...]
    return arr


def vertmix_tempsalt(vs, settings):
    """``vertmix_tempsalt`` (veros/core/thermodynamics.py:248-300) on one
    process, including its closing boundary exchange of the new temp and salt
    levels (:292-298), which copies the periodic x halo when the setting
    ``enable_cyclic_x`` is on (absent: off).

    Returns a dict with ``temp``, ``salt``, ``dtemp_vmix``, ``dsalt_vmix``.
    """
    dt = _settings_get(settings, "dt_tracer")
    nz = vs.dzt.shape[0]
    tp1 = vs.taup1
    dtemp_vmix = vs.temp[:, :, :, tp1].copy()
    dsalt_vmix = vs.salt[:, :, :, tp1].copy()
    shape = vs.kappaH[2:-2, 2:-2].shape
    a_tri = np.zeros(shape)
    b_tri = np.zeros(shape)
    c_tri = np.zeros(shape)
    delta = np.zeros(shape)
    _, water_mask, edge_mask = create_water_masks(vs.kbot[2:-2, 2:-2], nz)
    delta[:, :, :-1] = dt / vs.dzw[None, None, :-1] * vs.kappaH[2:-2, 2:-2, :-1]
    delta[:, :, -1] = 0.0
    a_tri[:, :, 1:] = -delta[:, :, :-1] / vs.dzt[None, None, 1:]
    b_tri[:, :, 1:] = 1 + (delta[:, :, 1:] + delta[:, :, :-1]) / vs.dzt[None, None, 1:]
    b_tri_edge = 1 + delta / vs.dzt[None, None, :]
    c_tri[:, :, :-1] = -delta[:, :, :-1] / vs.dzt[None, None, :-1]
    temp = vs.temp.copy()
    salt = vs.salt.copy()
    for tr, forc in ((temp, vs.forc_temp_surface), (salt, vs.forc_salt_surface)):
        d_tri = tr[2:-2, 2:-2, :, tp1].copy()
        d_tri[:, :, -1] += dt * forc[2:-2, 2:-2] / vs.dzt[-1]
        sol = solve_implicit(a_tri, b_tri, c_tri, d_tri, water_mask, edge_mask, b_edge=b_tri_edge)
        tr[2:-2, 2:-2, :, tp1] = np.where(water_mask, sol, tr[2:-2, 2:-2, :, tp1])
    dtemp_vmix = (temp[:, :, :, tp1] - dtemp_vmix) / dt
    dsalt_vmix = (salt[:, :, :, tp1] - dsalt_vmix) / dt
    cyclic = bool(settings.get("enable_cyclic_x", False) if isinstance(settings, dict)
                  else getattr(settings, "enable_cyclic_x", False))
    temp[..., tp1] = enforce_boundaries(temp[..., tp1], cyclic)
    salt[..., tp1] = enforce_boundaries(salt[..., tp1], cyclic)
    return dict(temp=temp, salt=salt, dtemp_vmix=dtemp_vmix, dsalt_vmix=dsalt_vmix)


def isoneutral_diag_streamfunction(vs):
    """``isoneutral_diag_streamfunction_kernel`` (veros/core/isoneutral/isoneutral.py:232-254).

    Returns a dict with ``B1_gm`` and ``B2_gm``; cells outside the written
    ranges keep the values of ``vs``.
    """
    K_gm_pad = pad_z_edges(vs.K_gm)
    B1 = vs.B1_gm.copy()
    B2 = vs.B2_gm.copy()
    diffloc = 0.25 * (K_gm_pad[1:-2, 2:-2, 1:-1] + K_gm_pad[1:-2, 2:-2, :-2]
                      + K_gm_pad[2:-1, 2:-2, 1:-1] + K_gm_pad[2:-1, 2:-2, :-2])
    B2[1:-2, 2:-2, :] = 0.25 * diffloc * np.sum(vs.Ai_ez[1:-2, 2:-2, ...], axis=(3, 4))
    diffloc = 0.25 * (K_gm_pad[2:-2, 1:-2, 1:-1] + K_gm_pad[2:-2, 1:-2, :-2]
                      + K_gm_pad[2:-2, 2:-1, 1:-1] + K_gm_pad[2:-2, 2:-1, :-2])
    B1[2:-2, 1:-2, :] = -0.25 * diffloc * np.sum(vs.Ai_nz[2:-2, 1:-2, ...], axis=(3, 4))
    return dict(B1_gm=B1, B2_gm=B2)
