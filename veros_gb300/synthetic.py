"""Seeded synthetic ocean states for the isoneutral mixing path.

No dataset is involved: every workload here is generated from a seed. The
grid and topography follow Veros's own construction so that the fields look
exactly like those of a ``VerosState`` after ``numerics.calc_grid`` and
``numerics.calc_topo``:

* halo fill of ``dxt/dyt`` and the u-centred staggering of x, y and z
  (veros/core/numerics.py:8-22 and :24-89),
* degree to metre conversion and the spherical metric factors ``cost/cosu``
  (veros/core/numerics.py:65-73 and :122-133),
* the closed 2-cell rim of ``kbot`` and the T/U/V/W masks
  (veros/core/numerics.py:181-224).

Arrays use the reference's logical layout: 3-D fields are ``(X, Y, Z)`` with
``X = nx + 4`` and ``Y = ny + 4``, tracers carry a trailing time axis of 3
levels, and the ``Ai_*`` tensors a trailing ``(2, 2)`` axis pair. ``kbot``
counts from 1 at the bottom level (k = 0) and 0 marks a land column.
"""

from dataclasses import dataclass, field

import numpy as np

PI = 3.14159265358979323846264338327950588
RADIUS = 6370e3
DEGTOM = RADIUS / 180.0 * PI

# equation-of-state constants shared by eq types 1-4
# (veros/core/density/linear_eq.py:10-16, nonlinear_eq2.py:11-20)
_RHO0 = 1024.0
_THETA0 = 283.0 - 273.15
_BETA_T = 1.67e-4
_BETA_TS_EQ3 = 1e-5
_BETA_TS_EQ24 = 1e-5 / 2.0
_BETA_S = 0.78e-3
_GAMMAS = 1.1e-8
_GRAV = 9.81


DEFAULT_SETTINGS = dict(
    iso_slopec=1e-3,
    iso_dslope=1e-3,
    K_iso_steep=0.0,
    dt_tracer=43200.0,
    grav=9.81,
    rho_0=1024.0,
    eq_of_state_type=1,
    enable_conserve_energy=False,
    enable_skew_diffusion=False,
    enable_neutral_diffusion=True,
    K_iso_0=1000.0,
    K_gm_0=1000.0,
)


@dataclass
class HostState:
    """A reference-layout state held in NumPy arrays (float64, bool, int32)."""

    nx: int
    ny: int
    nz: int
    settings: dict
    arrays: dict
    tau: int = 1
    taup1: int = 2
    taum1: int = 0
    meta: dict = field(default_factory=dict)

    def __getattr__(self, name):
        arrays = self.__dict__.get("arrays")
        if arrays is not None and name in arrays:
            return arrays[name]
        raise AttributeError(name)

    def copy(self):
        return HostState(
            self.nx, self.ny, self.nz, dict(self.settings), {k: v.copy() for k, v in self.arrays.items()},
            self.tau, self.taup1, self.taum1, dict(self.meta),
        )


def u_centered_grid(dyt):
    """Staggered positions and u-spacings from t-spacings.

    Follows veros/core/numerics.py:8-22: ``yu`` is the running sum of the
    t-spacings, ``yt`` the alternating-sum reconstruction of the centres and
    ``dyu`` the centre-to-centre distance with a mirrored last entry.
    """
    n = dyt.shape[0]
    yu = np.zeros(n)
    yu[1:] = np.cumsum(dyt[1:])
    yt = np.zeros(n)
    yt[0] = yu[0] - dyt[0] * 0.5
    yt[1:] = 2 * yu[:-1]
    alt = np.ones(n)
    alt[::2] = -1
    yt = alt * np.cumsum(alt * yt)
    dyu = np.zeros(n)
    dyu[:-1] = yt[1:] - yt[:-1]
    dyu[-1] = 2 * dyt[-1] - dyu[-2]
    return dyu, yt, yu


def calc_grid(dxt, dyt, dzt, x_origin, y_origin, coord_degree=True):
    """Grid spacings and metric factors (veros/core/numerics.py:24-133, non-cyclic)."""
    dxt = dxt.astype(np.float64).copy()
    dyt = dyt.astype(np.float64).copy()
    dxt[-2:] = dxt[-3]
    dxt[:2] = dxt[2]
    dyt[-2:] = dyt[-3]
    dyt[:2] = dyt[2]

    dxu, xt, xu = u_centered_grid(dxt)
    xt = xt + x_origin - xu[2]
    xu = xu + x_origin - xu[2]
    dyu, yt, yu = u_centered_grid(dyt)
    yt = yt + y_origin - yu[2]
    yu = yu + y_origin - yu[2]

    if coord_degree:
        dxt = dxt * DEGTOM
        dxu = dxu * DEGTOM
        dyt = dyt * DEGTOM
        dyu = dyu * DEGTOM

    dzw, zt, zw = u_centered_grid(dzt.astype(np.float64))
    zt = zt - zw[-1]
    zw = zw - zw[-1]

    if coord_degree:
        cost = np.cos(yt * PI / 180.0)
        cosu = np.cos(yu * PI / 180.0)
    else:
        cost = np.ones_like(yt)
        cosu = np.ones_like(yu)

    return dict(dxt=dxt, dxu=dxu, xt=xt, xu=xu, dyt=dyt, dyu=dyu, yt=yt, yu=yu,
                dzt=dzt.astype(np.float64).copy(), dzw=dzw, zt=zt, zw=zw, cost=cost, cosu=cosu)


def calc_topo(kbot, nz):
    """Closed rim and T/U/V/W masks from ``kbot`` (veros/core/numerics.py:181-224, non-cyclic)."""
    kbot = kbot.astype(np.int32).copy()
    kbot[:, :2] = 0
    kbot[:, -2:] = 0
    kbot[:2, :] = 0
    kbot[-2:, :] = 0
    ks = np.arange(nz)[None, None, :]
    maskT = (kbot > 0)[..., None] & (kbot[..., None] - 1 <= ks)
    maskU = maskT.copy()
    maskU[:-1] = np.minimum(maskT[:-1], maskT[1:])
    maskV = maskT.copy()
    maskV[:, :-1] = np.minimum(maskT[:, :-1], maskT[:, 1:])
    maskW = maskT.copy()
    maskW[:, :, :-1] = np.minimum(maskT[:, :, :-1], maskT[:, :, 1:])
    return kbot, maskT, maskU, maskV, maskW


def geometric_dz(nz, dz_top, dz_bottom):
    """Layer thicknesses growing geometrically from the surface to the bottom.

    Index 0 is the bottom level (Veros counts k upward), so the array runs from
    ``dz_bottom`` at k = 0 to ``dz_top`` at k = nz - 1.
    """
    if nz == 1:
        return np.array([dz_top], dtype=np.float64)
    ratio = (dz_bottom / dz_top) ** (1.0 / (nz - 1))
    surface_down = dz_top * ratio ** np.arange(nz)
    return surface_down[::-1].copy()


def eos_int_drhodT(eq_type, temp, p):
    """``int_z^0 drho/dT`` used by the energy branch (veros/core/density/get_rho.py:136-155)."""
    zz = -p
    thetas = temp - _THETA0
    if eq_type == 1:
        return p * (-_BETA_T * _RHO0)
    if eq_type in (2, 4):
        return p * (-(_BETA_T + 2 * _BETA_TS_EQ24 * thetas) * _RHO0)
    if eq_type == 3:
        return _RHO0 * zz * (_BETA_T + _BETA_TS_EQ3 * thetas) - _RHO0 * _BETA_T * _GAMMAS * _GRAV * _RHO0 * zz**2 / 2
    raise ValueError(f"unsupported eq_of_state_type {eq_type}")


def eos_int_drhodS(eq_type, p):
    zz = -p
    if eq_type == 1:
        return p * (_BETA_S * _RHO0)
    if eq_type == 2:
        return p * (_BETA_S * _RHO0)
    if eq_type == 3:
        return -_BETA_S * _RHO0 * zz
    if eq_type == 4:
        return p * 0.0
    raise ValueError(f"unsupported eq_of_state_type {eq_type}")


def make_state(nx, ny, nz, *, seed=0, dx_deg=1.0, dy_deg=1.0, x_origin=0.0, y_origin=-60.0,
               dz_top=10.0, dz_bottom=400.0, land_fraction=0.15, eq_of_state_type=1,
               k_iso_lognormal_sigma=None, settings=None, stable_caps=False, lean=False):
    """Build one seeded synthetic state.

    * ``kbot``: each interior column is land with probability ``land_fraction``,
      otherwise ``kbot ~ U{1..nz}``; the 2-cell rim is closed.
    * ``temp = 2 + 20 exp(zt/800) + N(0, 0.1)``, ``salt = 35 + 0.5 exp(zt/500) + N(0, 0.01)``,
      identical on the three time levels and multiplied by ``maskT``.
    * ``K_iso``: constant ``K_iso_0``, or lognormal with median ``K_iso_0`` when
      ``k_iso_lognormal_sigma`` is given.
    * ``stable_caps``: rows whose zonal spacing is below the stability limit
      of the explicit horizontal diffusion, ``K_iso dt / dx^2 <= 1/4`` with
      ``dx = dxt cos(lat)``, are land (the polar caps of a global grid, where
      cos(lat) -> 0; the reference's own 1-degree setup stops at 79S/81N,
      veros/setups/global_1deg/global_1deg.py:29-36).
    * ``lean``: leave out the all-zero output fields and ``int_drhodT/S``
      (a device state allocates its outputs itself); for large ensembles.
    """
    rng = np.random.default_rng(seed)
    X, Y, Z = nx + 4, ny + 4, nz
    s = dict(DEFAULT_SETTINGS)
    s.update(eq_of_state_type=int(eq_of_state_type), nx=nx, ny=ny, nz=nz)
    if settings:
        s.update(settings)

    grid = calc_grid(np.full(X, dx_deg), np.full(Y, dy_deg), geometric_dz(nz, dz_top, dz_bottom), x_origin, y_origin)

    kb = np.zeros((X, Y), dtype=np.int32)
    land = rng.random((nx, ny)) < land_fraction
    depth = rng.integers(1, nz + 1, size=(nx, ny))
    kb[2:-2, 2:-2] = np.where(land, 0, depth)
    if stable_caps:
        dx_min = np.minimum(grid["dxt"].min() * np.abs(grid["cost"]), grid["dyt"].min())
        unstable = s["K_iso_0"] * s["dt_tracer"] / dx_min**2 > 0.25
        kb[:, unstable] = 0
    kbot, maskT, maskU, maskV, maskW = calc_topo(kb, nz)

    zt = grid["zt"]
    temp3 = (2.0 + 20.0 * np.exp(zt / 800.0))[None, None, :] + rng.normal(0.0, 0.1, size=(X, Y, Z))
    salt3 = (35.0 + 0.5 * np.exp(zt / 500.0))[None, None, :] + rng.normal(0.0, 0.01, size=(X, Y, Z))
    temp3 = temp3 * maskT
    salt3 = salt3 * maskT
    temp = np.repeat(temp3[..., None], 3, axis=-1)
    salt = np.repeat(salt3[..., None], 3, axis=-1)

    if k_iso_lognormal_sigma is None:
        K_iso = np.full((X, Y, Z), s["K_iso_0"])
    else:
        K_iso = s["K_iso_0"] * np.exp(rng.normal(0.0, k_iso_lognormal_sigma, size=(X, Y, Z)))
    K_gm = np.full((X, Y, Z), s["K_gm_0"])

    meta = dict(seed=seed, land_fraction_realised=float(1.0 - (kbot[2:-2, 2:-2] > 0).mean()))
    if lean:
        arrays = dict(grid)
        arrays.update(kbot=kbot, maskT=maskT, maskU=maskU, maskV=maskV, maskW=maskW, temp=temp, salt=salt,
                      K_iso=K_iso, K_gm=K_gm)
        return HostState(nx, ny, nz, s, arrays, meta=meta)

    p = np.abs(zt)[None, None, :, None]
    int_drhodT = eos_int_drhodT(s["eq_of_state_type"], temp, p) * np.ones_like(temp)
    int_drhodS = eos_int_drhodS(s["eq_of_state_type"], p) * np.ones_like(salt)

    z3 = lambda: np.zeros((X, Y, Z))  # noqa: E731
    # inputs of the neighbouring vertical mixing: a vertical diffusivity of
    # 1e-4..1e-3 m^2/s on W points and small surface fluxes
    kappaH = 1e-4 * (1.0 + 9.0 * rng.random((X, Y, Z))) * maskW
    forc_temp_surface = 1e-5 * rng.standard_normal((X, Y))
    forc_salt_surface = 1e-6 * rng.standard_normal((X, Y))
    arrays = dict(grid)
    arrays.update(
        kbot=kbot, maskT=maskT, maskU=maskU, maskV=maskV, maskW=maskW,
        temp=temp, salt=salt, K_iso=K_iso, K_gm=K_gm,
        int_drhodT=int_drhodT, int_drhodS=int_drhodS,
        K_11=z3(), K_22=z3(), K_33=z3(),
        Ai_ez=np.zeros((X, Y, Z, 2, 2)), Ai_nz=np.zeros((X, Y, Z, 2, 2)),
        Ai_bx=np.zeros((X, Y, Z, 2, 2)), Ai_by=np.zeros((X, Y, Z, 2, 2)),
        dtemp_iso=z3(), dsalt_iso=z3(), P_diss_iso=z3(), P_diss_skew=z3(),
        kappaH=kappaH, forc_temp_surface=forc_temp_surface, forc_salt_surface=forc_salt_surface,
        dtemp_vmix=z3(), dsalt_vmix=z3(), B1_gm=z3(), B2_gm=z3(),
    )
    return HostState(nx, ny, nz, s, arrays, meta=meta)


# Workloads named by what they are. Sizes are interior cells; 2 halo cells per
# side are added in x and y.
def small_linear_state(seed=0):
    """64 x 48 x 20, 1 degree from 60S, dz 10-400 m, ~15% land, linear EOS."""
    return make_state(64, 48, 20, seed=seed, y_origin=-60.0, dz_top=10.0, dz_bottom=400.0,
                      land_fraction=0.15, eq_of_state_type=1)


def global_1deg_state(seed=0, nz=60, k_iso_lognormal_sigma=None):
    """360 x 180 x nz at 1 degree, -90..90, dz 10-250 m, ~30% land plus polar caps beyond 83 deg, nonlinear EOS."""
    return make_state(360, 180, nz, seed=seed, dx_deg=1.0, dy_deg=1.0, y_origin=-90.0, dz_top=10.0,
                      dz_bottom=250.0, land_fraction=0.30, eq_of_state_type=3,
                      k_iso_lognormal_sigma=k_iso_lognormal_sigma, stable_caps=True)


def global_quarter_deg_state(seed=0, lean=False):
    """1440 x 720 x 60 at 0.25 degree, -90..90, dz 10-250 m, ~30% land plus polar caps beyond 62 deg, nonlinear EOS."""
    return make_state(1440, 720, 60, seed=seed, dx_deg=0.25, dy_deg=0.25, y_origin=-90.0, dz_top=10.0,
                      dz_bottom=250.0, land_fraction=0.30, eq_of_state_type=3, stable_caps=True, lean=lean)


def ensemble_states(n=48, seed0=0, lean=True):
    """Ensemble members: nx ~ U{32..512}, ny ~ U{32..256}, nz from {15, 30, 45, 60},
    each with its own seed; kbot and tracers as in the small linear state
    (1 degree in x from 60S, dy = min(1, 120/ny) degrees, linear EOS)."""
    rng = np.random.default_rng(1234 + seed0)
    members = []
    for m in range(n):
        nx = int(rng.integers(32, 513))
        ny = int(rng.integers(32, 257))
        nz = int(rng.choice([15, 30, 45, 60]))
        dy = min(1.0, 120.0 / ny)  # every member stays within 60S..60N
        members.append(make_state(nx, ny, nz, seed=seed0 + m, dy_deg=dy, y_origin=-60.0, dz_top=10.0,
                                  dz_bottom=400.0, land_fraction=0.15, eq_of_state_type=1, lean=lean))
    return members
