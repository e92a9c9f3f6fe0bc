// Adjoint of one FP64 isoneutral step (the step of vg_isoneutral_step_f64:
// veros/core/thermodynamics.py:226-241 with zero advection, then
// isoneutral_diffusion_pre and isoneutral_diffusion of temp and salt,
// veros/core/isoneutral/isoneutral.py:18-229 and diffusion.py:9-283).
//
// Given dL/dT_{n+1} and dL/dS_{n+1} it returns dL/dT_n and dL/dS_n and adds
// dL/dK_iso. The step's inputs T_n, S_n and outputs T_{n+1}, S_{n+1} are the
// caller's checkpoints; the diffusion tensor is recomputed from them.
//
// Per-slope formulation: every slope of the tensor is attached to a T point
// P, one of its horizontal faces h (east, west, north, south) and one of its
// vertical faces v (below, above),
//   s = -(drdT(P) dT/dh + drdS(P) dS/dh) / (min(0, drdT(P) dT/dz(v) + drdS(P) dS/dz(v)) - epsln),
// and enters two terms of the forward with the same value: the term of face h
// (Ai_ez / Ai_nz, K_11 / K_22; isoneutral.py:100-168) and the term of face v
// (Ai_bx / Ai_by, K_33; :173-224). The adjoint visits each of the eight
// slopes of a point once.
//
// Launches (one stream, in order):
//   1. adj_tables_kernel     reciprocal grid factors
//   2. pre_span_kernel       the step's tensor K_11, K_22, K_33 (the forward kernel), and
//                            per point its 8 tapers, 8 slopes and 2 clamped reciprocals
//   3. adj_implicit_kernel   per water column: the transposed tridiagonal
//                            system A^T y = dL/dx (temp and salt on two
//                            threads sharing the Thomas factorisation, columns
//                            deepest first) and dL/dK_33 from
//                            dL/ddelta_k = (x_{k+1} - x_k)(y_k/dzt_k - y_{k+1}/dzt_{k+1})
//   4. adj_active_kernel     per point whether its faces carry a term (an
//                            activity map); the points that do, listed
//      adj_slope_kernel      per listed point: the eight slope adjoints (from the
//                            stored tapers and slopes), written as per-point
//                            partial sums onto the point's faces
//   5. adj_gather_kernel     per point: sums the partials of the faces around
//                            it (those of active points; the others are zero)
//                            into dL/dT_n, dL/dS_n and dL/dK_iso
//
// Every partial is written exactly once by the point that owns it and read
// by its neighbours in the next launch: no atomics, results are deterministic.
#include <algorithm>
#include <climits>

#include "common.cuh"
#include "pre_kernels.cuh"

namespace vg {
namespace adj {

using detail::kEpsln;

// reciprocal grid tables (scratch tail)
struct GridInv {
  const double *inv_dxu, *inv_dxt, *qinv_dxt;                // X
  const double *inv_dyu, *inv_dyt, *inv_cost, *qinv_dyt_cost;  // Y
  const double *inv_dzw, *inv_dzt, *qinv_dzt;                 // Z
};

constexpr int kTensorFields = 19;  // K_11, K_22, K_33, 4 x 4 Ai components
enum { F_GTP = kTensorFields, F_GSP, F_GK33, F_PART };
// partial sums written by the slope pass, one field each
// per point: LRT the adjoint of drho/dT; WT/WS (per horizontal face h) the
// face's tracer-difference adjoint from this point's slopes and fluxes, scaled
// by the face's masked metric factor where it multiplies a gradient; GZT/GZS
// (per vertical face v) likewise for the vertical gradients; LVD (tracer, v)
// the vertical differences of the fluxes; LDL (h) diffloc; LKW (v) K_iso at
// the vertical faces
enum { P_LRT = 0, P_WT = 1, P_WS = 5, P_GZT = 9, P_GZS = 11, P_LVD = 13, P_LDL = 17, P_LKW = 21, P_N = 23 };
// the forward's per-point tapers, slopes and reciprocals (detail::SLOPE_*)
constexpr int F_SLOPES = F_PART + P_N;
// mu = dt dL/dT_p on interior wet cells, scaled per direction: mu / (cost dxt),
// mu / (cost dyt), mu / dzt for temp (0..2) and salt (3..5)
constexpr int F_NU = F_SLOPES + detail::SLOPE_FIELDS;
constexpr int kFields = F_NU + 6;

inline size_t table_doubles(const Layout &L) { return 3 * (size_t)L.X + 4 * (size_t)L.Y + 3 * (size_t)L.Z; }

inline size_t field_doubles(const Layout &L) { return (size_t)L.plane * L.Z; }

// doubles before the active-point list (fields, then the grid tables)
inline size_t list_offset(const Layout &L) { return (size_t)kFields * field_doubles(L) + table_doubles(L); }

// fields, tables, then the active-point list (one int32 per point) and its
// count, then one activity byte per point
inline size_t scratch_bytes(const Layout &L) {
  size_t n = list_offset(L) * sizeof(double) + (field_doubles(L) + 1) * sizeof(int32_t) + field_doubles(L);
  return (n + 255) & ~(size_t)255;
}

GridInv tables_of(const Layout &L, const double *t) {
  GridInv g;
  g.inv_dxu = t;
  g.inv_dxt = t + L.X;
  g.qinv_dxt = t + 2 * L.X;
  const double *ty = t + 3 * L.X;
  g.inv_dyu = ty;
  g.inv_dyt = ty + L.Y;
  g.inv_cost = ty + 2 * L.Y;
  g.qinv_dyt_cost = ty + 3 * L.Y;
  const double *tz = ty + 4 * L.Y;
  g.inv_dzw = tz;
  g.inv_dzt = tz + L.Z;
  g.qinv_dzt = tz + 2 * L.Z;
  return g;
}

__global__ void adj_tables_kernel(Layout L, Grid g, double *t) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  const int X = L.X, Y = L.Y, Z = L.Z;
  if (n < X) {
    t[n] = 1.0 / g.dxu[n];
    t[X + n] = 1.0 / g.dxt[n];
    t[2 * X + n] = 1.0 / (4.0 * g.dxt[n]);
  }
  double *ty = t + 3 * X;
  if (n < Y) {
    ty[n] = 1.0 / g.dyu[n];
    ty[Y + n] = 1.0 / g.dyt[n];
    ty[2 * Y + n] = 1.0 / g.cost[n];
    ty[3 * Y + n] = 1.0 / (4.0 * g.dyt[n] * g.cost[n]);
  }
  double *tz = ty + 4 * Y;
  if (n < Z) {
    tz[n] = 1.0 / g.dzw[n];
    tz[Z + n] = 1.0 / g.dzt[n];
    tz[2 * Z + n] = 1.0 / (4.0 * g.dzt[n]);
  }
}

// d(drho/dT)/dT (veros/core/density/get_rho.py:93-111)
__device__ __forceinline__ double drdT_dT(int eos) {
  if (eos == 1) return 0.0;
  if (eos == 3) return -Eos::betaTs3 * Eos::rho0;
  return -2.0 * Eos::betaTs24 * Eos::rho0;
}

// ---------------------------------------------------------------------------
// 3. implicit part (diffusion.py:142-169)
// ---------------------------------------------------------------------------
struct ImpArgs {
  Layout L;
  GridInv gi;
  double dt;
  const int32_t *__restrict__ kbot;
  const double *__restrict__ K33;
  const double *__restrict__ xT;  // T_{n+1}: the solution of the forward solve
  const double *__restrict__ xS;
  const double *__restrict__ gTn;  // dL/dT_{n+1}
  const double *__restrict__ gSn;
  double *gTp, *gSp, *gK33;  // dL/d(right-hand side), dL/dK_33
  double *nu;                // the scaled adjoint sources of the explicit part (F_NU)
  long long field;
  const int32_t *__restrict__ col_order;  // interior columns, deepest first (optional)
};

// Row k of the forward matrix: a_k = -delta_{k-1}/dzt_k, c_k = -delta_k/dzt_k,
// b_k = 1 + (delta_k + delta_{k-1})/dzt_k (no delta_{k-1} on the bottom row
// ks), delta_k = dt K_33/dzw_k (0 on the top level). The transposed system
// has sub-diagonal c_{k-1} and super-diagonal a_{k+1}; A is row diagonally
// dominant, so A^T is column diagonally dominant and needs no pivoting.
// Temp and salt of a column on two neighbouring threads (lane 2c: temp,
// 2c+1: salt), which both form the shared factorisation; the lane of temp
// stores c'_k, each lane its own d'_k, so a CTA holds 1.5 Z doubles per
// thread in shared memory and twice the warps hide the recurrence.
__global__ void __launch_bounds__(128) adj_implicit_kernel(ImpArgs a) {
  extern __shared__ double smem[];
  const Layout &L = a.L;
  const int Z = L.Z, nb = blockDim.x, nc = nb / 2, t = threadIdx.x, c = t >> 1, r = t & 1;
  const unsigned pair = 3u << ((t & 31) & ~1);
  double *cps = smem;                   // [k][column]
  double *dps = smem + (size_t)Z * nc;  // [k][thread]
  // slots: the interior columns (in col_order: the lanes of a warp then walk
  // columns of similar depth), then the two-column rim
  const int slot = blockIdx.x * nc + c;
  if (slot >= L.X * L.Y) return;
  const int nx = L.X - 4, nint = nx * (L.Y - 4);
  int i, j;
  if (slot < nint) {
    const int col = a.col_order ? __ldg(a.col_order + slot) : slot;
    i = 2 + col % nx;
    j = 2 + col / nx;
  } else if (slot - nint < 4 * L.X) {
    const int q = slot - nint, jr = q / L.X;
    i = q % L.X;
    j = jr < 2 ? jr : L.Y - 4 + jr;
  } else {
    const int q = slot - nint - 4 * L.X, cc = q % 4;
    i = cc < 2 ? cc : L.X - 4 + cc;
    j = 2 + q / 4;
  }
  const long long base = L.at2(i, j);
  const bool interior = i >= 2 && i < L.X - 2 && j >= 2 && j < L.Y - 2;
  const int ks = interior ? a.kbot[base] - 1 : -1;  // create_water_masks (utilities.py:38-48)
  const int kw = (ks >= 0 && ks < Z) ? ks : Z;
  const long long F = a.field;
  const double *gn = r ? a.gSn : a.gTn;  // this lane's tracer
  const double *xn = r ? a.xS : a.xT;
  double *gp = r ? a.gSp : a.gTp;
  double *nu = a.nu + 3 * r * F;
  // cells outside the solve pass their adjoint through; dry or halo cells have no explicit part
  for (int k = 0; k < kw; ++k) {
    const long long o = base + (long long)k * L.plane;
    gp[o] = gn[o];
    if (r == 0) a.gK33[o] = 0.0;
#pragma unroll
    for (int n = 0; n < 3; ++n) nu[n * F + o] = 0.0;
  }
  if (kw == Z) return;
  // the explicit tendency's metric factors (diffusion.py:116-139)
  const double fx = a.dt * a.gi.inv_dxt[i] * a.gi.inv_cost[j], fy = a.dt * a.gi.inv_dyt[j] * a.gi.inv_cost[j];

  double cp = 0.0, dp = 0.0, delta_prev = 0.0;
  for (int k = ks; k < Z; ++k) {
    const long long o = base + (long long)k * L.plane;
    const double delta = k < Z - 1 ? a.dt * a.gi.inv_dzw[k] * a.K33[o] : 0.0;
    const double b = 1.0 + (delta + (k > ks ? delta_prev : 0.0)) * a.gi.inv_dzt[k];
    const double sub = k > ks ? -delta_prev * a.gi.inv_dzt[k - 1] : 0.0;
    const double sup = k < Z - 1 ? -delta * a.gi.inv_dzt[k + 1] : 0.0;
    const double inv = 1.0 / (b - sub * cp);
    cp = sup * inv;
    dp = (gn[o] - sub * dp) * inv;
    if (r == 0) cps[(size_t)k * nc + c] = cp;
    dps[(size_t)k * nb + t] = dp;
    delta_prev = delta;
  }
  __syncwarp(pair);  // c'_k of the temp lane is visible to the salt lane
  double y = 0.0, xu = 0.0;  // values one level up
  for (int k = Z - 1; k >= ks; --k) {
    const long long o = base + (long long)k * L.plane;
    const double n = dps[(size_t)k * nb + t] - cps[(size_t)k * nc + c] * y;
    const double x = xn[o];
    // dL/ddelta_k = sum over the tracers of (x_{k+1} - x_k)(y_k/dzt_k - y_{k+1}/dzt_{k+1})
    const double part = k < Z - 1 ? (xu - x) * (n * a.gi.inv_dzt[k] - y * a.gi.inv_dzt[k + 1]) : 0.0;
    const double other = __shfl_xor_sync(pair, part, 1);
    if (r == 0) a.gK33[o] = k < Z - 1 ? (part + other) * a.dt * a.gi.inv_dzw[k] : 0.0;
    gp[o] = n;
    nu[o] = n * fx;
    nu[F + o] = n * fy;
    nu[2 * F + o] = n * (a.dt * a.gi.inv_dzt[k]);
    y = n;
    xu = x;
  }
}

// ---------------------------------------------------------------------------
// 4. slope adjoints
// ---------------------------------------------------------------------------
struct SlopeArgs {
  Layout L;
  Grid g;
  GridInv gi;
  int eos;
  double slopec, inv_dslope, ksteep;
  const double *__restrict__ T;
  const double *__restrict__ S;
  const double *__restrict__ K;
  const double *__restrict__ gK33;
  const uint8_t *__restrict__ m;
  const double *__restrict__ slopes;  // the forward's tapers, slopes and reciprocals
  const double *__restrict__ nu;      // the scaled adjoint sources of the explicit part
  const double *__restrict__ K11;     // the forward's tensor
  const double *__restrict__ K22;
  double *part;
  long long field;
};

// Which faces of point (i, j, k) carry a term of the forward: face h (the
// east/north terms, vE) and face v (the top terms, vT), from the masks and
// the position alone. A point with none has all its partial sums zero.
struct SlopeFaces {
  bool mH[4], mWv[2], vE[4], vT[2];
  __device__ __forceinline__ bool any() const { return vE[0] || vE[1] || vE[2] || vE[3] || vT[0] || vT[1]; }
};

__device__ __forceinline__ SlopeFaces slope_faces(const Layout &L, const uint8_t *m, int i, int j, int k) {
  const int X = L.X, Y = L.Y, Z = L.Z;
  const long long o = L.at(i, j, k), PW = L.pitch, PL = L.plane;
  const unsigned mk = __ldg(m + o);
  const bool hasE = i < X - 1, hasW = i > 0, hasN = j < Y - 1, hasS = j > 0, hasU = k < Z - 1, hasD = k > 0;
  const bool inter = i >= 2 && i < X - 2 && j >= 2 && j < Y - 2;
  const bool rowE = j >= 2 && j < Y - 2, colN = i >= 2 && i < X - 2;
  SlopeFaces f;
  f.mH[0] = hasE && (mk & VG_MASK_U);
  f.mH[1] = hasW && (__ldg(m + o - 1) & VG_MASK_U);
  f.mH[2] = hasN && (mk & VG_MASK_V);
  f.mH[3] = hasS && (__ldg(m + o - PW) & VG_MASK_V);
  f.mWv[0] = hasD && (__ldg(m + o - PL) & VG_MASK_W);
  f.mWv[1] = hasU && (mk & VG_MASK_W);
  f.vE[0] = rowE && i >= 1 && i < X - 2 && f.mH[0];
  f.vE[1] = rowE && i >= 2 && i < X - 1 && f.mH[1];
  f.vE[2] = colN && j >= 1 && j < Y - 2 && f.mH[2];
  f.vE[3] = colN && j >= 2 && j < Y - 1 && f.mH[3];
  f.vT[0] = inter && f.mWv[0];
  f.vT[1] = inter && f.mWv[1];
  return f;
}

// The slope adjoints of one point whose faces carry a term
__device__ __forceinline__ void adj_slope_point(const SlopeArgs &a, const SlopeFaces &sf, int i, int j, int k) {
  const Layout &L = a.L;
  const int X = L.X, Y = L.Y, Z = L.Z;
  const long long o = L.at(i, j, k), PW = L.pitch, PL = L.plane;
  const GridInv &gi = a.gi;
  const uint8_t *m = a.m;
  const unsigned mk = __ldg(m + o);
  const bool hasE = i < X - 1, hasW = i > 0, hasN = j < Y - 1, hasS = j > 0, hasU = k < Z - 1, hasD = k > 0;
  const bool inter = i >= 2 && i < X - 2 && j >= 2 && j < Y - 2;
  const double Tc = __ldg(a.T + o), Sc = __ldg(a.S + o);
  const long long F = a.field;
  // tracer differences across the faces (unmasked) and the face masks
  double hdT[4], hdS[4], vdT[2], vdS[2];
  hdT[0] = hasE ? __ldg(a.T + o + 1) - Tc : 0.0;
  hdS[0] = hasE ? __ldg(a.S + o + 1) - Sc : 0.0;
  hdT[1] = hasW ? Tc - __ldg(a.T + o - 1) : 0.0;
  hdS[1] = hasW ? Sc - __ldg(a.S + o - 1) : 0.0;
  hdT[2] = hasN ? __ldg(a.T + o + PW) - Tc : 0.0;
  hdS[2] = hasN ? __ldg(a.S + o + PW) - Sc : 0.0;
  hdT[3] = hasS ? Tc - __ldg(a.T + o - PW) : 0.0;
  hdS[3] = hasS ? Sc - __ldg(a.S + o - PW) : 0.0;
  vdT[0] = hasD ? Tc - __ldg(a.T + o - PL) : 0.0;
  vdS[0] = hasD ? Sc - __ldg(a.S + o - PL) : 0.0;
  vdT[1] = hasU ? __ldg(a.T + o + PL) - Tc : 0.0;
  vdS[1] = hasU ? __ldg(a.S + o + PL) - Sc : 0.0;
  const bool *mH = sf.mH, *mWv = sf.mWv;

  // masked metric factors of the face gradients and the temperature gradients (isoneutral.py:46-95)
  const double icx = gi.inv_cost[j];
  const double fx[4] = {mH[0] ? gi.inv_dxu[i] * icx : 0.0, mH[1] ? gi.inv_dxu[i - 1] * icx : 0.0,
                        mH[2] ? gi.inv_dyu[j] : 0.0, mH[3] ? gi.inv_dyu[j - 1] : 0.0};
  const double fz[2] = {mWv[0] ? gi.inv_dzw[k - 1] : 0.0, mWv[1] ? gi.inv_dzw[k] : 0.0};
  double gxT[4], gzT[2];
#pragma unroll
  for (int h = 0; h < 4; ++h) gxT[h] = hdT[h] * fx[h];
  gzT[0] = vdT[0] * fz[0];
  gzT[1] = vdT[1] * fz[1];
  const bool wetP = mk & VG_MASK_T;
  const Eos eos{a.eos};
  const double rT = wetP ? eos.drdT(Tc, a.g.zt[k]) : 0.0, rS = wetP ? eos.drdS() : 0.0;
  // the clamped reciprocals 1/(min(0, G) - epsln) of the forward; G >= 0 gives exactly R_flat
  const long long R_flat_bits = __double_as_longlong(detail::recip_neg(fmin0(0.0) - kEpsln));
  const double c2 = -2.0 * a.inv_dslope;
  const double R[2] = {__ldg(a.slopes + o + detail::SLOPE_R * F), __ldg(a.slopes + o + (detail::SLOPE_R + 1) * F)};

  // which faces carry a term: face h (east/north terms) and face v (top terms)
  const bool *vE = sf.vE, *vT = sf.vT;

  // adjoints of the fluxes on the faces (diffusion.py:116-139) from the
  // scaled sources nu: lambda_fe(i) = nu_x(i) - nu_x(i+1), and so on
  double lfT[4] = {0, 0, 0, 0}, lfS[4] = {0, 0, 0, 0}, lftT[2] = {0, 0}, lftS[2] = {0, 0};
  {
    const double *nu = a.nu + o;
    auto nT = [&](int n, long long off) { return __ldg(nu + n * F + off); };
    if (vE[0]) {
      lfT[0] = nT(0, 0) - nT(0, 1);
      lfS[0] = nT(3, 0) - nT(3, 1);
    }
    if (vE[1]) {
      lfT[1] = nT(0, -1) - nT(0, 0);
      lfS[1] = nT(3, -1) - nT(3, 0);
    }
    if (vE[2]) {
      lfT[2] = a.g.cosu[j] * (nT(1, 0) - nT(1, PW));
      lfS[2] = a.g.cosu[j] * (nT(4, 0) - nT(4, PW));
    }
    if (vE[3]) {
      lfT[3] = a.g.cosu[j - 1] * (nT(1, -PW) - nT(1, 0));
      lfS[3] = a.g.cosu[j - 1] * (nT(4, -PW) - nT(4, 0));
    }
    if (vT[0]) {
      lftT[0] = nT(2, -PL) - nT(2, 0);
      lftS[0] = nT(5, -PL) - nT(5, 0);
    }
    if (vT[1]) {
      lftT[1] = nT(2, 0) - nT(2, PL);
      lftS[1] = nT(5, 0) - nT(5, PL);
    }
  }

  // face-level factors of the two terms
  double dl[4] = {0, 0, 0, 0}, gKh[4] = {0, 0, 0, 0}, c[4] = {0, 0, 0, 0}, cp[4] = {0, 0, 0, 0};
  {
    const double *K = a.K;
    // diffloc of the face, isoneutral.py:101-104 and :138-141 (k = 0: :104)
    auto dl_of = [&](long long ow, long long off) {
      return hasD ? 0.25 * (__ldg(K + ow) + __ldg(K + ow - PL) + __ldg(K + ow + off) + __ldg(K + ow + off - PL))
                  : 0.5 * (__ldg(K + ow) + __ldg(K + ow + off));
    };
    if (vE[0]) {
      dl[0] = dl_of(o, 1);
      gKh[0] = (lfT[0] * hdT[0] + lfS[0] * hdS[0]) * (gi.inv_dxu[i] * icx);
    }
    if (vE[1]) {
      dl[1] = dl_of(o - 1, 1);
      gKh[1] = (lfT[1] * hdT[1] + lfS[1] * hdS[1]) * (gi.inv_dxu[i - 1] * icx);
    }
    if (vE[2]) {
      dl[2] = dl_of(o, PW);
      gKh[2] = (lfT[2] * hdT[2] + lfS[2] * hdS[2]) * gi.inv_dyu[j];
    }
    if (vE[3]) {
      dl[3] = dl_of(o - PW, PW);
      gKh[3] = (lfT[3] * hdT[3] + lfS[3] * hdS[3]) * gi.inv_dyu[j - 1];
    }
    if (inter) {
      c[0] = a.g.dxu[i] * gi.qinv_dxt[i];
      c[1] = a.g.dxu[i - 1] * gi.qinv_dxt[i];
      cp[0] = cp[1] = icx * gi.qinv_dxt[i];
      c[2] = a.g.cosu[j] * a.g.dyu[j] * gi.qinv_dyt_cost[j];
      c[3] = a.g.cosu[j - 1] * a.g.dyu[j - 1] * gi.qinv_dyt_cost[j];
      cp[2] = a.g.cosu[j] * gi.qinv_dyt_cost[j];
      cp[3] = a.g.cosu[j - 1] * gi.qinv_dyt_cost[j];
    }
  }
  const double KW[2] = {vT[0] ? __ldg(a.K + o - PL) : 0.0, vT[1] ? __ldg(a.K + o) : 0.0};
  const double gK33W[2] = {vT[0] ? __ldg(a.gK33 + o - PL) : 0.0, vT[1] ? __ldg(a.gK33 + o) : 0.0};
  const double dzwv[2] = {hasD ? a.g.dzw[k - 1] : 0.0, a.g.dzw[k]};
  const double q = gi.qinv_dzt[k];

  double lrT = 0.0, nsum[4] = {0, 0, 0, 0}, lG[2] = {0, 0}, lvd[2][2] = {{0, 0}, {0, 0}};
  double lhd[2][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}}, ldl[4] = {0, 0, 0, 0}, lKw[2] = {0, 0};
#pragma unroll
  for (int h = 0; h < 4; ++h) {
#pragma unroll
    for (int v = 0; v < 2; ++v) {
      const bool Ef = vE[h] && (v == 1 || hasD);
      const bool Tf = vT[v];
      if (!Ef && !Tf) continue;
      const double s = __ldg(a.slopes + o + (detail::SLOPE_S + h * 2 + v) * F);
      const double t = __ldg(a.slopes + o + (detail::SLOPE_T + h * 2 + v) * F);
      // d taper / ds = -2 sign(s) t (1 - t) / dslope (0 at s = 0); the sign by integer operations
      const long long sb = __double_as_longlong(s);
      const double tq = t * (1.0 - t) * c2;
      const double tp = (sb & 0x7FFFFFFFFFFFFFFFLL) ? __longlong_as_double(__double_as_longlong(tq) ^
                                                                            (sb & (long long)0x8000000000000000ULL))
                                                    : 0.0;
      const double tst = t + s * tp;                              // d (taper s) / ds
      const double ts = t * s;
      double gs = 0.0;
      if (Ef) {
        // Ai = taper s, K_11 += dzw max(K_iso_steep, diffloc taper) / (4 dzt)
        const double lfv = lfT[h] * vdT[v] + lfS[h] * vdS[v];
        const double dlq = dl[h] * q;
        const double kq = dgt(dl[h] * t, a.ksteep) ? gKh[h] * dzwv[v] * q : 0.0;
        gs += lfv * dlq * tst + kq * dl[h] * tp;
        ldl[h] += kq * t + lfv * ts * q;
        lvd[0][v] += lfT[h] * ts * dlq;
        lvd[1][v] += lfS[h] * ts * dlq;
      }
      if (Tf) {
        // Ai_b = taper s, K_33 += c K_iso taper s^2
        const double lfh = lftT[v] * hdT[h] + lftS[v] * hdS[h];
        const double kc = gK33W[v] * c[h];
        gs += lfh * KW[v] * cp[h] * tst + kc * KW[v] * (tp * s * s + 2.0 * ts);
        lKw[v] += kc * ts * s + lfh * ts * cp[h];
        const double f = KW[v] * ts * cp[h];
        lhd[0][h] += lftT[v] * f;
        lhd[1][h] += lftS[v] * f;
      }
      const double lN = -gs * R[v];
      if (__double_as_longlong(R[v]) != R_flat_bits) lG[v] -= gs * s * R[v];  // d min(0, G)/dG = 1 where G < 0
      lrT += lN * gxT[h];
      nsum[h] += lN;
    }
  }
  lrT += lG[0] * gzT[0] + lG[1] * gzT[1];
  // the K_11 / K_22 terms of the east and north fluxes (diffusion.py:31-33, :57-60), added
  // once per face by the point west / south of it
  if (vE[0]) {
    const double k11 = __ldg(a.K11 + o) * (gi.inv_dxu[i] * icx);
    lhd[0][0] += lfT[0] * k11;
    lhd[1][0] += lfS[0] * k11;
  }
  if (vE[2]) {
    const double k22 = __ldg(a.K22 + o) * gi.inv_dyu[j];
    lhd[0][2] += lfT[2] * k22;
    lhd[1][2] += lfS[2] * k22;
  }

  double *p = a.part + o;
  p[P_LRT * F] = lrT;
#pragma unroll
  for (int h = 0; h < 4; ++h) {
    p[(P_WT + h) * F] = nsum[h] * rT * fx[h] + lhd[0][h];
    p[(P_WS + h) * F] = nsum[h] * rS * fx[h] + lhd[1][h];
    p[(P_LDL + h) * F] = ldl[h];
  }
#pragma unroll
  for (int v = 0; v < 2; ++v) {
    p[(P_GZT + v) * F] = lG[v] * rT * fz[v];
    p[(P_GZS + v) * F] = lG[v] * rS * fz[v];
    p[(P_LVD + v) * F] = lvd[0][v];
    p[(P_LVD + 2 + v) * F] = lvd[1][v];
    p[(P_LKW + v) * F] = lKw[v];
  }
}

// Active-point list: a point whose faces carry no term has all its partial
// sums zero; it is marked so in the activity map (which the gather reads
// instead of its partials) and the others are appended to the list (one
// atomic per warp, the lanes of a warp in x order), so that the slope pass
// runs whole warps of points with terms: an FP64 warp instruction costs the
// same however few of its lanes are active, and most points of a warp row are
// dry on most levels. Block (32, 4): a warp is one x row.
__global__ void __launch_bounds__(128) adj_active_kernel(Layout L, const uint8_t *__restrict__ m, uint8_t *active,
                                                         int32_t *list, int *count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  const bool in = i < L.X && j < L.Y;
  const bool act = in && slope_faces(L, m, i, j, k).any();
  const long long o = in ? L.at(i, j, k) : 0;
  if (in) active[o] = act ? 1 : 0;
  const unsigned ball = __ballot_sync(0xffffffffu, act);
  if (!ball) return;
  const int lane = threadIdx.x & 31, leader = __ffs(ball) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(count, __popc(ball));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (act) list[base + __popc(ball & ((1u << lane) - 1u))] = (int32_t)o;
}

// The slope pass over the active list: persistent threads, grid-stride.
// Three CTAs per SM: 168 registers (14.8 against 15.0 ms for the 8-step
// backward at 360 x 180 x 30 with the unbounded 184).
__global__ void __launch_bounds__(128, 3) adj_slope_kernel(SlopeArgs a, const int32_t *__restrict__ list,
                                                        const int *__restrict__ count) {
  const int n = *count;
  const Layout &L = a.L;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const long long o = __ldg(list + t);
    const int k = (int)(o / L.plane);
    const long long r = o - (long long)k * L.plane;
    const int j = (int)(r / L.pitch), i = (int)(r - (long long)j * L.pitch);
    adj_slope_point(a, slope_faces(L, a.m, i, j, k), i, j, k);
  }
}

// ---------------------------------------------------------------------------
// 5. gather onto points
// ---------------------------------------------------------------------------
struct GatherArgs {
  Layout L;
  Grid g;
  GridInv gi;
  int eos;
  const double *__restrict__ gTp;
  const double *__restrict__ gSp;
  const uint8_t *__restrict__ m;
  const double *__restrict__ part;
  long long field;
  double *gT, *gS, *gK;
  const uint8_t *__restrict__ active;  // points whose partials the slope pass wrote (the others are zero)
};

__global__ void __launch_bounds__(128) adj_gather_kernel(GatherArgs a) {
  const Layout &L = a.L;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= L.X || j >= L.Y) return;
  const int X = L.X, Y = L.Y, Z = L.Z;
  const long long o = L.at(i, j, k), PW = L.pitch, PL = L.plane, F = a.field;
  const uint8_t *m = a.m;
  auto part = [&](int comp, long long at) { return __ldg(a.active + at) ? __ldg(a.part + comp * F + at) : 0.0; };

  const bool wet = __ldg(m + o) & VG_MASK_T;
  double lamT = wet ? __ldg(a.gTp + o) + drdT_dT(a.eos) * part(P_LRT, o) : 0.0;
  double lamS = wet ? __ldg(a.gSp + o) : 0.0;
  double gk = part(P_LKW + 1, o) + (k < Z - 1 ? part(P_LKW + 0, o + PL) : 0.0);
  const double wk = k >= 1 ? 0.25 : 0.5;

  // x-faces f = i-1 (this point is east of it) and f = i (west of it): the
  // face's difference T(f+1) - T(f) takes the partials of both its points
#pragma unroll
  for (int side = 0; side < 2; ++side) {
    const int f = i - 1 + side;
    if (f < 0 || f > X - 2) continue;
    const long long ow = o - 1 + side, oe = ow + 1;
    const double wT = part(P_WT + 0, ow) + part(P_WT + 1, oe), wS = part(P_WS + 0, ow) + part(P_WS + 1, oe);
    lamT += side == 0 ? wT : -wT;
    lamS += side == 0 ? wS : -wS;
    gk += wk * (part(P_LDL + 0, ow) + part(P_LDL + 1, oe));
    if (k < Z - 1) gk += 0.25 * (part(P_LDL + 0, ow + PL) + part(P_LDL + 1, oe + PL));
  }
  // y-faces f = j-1, j
#pragma unroll
  for (int side = 0; side < 2; ++side) {
    const int f = j - 1 + side;
    if (f < 0 || f > Y - 2) continue;
    const long long os = o + (side - 1) * PW, on = os + PW;
    const double wT = part(P_WT + 2, os) + part(P_WT + 3, on), wS = part(P_WS + 2, os) + part(P_WS + 3, on);
    lamT += side == 0 ? wT : -wT;
    lamS += side == 0 ? wS : -wS;
    gk += wk * (part(P_LDL + 2, os) + part(P_LDL + 3, on));
    if (k < Z - 1) gk += 0.25 * (part(P_LDL + 2, os + PL) + part(P_LDL + 3, on + PL));
  }
  // z-faces f = k-1, k
#pragma unroll
  for (int side = 0; side < 2; ++side) {
    const int f = k - 1 + side;
    if (f < 0 || f > Z - 2) continue;
    const long long od = o + (side - 1) * PL, ou = od + PL;
    const double gT = part(P_GZT + 1, od) + part(P_GZT + 0, ou), gS = part(P_GZS + 1, od) + part(P_GZS + 0, ou);
    lamT += side == 0 ? gT : -gT;
    lamS += side == 0 ? gS : -gS;
  }
  // vertical tracer differences of the isoneutral fluxes (edge-padded in z)
  if (k >= 1) {
    lamT += part(P_LVD + 0, o) + part(P_LVD + 1, o - PL);
    lamS += part(P_LVD + 2, o) + part(P_LVD + 3, o - PL);
  }
  if (k < Z - 1) {
    lamT -= part(P_LVD + 1, o) + part(P_LVD + 0, o + PL);
    lamS -= part(P_LVD + 3, o) + part(P_LVD + 2, o + PL);
  }
  a.gT[o] = lamT;
  a.gS[o] = lamS;
  a.gK[o] += gk;
}

}  // namespace adj
}  // namespace vg

using namespace vg;

extern "C" size_t vg_isoneutral_step_adjoint_scratch_bytes(const VgDomain *dom) {
  if (validate_domain(dom)) return 0;
  return adj::scratch_bytes(layout_of(dom));
}

extern "C" int vg_isoneutral_step_adjoint_f64(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set,
                                              const VgAdjointFields *f, void *scratch, size_t scratch_bytes,
                                              void *stream) {
  clear_error();
  int st = validate_domain(dom);
  if (st) return st;
  if (!grid_complete(grid) || !set || !f || !f->temp || !f->salt || !f->temp_new || !f->salt_new || !f->K_iso ||
      !f->mask_bits || !f->kbot || !f->gtemp_new || !f->gsalt_new || !f->gtemp || !f->gsalt || !f->gK_iso)
    return fail(VG_ERR_ARG, "vg_isoneutral_step_adjoint_f64: NULL pointer argument");
  if (!(set->iso_dslope > 0.0)) return fail(VG_ERR_ARG, "iso_dslope must be positive");
  if (set->eq_of_state_type < 1 || set->eq_of_state_type > 4)
    return fail(VG_ERR_ARG, "eq_of_state_type %d not supported", set->eq_of_state_type);
  const Layout L = layout_of(dom);
  const size_t need = adj::scratch_bytes(L);
  if (!scratch || scratch_bytes < need)
    return fail(VG_ERR_SCRATCH, "adjoint scratch of %zu bytes given, %zu needed", scratch_bytes, need);
  if (L.Z > 200) return fail(VG_ERR_SHAPE, "Z=%d above the 200 levels supported", L.Z);
  if (adj::field_doubles(L) >= (size_t)INT_MAX)
    return fail(VG_ERR_SHAPE, "%zu points per field: the active-point list indexes below 2^31", adj::field_doubles(L));
  cudaStream_t s = as_stream(stream);
  double *base = static_cast<double *>(scratch);
  const long long F = (long long)adj::field_doubles(L);
  double *tables = base + adj::kFields * F;
  const adj::GridInv gi = adj::tables_of(L, tables);
  const Grid g = grid_of(grid);

  // 1. reciprocal grid tables
  {
    const int n = L.X > L.Y ? (L.X > L.Z ? L.X : L.Z) : (L.Y > L.Z ? L.Y : L.Z);
    adj::adj_tables_kernel<<<(n + 127) / 128, 128, 0, s>>>(L, g, tables);
    if ((st = check_launch("adj_tables_kernel"))) return st;
  }
  // 2. the step's tensor
  VgTensorFields ten;
  ten.K_11 = base;
  ten.K_22 = base + F;
  ten.K_33 = base + 2 * F;
  ten.Ai_ez = base + 3 * F;
  ten.Ai_nz = base + 7 * F;
  ten.Ai_bx = base + 11 * F;
  ten.Ai_by = base + 15 * F;
  ten.ai_stride_p = 2 * F;
  ten.ai_stride_r = F;
  double *slopes = base + adj::F_SLOPES * F;
  if ((st = pre_f64_with_slopes(dom, grid, set, f->temp, f->salt, f->K_iso, f->mask_bits, &ten, slopes, stream)))
    return st;
  double *gTp = base + adj::F_GTP * F, *gSp = base + adj::F_GSP * F, *gK33 = base + adj::F_GK33 * F;
  double *part = base + adj::F_PART * F;
  double *nu = base + adj::F_NU * F;

  // 3. implicit part
  {
    adj::ImpArgs a{L,   gi,  set->dt_tracer, f->kbot, ten.K_33, f->temp_new, f->salt_new, f->gtemp_new,
                   f->gsalt_new, gTp, gSp, gK33, nu, F, f->column_order};
    // two threads per column, c' per column and d' per thread in shared memory
    int nb = 128;
    while (nb > 32 && 3 * (size_t)L.Z * (nb / 2) * sizeof(double) > 160 * 1024) nb /= 2;
    const size_t smem = 3 * (size_t)L.Z * (nb / 2) * sizeof(double);
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(adj::adj_implicit_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem);
      if (e != cudaSuccess) return fail(VG_ERR_LAUNCH, "adj_implicit_kernel smem %zu: %s", smem, cudaGetErrorString(e));
    }
    const int ncols = L.X * L.Y, nc = nb / 2;
    adj::adj_implicit_kernel<<<(ncols + nc - 1) / nc, nb, smem, s>>>(a);
    if ((st = check_launch("adj_implicit_kernel"))) return st;
  }
  const dim3 block(32, 4), grd((L.X + 31) / 32, (L.Y + 3) / 4, L.Z);
  // 4. slope adjoints: the points whose faces carry terms, listed, then the slope pass over the list
  {
    int32_t *list = reinterpret_cast<int32_t *>(base + adj::list_offset(L));
    int *count = list + F;
    uint8_t *active = reinterpret_cast<uint8_t *>(count + 1);
    cudaError_t e = cudaMemsetAsync(count, 0, sizeof(int), s);
    if (e != cudaSuccess) return fail(VG_ERR_LAUNCH, "adjoint list count: %s", cudaGetErrorString(e));
    adj::adj_active_kernel<<<grd, block, 0, s>>>(L, f->mask_bits, active, list, count);
    if ((st = check_launch("adj_active_kernel"))) return st;
    adj::SlopeArgs a{L,      g,    gi,       set->eq_of_state_type, set->iso_slopec, 1.0 / set->iso_dslope,
                     set->K_iso_steep, f->temp, f->salt, f->K_iso, gK33, f->mask_bits, slopes, nu, ten.K_11,
                     ten.K_22, part, F};
    int dev = 0, sms = 0, per = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, adj::adj_slope_kernel, 128, 0) != cudaSuccess || per < 1)
      return fail(VG_ERR_LAUNCH, "adj_slope_kernel: occupancy query failed");
    const long long want = ((long long)F + 127) / 128;
    const int nblk = (int)std::min<long long>(want, (long long)sms * per);
    adj::adj_slope_kernel<<<nblk, 128, 0, s>>>(a, list, count);
    if ((st = check_launch("adj_slope_kernel"))) return st;
  }
  // 5. gather
  {
    const uint8_t *active = reinterpret_cast<const uint8_t *>(
        reinterpret_cast<const int32_t *>(base + adj::list_offset(L)) + F + 1);
    adj::GatherArgs a{L, g, gi, set->eq_of_state_type, gTp, gSp, f->mask_bits, part, F, f->gtemp, f->gsalt,
                      f->gK_iso, active};
    adj::adj_gather_kernel<<<grd, block, 0, s>>>(a);
    if ((st = check_launch("adj_gather_kernel"))) return st;
  }
  return VG_OK;
}
