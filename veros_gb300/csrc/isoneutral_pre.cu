// Isoneutral slopes and diffusion tensor (FP64), the work of
// veros/core/isoneutral/isoneutral.py:18-229.
//
// One thread per cell (i, j, k). Every thread derives the face gradients and
// density derivatives it needs from temp/salt directly; neighbouring threads
// read the same cache lines, which L1/L2 serve. Outputs are written only on
// the reference's sub-ranges so that all other cells keep their contents.
#include "common.cuh"

namespace vg {

namespace {

constexpr double kEpsln = 1e-20;  // isoneutral.py:28

struct PreArgs {
  Layout L;
  Grid g;
  Eos eos;
  double slopec, dslope, ksteep;
  const double *__restrict__ T;
  const double *__restrict__ S;
  const double *__restrict__ K;
  const uint8_t *__restrict__ m;
  double *K11, *K22, *K33, *Aez, *Anz, *Abx, *Aby;
  long long sp, sr;
};

struct Fields {
  const PreArgs &a;
  __device__ __forceinline__ double T(int i, int j, int k) const { return __ldg(a.T + a.L.at(i, j, k)); }
  __device__ __forceinline__ double S(int i, int j, int k) const { return __ldg(a.S + a.L.at(i, j, k)); }
  __device__ __forceinline__ unsigned M(int i, int j, int k) const { return __ldg(a.m + a.L.at(i, j, k)); }
  // drho/dT and drho/dS at T points, masked (isoneutral.py:40-41)
  __device__ __forceinline__ double drdT(int i, int j, int k) const {
    return (M(i, j, k) & VG_MASK_T) ? a.eos.drdT(T(i, j, k), a.g.zt[k]) : 0.0;
  }
  __device__ __forceinline__ double drdS(int i, int j, int k) const {
    return (M(i, j, k) & VG_MASK_T) ? a.eos.drdS() : 0.0;
  }
  // gradients at the top face (isoneutral.py:46-59); zero on the top level
  __device__ __forceinline__ double dTdz(int i, int j, int k) const {
    if (k >= a.L.Z - 1 || !(M(i, j, k) & VG_MASK_W)) return 0.0;
    return (T(i, j, k + 1) - T(i, j, k)) / a.g.dzw[k];
  }
  __device__ __forceinline__ double dSdz(int i, int j, int k) const {
    if (k >= a.L.Z - 1 || !(M(i, j, k) & VG_MASK_W)) return 0.0;
    return (S(i, j, k + 1) - S(i, j, k)) / a.g.dzw[k];
  }
  // gradients at the east face (isoneutral.py:64-77); zero on the last column
  __device__ __forceinline__ double dTdx(int i, int j, int k) const {
    if (i >= a.L.X - 1 || !(M(i, j, k) & VG_MASK_U)) return 0.0;
    return (T(i + 1, j, k) - T(i, j, k)) / (a.g.dxu[i] * a.g.cost[j]);
  }
  __device__ __forceinline__ double dSdx(int i, int j, int k) const {
    if (i >= a.L.X - 1 || !(M(i, j, k) & VG_MASK_U)) return 0.0;
    return (S(i + 1, j, k) - S(i, j, k)) / (a.g.dxu[i] * a.g.cost[j]);
  }
  // gradients at the north face (isoneutral.py:82-95); zero on the last row
  __device__ __forceinline__ double dTdy(int i, int j, int k) const {
    if (j >= a.L.Y - 1 || !(M(i, j, k) & VG_MASK_V)) return 0.0;
    return (T(i, j + 1, k) - T(i, j, k)) / a.g.dyu[j];
  }
  __device__ __forceinline__ double dSdy(int i, int j, int k) const {
    if (j >= a.L.Y - 1 || !(M(i, j, k) & VG_MASK_V)) return 0.0;
    return (S(i, j + 1, k) - S(i, j, k)) / a.g.dyu[j];
  }
};

// dm_taper (isoneutral.py:10-15)
__device__ __forceinline__ double taper_of(double sx, double slopec, double dslope) {
  return 0.5 * (1.0 + tanh((-fabs(sx) + slopec) / dslope));
}

__device__ __forceinline__ double slope_of(double num, double den) { return -num / (fmin(0.0, den) - kEpsln); }

__global__ void __launch_bounds__(128) pre_cell_kernel(PreArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  const int k = blockIdx.z;
  const Layout &L = a.L;
  if (i >= L.X) return;
  Fields f{a};
  const long long o = L.at(i, j, k);

  // K_33 on the top level is zero everywhere (isoneutral.py:225)
  if (k == L.Z - 1) a.K33[o] = 0.0;

  // east face: Ai_ez and K_11 (isoneutral.py:100-132)
  if (i >= 1 && i < L.X - 2 && j >= 2 && j < L.Y - 2) {
    const bool mU = f.M(i, j, k) & VG_MASK_U;
    double diffloc;
    if (k >= 1)
      diffloc = 0.25 * (__ldg(a.K + o) + __ldg(a.K + L.at(i, j, k - 1)) + __ldg(a.K + L.at(i + 1, j, k)) +
                        __ldg(a.K + L.at(i + 1, j, k - 1)));
    else
      diffloc = 0.5 * (__ldg(a.K + o) + __ldg(a.K + L.at(i + 1, j, 0)));
    const double dTx = f.dTdx(i, j, k), dSx = f.dSdx(i, j, k);
    double sumz = 0.0;
#pragma unroll
    for (int kr = 0; kr < 2; ++kr) {
      const int ki = kr == 1 ? 0 : 1;
      if (k < ki) continue;
#pragma unroll
      for (int ip = 0; ip < 2; ++ip) {
        const double rT = f.drdT(i + ip, j, k), rS = f.drdS(i + ip, j, k);
        const double drodxe = rT * dTx + rS * dSx;
        const double drodze = rT * f.dTdz(i + ip, j, k - 1 + kr) + rS * f.dSdz(i + ip, j, k - 1 + kr);
        const double sxe = slope_of(drodxe, drodze);
        const double taper = taper_of(sxe, a.slopec, a.dslope);
        sumz += a.g.dzw[k - 1 + kr] * (mU ? 1.0 : 0.0) * fmax(a.ksteep, diffloc * taper);
        a.Aez[o + ip * a.sp + kr * a.sr] = taper * sxe * (mU ? 1.0 : 0.0);
      }
    }
    a.K11[o] = sumz / (4.0 * a.g.dzt[k]);
  }

  // north face: Ai_nz and K_22 (isoneutral.py:137-168)
  if (i >= 2 && i < L.X - 2 && j >= 1 && j < L.Y - 2) {
    const bool mV = f.M(i, j, k) & VG_MASK_V;
    double diffloc;
    if (k >= 1)
      diffloc = 0.25 * (__ldg(a.K + o) + __ldg(a.K + L.at(i, j, k - 1)) + __ldg(a.K + L.at(i, j + 1, k)) +
                        __ldg(a.K + L.at(i, j + 1, k - 1)));
    else
      diffloc = 0.5 * (__ldg(a.K + o) + __ldg(a.K + L.at(i, j + 1, 0)));
    const double dTy = f.dTdy(i, j, k), dSy = f.dSdy(i, j, k);
    double sumz = 0.0;
#pragma unroll
    for (int kr = 0; kr < 2; ++kr) {
      const int ki = kr == 1 ? 0 : 1;
      if (k < ki) continue;
#pragma unroll
      for (int jp = 0; jp < 2; ++jp) {
        const double rT = f.drdT(i, j + jp, k), rS = f.drdS(i, j + jp, k);
        const double drodyn = rT * dTy + rS * dSy;
        const double drodzn = rT * f.dTdz(i, j + jp, k - 1 + kr) + rS * f.dSdz(i, j + jp, k - 1 + kr);
        const double syn = slope_of(drodyn, drodzn);
        const double taper = taper_of(syn, a.slopec, a.dslope);
        sumz += a.g.dzw[k - 1 + kr] * (mV ? 1.0 : 0.0) * fmax(a.ksteep, diffloc * taper);
        a.Anz[o + jp * a.sp + kr * a.sr] = taper * syn * (mV ? 1.0 : 0.0);
      }
    }
    a.K22[o] = sumz / (4.0 * a.g.dzt[k]);
  }

  // top face: Ai_bx, Ai_by and K_33 (isoneutral.py:173-224)
  if (i >= 2 && i < L.X - 2 && j >= 2 && j < L.Y - 2 && k < L.Z - 1) {
    const bool mW = f.M(i, j, k) & VG_MASK_W;
    const double wm = mW ? 1.0 : 0.0;
    const double Kc = __ldg(a.K + o);
    const double dTz = f.dTdz(i, j, k), dSz = f.dSdz(i, j, k);
    double sumx = 0.0, sumy = 0.0;
#pragma unroll
    for (int kr = 0; kr < 2; ++kr) {
      const double rT = f.drdT(i, j, k + kr), rS = f.drdS(i, j, k + kr);
      const double drodzb = rT * dTz + rS * dSz;
#pragma unroll
      for (int ip = 0; ip < 2; ++ip) {
        const double drodxb = rT * f.dTdx(i - 1 + ip, j, k + kr) + rS * f.dSdx(i - 1 + ip, j, k + kr);
        const double sxb = slope_of(drodxb, drodzb);
        const double taper = taper_of(sxb, a.slopec, a.dslope);
        sumx = sumx + a.g.dxu[i - 1 + ip] * Kc * taper * (sxb * sxb) * wm;
        a.Abx[o + ip * a.sp + kr * a.sr] = taper * sxb * wm;
      }
#pragma unroll
      for (int jp = 0; jp < 2; ++jp) {
        const double facty = a.g.cosu[j - 1 + jp] * a.g.dyu[j - 1 + jp];
        const double drodyb = rT * f.dTdy(i, j - 1 + jp, k + kr) + rS * f.dSdy(i, j - 1 + jp, k + kr);
        const double syb = slope_of(drodyb, drodzb);
        const double taper = taper_of(syb, a.slopec, a.dslope);
        sumy = sumy + facty * Kc * taper * (syb * syb) * wm;
        a.Aby[o + jp * a.sp + kr * a.sr] = taper * syb * wm;
      }
    }
    a.K33[o] = sumx / (4.0 * a.g.dxt[i]) + sumy / (4.0 * a.g.dyt[j] * a.g.cost[j]);
  }
}

}  // namespace

}  // namespace vg

using namespace vg;

extern "C" int vg_isoneutral_pre_f64(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set,
                                     const double *temp_tau, const double *salt_tau, const double *K_iso,
                                     const uint8_t *mask_bits, const VgTensorFields *out, void *stream) {
  clear_error();
  int st = validate_domain(dom);
  if (st) return st;
  if (!grid_complete(grid) || !set || !temp_tau || !salt_tau || !K_iso || !mask_bits || !out || !out->K_11 ||
      !out->K_22 || !out->K_33 || !out->Ai_ez || !out->Ai_nz || !out->Ai_bx || !out->Ai_by)
    return fail(VG_ERR_ARG, "vg_isoneutral_pre_f64: NULL pointer argument");
  if (set->eq_of_state_type < 1 || set->eq_of_state_type > 4)
    return fail(VG_ERR_UNSUPPORTED, "eq_of_state_type %d not implemented (1-4 are)", set->eq_of_state_type);
  if (!(set->iso_dslope != 0.0)) return fail(VG_ERR_ARG, "iso_dslope must be non-zero");
  PreArgs a;
  a.L = layout_of(dom);
  a.g = grid_of(grid);
  a.eos = Eos{set->eq_of_state_type};
  a.slopec = set->iso_slopec;
  a.dslope = set->iso_dslope;
  a.ksteep = set->K_iso_steep;
  a.T = temp_tau;
  a.S = salt_tau;
  a.K = K_iso;
  a.m = mask_bits;
  a.K11 = out->K_11;
  a.K22 = out->K_22;
  a.K33 = out->K_33;
  a.Aez = out->Ai_ez;
  a.Anz = out->Ai_nz;
  a.Abx = out->Ai_bx;
  a.Aby = out->Ai_by;
  a.sp = out->ai_stride_p;
  a.sr = out->ai_stride_r;
  dim3 block(128);
  dim3 g((a.L.X + 127) / 128, a.L.Y, a.L.Z);
  pre_cell_kernel<<<g, block, 0, as_stream(stream)>>>(a);
  return check_launch("pre_cell_kernel");
}
