// Isoneutral tracer diffusion (FP64), the work of
// veros/core/isoneutral/diffusion.py:9-295 and veros/core/diffusion.py:9-62.
//
// Three launches per tracer:
//  1. flux_kernel   one thread per cell: east, north and top fluxes
//                   (diffusion.py:9-113) into a scratch triple; zero where the
//                   reference leaves them unset.
//  2. column_kernel one thread per interior column, walking k upward: flux
//                   divergence (diffusion.py:116-139), explicit update, the
//                   implicit K_33 solve in the operation order of LAPACK dgtsv
//                   (the solver behind the reference's solve_implicit), with
//                   the eliminated rows in shared memory (diffusion.py:142-169),
//                   and the dtracer_iso accumulation (diffusion.py:196-205).
//  3. energy_kernel (enable_conserve_energy only) one thread per cell:
//                   dissipation on the W grid and the vertical-mixing term
//                   added to P_diss (diffusion.py:234-281).
#include "common.cuh"
#include "dgtsv.cuh"

namespace vg {

namespace {

struct DiffArgs {
  Layout L;
  Grid g;
  double dt, grav, rho0;
  const double *__restrict__ K;  // K_iso (iso) or K_gm (skew)
  double s1, s2;                 // K1 = s1*K, K2 = s2*K (diffusion.py:15-16)
  const double *__restrict__ K11;
  const double *__restrict__ K22;
  const double *__restrict__ K33;
  const double *__restrict__ Aez;
  const double *__restrict__ Anz;
  const double *__restrict__ Abx;
  const double *__restrict__ Aby;
  long long sp, sr;
  const uint8_t *__restrict__ m;
  const int32_t *__restrict__ kbot;
  const double *__restrict__ tr;  // tau
  double *trp;                    // taup1
  double *dtr_iso;
  const double *__restrict__ idr;  // int_drhodX at tau
  double *P;
  double *fe, *fn, *ft;  // scratch fluxes
  int iso;
};

__device__ __forceinline__ double ld(const double *p, long long o) { return __ldg(p + o); }

__global__ void __launch_bounds__(128) flux_kernel(DiffArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  const int k = blockIdx.z;
  const Layout &L = a.L;
  if (i >= L.X) return;
  const long long o = L.at(i, j, k);
  const int Z = L.Z;
  const int km = k > 0 ? k - 1 : 0;      // edge padding in z (utilities.py:24-35)
  const int kp = k < Z - 1 ? k + 1 : Z - 1;

  // east face (diffusion.py:25-47)
  double fe = 0.0;
  if (i >= 1 && i < L.X - 2 && j >= 2 && j < L.Y - 2) {
    const double K1c = a.s1 * ld(a.K, o), K1e = a.s1 * ld(a.K, L.at(i + 1, j, k));
    double diffloc;
    if (k >= 1)
      diffloc = 0.25 * (K1c + a.s1 * ld(a.K, L.at(i, j, k - 1)) + K1e + a.s1 * ld(a.K, L.at(i + 1, j, k - 1)));
    else
      diffloc = 0.5 * (K1c + K1e);
    double sumz = 0.0;
#pragma unroll
    for (int kr = 0; kr < 2; ++kr) {
#pragma unroll
      for (int ip = 0; ip < 2; ++ip) {
        const double hi = ld(a.tr, L.at(i + ip, j, kr ? kp : k));
        const double lo = ld(a.tr, L.at(i + ip, j, kr ? k : km));
        sumz = sumz + diffloc * ld(a.Aez, o + ip * a.sp + kr * a.sr) * (hi - lo);
      }
    }
    const double tc = ld(a.tr, o), te = ld(a.tr, L.at(i + 1, j, k));
    fe = sumz / (4.0 * a.g.dzt[k]) + (te - tc) / (a.g.cost[j] * a.g.dxu[i]) * ld(a.K11, o);
  }
  a.fe[o] = fe;

  // north face (diffusion.py:52-77)
  double fn = 0.0;
  if (i >= 2 && i < L.X - 2 && j >= 1 && j < L.Y - 2) {
    const double K1c = a.s1 * ld(a.K, o), K1n = a.s1 * ld(a.K, L.at(i, j + 1, k));
    double diffloc;
    if (k >= 1)
      diffloc = 0.25 * (K1c + a.s1 * ld(a.K, L.at(i, j, k - 1)) + K1n + a.s1 * ld(a.K, L.at(i, j + 1, k - 1)));
    else
      diffloc = 0.5 * (K1c + K1n);
    double sumz = 0.0;
#pragma unroll
    for (int kr = 0; kr < 2; ++kr) {
#pragma unroll
      for (int jp = 0; jp < 2; ++jp) {
        const double hi = ld(a.tr, L.at(i, j + jp, kr ? kp : k));
        const double lo = ld(a.tr, L.at(i, j + jp, kr ? k : km));
        sumz = sumz + diffloc * ld(a.Anz, o + jp * a.sp + kr * a.sr) * (hi - lo);
      }
    }
    const double tc = ld(a.tr, o), tn = ld(a.tr, L.at(i, j + 1, k));
    fn = a.g.cosu[j] * (sumz / (4.0 * a.g.dzt[k]) + (tn - tc) / a.g.dyu[j] * ld(a.K22, o));
  }
  a.fn[o] = fn;

  // top face (diffusion.py:85-111)
  double ft = 0.0;
  if (i >= 2 && i < L.X - 2 && j >= 2 && j < L.Y - 2 && k < Z - 1) {
    const double diffloc = a.s2 * ld(a.K, o);
    const double cost = a.g.cost[j];
    double sumx = 0.0;
#pragma unroll
    for (int ip = 0; ip < 2; ++ip) {
#pragma unroll
      for (int kr = 0; kr < 2; ++kr) {
        const double d = ld(a.tr, L.at(i + ip, j, k + kr)) - ld(a.tr, L.at(i - 1 + ip, j, k + kr));
        sumx = sumx + diffloc * ld(a.Abx, o + ip * a.sp + kr * a.sr) / cost * d;
      }
    }
    double sumy = 0.0;
#pragma unroll
    for (int jp = 0; jp < 2; ++jp) {
#pragma unroll
      for (int kr = 0; kr < 2; ++kr) {
        const double d = ld(a.tr, L.at(i, j + jp, k + kr)) - ld(a.tr, L.at(i, j - 1 + jp, k + kr));
        sumy = sumy + diffloc * ld(a.Aby, o + jp * a.sp + kr * a.sr) * a.g.cosu[j - 1 + jp] * d;
      }
    }
    ft = sumx / (4.0 * a.g.dxt[i]) + sumy / (4.0 * a.g.dyt[j] * cost);
  }
  a.ft[o] = ft;
}

// Row source of one column's implicit system (diffusion.py:154-164), read
// back from global memory for the interchange path.
struct ColSrc {
  const DiffArgs &a;
  long long base;
  int ks, Z;
  __device__ double delta(int k) const {
    return k < Z - 1 ? rmul(rdiv(a.dt, a.g.dzw[k]), a.K33[base + (long long)k * a.L.plane]) : 0.0;
  }
  __device__ double a_(int k) const { return rdiv(-delta(k - 1), a.g.dzt[k]); }
  __device__ double b(int k) const {
    return k == ks ? radd(1.0, rdiv(delta(k), a.g.dzt[k])) : radd(1.0, rdiv(radd(delta(k), delta(k - 1)), a.g.dzt[k]));
  }
  __device__ double c(int k) const { return rdiv(-delta(k), a.g.dzt[k]); }
  __device__ double d(int k) const { return a.trp[base + (long long)k * a.L.plane]; }
};
struct ColSrcView {
  const ColSrc &s;
  __device__ double a(int k) const { return s.a_(k); }
  __device__ double b(int k) const { return s.b(k); }
  __device__ double c(int k) const { return s.c(k); }
  __device__ double d(int k) const { return s.d(k); }
};

// Per interior column: explicit divergence, explicit update and (iso) the
// implicit vertical solve in dgtsv's operation order. Shared memory holds the
// eliminated diagonal and right-hand side of each thread's column, 2 * Z
// doubles laid out [k][thread]; tr1 and the partial tendency are parked in
// the output arrays between the two sweeps.
__global__ void __launch_bounds__(64) column_kernel(DiffArgs a, int ncols_x, int ncols) {
  extern __shared__ double smem[];
  const int t = threadIdx.x;
  const int col = blockIdx.x * blockDim.x + t;
  if (col >= ncols) return;
  const Layout &L = a.L;
  const int Z = L.Z;
  const int i = 2 + col % ncols_x;
  const int j = 2 + col / ncols_x;
  const int nb = blockDim.x;
  double *Ds = smem;
  double *Bs = smem + (size_t)Z * nb;

  const double cost = a.g.cost[j];
  const double fx = cost * a.g.dxt[i];
  const double fy = cost * a.g.dyt[j];
  const int ks = a.kbot[L.at2(i, j)] - 1;  // create_water_masks (utilities.py:38-48)
  const bool solve = a.iso && ks >= 0;

  double ft_prev = 0.0, delta_prev = 0.0, Dp = 0.0, Bp = 0.0, cp = 0.0;
  bool interchange = false;
  for (int k = 0; k < Z; ++k) {
    const long long o = L.at(i, j, k);
    const double mT = (__ldg(a.m + o) & VG_MASK_T) ? 1.0 : 0.0;
    const double ftk = a.ft[o];
    double e = mT * ((a.fe[o] - a.fe[o - 1]) / fx + (a.fn[o] - a.fn[o - L.pitch]) / fy);
    if (k == 0)
      e = e + mT * ftk / a.g.dzt[0];
    else
      e = e + mT * (ftk - ft_prev) / a.g.dzt[k];
    ft_prev = ftk;
    const double d1 = radd(a.dtr_iso[o], e);
    const double tr1 = radd(a.trp[o], rmul(a.dt, e));
    a.dtr_iso[o] = d1;
    a.trp[o] = tr1;
    if (solve) {
      const double dzt = a.g.dzt[k];
      const double delta = k < Z - 1 ? rmul(rdiv(a.dt, a.g.dzw[k]), ld(a.K33, o)) : 0.0;
      if (k >= ks) {
        const double ck = rdiv(-delta, dzt);
        double Dk, Bk;
        if (k == ks) {
          Dk = radd(1.0, rdiv(delta, dzt));
          Bk = tr1;
        } else {
          const double dl = rdiv(-delta_prev, dzt);
          const double bk = radd(1.0, rdiv(radd(delta, delta_prev), dzt));
          if (fabs(Dp) < fabs(dl)) interchange = true;
          const double fact = rdiv(dl, Dp);
          Dk = rsub(bk, rmul(fact, cp));
          Bk = rsub(tr1, rmul(fact, Bp));
        }
        Ds[(size_t)k * nb + t] = Dk;
        Bs[(size_t)k * nb + t] = Bk;
        Dp = Dk;
        Bp = Bk;
        cp = ck;
      }
      delta_prev = delta;
    }
  }
  if (!solve) return;
  const long long base = L.at2(i, j);
  if (interchange) {
    // rows that dgtsv would interchange: replay the elimination with pivoting
    ColSrc src{a, base, ks, Z};
    dgtsv_slow_solve(ColSrcView{src}, ks, Z, Ds + t, nb);
  } else {
    double x = 0.0;
    for (int k = Z - 1; k >= ks; --k) {
      const double Dk = Ds[(size_t)k * nb + t], Bk = Bs[(size_t)k * nb + t];
      if (k == Z - 1) {
        x = rdiv(Bk, Dk);
      } else {
        const double delta = rmul(rdiv(a.dt, a.g.dzw[k]), ld(a.K33, base + (long long)k * L.plane));
        x = rdiv(rsub(Bk, rmul(rdiv(-delta, a.g.dzt[k]), x)), Dk);
      }
      Ds[(size_t)k * nb + t] = x;
    }
  }
  for (int k = Z - 1; k >= ks; --k) {
    const long long o = base + (long long)k * L.plane;
    const double x = Ds[(size_t)k * nb + t];
    const double tr1 = a.trp[o];
    a.trp[o] = x;
    a.dtr_iso[o] = radd(a.dtr_iso[o], rdiv(rsub(x, tr1), a.dt));
  }
}

// Dissipation at T points (veros/core/diffusion.py:9-36); zero on the outer ring.
__device__ __forceinline__ double diss_at(const DiffArgs &a, int i, int j, int k) {
  const Layout &L = a.L;
  const long long o = L.at(i, j, k);
  const double c = 0.5 * a.grav / a.rho0;
  const double I0 = ld(a.idr, o);
  const double ex = (ld(a.idr, o + 1) - I0) * a.fe[o] + (I0 - ld(a.idr, o - 1)) * a.fe[o - 1];
  const double ny = (ld(a.idr, o + L.pitch) - I0) * a.fn[o] + (I0 - ld(a.idr, o - L.pitch)) * a.fn[o - L.pitch];
  const double cost = a.g.cost[j];
  return c * ex / (a.g.dxt[i] * cost) + c * ny / (a.g.dyt[j] * cost);
}

__global__ void __launch_bounds__(128) energy_kernel(DiffArgs a) {
  const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = 1 + blockIdx.y;
  const int k = blockIdx.z;
  const Layout &L = a.L;
  if (i >= L.X - 1) return;
  const int Z = L.Z;
  const long long o = L.at(i, j, k);
  const int ks = a.kbot[L.at2(i, j)] - 1;
  const bool land = ks >= 0;  // "land_mask" of create_water_masks: column has water

  // dissipation_on_wgrid (veros/core/diffusion.py:39-62)
  const double d0 = diss_at(a, i, j, k);
  double dw;
  if (k < Z - 1) {
    const double d1 = diss_at(a, i, j, k + 1);
    const double edge = (land && k == ks) ? 1.0 : 0.0;
    const double water = (land && k > ks) ? 1.0 : 0.0;
    const double dzw_pad = a.g.dzw[k > 0 ? k - 1 : 0];
    dw = (0.5 * (d0 + d1) + 0.5 * (d0 * dzw_pad / a.g.dzw[k])) * edge + 0.5 * (d0 + d1) * water;
  } else {
    dw = d0 * (land ? 1.0 : 0.0);
  }
  double P = a.P[o] + dw;

  // vertical-mixing term (diffusion.py:254-279)
  if (i >= 2 && i < L.X - 2 && j >= 2 && j < L.Y - 2 && k < Z - 1) {
    const double mW = (__ldg(a.m + o) & VG_MASK_W) ? 1.0 : 0.0;
    const double fxa = (-ld(a.idr, o + L.plane) + ld(a.idr, o)) / a.g.dzw[k];
    const double g = -a.grav / a.rho0 * fxa;
    if (a.iso) {
      const double dtrz = a.trp[o + L.plane] - a.trp[o];
      P = P + g * (a.ft[o] * mW + ld(a.K33, o) * dtrz / a.g.dzw[k] * mW);
    } else {
      P = P + g * a.ft[o] * mW;
    }
  }
  a.P[o] = P;
}

}  // namespace

}  // namespace vg

using namespace vg;

extern "C" size_t vg_isoneutral_diffusion_scratch_bytes(const VgDomain *dom) {
  if (!dom || dom->plane <= 0 || dom->Z <= 0) return 0;
  return 3 * (size_t)dom->plane * (size_t)dom->Z * sizeof(double);
}

extern "C" int vg_isoneutral_diffusion_f64(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set,
                                           const VgTensorFields *ten, const double *K_field,
                                           const uint8_t *mask_bits, const int32_t *kbot, const VgTracerArgs *tr,
                                           int skew, void *scratch, size_t scratch_bytes, void *stream) {
  clear_error();
  int st = validate_domain(dom);
  if (st) return st;
  if (!grid_complete(grid) || !set || !ten || !K_field || !mask_bits || !kbot || !tr || !tr->tr_tau ||
      !tr->tr_taup1 || !tr->dtracer_iso || !ten->K_11 || !ten->K_22 || !ten->K_33 || !ten->Ai_ez ||
      !ten->Ai_nz || !ten->Ai_bx || !ten->Ai_by)
    return fail(VG_ERR_ARG, "vg_isoneutral_diffusion_f64: NULL pointer argument");
  if (skew != 0 && skew != 1) return fail(VG_ERR_ARG, "skew must be 0 or 1");
  if (set->enable_conserve_energy && (!tr->int_drhodX_tau || !tr->P_diss))
    return fail(VG_ERR_ARG, "enable_conserve_energy needs int_drhodX_tau and P_diss");
  if (!(set->dt_tracer != 0.0)) return fail(VG_ERR_ARG, "dt_tracer must be non-zero");
  const size_t need = vg_isoneutral_diffusion_scratch_bytes(dom);
  if (!scratch || scratch_bytes < need)
    return fail(VG_ERR_SCRATCH, "scratch of %zu bytes given, %zu needed", scratch_bytes, need);

  DiffArgs a;
  a.L = layout_of(dom);
  a.g = grid_of(grid);
  a.dt = set->dt_tracer;
  a.grav = set->grav;
  a.rho0 = set->rho_0;
  a.K = K_field;
  a.s1 = skew ? -1.0 : 1.0;
  a.s2 = 1.0;
  a.K11 = ten->K_11;
  a.K22 = ten->K_22;
  a.K33 = ten->K_33;
  a.Aez = ten->Ai_ez;
  a.Anz = ten->Ai_nz;
  a.Abx = ten->Ai_bx;
  a.Aby = ten->Ai_by;
  a.sp = ten->ai_stride_p;
  a.sr = ten->ai_stride_r;
  a.m = mask_bits;
  a.kbot = kbot;
  a.tr = tr->tr_tau;
  a.trp = tr->tr_taup1;
  a.dtr_iso = tr->dtracer_iso;
  a.idr = tr->int_drhodX_tau;
  a.P = tr->P_diss;
  const size_t fsz = (size_t)a.L.plane * a.L.Z;
  a.fe = static_cast<double *>(scratch);
  a.fn = a.fe + fsz;
  a.ft = a.fn + fsz;
  a.iso = skew ? 0 : 1;
  cudaStream_t s = as_stream(stream);

  {
    dim3 block(128);
    dim3 g((a.L.X + 127) / 128, a.L.Y, a.L.Z);
    flux_kernel<<<g, block, 0, s>>>(a);
    if ((st = check_launch("flux_kernel"))) return st;
  }
  {
    const int ncols_x = a.L.X - 4, ncols = ncols_x * (a.L.Y - 4);
    const int nb = 64;
    const size_t smem = 2 * (size_t)a.L.Z * nb * sizeof(double);
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(column_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return fail(VG_ERR_LAUNCH, "column_kernel smem %zu: %s", smem, cudaGetErrorString(e));
    }
    column_kernel<<<(ncols + nb - 1) / nb, nb, smem, s>>>(a, ncols_x, ncols);
    if ((st = check_launch("column_kernel"))) return st;
  }
  if (set->enable_conserve_energy) {
    dim3 block(128);
    dim3 g((a.L.X - 2 + 127) / 128, a.L.Y - 2, a.L.Z);
    energy_kernel<<<g, block, 0, s>>>(a);
    if ((st = check_launch("energy_kernel"))) return st;
  }
  return VG_OK;
}
