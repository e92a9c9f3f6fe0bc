// The two neighbours of the isoneutral path (FP64):
//
// * vg_vertmix_tempsalt_f64: implicit vertical mixing of temp and salt with
//   the diffusivity kappaH and the surface forcing
//   (veros/core/thermodynamics.py:248-300). One thread per column; temp and
//   salt share one Thomas factorisation of the matrix (the same system as the
//   isoneutral implicit part with kappaH for K_33, diffusion.py:154-164); the
//   surface forcing enters the top row's right-hand side. dtemp_vmix and
//   dsalt_vmix are written on the whole array ((new - old)/dt, zero outside
//   the water columns). With enable_cyclic_x the call ends with the
//   reference's closing boundary exchange of the new levels
//   (thermodynamics.py:292-298) in its single-process form: the periodic
//   copy of the x halo columns (veros/core/utilities.py:7-16).
// * vg_enforce_boundaries_f64: that copy on its own for one field.
// * vg_isoneutral_streamfunction_f64: the GM streamfunction diagnostics B1_gm
//   and B2_gm (veros/core/isoneutral/isoneutral.py:232-254), elementwise.
#include "common.cuh"
#include "dgtsv.cuh"

namespace vg {
namespace {

struct VmixArgs {
  Layout L;
  Grid g;
  double dt;
  const double *__restrict__ kappaH;
  const int32_t *__restrict__ kbot;
  double *tr[2];
  const double *forc[2];
  double *dvmix[2];
};

__device__ __forceinline__ double vm_mul(double x, double y) { return __dmul_rn(x, y); }
__device__ __forceinline__ double vm_fma(double x, double y, double z) { return __fma_rn(x, y, z); }

// One thread per column. Shared memory holds the per-level tables dt/dzw
// (the reference's own quotient, so delta keeps its rounding) and 1/dzt, and
// the eliminated c' of the CTA's columns, laid out [k][thread]; the
// eliminated right-hand sides d' go to dtemp_vmix / dsalt_vmix, which the
// back substitution then overwrites with the tendencies (the column stays in
// L2 between the two sweeps). Divisions by dzt are multiplications by the
// table's reciprocals and each pivot costs one reciprocal (an FP32 seed
// refined by Newton steps). Both sweeps load PF levels ahead of their serial
// chain, so the chain waits for FP64 latency rather than for memory.
constexpr int kVmixThreads = 128;

__global__ void __launch_bounds__(kVmixThreads) vertmix_kernel(VmixArgs a) {
  extern __shared__ double smem[];
  const Layout &L = a.L;
  const int Z = L.Z;
  const int t = threadIdx.x, nb = blockDim.x;
  double *dtdzw = smem, *inv_dzt = smem + Z;
  double *cps = smem + 2 * Z;
  for (int k = t; k < Z; k += nb) {
    dtdzw[k] = a.dt / a.g.dzw[k];
    inv_dzt[k] = 1.0 / a.g.dzt[k];
  }
  // The CTA's columns ranked by their number of water levels (most first,
  // ties by position), so that the lanes of a warp walk columns of similar
  // length: each thread counts the columns ahead of its own and the thread of
  // that rank takes it.
  __shared__ int nlev_s[kVmixThreads];
  __shared__ int perm_s[kVmixThreads];
  const int ncols = L.X * L.Y;
  auto ks_of = [&](int c) {
    const int ci = c % L.X, cj = c / L.X;
    const bool interior = ci >= 2 && ci < L.X - 2 && cj >= 2 && cj < L.Y - 2;
    return interior ? a.kbot[L.at2(ci, cj)] - 1 : -1;  // create_water_masks (utilities.py:38-48)
  };
  {
    const int c = blockIdx.x * nb + t;
    const int k = c < ncols ? ks_of(c) : -1;
    nlev_s[t] = (k >= 0 && k < Z) ? Z - k : 0;
  }
  __syncthreads();
  {
    const int n = nlev_s[t];
    int rank = 0;
    for (int u = 0; u < nb; ++u) {
      const int m = nlev_s[u];
      rank += (m > n) || (m == n && u < t);
    }
    perm_s[rank] = t;
  }
  __syncthreads();
  const int col = blockIdx.x * nb + perm_s[t];
  if (col >= ncols) return;
  const int i = col % L.X, j = col / L.X;
  const long long base = L.at2(i, j);
  const int ks = ks_of(col);
  // dtemp_vmix starts as the old level; outside the water cells the update is (old - old)/dt = 0
  for (int k = 0; k < (ks >= 0 && ks < Z ? ks : Z); ++k) {
    const long long o = base + (long long)k * L.plane;
    a.dvmix[0][o] = 0.0;
    a.dvmix[1][o] = 0.0;
  }
  if (ks < 0 || ks >= Z) return;

  constexpr int PF = 8;
  double qK[PF], qT[PF][2];
#pragma unroll
  for (int u = 0; u < PF; ++u) {
    const int k = ks + u;
    const long long o = base + (long long)min(k, Z - 1) * L.plane;
    qK[u] = k < Z - 1 ? a.kappaH[o] : 0.0;
    qT[u][0] = k < Z ? a.tr[0][o] : 0.0;
    qT[u][1] = k < Z ? a.tr[1][o] : 0.0;
  }
  double delta_prev = 0.0, cp = 0.0, dp[2] = {0.0, 0.0};
  for (int k0 = ks; k0 < Z; k0 += PF) {
#pragma unroll
    for (int u = 0; u < PF; ++u) {
      const int k = k0 + u;
      if (k < Z) {
        const long long o = base + (long long)k * L.plane;
        const double idzt = inv_dzt[k];
        const double delta = k < Z - 1 ? vm_mul(dtdzw[k], qK[u]) : 0.0;  // thermodynamics.py:267-270
        double d[2] = {qT[u][0], qT[u][1]};
        const int kn = k + PF;
        if (kn < Z) {
          const long long on = base + (long long)kn * L.plane;
          qK[u] = kn < Z - 1 ? a.kappaH[on] : 0.0;
          qT[u][0] = a.tr[0][on];
          qT[u][1] = a.tr[1][on];
        }
        const double ak = k == ks ? 0.0 : vm_mul(-delta_prev, idzt);  // a_tri, zero at the edge (operators.py:72)
        const double bk = vm_fma(k == ks ? delta : delta + delta_prev, idzt, 1.0);  // b_tri, b_tri_edge at ks
        const double ck = vm_mul(-delta, idzt);                                      // c_tri (0 on the top level)
        const double den = recip_newton(vm_fma(-ak, cp, bk));  // pivot >= the diagonal's excess over 1
        cp = vm_mul(ck, den);
        cps[(size_t)k * nb + t] = cp;
#pragma unroll
        for (int r = 0; r < 2; ++r) {
          if (k == Z - 1) d[r] = vm_fma(vm_mul(a.dt, a.forc[r][base]), idzt, d[r]);  // thermodynamics.py:279, :287
          dp[r] = vm_mul(vm_fma(-ak, dp[r], d[r]), den);
          a.dvmix[r][o] = dp[r];
        }
        delta_prev = delta;
      }
    }
  }
  // back substitution from the top level down to ks; slot u holds level k - u
  double qD[PF][2], qO[PF][2];
#pragma unroll
  for (int u = 0; u < PF; ++u) {
    const int k = Z - 1 - u;
    const long long o = base + (long long)max(k, ks) * L.plane;
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      qD[u][r] = k >= ks ? a.dvmix[r][o] : 0.0;
      qO[u][r] = k >= ks ? a.tr[r][o] : 0.0;
    }
  }
  double x[2] = {0.0, 0.0};
  const double inv_dt = 1.0 / a.dt;
  for (int k0 = Z - 1; k0 >= ks; k0 -= PF) {
#pragma unroll
    for (int u = 0; u < PF; ++u) {
      const int k = k0 - u;
      if (k >= ks) {
        const long long o = base + (long long)k * L.plane;
        const double c = cps[(size_t)k * nb + t];
        double dk[2], old[2];
#pragma unroll
        for (int r = 0; r < 2; ++r) {
          dk[r] = qD[u][r];
          old[r] = qO[u][r];
        }
        const int kn = k - PF;
        if (kn >= ks) {
          const long long on = base + (long long)kn * L.plane;
#pragma unroll
          for (int r = 0; r < 2; ++r) {
            qD[u][r] = a.dvmix[r][on];
            qO[u][r] = a.tr[r][on];
          }
        }
#pragma unroll
        for (int r = 0; r < 2; ++r) {
          x[r] = vm_fma(-c, x[r], dk[r]);
          a.tr[r][o] = x[r];
          a.dvmix[r][o] = vm_mul(x[r] - old[r], inv_dt);  // thermodynamics.py:289-290
        }
      }
    }
  }
}

// enforce_boundaries (veros/core/utilities.py:7-16) on one process:
// arr[-2:] = arr[2:4], then arr[:2] = arr[-4:-2], for every (j, k) row of up
// to two fields. One thread per row reads its four source cells before it
// writes, which is what NumPy's overlap-safe assignment gives for the
// narrowest domain (X = 5), where the sources and destinations meet; for
// X >= 6 the two copies touch disjoint cells.
__global__ void __launch_bounds__(256) cyclic_x_kernel(Layout L, double *f0, double *f1) {
  const long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= (long long)L.Y * L.Z) return;
  const int j = (int)(row % L.Y), k = (int)(row / L.Y);
  const int X = L.X;
  for (int f = 0; f < 2; ++f) {
    double *p = f == 0 ? f0 : f1;
    if (!p) continue;
    double *r = p + L.at(0, j, k);
    const double s2 = r[2], s3 = r[3], t0 = r[X - 4], t1 = r[X - 3];
    r[X - 2] = s2;
    r[X - 1] = s3;
    r[0] = t0;
    r[1] = t1;
  }
}

int launch_cyclic_x(const Layout &L, double *f0, double *f1, cudaStream_t s) {
  const long long rows = (long long)L.Y * L.Z;
  cyclic_x_kernel<<<(unsigned)((rows + 255) / 256), 256, 0, s>>>(L, f0, f1);
  return check_launch("cyclic_x_kernel");
}

struct SfArgs {
  Layout L;
  const double *__restrict__ Kgm;
  const double *__restrict__ Aez;
  const double *__restrict__ Anz;
  long long sp, sr;
  double *B1, *B2;
};

// x / 16 through the exponent field: exact, as the multiplication by 2^-4
// is, whenever the result is a normal number; zeros, subnormal results, inf
// and NaN take the multiplication. An integer subtraction instead of an FP64
// multiply (the FP64 pipe bounds this kernel).
__device__ __forceinline__ double div16(double x) {
  const long long b = __double_as_longlong(x);
  const long long e = (b >> 52) & 0x7FF;
  return (e > 4 && e < 0x7FF) ? __longlong_as_double(b - (4LL << 52)) : x * 0.0625;
}

// Sum of the four K_gm around a face, K_gm edge-padded in z (utilities.py:24-35),
// added in the reference's order; the face value is this sum / 4.
__device__ __forceinline__ double kgm_sum(const SfArgs &a, long long o, long long dn, int k) {
  const long long up = k > 0 ? -a.L.plane : 0;  // pad: level k-1 clamps to 0
  return a.Kgm[o] + a.Kgm[o + up] + a.Kgm[o + dn] + a.Kgm[o + dn + up];
}

// 0.25 * (0.25 * sum) * s = (sum * s) / 16 exactly: both quarter scalings are
// exact, so one product and an exponent shift give the reference's bits.
__global__ void __launch_bounds__(128) streamfunction_kernel(SfArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y, k = blockIdx.z;
  const Layout &L = a.L;
  if (i >= L.X) return;
  const long long o = L.at(i, j, k);
  // B2_gm[1:-2, 2:-2] (isoneutral.py:241-244)
  if (i >= 1 && i < L.X - 2 && j >= 2 && j < L.Y - 2) {
    const double s = a.Aez[o] + a.Aez[o + a.sr] + a.Aez[o + a.sp] + a.Aez[o + a.sp + a.sr];
    a.B2[o] = div16(kgm_sum(a, o, 1, k) * s);
  }
  // B1_gm[2:-2, 1:-2] (isoneutral.py:249-252)
  if (i >= 2 && i < L.X - 2 && j >= 1 && j < L.Y - 2) {
    const double s = a.Anz[o] + a.Anz[o + a.sr] + a.Anz[o + a.sp] + a.Anz[o + a.sp + a.sr];
    a.B1[o] = div16(kgm_sum(a, o, L.pitch, k) * -s);
  }
}

}  // namespace
}  // namespace vg

using namespace vg;

extern "C" int vg_vertmix_tempsalt_f64(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set,
                                       const double *kappaH, const int32_t *kbot, double *temp_taup1,
                                       double *salt_taup1, const double *forc_temp_surface,
                                       const double *forc_salt_surface, double *dtemp_vmix, double *dsalt_vmix,
                                       int enable_cyclic_x, void *stream) {
  clear_error();
  int st = validate_domain(dom);
  if (st) return st;
  if (!grid_complete(grid) || !set || !kappaH || !kbot || !temp_taup1 || !salt_taup1 || !forc_temp_surface ||
      !forc_salt_surface || !dtemp_vmix || !dsalt_vmix)
    return fail(VG_ERR_ARG, "vg_vertmix_tempsalt_f64: NULL pointer argument");
  if (!(set->dt_tracer != 0.0)) return fail(VG_ERR_ARG, "dt_tracer must be non-zero");
  if (dom->Z > 512) return fail(VG_ERR_SHAPE, "Z=%d above the 512 levels supported", dom->Z);
  VmixArgs a;
  a.L = layout_of(dom);
  a.g = grid_of(grid);
  a.dt = set->dt_tracer;
  a.kappaH = kappaH;
  a.kbot = kbot;
  a.tr[0] = temp_taup1;
  a.tr[1] = salt_taup1;
  a.forc[0] = forc_temp_surface;
  a.forc[1] = forc_salt_surface;
  a.dvmix[0] = dtemp_vmix;
  a.dvmix[1] = dsalt_vmix;
  // columns per CTA: 128, fewer where the c' of 128 deep columns would not fit
  int nb = kVmixThreads;
  while (nb > 32 && (2 + (size_t)nb) * a.L.Z * sizeof(double) > 100 * 1024) nb /= 2;
  const size_t smem = (2 + (size_t)nb) * a.L.Z * sizeof(double);
  if (smem > 227 * 1024)
    return fail(VG_ERR_SHAPE, "vg_vertmix_tempsalt_f64: Z=%d too deep for the shared-memory factorisation", a.L.Z);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(vertmix_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return fail(VG_ERR_LAUNCH, "vertmix_kernel smem %zu: %s", smem, cudaGetErrorString(e));
  }
  const int ncols = a.L.X * a.L.Y;
  vertmix_kernel<<<(ncols + nb - 1) / nb, nb, smem, as_stream(stream)>>>(a);
  st = check_launch("vertmix_kernel");
  if (st || !enable_cyclic_x) return st;
  // thermodynamics.py:292-298: after dtemp_vmix / dsalt_vmix, so the
  // tendencies keep the halo columns' (new - old) / dt of the solve
  return launch_cyclic_x(a.L, temp_taup1, salt_taup1, as_stream(stream));
}

extern "C" int vg_enforce_boundaries_f64(const VgDomain *dom, double *arr, int enable_cyclic_x, void *stream) {
  clear_error();
  int st = validate_domain(dom);
  if (st) return st;
  if (!arr) return fail(VG_ERR_ARG, "vg_enforce_boundaries_f64: NULL pointer argument");
  if (!enable_cyclic_x) return VG_OK;
  return launch_cyclic_x(layout_of(dom), arr, nullptr, as_stream(stream));
}

extern "C" int vg_isoneutral_streamfunction_f64(const VgDomain *dom, const double *K_gm, const double *Ai_ez,
                                                const double *Ai_nz, long long ai_stride_p, long long ai_stride_r,
                                                double *B1_gm, double *B2_gm, void *stream) {
  clear_error();
  int st = validate_domain(dom);
  if (st) return st;
  if (!K_gm || !Ai_ez || !Ai_nz || !B1_gm || !B2_gm)
    return fail(VG_ERR_ARG, "vg_isoneutral_streamfunction_f64: NULL pointer argument");
  SfArgs a{layout_of(dom), K_gm, Ai_ez, Ai_nz, ai_stride_p, ai_stride_r, B1_gm, B2_gm};
  dim3 block(128), g((a.L.X + 127) / 128, a.L.Y, a.L.Z);
  streamfunction_kernel<<<g, block, 0, as_stream(stream)>>>(a);
  return check_launch("streamfunction_kernel");
}
