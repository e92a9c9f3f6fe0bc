// The two neighbours of the isoneutral path (FP64):
//
// * vg_vertmix_tempsalt_f64: implicit vertical mixing of temp and salt with
//   the diffusivity kappaH and the surface forcing
//   (veros/core/thermodynamics.py:248-300). One thread per column; temp and
//   salt share one Thomas factorisation of the matrix (the same system as the
//   isoneutral implicit part with kappaH for K_33, diffusion.py:154-164); the
//   surface forcing enters the top row's right-hand side. dtemp_vmix and
//   dsalt_vmix are written on the whole array ((new - old)/dt, zero outside
//   the water columns). Single-process, non-cyclic: the closing boundary
//   exchange (thermodynamics.py:292-298) is then a no-op.
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

__global__ void __launch_bounds__(64) vertmix_kernel(VmixArgs a) {
  extern __shared__ double smem[];
  const Layout &L = a.L;
  const int Z = L.Z;
  const int t = threadIdx.x, nb = blockDim.x;
  double *cps = smem;
  double *dps = smem + (size_t)Z * nb;  // [r][k][thread]
  const int col = blockIdx.x * nb + t;
  if (col >= L.X * L.Y) return;
  const int i = col % L.X, j = col / L.X;
  const long long base = L.at2(i, j);
  const bool interior = i >= 2 && i < L.X - 2 && j >= 2 && j < L.Y - 2;
  const int ks = interior ? a.kbot[base] - 1 : -1;  // create_water_masks (utilities.py:38-48)
  // dtemp_vmix starts as the old level; outside the water cells the update is (old - old)/dt = 0
  for (int k = 0; k < (ks >= 0 && ks < Z ? ks : Z); ++k) {
    const long long o = base + (long long)k * L.plane;
    a.dvmix[0][o] = 0.0;
    a.dvmix[1][o] = 0.0;
  }
  if (ks < 0 || ks >= Z) return;

  double delta_prev = 0.0, cp = 0.0, dp[2] = {0.0, 0.0};
  for (int k = ks; k < Z; ++k) {
    const long long o = base + (long long)k * L.plane;
    const double dzt = a.g.dzt[k];
    const double delta = k < Z - 1 ? rmul(rdiv(a.dt, a.g.dzw[k]), a.kappaH[o]) : 0.0;
    const double ak = k == ks ? 0.0 : rdiv(-delta_prev, dzt);  // a_tri, zero at the edge (operators.py:72)
    const double bk = k == ks ? radd(1.0, rdiv(delta, dzt)) : radd(1.0, rdiv(radd(delta, delta_prev), dzt));
    const double ck = k < Z - 1 ? rdiv(-delta, dzt) : 0.0;
    const double den = 1.0 / (bk - ak * cp);
    cp = ck * den;
    cps[(size_t)k * nb + t] = cp;
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      double d = a.tr[r][o];
      if (k == Z - 1) d = radd(d, rdiv(rmul(a.dt, a.forc[r][base]), dzt));  // thermodynamics.py:279, :287
      dp[r] = (d - ak * dp[r]) * den;
      dps[((size_t)r * Z + k) * nb + t] = dp[r];
    }
    delta_prev = delta;
  }
  double x[2] = {0.0, 0.0};
  const double inv_dt = 1.0 / a.dt;
  for (int k = Z - 1; k >= ks; --k) {
    const long long o = base + (long long)k * L.plane;
    const double c = cps[(size_t)k * nb + t];
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      x[r] = dps[((size_t)r * Z + k) * nb + t] - c * x[r];
      const double old = a.tr[r][o];
      a.tr[r][o] = x[r];
      a.dvmix[r][o] = (x[r] - old) * inv_dt;  // thermodynamics.py:289-290
    }
  }
}

struct SfArgs {
  Layout L;
  const double *__restrict__ Kgm;
  const double *__restrict__ Aez;
  const double *__restrict__ Anz;
  long long sp, sr;
  double *B1, *B2;
};

// K_gm edge-padded in z (utilities.py:24-35), averaged onto the face
__device__ __forceinline__ double kgm_face(const SfArgs &a, long long o, long long dn, int k) {
  const long long up = k > 0 ? -a.L.plane : 0;  // pad: level k-1 clamps to 0
  return 0.25 * (a.Kgm[o] + a.Kgm[o + up] + a.Kgm[o + dn] + a.Kgm[o + dn + up]);
}

__global__ void __launch_bounds__(128) streamfunction_kernel(SfArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y, k = blockIdx.z;
  const Layout &L = a.L;
  if (i >= L.X) return;
  const long long o = L.at(i, j, k);
  // B2_gm[1:-2, 2:-2] (isoneutral.py:241-244)
  if (i >= 1 && i < L.X - 2 && j >= 2 && j < L.Y - 2) {
    const double diffloc = kgm_face(a, o, 1, k);
    const double s = a.Aez[o] + a.Aez[o + a.sr] + a.Aez[o + a.sp] + a.Aez[o + a.sp + a.sr];
    a.B2[o] = 0.25 * diffloc * s;
  }
  // B1_gm[2:-2, 1:-2] (isoneutral.py:249-252)
  if (i >= 2 && i < L.X - 2 && j >= 1 && j < L.Y - 2) {
    const double diffloc = kgm_face(a, o, L.pitch, k);
    const double s = a.Anz[o] + a.Anz[o + a.sr] + a.Anz[o + a.sp] + a.Anz[o + a.sp + a.sr];
    a.B1[o] = -0.25 * diffloc * s;
  }
}

}  // namespace
}  // namespace vg

using namespace vg;

extern "C" int vg_vertmix_tempsalt_f64(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set,
                                       const double *kappaH, const int32_t *kbot, double *temp_taup1,
                                       double *salt_taup1, const double *forc_temp_surface,
                                       const double *forc_salt_surface, double *dtemp_vmix, double *dsalt_vmix,
                                       void *stream) {
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
  const int nb = 64;
  const size_t smem = 3 * (size_t)a.L.Z * nb * sizeof(double);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(vertmix_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return fail(VG_ERR_LAUNCH, "vertmix_kernel smem %zu: %s", smem, cudaGetErrorString(e));
  }
  const int ncols = a.L.X * a.L.Y;
  vertmix_kernel<<<(ncols + nb - 1) / nb, nb, smem, as_stream(stream)>>>(a);
  return check_launch("vertmix_kernel");
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
