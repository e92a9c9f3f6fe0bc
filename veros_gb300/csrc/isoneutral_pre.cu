// Launchers and C entry points of the slope/tensor kernel (pre_kernels.cuh).
#include "pre_kernels.cuh"

using namespace vg;

namespace vg {
namespace {

using namespace detail;

// tiles of 32 x 8 columns (FP64: two CTAs of 8 warps per SM) or 32 x 4
// (split form: four CTAs of 4 warps, whose level barriers overlap); one CTA
// per tile on large domains, else every resident CTA with a share of the
// tile-levels. The FP64 form on 32 x 4 tiles measured 1.04 against 0.85 ms
// at 1 degree: its halo rows then cost more FP64 work than the overlapping
// barriers save.
template <typename F>
struct PreGeometry {
  static constexpr int TY = sizeof(F) == sizeof(double) ? 8 : 4, TX = 32;
  int nbx, nby, nc;
  bool per_tile;  // one CTA per tile (no shares)
  size_t smem;
};

template <typename F>
int pre_geometry(const Layout &L, PreGeometry<F> &g) {
  constexpr int TY = PreGeometry<F>::TY, TX = PreGeometry<F>::TX;
  g.nbx = (L.X - 3 + TX - 1) / TX;
  g.nby = (L.Y - 3 + TY - 1) / TY;
  g.smem = pre_smem_bytes<F, TY>(L.Z);
  cudaError_t e =
      cudaFuncSetAttribute(pre_span_kernel<F, TY>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g.smem);
  if (e != cudaSuccess) return fail(VG_ERR_LAUNCH, "pre_span_kernel smem %zu: %s", g.smem, cudaGetErrorString(e));
  g.nc = span_ctas(pre_span_kernel<F, TY>, TX * TY, g.smem, g.nbx * g.nby, L.Z, 8, &g.per_tile);
  if (g.nc < 1) return fail(VG_ERR_LAUNCH, "pre_span_kernel: occupancy query failed");
  return VG_OK;
}

template <typename F, typename Out>
int launch_pre(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set, const double *temp_tau,
               const double *salt_tau, const F *K_iso, const uint8_t *mask_bits, const Out *out, void *stream,
               const char *name, double *slopes = nullptr, const long long *starts = nullptr, int nstarts = 0) {
  clear_error();
  int st = validate_domain(dom);
  if (st) return st;
  if (!grid_complete(grid) || !set || !temp_tau || !salt_tau || !K_iso || !mask_bits || !out || !out->K_11 ||
      !out->K_22 || !out->K_33 || !out->Ai_ez || !out->Ai_nz || !out->Ai_bx || !out->Ai_by)
    return fail(VG_ERR_ARG, "%s: NULL pointer argument", name);
  if (set->eq_of_state_type < 1 || set->eq_of_state_type > 4)
    return fail(VG_ERR_UNSUPPORTED, "eq_of_state_type %d not implemented (1-4 are)", set->eq_of_state_type);
  if (!(set->iso_dslope != 0.0)) return fail(VG_ERR_ARG, "iso_dslope must be non-zero");
  if (dom->Z > 512) return fail(VG_ERR_SHAPE, "Z=%d above the 512 levels the per-CTA tables hold", dom->Z);
  PreArgs<F> a;
  a.L = layout_of(dom);
  a.g = grid_of(grid);
  a.eos_type = set->eq_of_state_type;
  a.slopec = set->iso_slopec;
  a.inv_dslope = 1.0 / set->iso_dslope;
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
  a.slopes = slopes;
  a.slope_field = (long long)a.L.plane * a.L.Z;
  a.stage_ok = pre_stage_ok(a);
  PreGeometry<F> g;
  if ((st = pre_geometry<F>(a.L, g))) return st;
  constexpr int TY = PreGeometry<F>::TY, TX = PreGeometry<F>::TX;
  a.kchunk = a.L.Z;
  // shares apply where the CTAs split the tile-levels (not one CTA per tile)
  const long long *sh = !g.per_tile && nstarts == g.nc ? starts : nullptr;
  pre_span_kernel<F, TY><<<g.nc, TX * TY, g.smem, as_stream(stream)>>>(a, g.nbx, g.nbx * g.nby, sh);
  return check_launch("pre_span_kernel");
}

}  // namespace

// The pre kernel's tiling on this device: tiles along x, tiles in all, and
// CTAs (as many as tiles where it runs one CTA per tile).
template <typename F>
int pre_span_plan(const VgDomain *dom, int *ntx, int *ntiles, int *nctas) {
  PreGeometry<F> g;
  const int st = pre_geometry<F>(layout_of(dom), g);
  if (st) return st;
  *ntx = g.nbx;
  *ntiles = g.nbx * g.nby;
  *nctas = g.per_tile ? 0 : g.nc;
  return VG_OK;
}
template int pre_span_plan<double>(const VgDomain *, int *, int *, int *);
template int pre_span_plan<float>(const VgDomain *, int *, int *, int *);

int pre_for_step_f64(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set, const double *temp_tau,
                     const double *salt_tau, const double *K_iso, const uint8_t *mask_bits,
                     const VgTensorFields *out, const long long *starts, int nstarts, void *stream) {
  return launch_pre<double>(dom, grid, set, temp_tau, salt_tau, K_iso, mask_bits, out, stream,
                            "vg_isoneutral_step_stage_f64 (pre)", nullptr, starts, nstarts);
}

int pre_for_step_f32split(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set, const double *temp_tau,
                          const double *salt_tau, const float *K_iso, const uint8_t *mask_bits,
                          const VgTensorFieldsF32 *out, const long long *starts, int nstarts, void *stream) {
  return launch_pre<float>(dom, grid, set, temp_tau, salt_tau, K_iso, mask_bits, out, stream,
                           "vg_isoneutral_step_stage_f32split (pre)", nullptr, starts, nstarts);
}

int pre_f64_with_slopes(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set, const double *temp_tau,
                        const double *salt_tau, const double *K_iso, const uint8_t *mask_bits,
                        const VgTensorFields *out, double *slopes, void *stream) {
  return launch_pre<double>(dom, grid, set, temp_tau, salt_tau, K_iso, mask_bits, out, stream, "pre (adjoint)",
                            slopes);
}

}  // namespace vg

extern "C" int vg_isoneutral_pre_f64(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set,
                                     const double *temp_tau, const double *salt_tau, const double *K_iso,
                                     const uint8_t *mask_bits, const VgTensorFields *out, void *stream) {
  return launch_pre<double>(dom, grid, set, temp_tau, salt_tau, K_iso, mask_bits, out, stream,
                            "vg_isoneutral_pre_f64");
}

extern "C" int vg_isoneutral_pre_f32split(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set,
                                          const double *temp_tau, const double *salt_tau, const float *K_iso,
                                          const uint8_t *mask_bits, const VgTensorFieldsF32 *out, void *stream) {
  return launch_pre<float>(dom, grid, set, temp_tau, salt_tau, K_iso, mask_bits, out, stream,
                           "vg_isoneutral_pre_f32split");
}
