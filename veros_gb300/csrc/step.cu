// One isoneutral step of a rollout as a single C call: the caller-side
// sequence of veros/core/thermodynamics.py:226-241 (zero advection: the new
// level is the old one, masked) and :425-432 (zero the iso tendencies, pre,
// diffusion of temp then salt). Time levels rotate on the host by swapping
// the level pointers (veros/veros.py:321-322).
#include "common.cuh"

namespace vg {
namespace {

template <typename F>
__global__ void prepare_kernel(Layout L, const uint8_t *__restrict__ m, const double *__restrict__ T0, double *T1,
                               const double *__restrict__ S0, double *S1, F *dT, F *dS, F *P) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y, k = blockIdx.z;
  if (i >= L.X) return;
  const long long o = L.at(i, j, k);
  const double mT = (__ldg(m + o) & VG_MASK_T) ? 1.0 : 0.0;
  T1[o] = T0[o] * mT;
  S1[o] = S0[o] * mT;
  dT[o] = F(0.0);
  dS[o] = F(0.0);
  if (P) P[o] = F(0.0);
}

template <typename F, typename Fields>
int prepare(const VgDomain *dom, const Fields *f, void *stream, const char *name) {
  clear_error();
  int st = validate_domain(dom);
  if (st) return st;
  if (!f || !f->temp_tau || !f->temp_taup1 || !f->salt_tau || !f->salt_taup1 || !f->mask_bits || !f->dtemp_iso ||
      !f->dsalt_iso)
    return fail(VG_ERR_ARG, "%s: NULL pointer argument", name);
  Layout L = layout_of(dom);
  dim3 block(128), g((L.X + 127) / 128, L.Y, L.Z);
  prepare_kernel<F><<<g, block, 0, as_stream(stream)>>>(L, f->mask_bits, f->temp_tau, f->temp_taup1, f->salt_tau,
                                                        f->salt_taup1, f->dtemp_iso, f->dsalt_iso, f->P_diss_iso);
  return check_launch("prepare_kernel");
}

}  // namespace
}  // namespace vg

using namespace vg;

extern "C" int vg_isoneutral_step_prepare_f64(const VgDomain *dom, const VgStepFields *f, void *stream) {
  return prepare<double>(dom, f, stream, "vg_isoneutral_step_prepare_f64");
}

extern "C" int vg_isoneutral_step_prepare_f32split(const VgDomain *dom, const VgStepFieldsF32 *f, void *stream) {
  return prepare<float>(dom, f, stream, "vg_isoneutral_step_prepare_f32split");
}

namespace vg {
namespace {

// The step's preparation of the cells the fused diffusion does not cover:
// the two-cell rim of every level (i < 2, i >= X-2, j < 2, j >= Y-2).
template <typename F>
// One thread per rim cell of a level: the two full rows at each end of y,
// then the two columns at each end of x on the rows between.
__global__ void prepare_rim_kernel(Layout L, const uint8_t *__restrict__ m, const double *__restrict__ T0,
                                   double *T1, const double *__restrict__ S0, double *S1, F *dT, F *dS, F *P) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y;
  if (r >= 4 * L.X + 4 * (L.Y - 4)) return;
  int i, j;
  if (r < 4 * L.X) {
    const int jr = r / L.X;
    i = r % L.X;
    j = jr < 2 ? jr : L.Y - 4 + jr;
  } else {
    const int q = r - 4 * L.X, c = q % 4;
    i = c < 2 ? c : L.X - 4 + c;
    j = 2 + q / 4;
  }
  const long long o = L.at(i, j, k);
  const double mT = (__ldg(m + o) & VG_MASK_T) ? 1.0 : 0.0;
  T1[o] = T0[o] * mT;
  S1[o] = S0[o] * mT;
  dT[o] = F(0.0);
  dS[o] = F(0.0);
  if (P) P[o] = F(0.0);
}

// Stage 0: the rim's preparation; 1: pre; 2: diffusion of temp and salt with
// the interior's preparation fused into the flux kernel. Together the same
// results as the separate preparation, pre and diffusion, bit for bit.
template <typename F, typename Fields, typename TrA>
int step_stage(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set, const Fields *f, void *scratch,
               size_t scratch_bytes, int stage, void *stream, const char *name) {
  clear_error();
  int st = validate_domain(dom);
  if (st) return st;
  if (!f || !set) return fail(VG_ERR_ARG, "%s: NULL pointer argument", name);
  if (set->enable_conserve_energy && (!f->P_diss_iso || !f->int_drhodT_tau || !f->int_drhodS_tau))
    return fail(VG_ERR_ARG, "enable_conserve_energy needs P_diss_iso and int_drhodT/S");
  if (stage == 0) {
    if (!f->temp_tau || !f->temp_taup1 || !f->salt_tau || !f->salt_taup1 || !f->mask_bits || !f->dtemp_iso ||
        !f->dsalt_iso)
      return fail(VG_ERR_ARG, "%s: NULL pointer argument", name);
    const Layout L = layout_of(dom);
    const int nrim = 4 * L.X + 4 * (L.Y - 4);
    prepare_rim_kernel<F><<<dim3((nrim + 127) / 128, L.Z), 128, 0, as_stream(stream)>>>(
        L, f->mask_bits, f->temp_tau, f->temp_taup1, f->salt_tau, f->salt_taup1, f->dtemp_iso, f->dsalt_iso,
        f->P_diss_iso);
    return check_launch("prepare_rim_kernel");
  }
  if (stage == 1) {
    if constexpr (sizeof(F) == sizeof(double))
      return pre_for_step_f64(dom, grid, set, f->temp_tau, f->salt_tau, f->K_iso, f->mask_bits, &f->ten,
                              f->pre_shares, f->pre_shares_n, stream);
    else
      return pre_for_step_f32split(dom, grid, set, f->temp_tau, f->salt_tau, f->K_iso, f->mask_bits, &f->ten,
                                   f->pre_shares, f->pre_shares_n, stream);
  }
  if (stage != 2) return fail(VG_ERR_ARG, "%s: stage %d not in 0..2", name, stage);
  TrA trT{f->temp_tau, f->temp_taup1, f->dtemp_iso, f->int_drhodT_tau, f->P_diss_iso};
  TrA trS{f->salt_tau, f->salt_taup1, f->dsalt_iso, f->int_drhodS_tau, f->P_diss_iso};
  if constexpr (sizeof(F) == sizeof(double))
    return diffusion_pair_ordered_f64(dom, grid, set, &f->ten, f->K_iso, f->mask_bits, f->kbot, &trT, &trS,
                                      f->column_order, scratch, scratch_bytes, stream, 1, f->flux_shares,
                                      f->flux_shares_n);
  else
    return diffusion_pair_ordered_f32split(dom, grid, set, &f->ten, f->K_iso, f->mask_bits, f->kbot, &trT, &trS,
                                           f->column_order, scratch, scratch_bytes, stream, 1, f->flux_shares,
                                           f->flux_shares_n);
}

}  // namespace
}  // namespace vg

extern "C" int vg_isoneutral_step_stage_f64(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set,
                                            const VgStepFields *f, void *scratch, size_t scratch_bytes, int stage,
                                            void *stream) {
  return step_stage<double, VgStepFields, VgTracerArgs>(dom, grid, set, f, scratch, scratch_bytes, stage, stream,
                                                        "vg_isoneutral_step_stage_f64");
}

extern "C" int vg_isoneutral_step_stage_f32split(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set,
                                                 const VgStepFieldsF32 *f, void *scratch, size_t scratch_bytes,
                                                 int stage, void *stream) {
  return step_stage<float, VgStepFieldsF32, VgTracerArgsF32>(dom, grid, set, f, scratch, scratch_bytes, stage,
                                                             stream, "vg_isoneutral_step_stage_f32split");
}

extern "C" int vg_isoneutral_step_f64(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set,
                                      const VgStepFields *f, void *scratch, size_t scratch_bytes, void *stream) {
  int st = 0;
  for (int stage = 0; stage < 3 && !st; ++stage)
    st = vg_isoneutral_step_stage_f64(dom, grid, set, f, scratch, scratch_bytes, stage, stream);
  return st;
}

extern "C" int vg_isoneutral_step_f32split(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set,
                                           const VgStepFieldsF32 *f, void *scratch, size_t scratch_bytes,
                                           void *stream) {
  int st = 0;
  for (int stage = 0; stage < 3 && !st; ++stage)
    st = vg_isoneutral_step_stage_f32split(dom, grid, set, f, scratch, scratch_bytes, stage, stream);
  return st;
}
