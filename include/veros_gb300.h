/*
 * veros_gb300 — C ABI of the GB300 (sm_103a) isoneutral mixing path.
 *
 * Plain pointers and sizes; no framework types. Every entry point returns an
 * int status (VG_OK on success) and never exits the process; the message of
 * the last failure on the calling thread is available from vg_last_error().
 * All work is enqueued on the caller's CUDA stream (passed as void*, a
 * cudaStream_t; NULL = legacy default stream) and no call synchronises the
 * host, except where stated.
 *
 * Device layout of one domain ("canonical layout"): a 3-D field f(i, j, k)
 * with i in [0, X), j in [0, Y), k in [0, Z) lives at
 *     base[i + j * pitch + k * plane]
 * (x fastest). X = nx + 4 and Y = ny + 4 include the two halo cells on each
 * side; k = 0 is the bottom level. Fields with a time axis are passed as the
 * pointer of one level. The (2, 2) tensors Ai_* hold component (p, r)
 * (p = ip or jp, r = kr) at base + p * ai_stride_p + r * ai_stride_r.
 * kbot is an int32 (X, Y) plane with the same pitch. The four boolean masks
 * are packed into one byte per cell (bit 0 T, bit 1 U, bit 2 V, bit 3 W).
 */
#ifndef VEROS_GB300_H
#define VEROS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  VG_OK = 0,
  VG_ERR_SHAPE = 1,       /* extents out of range or inconsistent */
  VG_ERR_STRIDE = 2,      /* pitch/plane/component strides not usable */
  VG_ERR_ARG = 3,         /* NULL pointer or bad flag */
  VG_ERR_LAUNCH = 4,      /* CUDA launch or runtime error */
  VG_ERR_TIMEOUT = 5,     /* a bounded device wait gave up */
  VG_ERR_UNSUPPORTED = 6, /* setting outside what the kernels implement */
  VG_ERR_SCRATCH = 7      /* scratch buffer too small */
};

#define VG_MASK_T 1u
#define VG_MASK_U 2u
#define VG_MASK_V 4u
#define VG_MASK_W 8u

typedef struct VgDomain {
  int X, Y, Z;          /* extents including halos */
  long long pitch;      /* elements between consecutive j rows (>= X) */
  long long plane;      /* elements between consecutive k levels (>= pitch * Y) */
} VgDomain;

typedef struct VgGrid {
  const double *dxt, *dxu;               /* length X */
  const double *dyt, *dyu, *cost, *cosu; /* length Y */
  const double *dzt, *dzw, *zt;          /* length Z */
} VgGrid;

typedef struct VgIsoSettings {
  double iso_slopec, iso_dslope, K_iso_steep, dt_tracer, grav, rho_0;
  int eq_of_state_type;        /* 1..4 */
  int enable_conserve_energy;  /* 0/1 */
} VgIsoSettings;

typedef struct VgTensorFields {
  double *K_11, *K_22, *K_33;
  double *Ai_ez, *Ai_nz, *Ai_bx, *Ai_by;
  long long ai_stride_p, ai_stride_r;
} VgTensorFields;

/* Derived fields of the split form (same layout, float elements). The
 * tracers stay FP64 in the split form too: the slopes divide by vertical
 * density gradients, differences of nearby tracer values, which FP32 storage
 * would already blur at the 1e-6 K level. */
typedef struct VgTensorFieldsF32 {
  float *K_11, *K_22, *K_33;
  float *Ai_ez, *Ai_nz, *Ai_bx, *Ai_by;
  long long ai_stride_p, ai_stride_r;
} VgTensorFieldsF32;

typedef struct VgTracerArgsF32 {
  const double *tr_tau;
  double *tr_taup1;
  float *dtracer_iso;
  const float *int_drhodX_tau;
  float *P_diss;
} VgTracerArgsF32;

typedef struct VgTracerArgs {
  const double *tr_tau;         /* tracer at level tau (read) */
  double *tr_taup1;             /* tracer at level taup1 (read, updated) */
  double *dtracer_iso;          /* dtemp_iso or dsalt_iso (updated) */
  const double *int_drhodX_tau; /* int_drhodT or int_drhodS at tau; energy branch only */
  double *P_diss;               /* P_diss_iso (iso) or P_diss_skew (skew); energy branch only */
} VgTracerArgs;

/* Message of the last failure on this thread ("" if none). */
const char *vg_last_error(void);
/* Library version string. */
const char *vg_version(void);

/* Pack four bool (0/1 byte) masks in canonical layout into the mask byte plane.
 * No reference counterpart: Veros keeps maskT/U/V/W as separate bool arrays
 * (veros/variables.py:255-292); packing is this library's layout choice. */
int vg_pack_masks(const VgDomain *dom, const uint8_t *maskT, const uint8_t *maskU,
                  const uint8_t *maskV, const uint8_t *maskW, uint8_t *mask_bits, void *stream);

/* Replaces veros.core.isoneutral.isoneutral_diffusion_pre
 * (veros/core/isoneutral/isoneutral.py:18-229): slopes, taper and the
 * diffusion tensor. Writes K_11[1:-2,2:-2,:], K_22[2:-2,1:-2,:],
 * K_33[2:-2,2:-2,:-1] and K_33[...,-1] = 0, Ai_ez/Ai_nz/Ai_bx/Ai_by on the
 * reference's sub-ranges; every other cell of the outputs is left untouched. */
int vg_isoneutral_pre_f64(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set,
                          const double *temp_tau, const double *salt_tau, const double *K_iso,
                          const uint8_t *mask_bits, const VgTensorFields *out, void *stream);

/* FP32/FP64-split form of vg_isoneutral_pre_f64: derived fields (K_iso in,
 * K and Ai out) and their arithmetic in FP32; tracer gradients, the vertical
 * density gradients (the clamped slope denominators), the slope numerators
 * and the slopes in FP64; the taper evaluated in FP32 from the FP64 slope.
 * Tracers and grid stay FP64. No reference counterpart (the reference runs in
 * its float_type throughout). */
int vg_isoneutral_pre_f32split(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set,
                               const double *temp_tau, const double *salt_tau, const float *K_iso,
                               const uint8_t *mask_bits, const VgTensorFieldsF32 *out, void *stream);

/* Scratch bytes vg_isoneutral_diffusion_f64 needs for one domain. */
size_t vg_isoneutral_diffusion_scratch_bytes(const VgDomain *dom);

/* Replaces veros.core.isoneutral.isoneutral_diffusion (skew = 0,
 * veros/core/isoneutral/diffusion.py:286-295) and isoneutral_skew_diffusion
 * (skew = 1, :298-307) through isoneutral_diffusion_kernel (:210-283):
 * explicit flux divergence, implicit vertical K_33 solve (iso only),
 * dtracer_iso update and, when enable_conserve_energy, the P_diss update.
 * K_field is K_iso (iso) or K_gm (skew). */
int vg_isoneutral_diffusion_f64(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set,
                                const VgTensorFields *ten, const double *K_field,
                                const uint8_t *mask_bits, const int32_t *kbot,
                                const VgTracerArgs *tr, int skew,
                                void *scratch, size_t scratch_bytes, void *stream);

/* Diffusion of temp and then salt with one shared factorisation of the
 * implicit K_33 system (both tracers solve the same matrix): the same results
 * as vg_isoneutral_diffusion_f64 for temp followed by salt
 * (veros/core/thermodynamics.py:431-432), with fewer FP64 operations. Scratch:
 * vg_isoneutral_diffusion_pair_scratch_bytes. */
size_t vg_isoneutral_diffusion_pair_scratch_bytes(const VgDomain *dom);
int vg_isoneutral_diffusion_pair_f64(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set,
                                     const VgTensorFields *ten, const double *K_iso,
                                     const uint8_t *mask_bits, const int32_t *kbot,
                                     const VgTracerArgs *temp, const VgTracerArgs *salt,
                                     void *scratch, size_t scratch_bytes, void *stream);

/* FP32/FP64-split forms of the diffusion calls: fluxes and divergence in FP32
 * from FP64 tracer differences, the tracer update and the implicit K_33 solve
 * in FP64; tendencies and dissipation stored FP32.
 * Same scratch sizes as the FP64 calls (of which they use half). */
int vg_isoneutral_diffusion_f32split(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set,
                                     const VgTensorFieldsF32 *ten, const float *K_field,
                                     const uint8_t *mask_bits, const int32_t *kbot,
                                     const VgTracerArgsF32 *tr, int skew,
                                     void *scratch, size_t scratch_bytes, void *stream);
int vg_isoneutral_diffusion_pair_f32split(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set,
                                          const VgTensorFieldsF32 *ten, const float *K_iso,
                                          const uint8_t *mask_bits, const int32_t *kbot,
                                          const VgTracerArgsF32 *temp, const VgTracerArgsF32 *salt,
                                          void *scratch, size_t scratch_bytes, void *stream);

/* The pair calls with the implicit solve's interior columns taken in the
 * order column_order (indices (i-2) + (j-2)*(X-4), a permutation of all
 * (X-4)*(Y-4) interior columns; deepest first keeps the lanes of a warp on
 * columns of similar length; NULL: natural order). Results are identical to
 * the unordered calls. */
int vg_isoneutral_diffusion_pair_ordered_f64(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set,
                                             const VgTensorFields *ten, const double *K_iso,
                                             const uint8_t *mask_bits, const int32_t *kbot,
                                             const VgTracerArgs *temp, const VgTracerArgs *salt,
                                             const int32_t *column_order, void *scratch, size_t scratch_bytes,
                                             void *stream);
int vg_isoneutral_diffusion_pair_ordered_f32split(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set,
                                                  const VgTensorFieldsF32 *ten, const float *K_iso,
                                                  const uint8_t *mask_bits, const int32_t *kbot,
                                                  const VgTracerArgsF32 *temp, const VgTracerArgsF32 *salt,
                                                  const int32_t *column_order, void *scratch,
                                                  size_t scratch_bytes, void *stream);

/* Scratch-free variant of vg_isoneutral_diffusion_f64 for callers that cannot
 * allocate device memory (an XLA custom-call or FFI handler working only with
 * the buffers it is handed, or a host model that fixes its device memory at
 * start-up). No counterpart in the reference. The scratch is a 32 MiB
 * file-scope device array held by every GPU that loads the library; domains
 * needing more (3 * plane * Z * 8 bytes) get VG_ERR_SCRATCH. The first call
 * on a device looks up the array's address (make it before any stream
 * capture); all calls share the array, so calls overlapping on the GPU race.
 * Allocates nothing. */
int vg_isoneutral_diffusion_noalloc_f64(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set,
                                        const VgTensorFields *ten, const double *K_field,
                                        const uint8_t *mask_bits, const int32_t *kbot,
                                        const VgTracerArgs *tr, int skew, void *stream);
/* Bytes of the static scratch array vg_isoneutral_diffusion_noalloc_f64 uses. */
size_t vg_isoneutral_diffusion_noalloc_capacity(void);
/* Forget the cached device addresses of that array (no GPU work). The address
 * belongs to a device's context: a caller that resets a device
 * (cudaDeviceReset unloads the library's device code) calls this before the
 * next scratch-free call on it. No counterpart in the reference. */
void vg_isoneutral_diffusion_noalloc_reset(void);

/* Fields of one rollout step (vg_isoneutral_step_f64). */
typedef struct VgStepFields {
  const double *temp_tau;
  double *temp_taup1;
  const double *salt_tau;
  double *salt_taup1;
  const double *K_iso;
  const uint8_t *mask_bits;
  const int32_t *kbot;
  VgTensorFields ten;
  double *dtemp_iso, *dsalt_iso;
  const double *int_drhodT_tau, *int_drhodS_tau; /* energy branch only */
  double *P_diss_iso;                            /* may be NULL without the energy branch */
  /* optional (NULL: natural order): the interior columns, as indices
   * (i-2) + (j-2)*(X-4), in the order the implicit solve takes them; deepest
   * first keeps the lanes of a warp on columns of similar length. A
   * permutation of all (X-4)*(Y-4) interior columns. */
  const int32_t *column_order;
  /* optional (NULL: equal counts of tile-levels per CTA): the work shares of
   * the pre and flux kernels' CTAs, written by vg_isoneutral_step_shares for
   * these masks on this device, n + 1 tile-level starts each, with the n of
   * vg_isoneutral_step_shares_size; a kernel whose CTA count is not its n
   * takes equal counts instead. Only the distribution of the work depends on
   * them, not the results. */
  const long long *pre_shares, *flux_shares;
  int pre_shares_n, flux_shares_n;
} VgStepFields;

/* One isoneutral step as the reference's caller runs it
 * (veros/core/thermodynamics.py:226-241 with zero advection, then :425-432):
 * tr[taup1] = tr[tau] * maskT for temp and salt; dtemp_iso = dsalt_iso = 0
 * and P_diss_iso = 0 (if given; needed with the energy branch); pre; diffusion of temp; diffusion
 * of salt. The caller rotates the time levels (veros/veros.py:321-322).
 * Scratch as for vg_isoneutral_diffusion_pair_f64. */
int vg_isoneutral_step_f64(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set,
                           const VgStepFields *f, void *scratch, size_t scratch_bytes, void *stream);

/* Work shares of a step's persistent pre and flux kernels (no reference
 * counterpart). precision 0: vg_isoneutral_step_f64, 1: the split form.
 * With equal counts of tile-levels per CTA, CTAs holding dry tile-levels
 * finish early; the shares give each CTA an equal part of a + (busy warps)
 * summed over its tile-levels, the busy warps of a level being the wet points
 * of the tile / 32, rounded up. vg_isoneutral_step_shares_size gives the
 * number of CTAs of each kernel (0 for a kernel that takes no shares: one
 * CTA per tile on large domains, and the split form's flux kernel) and the
 * scratch bytes; vg_isoneutral_step_shares writes n + 1 tile-level starts
 * per kernel into device arrays, on the stream, from the packed masks.
 * Recompute them when the masks change; stale shares only cost time. */
int vg_isoneutral_step_shares_size(const VgDomain *dom, int precision, int *n_pre, int *n_flux,
                                   size_t *scratch_bytes);
int vg_isoneutral_step_shares(const VgDomain *dom, int precision, const uint8_t *mask_bits, long long *pre_starts,
                              long long *flux_starts, void *scratch, size_t scratch_bytes, void *stream);

/* FP32 fields of one rollout step of the split form. */
typedef struct VgStepFieldsF32 {
  const double *temp_tau;
  double *temp_taup1;
  const double *salt_tau;
  double *salt_taup1;
  const float *K_iso;
  const uint8_t *mask_bits;
  const int32_t *kbot;
  VgTensorFieldsF32 ten;
  float *dtemp_iso, *dsalt_iso;
  const float *int_drhodT_tau, *int_drhodS_tau;
  float *P_diss_iso;
  const int32_t *column_order;               /* as in VgStepFields */
  const long long *pre_shares, *flux_shares; /* as in VgStepFields */
  int pre_shares_n, flux_shares_n;
} VgStepFieldsF32;

/* One isoneutral step of the FP32/FP64-split form (see vg_isoneutral_step_f64). */
int vg_isoneutral_step_f32split(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set,
                                const VgStepFieldsF32 *f, void *scratch, size_t scratch_bytes, void *stream);
int vg_isoneutral_step_prepare_f32split(const VgDomain *dom, const VgStepFieldsF32 *f, void *stream);

/* The new time level and zeroed tendencies of a step on every cell, as a
 * separate kernel (what vg_isoneutral_step_f64 fuses into its flux kernel).
 * With vg_isoneutral_pre_f64 and vg_isoneutral_diffusion_pair_ordered_f64 it
 * makes the unfused form of the step, with the same results bit for bit. */
int vg_isoneutral_step_prepare_f64(const VgDomain *dom, const VgStepFields *f, void *stream);

/* One stage of vg_isoneutral_step_f64, for callers that time or interleave
 * the stages; stages 0, 1, 2 in order make one step. 0: the new time level
 * and zeroed tendencies on the two-cell rim of every level; 1: pre; 2:
 * diffusion of temp and salt, whose flux kernel also prepares the interior
 * cells (each wet cell's new level and tendency written once, from tr[tau]
 * and its flux divergence, instead of a separate preparation followed by a
 * read-modify-write). Stage 2 reads the tensor stage 1 wrote for the same
 * masks: the faces of a cell without mask bits carry zero coefficients
 * there, and the flux kernel does not read them. */
int vg_isoneutral_step_stage_f64(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set,
                                 const VgStepFields *f, void *scratch, size_t scratch_bytes, int stage,
                                 void *stream);
int vg_isoneutral_step_stage_f32split(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set,
                                      const VgStepFieldsF32 *f, void *scratch, size_t scratch_bytes, int stage,
                                      void *stream);

/* Replaces veros.core.thermodynamics.vertmix_tempsalt
 * (veros/core/thermodynamics.py:248-300): implicit vertical mixing of temp and
 * salt at level taup1 with the diffusivity kappaH and the surface forcing
 * forc_temp_surface / forc_salt_surface ((X, Y) planes, canonical pitch);
 * writes the new levels and dtemp_vmix / dsalt_vmix on the whole array.
 * enable_cyclic_x (settings.enable_cyclic_x): end with the closing boundary
 * exchange of the new temp and salt levels (thermodynamics.py:292-298) as one
 * process runs it, the periodic x-halo copy of vg_enforce_boundaries_f64.
 * Domain decompositions over several processes are not supported. */
int vg_vertmix_tempsalt_f64(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set,
                            const double *kappaH, const int32_t *kbot, double *temp_taup1, double *salt_taup1,
                            const double *forc_temp_surface, const double *forc_salt_surface,
                            double *dtemp_vmix, double *dsalt_vmix, int enable_cyclic_x, void *stream);

/* Replaces veros.core.utilities.enforce_boundaries (veros/core/utilities.py:7-21)
 * for one process: with enable_cyclic_x, arr[-2:, ...] = arr[2:4, ...] and then
 * arr[:2, ...] = arr[-4:-2, ...] over every (j, k) of one (X, Y, Z) field in
 * the canonical layout; without it nothing is done (as the reference). */
int vg_enforce_boundaries_f64(const VgDomain *dom, double *arr, int enable_cyclic_x, void *stream);

/* Replaces isoneutral_diag_streamfunction_kernel
 * (veros/core/isoneutral/isoneutral.py:232-254): B1_gm[2:-2,1:-2] and
 * B2_gm[1:-2,2:-2] from K_gm and Ai_nz / Ai_ez; other cells untouched. */
int vg_isoneutral_streamfunction_f64(const VgDomain *dom, const double *K_gm, const double *Ai_ez,
                                     const double *Ai_nz, long long ai_stride_p, long long ai_stride_r,
                                     double *B1_gm, double *B2_gm, void *stream);

/* Host-layout conversion for callers that exchange fields with the reference's
 * (X, Y, Z) arrays in NumPy's default C order (z fastest): nfields (1..8)
 * FP64 fields from src[n] to dst[n], element (i, j, k) at
 * (i*Y + j)*Z + k on the reference side and i + j*pitch + k*plane on the
 * canonical side. No reference counterpart (Veros keeps one layout). */
int vg_layout_to_canonical_f64(const VgDomain *dom, int nfields, const double *const *src, double *const *dst,
                               void *stream);
int vg_layout_from_canonical_f64(const VgDomain *dom, int nfields, const double *const *src, double *const *dst,
                                 void *stream);

/* ---- Batched ensemble ------------------------------------------------------
 * One isoneutral step of many domains (uneven extents and kbot) with one
 * persistent launch per stage. No reference counterpart: Veros steps one
 * domain per process. Each member gives its domain, grid, settings and its
 * step fields for the three time-level phases (phase p = the pointers after p
 * rotations). The energy branch is not batched (VG_ERR_UNSUPPORTED). */
typedef struct VgEnsembleTuning {
  int pre_rows;       /* columns per CTA / 32 of the slope kernel: 4 or 8 */
  int pre_kchunk;     /* levels per item of the slope kernel, 0 = whole column, -1 = equal shares of
                         all members' tile-levels per resident CTA (static, no work counter) */
  int flux_rows;      /* columns per CTA / 32 of the flux kernel: 4 or 8 */
  int flux_kchunk;    /* levels per item of the flux kernel, as pre_kchunk */
  int solve_threads;  /* columns per CTA of the implicit solve: 32 or 64 */
} VgEnsembleTuning;

typedef struct VgEnsembleMember {
  VgDomain dom;
  VgGrid grid;
  VgIsoSettings set;
  VgStepFields phase[3];
} VgEnsembleMember;

typedef struct VgEnsembleMemberF32 {
  VgDomain dom;
  VgGrid grid;
  VgIsoSettings set;
  VgStepFieldsF32 phase[3];
} VgEnsembleMemberF32;

/* Build the device tables (allocates device memory); *handle receives the ensemble. */
int vg_ensemble_create_f64(const VgEnsembleMember *members, int n, const VgEnsembleTuning *tuning, void **handle);
int vg_ensemble_create_f32split(const VgEnsembleMemberF32 *members, int n, const VgEnsembleTuning *tuning,
                                void **handle);
/* Re-tile the work lists (the autotuner's knob). */
int vg_ensemble_tune(void *handle, const VgEnsembleTuning *tuning);
/* One step of every member at time-level phase 0..2: a counter reset and four launches. */
int vg_ensemble_step(void *handle, int phase, void *stream);
int vg_ensemble_destroy(void *handle);

/* Adjoint of one FP64 step of vg_isoneutral_step_f64 (no reference
 * counterpart: Veros defines no derivative of this path). The step maps
 * (temp, salt, K_iso) to (temp_new, salt_new); given dL/dtemp_new and
 * dL/dsalt_new this writes dL/dtemp and dL/dsalt and ADDS dL/dK_iso into
 * gK_iso (so a rollout accumulates it over its steps). temp/salt and
 * temp_new/salt_new are the step's input and output levels (the caller's
 * per-step checkpoints); the diffusion tensor is recomputed from them. The
 * energy branch does not change the tracers and takes no part. All fields
 * canonical; the gradients may not alias the inputs. */
typedef struct VgAdjointFields {
  const double *temp, *salt;
  const double *temp_new, *salt_new;
  const double *K_iso;
  const uint8_t *mask_bits;
  const int32_t *kbot;
  const double *gtemp_new, *gsalt_new;
  double *gtemp, *gsalt;
  double *gK_iso;
  /* optional (NULL: natural order): the interior columns in the order the
   * transposed solve takes them, as VgStepFields.column_order */
  const int32_t *column_order;
} VgAdjointFields;

size_t vg_isoneutral_step_adjoint_scratch_bytes(const VgDomain *dom);
int vg_isoneutral_step_adjoint_f64(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set,
                                   const VgAdjointFields *f, void *scratch, size_t scratch_bytes, void *stream);

/* Replaces veros.core.utilities.solve_implicit (veros/core/utilities.py:51-59)
 * and veros.core.operators.solve_tridiagonal (veros/core/operators.py:60-77,
 * :102-156). nsys columns of nz levels; element (s, k) of every array is at
 * s_x * (s % nsx) + s_y * (s / nsx) + s_z * k with nsys = nsx * nsy.
 * water/edge are 0/1 bytes as produced by create_water_masks
 * (veros/core/utilities.py:38-48): per column, water is k >= ks and edge is
 * k == ks. b_edge/d_edge may be NULL. Outside water the output is 0.
 * Columns whose masks do not have that form are counted into *bad_columns
 * (device int, may be NULL) and solved over their water cells only.
 * Elimination uses partial pivoting, as LAPACK dgtsv does. out may not
 * overlap an input (VG_ERR_ARG). */
int vg_solve_implicit_f64(int nsx, int nsy, int nz, long long s_x, long long s_y, long long s_z,
                          const double *a, const double *b, const double *c, const double *d,
                          const uint8_t *water, const uint8_t *edge,
                          const double *b_edge, const double *d_edge, double *out,
                          int *bad_columns, void *stream);

/* The same drop-in for float32 systems (runtime_settings.float_type =
 * "float32", veros/runtime.py:93). The reference's NumPy solve passes float32
 * arrays to LAPACK dgtsv, which computes on float64 copies, and stores the
 * solution into a float32 array (veros/core/operators.py:64, :75-76): this
 * call widens each entry to double, eliminates in double in dgtsv's order
 * and rounds each solution value to float once. */
int vg_solve_implicit_f32(int nsx, int nsy, int nz, long long s_x, long long s_y, long long s_z,
                          const float *a, const float *b, const float *c, const float *d,
                          const uint8_t *water, const uint8_t *edge,
                          const float *b_edge, const float *d_edge, float *out,
                          int *bad_columns, void *stream);

/* Drop-in for the XLA GPU custom-call targets tdma_cuda_double / tdma_cuda_float
 * (veros/core/special/cuda_tdma_kernels.cu:103-111, registered in
 * veros/core/special/tdma_.py:35-37): buffers = {a, b, c, d, out, workspace},
 * opaque = {int num_systems; int system_depth}, operands system-fastest
 * ((k, s) at k * num_systems + s). On error the message is kept for
 * vg_last_error() instead of exiting the process. The workspace is not used. */
void vg_tdma_cuda_double(void *stream, void **buffers, const char *opaque, size_t opaque_len);
void vg_tdma_cuda_float(void *stream, void **buffers, const char *opaque, size_t opaque_len);

#ifdef __cplusplus
}
#endif

#endif /* VEROS_GB300_H */
