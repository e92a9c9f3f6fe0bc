// Shared helpers of the veros_gb300 CUDA library: status handling, layout
// indexing and small device utilities.
#pragma once

#include <algorithm>

#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>

#include "../../include/veros_gb300.h"

namespace vg {

// Sets the thread's last-error message and returns `code`.
int fail(int code, const char *fmt, ...);
void clear_error();

// Converts a CUDA error after a launch into a status.
inline int check_launch(const char *what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(VG_ERR_LAUNCH, "%s: %s", what, cudaGetErrorString(e));
  return VG_OK;
}

int validate_domain(const VgDomain *dom);

// CTAs for a span kernel over ntiles x Z tile-levels (an even share per
// CTA). With at least four tiles per resident CTA slot, one CTA per tile: the
// hardware then runs neighbouring tiles side by side (their halo reads meet
// in L2) and its tail is short against the many waves. Otherwise every CTA
// the device holds at once, each with a share (at least min_levels
// tile-levels), so that no SM idles through a partial last wave. 0 on error.
// *per_tile (optional) tells which of the two.
template <typename K>
inline int span_ctas(K kernel, int threads, size_t smem, int ntiles, int Z, int min_levels,
                     bool *per_tile = nullptr) {
  int dev = 0, sms = 0, per = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, smem) != cudaSuccess || per < 1)
    return 0;
  const long long slots = (long long)sms * per;
  if (per_tile) *per_tile = ntiles >= 4 * slots;
  if (ntiles >= 4 * slots) return ntiles;
  const long long by_units = ((long long)ntiles * Z + min_levels - 1) / min_levels;
  return (int)std::max(1LL, std::min(slots, by_units));
}

// Index of this thread's "virtual" warp for kernels that hand their work to
// warps in a priority order (the busiest entries to virtual warp 0). Warp
// slot w of an SM issues on sub-partition w % 4, so co-resident CTAs whose
// busy warps have the same index would share the sub-partitions' FP64 pipes
// while others idle; the CTA's warp-slot base (%warpid of its warp 0, shared
// by the caller through shared memory) rotates the order so that the CTA in
// slot group g starts on sub-partition g * nw / 4. Only a performance
// choice: any permutation of the work over the warps gives the same results.
__device__ __forceinline__ unsigned hw_warp_slot() {
  unsigned w;
  asm volatile("mov.u32 %0, %%warpid;" : "=r"(w));
  return w;
}
__device__ __forceinline__ int virtual_warp(int warp, int nw, unsigned slot0) {
  // virtual warp v runs on physical warp p = v + c (mod nw), whose
  // sub-partition (slot0 + p) % 4 is then (v + g * nw / 4) % 4
  const int g = (int)(slot0 / (unsigned)nw);
  const int c = ((g * (nw / 4) - (int)(slot0 % 4u)) % nw + nw) % nw;
  return (warp - c + nw) % nw;
}

// Asynchronous 16-byte global -> shared copies (cp.async, bypassing L1):
// both addresses 16-byte aligned. wait_all waits for all of this thread's
// copies; other threads see them after a barrier.
__device__ __forceinline__ void cp_async16(void *smem_dst, const void *gsrc) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }
// A hint to bring the line holding p into L2 ahead of its load; p must point
// into an allocation (callers keep it in bounds).
__device__ __forceinline__ void prefetch_l2(const void *p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

struct Layout {
  int X, Y, Z;
  long long pitch, plane;
  __host__ __device__ __forceinline__ long long at(int i, int j, int k) const {
    return (long long)i + (long long)j * pitch + (long long)k * plane;
  }
  __host__ __device__ __forceinline__ long long at2(int i, int j) const {
    return (long long)i + (long long)j * pitch;
  }
};

inline Layout layout_of(const VgDomain *d) { return Layout{d->X, d->Y, d->Z, d->pitch, d->plane}; }

struct Grid {
  const double *dxt, *dxu, *dyt, *dyu, *cost, *cosu, *dzt, *dzw, *zt;
};

inline Grid grid_of(const VgGrid *g) {
  return Grid{g->dxt, g->dxu, g->dyt, g->dyu, g->cost, g->cosu, g->dzt, g->dzw, g->zt};
}

inline bool grid_complete(const VgGrid *g) {
  return g && g->dxt && g->dxu && g->dyt && g->dyu && g->cost && g->cosu && g->dzt && g->dzw && g->zt;
}

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// FP64 helpers that keep work off the FP64 pipe (one FP64 warp instruction
// costs tens of issue cycles on GB300; integer and FP32 instructions do not
// compete for that pipe).

// min(0, x) from the sign bit
__device__ __forceinline__ double fmin0(double x) { return __double_as_longlong(x) < 0 ? x : 0.0; }

// max(a, b) by an integer comparison of the bit patterns mapped to a monotone order
__device__ __forceinline__ double dmax(double a, double b) {
  long long ia = __double_as_longlong(a), ib = __double_as_longlong(b);
  ia ^= (ia >> 63) & 0x7FFFFFFFFFFFFFFFLL;
  ib ^= (ib >> 63) & 0x7FFFFFFFFFFFFFFFLL;
  return ia >= ib ? a : b;
}

// a > b by an integer comparison of the bit patterns mapped to a monotone order
__device__ __forceinline__ bool dgt(double a, double b) {
  long long ia = __double_as_longlong(a), ib = __double_as_longlong(b);
  ia ^= (ia >> 63) & 0x7FFFFFFFFFFFFFFFLL;
  ib ^= (ib >> 63) & 0x7FFFFFFFFFFFFFFFLL;
  return ia > ib;
}

// double -> float by truncating the mantissa (|x| within the FP32 normal range)
__device__ __forceinline__ float dtof_trunc(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
  const unsigned e = (unsigned)((int)((b >> 52) & 0x7FF) - 1023 + 127);
  const unsigned m = (unsigned)(b >> 29) & 0x7FFFFFu;
  return __uint_as_float(sign | (e << 23) | m);
}

// float -> double, exact for FP32 normal numbers
__device__ __forceinline__ double ftod(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
  const unsigned long long e = (unsigned long long)(((u >> 23) & 0xFFu) - 127 + 1023) << 52;
  const unsigned long long m = (unsigned long long)(u & 0x7FFFFFu) << 29;
  return __longlong_as_double((long long)(sign | e | m));
}

// 1/d for d of FP32-normal magnitude: an FP32 reciprocal of the truncated d,
// refined by two Newton-Raphson steps r <- r + r (1 - d r), each of which
// squares the relative error (2^-22 -> 2^-44 -> below the final rounding).
__device__ __forceinline__ double recip_newton(double d) {
  double r = ftod(__frcp_rn(dtof_trunc(d)));
  double e = fma(-d, r, 1.0);
  r = fma(r, e, r);
  e = fma(-d, r, 1.0);
  return fma(r, e, r);
}

// 1/d for any d: recip_newton where the FP32 seed is a normal number
// (|d| in [2^-125, 2^125)), the IEEE quotient elsewhere (zero, subnormal,
// huge, inf, NaN), chosen by an integer test of the exponent field.
__device__ __forceinline__ double recip_any(double d) {
  const unsigned e = (unsigned)((unsigned long long)__double_as_longlong(d) >> 52) & 0x7FFu;
  return (e - (1023u - 125u) < 250u) ? recip_newton(d) : 1.0 / d;
}

// FP64 -> FP32 rounded to nearest (ties away from zero) by integer
// operations; magnitudes below the FP32 normal range flush to a signed zero,
// above it to infinity. The split form's conversions use it.
__device__ __forceinline__ float d2f_int(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
  const int e = (int)((b >> 52) & 0x7FF) - 1023 + 127;
  const unsigned long long m = (b & 0xFFFFFFFFFFFFFULL) + (1ULL << 28);  // round at FP32's last bit
  const int e2 = e + (int)(m >> 52);                                      // carry into the exponent
  if (e2 <= 0) return __uint_as_float(sign);
  if (e2 >= 255) return __uint_as_float(sign | 0x7F800000u);
  return __uint_as_float(sign | ((unsigned)e2 << 23) | ((unsigned)(m >> 29) & 0x7FFFFFu));
}

// FP32 -> FP64 by integer operations, exact (FP32 denormals flush to zero)
__device__ __forceinline__ double f2d_int(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned ef = (u >> 23) & 0xFFu;
  const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
  const unsigned long long m = (unsigned long long)(u & 0x7FFFFFu) << 29;
  if (ef == 0) return __longlong_as_double((long long)sign);
  if (ef == 255) return __longlong_as_double((long long)(sign | 0x7FF0000000000000ULL | m));
  return __longlong_as_double((long long)(sign | ((unsigned long long)(ef - 127 + 1023) << 52) | m));
}

// Conversions between the FP64 path and the derived-field type F
template <typename F>
__device__ __forceinline__ F to_F(double x);
template <>
__device__ __forceinline__ double to_F<double>(double x) {
  return x;
}
template <>
__device__ __forceinline__ float to_F<float>(double x) {
  return d2f_int(x);
}
// D (FP64 or F) to F
template <typename F, typename D>
__device__ __forceinline__ F as_F(D x) {
  if constexpr (sizeof(D) == sizeof(F))
    return x;
  else
    return to_F<F>(x);
}
__device__ __forceinline__ double to_D(double x) { return x; }
__device__ __forceinline__ double to_D(float x) { return f2d_int(x); }

// Equation-of-state derivatives for eq types 1-4
// (veros/core/density/linear_eq.py:36-43, nonlinear_eq1.py:39-47,
//  nonlinear_eq2.py:57-66, nonlinear_eq3.py:39-47).
struct Eos {
  int type;
  static constexpr double rho0 = 1024.0;
  static constexpr double theta0 = 283.0 - 273.15;
  static constexpr double betaT = 1.67e-4;
  static constexpr double betaS = 0.78e-3;
  static constexpr double betaTs3 = 1e-5;
  static constexpr double betaTs24 = 1e-5 / 2.0;
  static constexpr double gammas = 1.1e-8;
  static constexpr double grav = 9.81;

  __device__ __forceinline__ double drdT(double T, double zt) const {
    if (type == 1) return -betaT * rho0;
    if (type == 3) {
      double zz = -fabs(zt) - 0.0;
      double thetas = T - theta0;
      return -(betaTs3 * thetas + betaT * (1.0 - gammas * grav * zz * rho0)) * rho0;
    }
    return -(betaT + 2.0 * betaTs24 * (T - theta0)) * rho0;  // types 2 and 4
  }
  __device__ __forceinline__ double drdS() const { return type == 4 ? 0.0 * rho0 : betaS * rho0; }
};

// The temp+salt diffusion of vg_isoneutral_diffusion_pair_* with the
// implicit solve's columns taken in the order column_order (interior column
// indices (i-2) + (j-2)*(X-4); NULL: natural order). fuse_prepare: the flux
// kernel also does a step's preparation of the interior cells (the step's
// rim is prepared separately), instead of updating what a separate
// preparation wrote.
// flux_starts: optional work shares of the flux kernel's CTAs (span_shares.cu).
int diffusion_pair_ordered_f64(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set,
                               const VgTensorFields *ten, const double *K_iso, const uint8_t *mask_bits,
                               const int32_t *kbot, const VgTracerArgs *temp, const VgTracerArgs *salt,
                               const int32_t *column_order, void *scratch, size_t scratch_bytes, void *stream,
                               int fuse_prepare = 0, const long long *flux_starts = nullptr, int flux_nstarts = 0);
int diffusion_pair_ordered_f32split(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set,
                                    const VgTensorFieldsF32 *ten, const float *K_iso, const uint8_t *mask_bits,
                                    const int32_t *kbot, const VgTracerArgsF32 *temp, const VgTracerArgsF32 *salt,
                                    const int32_t *column_order, void *scratch, size_t scratch_bytes,
                                    void *stream, int fuse_prepare = 0, const long long *flux_starts = nullptr,
                                    int flux_nstarts = 0);

// The pre and temp+salt flux kernels' tilings on this device: tiles along x,
// tiles in all, and the CTAs that share the tile-levels (0 where the kernel
// runs one CTA per tile); F = double or float (the split form).
template <typename F>
int pre_span_plan(const VgDomain *dom, int *ntx, int *ntiles, int *nctas);
template <typename F>
int flux_span_plan(const VgDomain *dom, int *ntx, int *ntiles, int *nctas);

// The pre kernel of a step, with optional work shares of its CTAs.
int pre_for_step_f64(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set, const double *temp_tau,
                     const double *salt_tau, const double *K_iso, const uint8_t *mask_bits,
                     const VgTensorFields *out, const long long *starts, int nstarts, void *stream);
int pre_for_step_f32split(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set, const double *temp_tau,
                          const double *salt_tau, const float *K_iso, const uint8_t *mask_bits,
                          const VgTensorFieldsF32 *out, const long long *starts, int nstarts, void *stream);

}  // namespace vg
