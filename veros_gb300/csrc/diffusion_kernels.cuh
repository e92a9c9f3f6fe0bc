// Isoneutral tracer diffusion (FP64), the work of
// veros/core/isoneutral/diffusion.py:9-295 and veros/core/diffusion.py:9-62.
//
// Two launches per tracer, or per temp-and-salt pair (one more with the
// energy branch):
//  1. flux_span_kernel 2.5-D tiled: a CTA owns 32 x 8 interior columns and
//                      walks k upward (a persistent CTA walks its share of
//                      the domain's tile-levels). Per level it forms the east, north and
//                      top fluxes (diffusion.py:9-113) of its faces plus the
//                      west/south halo faces, exchanges them through shared
//                      memory, and applies the divergence (:116-139), the
//                      explicit update of tr[taup1] and the dtracer_iso
//                      accumulation (:196-197). Grid divisions are
//                      multiplications by per-thread reciprocals.
//  2. implicit_kernel  (iso only) one thread per interior column: the
//                      implicit K_33 solve (:142-169) as a Thomas sweep whose
//                      c'/d' live in shared memory, shared by temp and salt
//                      when both are diffused together, and the second
//                      dtracer_iso term (:204).
//  3. energy_kernel    (enable_conserve_energy) one thread per column and
//                      chunk of levels: dissipation on the W grid and the
//                      vertical-mixing term added to P_diss (:234-281), from
//                      the fluxes step 1 saved in the scratch buffer.
#pragma once

#include "common.cuh"
#include "dgtsv.cuh"  // rounded arithmetic helpers

namespace vg {
namespace detail {

constexpr int TX = 32;  // one warp along x; TY (columns per CTA / 32) is a template parameter

// F is the type of the derived fields (tensors, tendencies, dissipation) and of
// the flux arithmetic: double for the FP64 drop-in, float for the split form.
// Tracers stay FP64 in both (their differences feed the fluxes and their
// increments are small against their values); the implicit solve is FP64.
template <typename F>
struct DiffArgs {
  Layout L;
  Grid g;
  double dt, grav, rho0;
  const F *__restrict__ K;  // K_iso (iso) or K_gm (skew)
  double s1, s2;            // K1 = s1*K, K2 = s2*K (diffusion.py:15-16)
  const F *__restrict__ K11;
  const F *__restrict__ K22;
  const F *__restrict__ K33;
  const F *__restrict__ Aez;
  const F *__restrict__ Anz;
  const F *__restrict__ Abx;
  const F *__restrict__ Aby;
  long long sp, sr;
  const uint8_t *__restrict__ m;
  const int32_t *__restrict__ kbot;
  const int32_t *__restrict__ col_order;  // implicit solve: interior columns in this order (NULL: natural)
  const double *__restrict__ tr;  // tau
  double *trp;                    // taup1
  F *dtr_iso;
  const F *__restrict__ idr;  // int_drhodX at tau
  F *P;
  F *fe, *fn, *ft;  // scratch fluxes (energy branch)
  int iso, save_fluxes, kchunk;
  // 1 inside a whole step (vg_isoneutral_step_*): the kernel also does the
  // step's preparation of its interior cells (tr[taup1] = tr[tau] * maskT,
  // zero tendencies and P_diss) instead of updating what a separate pass
  // wrote; the same values, bit for bit, without that pass
  int fuse_prepare;
  // 1 where the tensor was written by this library's pre kernel on the same
  // masks (a whole step): every face of a cell without mask bits then has
  // zero coefficients (+0), and the flux kernel reads none of them for the
  // levels below a column's first mask bit
  int tensor_from_pre;
};

// x * 0.0 by integer operations for finite x (the zero of x's sign), the
// product itself otherwise (inf and NaN give NaN)
__device__ __forceinline__ double times_zero(double x) {
  const long long b = __double_as_longlong(x);
  return ((b >> 52) & 0x7FF) == 0x7FF ? x * 0.0 : __longlong_as_double(b & (long long)0x8000000000000000ULL);
}

template <typename F>
__device__ __forceinline__ F ld(const F *p, long long o) { return __ldg(p + o); }

// x + y and x * y: explicitly rounded in FP64 (no contraction into the
// explicit update, which feeds the tendency's differencing), plain in FP32.
static __device__ __forceinline__ double add_(double x, double y) { return radd(x, y); }
static __device__ __forceinline__ double mul_(double x, double y) { return rmul(x, y); }
static __device__ __forceinline__ float add_(float x, float y) { return x + y; }
static __device__ __forceinline__ float mul_(float x, float y) { return x * y; }

// Multiplies and fused multiply-adds with their rounding fixed in the source,
// so that every instantiation of a flux (one tracer, two tracers, batched)
// performs the same operations whatever the compiler would contract.
static __device__ __forceinline__ double pm(double x, double y) { return __dmul_rn(x, y); }
static __device__ __forceinline__ float pm(float x, float y) { return __fmul_rn(x, y); }
static __device__ __forceinline__ double pfma(double x, double y, double z) { return __fma_rn(x, y, z); }
static __device__ __forceinline__ float pfma(float x, float y, float z) { return __fmaf_rn(x, y, z); }

// Face fluxes, split into the coefficients a face's tracers share (diffloc
// times the slope components, the K_11/K_22 factor) and the per-tracer
// differences, so that temp and salt diffused together load and multiply the
// tensor once. Operand order per tracer is the reference's.

// east face of cell (i, j, k), valid for i in [1, X-2), j in [2, Y-2) (diffusion.py:25-47)
// diffloc of an east/north face: the mean of K1 = s1 K over the face's two
// points on levels k and k-1 (diffusion.py:21-23, :48-50), from the pair sums
// K(P) + K(P') of the two levels (s1 = +-1)
template <typename F>
__device__ __forceinline__ F face_diffloc(F pair, F pair_below, int k, double s1) {
  const F q = s1 > 0.0 ? (k >= 1 ? F(0.25) : F(0.5)) : (k >= 1 ? F(-0.25) : F(-0.5));
  return q * (k >= 1 ? pair + pair_below : pair);
}

// c[0..3]: the four slope components of the face; c[4]: K_11 / (cost dxu);
// c[5]: diffloc / (4 dzt), which scales the sum of the four vertical terms
// once instead of each component.
template <typename F>
__device__ __forceinline__ void east_coef(const DiffArgs<F> &a, long long o, F diffloc, F inv_cost_dxu, F q_dzt,
                                          F c[6]) {
  c[0] = ld(a.Aez, o);
  c[1] = ld(a.Aez, o + a.sp);
  c[2] = ld(a.Aez, o + a.sr);
  c[3] = ld(a.Aez, o + a.sp + a.sr);
  c[4] = pm(inv_cost_dxu, ld(a.K11, o));
  c[5] = pm(diffloc, q_dzt);
}

// flux of one tracer through a face from the face coefficients and the
// tracer differences: the two lower and the two upper vertical differences
// of the face's points, and the difference across the face
// (differences in FP64 or already converted to F)
template <typename F, typename D>
__device__ __forceinline__ F face_flux(const F c[6], D z0m, D z1m, D z0p, D z1p, D h) {
  F sumz = pm(c[0], as_F<F>(z0m));
  sumz = pfma(c[1], as_F<F>(z1m), sumz);
  sumz = pfma(c[2], as_F<F>(z0p), sumz);
  sumz = pfma(c[3], as_F<F>(z1p), sumz);
  return pfma(sumz, c[5], pm(as_F<F>(h), c[4]));
}

template <typename F>
__device__ __forceinline__ F east_flux(const Layout &L, const double *tr, long long o, int k, const F c[6]) {
  const long long dm = k > 0 ? L.plane : 0;  // edge padding in z (utilities.py:24-35)
  const long long dp = k < L.Z - 1 ? L.plane : 0;
  const double t0 = __ldg(tr + o), t1 = __ldg(tr + o + 1);
  const double t0m = __ldg(tr + o - dm), t1m = __ldg(tr + o + 1 - dm);
  const double t0p = __ldg(tr + o + dp), t1p = __ldg(tr + o + 1 + dp);
  return face_flux(c, t0 - t0m, t1 - t1m, t0p - t0, t1p - t1, t1 - t0);
}

// north face of cell (i, j, k), valid for i in [2, X-2), j in [1, Y-2) (diffusion.py:52-77)
template <typename F>
__device__ __forceinline__ void north_coef(const DiffArgs<F> &a, long long o, F diffloc, F inv_dyu, F q_dzt,
                                           F c[6]) {
  c[0] = ld(a.Anz, o);
  c[1] = ld(a.Anz, o + a.sp);
  c[2] = ld(a.Anz, o + a.sr);
  c[3] = ld(a.Anz, o + a.sp + a.sr);
  c[4] = pm(inv_dyu, ld(a.K22, o));
  c[5] = pm(diffloc, q_dzt);
}

template <typename F>
__device__ __forceinline__ F north_flux(const Layout &L, const double *tr, long long o, int k, const F c[6],
                                        F cosu) {
  const long long P = L.pitch;
  const long long dm = k > 0 ? L.plane : 0;
  const long long dp = k < L.Z - 1 ? L.plane : 0;
  const double t0 = __ldg(tr + o), t1 = __ldg(tr + o + P);
  const double t0m = __ldg(tr + o - dm), t1m = __ldg(tr + o + P - dm);
  const double t0p = __ldg(tr + o + dp), t1p = __ldg(tr + o + P + dp);
  return pm(cosu, face_flux(c, t0 - t0m, t1 - t1m, t0p - t0, t1p - t1, t1 - t0));
}

// top face of interior cell (i, j, k < Z-1) (diffusion.py:85-111).
// c[0..3]: the x slope components; c[4..7]: the y slope components times
// cosu of their face; c[8] = K2 / (4 dxt cost) and c[9] = K2 / (4 dyt cost)
// scale the two sums once.
template <typename F>
__device__ __forceinline__ void top_coef(const DiffArgs<F> &a, long long o, F qx_cost, F q_dyt_cost, F cosu_s,
                                         F cosu_c, F c[10]) {
  const F diffloc = a.s2 == 1.0 ? ld(a.K, o) : to_F<F>(a.s2) * ld(a.K, o);  // K2 = s2 K (diffusion.py:16)
  c[0] = ld(a.Abx, o);
  c[1] = ld(a.Abx, o + a.sr);
  c[2] = ld(a.Abx, o + a.sp);
  c[3] = ld(a.Abx, o + a.sp + a.sr);
  c[4] = pm(cosu_s, ld(a.Aby, o));
  c[5] = pm(cosu_s, ld(a.Aby, o + a.sr));
  c[6] = pm(cosu_c, ld(a.Aby, o + a.sp));
  c[7] = pm(cosu_c, ld(a.Aby, o + a.sp + a.sr));
  c[8] = pm(diffloc, qx_cost);
  c[9] = pm(diffloc, q_dyt_cost);
}

// top flux of one tracer from the west, east, south and north differences on
// the face's lower (k) and upper (k+1) levels
template <typename F, typename D>
__device__ __forceinline__ F top_face_flux(const F c[10], D w0, D w1, D e0, D e1, D s0, D s1, D n0, D n1) {
  F sumx = pm(c[0], as_F<F>(w0));
  sumx = pfma(c[1], as_F<F>(w1), sumx);
  sumx = pfma(c[2], as_F<F>(e0), sumx);
  sumx = pfma(c[3], as_F<F>(e1), sumx);
  F sumy = pm(c[4], as_F<F>(s0));
  sumy = pfma(c[5], as_F<F>(s1), sumy);
  sumy = pfma(c[6], as_F<F>(n0), sumy);
  sumy = pfma(c[7], as_F<F>(n1), sumy);
  return pfma(sumx, c[8], pm(sumy, c[9]));
}

template <typename F>
__device__ __forceinline__ F top_flux(const Layout &L, const double *tr, long long o, const F c[10]) {
  const long long P = L.pitch, Q = L.plane;
  const double tc = __ldg(tr + o), tcu = __ldg(tr + o + Q);
  return top_face_flux(c, tc - __ldg(tr + o - 1), tcu - __ldg(tr + o - 1 + Q), __ldg(tr + o + 1) - tc,
                       __ldg(tr + o + 1 + Q) - tcu, tc - __ldg(tr + o - P), tcu - __ldg(tr + o - P + Q),
                       __ldg(tr + o + P) - tc, __ldg(tr + o + P + Q) - tcu);
}

// Dynamic shared memory of flux_div_body: 1/(4 dzt) and 1/dzt per level, then
// a (Z + 1)-entry int table for the wet-point ordering, then the two level
// tables in FP32 (used by the split form).
inline size_t flux_smem_bytes(int Z) {
  return 2 * (size_t)Z * sizeof(double) + ((size_t)Z + 1) * sizeof(int) + 2 * (size_t)Z * sizeof(float);
}

// True if any of n values loaded at p + off[m] is non-zero (either sign of
// zero counts as zero), by integer operations on the bit patterns.
template <typename F>
__device__ __forceinline__ bool any_nonzero(const F *p, long long o, const long long *off, int n) {
  unsigned long long acc = 0;
  for (int m = 0; m < n; ++m) {
    const F v = ld(p, o + off[m]);
    if constexpr (sizeof(F) == 8)
      acc |= (unsigned long long)__double_as_longlong((double)v) << 1;
    else
      acc |= (unsigned long long)(__float_as_uint((float)v) << 1);
  }
  return acc != 0;
}

// One tile (bx, by) and levels [kb, ke) of NTR tracers of one domain; the whole CTA
// (32 x TY threads) takes part. A[0..NTR-1] differ only in their tracer
// fields; geometry, tensor and masks come from A[0]. zq_dzt: dynamic shared
// memory of flux_smem_bytes(Z).
//
// Wet-point ordering. An FP64 warp instruction holds the FP64 pipe for its
// whole warp however few lanes are active, and on random topography most
// warps have a few wet and many dry columns on most levels. So the threads
// take the tile's columns in the order of their first level in [kb, ke) with
// a mask bit set (stable, one warp's counting sort): on each level the
// columns with a mask bit so far form a prefix of the order, and whole warps
// of dry columns skip the FP64 work. A column runs the full computation from
// its first wet level on (its carried values start there as at a segment
// start). Before it, the divergence is zero (maskT multiplies it), and the
// fluxes through its east, north and top faces are zero wherever their
// tensor coefficients are, as isoneutral_diffusion_pre writes them for a
// face whose mask is zero; a dry column checks that on the bit patterns of
// the coefficients and computes any face whose coefficients are not zero
// from freshly loaded tracers, so the result is the reference's for any
// tensor. The arithmetic of every face and cell is the same in all paths.
// Only the FP64 form orders its columns: the split form's fluxes are FP32,
// whose pipe the dry lanes hardly load, and the ordering would cost it more
// than it saves (measured 0.13 ms slower per step at 1 degree).
template <typename F, int TY, int NTR>
__device__ __forceinline__ void flux_div_body(const DiffArgs<F> *A, double *zq_dzt, int bx, int by, int kb, int ke) {
  constexpr int NT = TX * TY;
  __shared__ F fe_s[2][NTR][TY][TX + 1];  // east faces i0-1 .. i0+TX-1
  __shared__ F fn_s[2][NTR][TY + 1][TX];  // north faces j0-1 .. j0+TY-1
  __shared__ short okey[NT], olist[NT];
  __shared__ unsigned slot0;  // %warpid of warp 0 (virtual_warp)
  const DiffArgs<F> &a = A[0];
  const Layout &L = a.L;
  const int Z = L.Z;
  double *zinv_dzt = zq_dzt + Z;  // 1/(4 dzt[k]) then 1/dzt[k]
  int *hist = reinterpret_cast<int *>(zq_dzt + 2 * Z);
  const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
  const int i0 = 2 + bx * TX, j0 = 2 + by * TY;
  const int nkeys = ke - kb + 1;
  // the split form's FP32 copies of both tables (after the int table)
  float *zf = reinterpret_cast<float *>(hist + Z + 1);
  constexpr bool kF32 = sizeof(F) == sizeof(float);
  for (int k = tid; k < Z; k += NT) {
    zq_dzt[k] = 1.0 / (4.0 * a.g.dzt[k]);
    zinv_dzt[k] = 1.0 / a.g.dzt[k];
    if constexpr (kF32) {
      zf[k] = to_F<float>(zq_dzt[k]);
      zf[Z + k] = to_F<float>(zinv_dzt[k]);
    }
  }
  // 1/(4 dzt[k]) (t = 0) or 1/dzt[k] (t = 1) in F
  auto ztab = [&](int t, int k) -> F {
    if constexpr (kF32)
      return zf[t * Z + k];
    else
      return (t ? zinv_dzt : zq_dzt)[k];
  };
  constexpr bool kOrder = sizeof(F) == sizeof(double);
  if (kOrder) {
    for (int n = tid; n < nkeys; n += NT) hist[n] = 0;
    // fluxes of faces nobody computes on a level are zero
    for (int n = tid; n < 2 * NTR * TY * (TX + 1); n += NT) (&fe_s[0][0][0][0])[n] = F(0);
    for (int n = tid; n < 2 * NTR * (TY + 1) * TX; n += NT) (&fn_s[0][0][0][0])[n] = F(0);
  }
  if (kOrder) {
    // the first level of [kb, ke) with a mask bit of the column (ke - kb if none)
    const int ci = i0 + tid % TX, cj = j0 + tid / TX;
    int f = ke;
    if (ci < L.X - 2 && cj < L.Y - 2) {
      const uint8_t *mp = a.m + L.at(ci, cj, 0);
      for (int l0 = kb; l0 < ke && f >= ke; l0 += 8) {
        unsigned v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = l0 + u < ke ? __ldg(mp + (long long)(l0 + u) * L.plane) : 0u;
#pragma unroll
        for (int u = 0; u < 8; ++u)
          if (f >= ke && v[u]) f = l0 + u;
      }
    }
    okey[tid] = (short)(f - kb);
    __syncthreads();
    atomicAdd(&hist[okey[tid]], 1);
  } else {
    okey[tid] = 0;  // every column from the segment's first level, in tile order
    olist[tid] = (short)tid;
  }
  if (tid == 0) slot0 = hw_warp_slot();
  __syncthreads();
  if (kOrder && warp == 0) {
    // exclusive prefix sums of the key histogram, then the stable scatter
    int run = 0;
    for (int c0 = 0; c0 < nkeys; c0 += 32) {
      const int v = c0 + lane < nkeys ? hist[c0 + lane] : 0;
      int x = v;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= d) x += y;
      }
      if (c0 + lane < nkeys) hist[c0 + lane] = run + x - v;
      run += __shfl_sync(0xffffffffu, x, 31);
    }
    __syncwarp();
    for (int c0 = 0; c0 < NT; c0 += 32) {
      const int idx = c0 + lane;
      const int kk = okey[idx];
      const unsigned grp = __match_any_sync(0xffffffffu, kk);
      const int leader = __ffs(grp) - 1;
      const int rank = __popc(grp & ((1u << lane) - 1u));
      int base = lane == leader ? hist[kk] : 0;
      base = __shfl_sync(0xffffffffu, base, leader);
      olist[base + rank] = (short)idx;
      __syncwarp();
      if (lane == leader) hist[kk] = base + __popc(grp);
      __syncwarp();
    }
  }
  __syncthreads();
  // the busiest columns go to virtual warp 0 (virtual_warp spreads co-resident CTAs' busy warps
  // over the sub-partitions); the split form keeps the tile order
  const int oe = kOrder ? olist[virtual_warp(warp, NT / 32, slot0) * 32 + lane] : olist[tid];
  const int kact = kb + okey[oe];  // first level with a mask bit (ke: none)
  const int tx = oe % TX, ty = oe / TX;

  const int i = i0 + tx, j = j0 + ty;
  const bool own = i < L.X - 2 && j < L.Y - 2;
  const int ic = min(i, L.X - 3), jc = min(j, L.Y - 3);
  const double cost = a.g.cost[jc];
  const F inv_cost_dxu = F(1.0 / (cost * a.g.dxu[ic]));
  const F cosu_c = F(a.g.cosu[jc]), cosu_s = F(a.g.cosu[jc - 1]);
  const F inv_dyu = F(1.0 / a.g.dyu[jc]);
  const F inv_fx = F(1.0 / (cost * a.g.dxt[ic]));  // divergence factors (diffusion.py:127, :129)
  const F inv_fy = F(1.0 / (cost * a.g.dyt[jc]));
  const F qx_cost = F(1.0 / (4.0 * a.g.dxt[ic] * cost));
  const F q_dyt_cost = F(1.0 / (4.0 * a.g.dyt[jc] * cost));
  // halo faces: the last virtual warp the south row of north faces, the one before it the west
  // column of east faces (in the FP64 form those warps hold the tile's driest columns, so the
  // halo work does not lengthen the busiest warps' path to the level's barrier)
  const int hwarp = kOrder ? virtual_warp(warp, NT / 32, slot0) : warp;
  const int hi_n = i0 + lane;  // north face (hi_n, j0-1)
  const bool halo_n = hwarp == NT / 32 - 1 && hi_n < L.X - 2 && j0 - 1 < L.Y - 2;
  const int hj_e = j0 + lane;  // east face (i0-1, hj_e)
  const bool halo_e = hwarp == NT / 32 - 2 && lane < TY && hj_e < L.Y - 2 && i0 - 1 < L.X - 2;
  F h_cosu = 0, h_inv_dyu = 0, h_inv_cost_dxu = 0;
  if (halo_n) {
    h_cosu = F(a.g.cosu[j0 - 1]);
    h_inv_dyu = F(1.0 / a.g.dyu[j0 - 1]);
  }
  if (halo_e) h_inv_cost_dxu = F(1.0 / (a.g.cost[hj_e] * a.g.dxu[i0 - 1]));

  // Tracer values and differences of the own faces carried up the column:
  // per tracer the values at the own, east and north columns, their vertical
  // differences t(k) - t(k-1) (0 at k = 0, edge padding), and the four
  // horizontal differences around the own point; each level loads the level
  // above once and forms its differences once, in FP64, converted to F once
  // (each difference serves two levels' faces). The K pair sums of the east
  // and north faces are carried the same way. They start on the column's
  // first wet level (start_column), as on a segment's first level.
  const long long P = L.pitch, Q = L.plane;
  double vc[NTR], ve[NTR], vn[NTR];     // values at level k
  F dzc[NTR], dze[NTR], dzn[NTR];  // t(k) - t(k-1)
  F hw[NTR], hs[NTR], he[NTR], hn[NTR];  // west, south, east, north differences at level k
  F ft_prev[NTR];
  F pe_below = 0, pn_below = 0;  // K pair sums of the east / north face on level k-1
#pragma unroll
  for (int r = 0; r < NTR; ++r) {
    ft_prev[r] = 0.0;
    vc[r] = ve[r] = vn[r] = dzc[r] = dze[r] = dzn[r] = hw[r] = hs[r] = he[r] = hn[r] = 0.0;
  }
  auto start_column = [&](int k0) {
    const long long ob = L.at(i, j, k0);
#pragma unroll
    for (int r = 0; r < NTR; ++r) {
      const double *tr = A[r].tr;
      vc[r] = __ldg(tr + ob);
      ve[r] = __ldg(tr + ob + 1);
      vn[r] = __ldg(tr + ob + P);
      hw[r] = to_F<F>(vc[r] - __ldg(tr + ob - 1));
      hs[r] = to_F<F>(vc[r] - __ldg(tr + ob - P));
      he[r] = to_F<F>(ve[r] - vc[r]);
      hn[r] = to_F<F>(vn[r] - vc[r]);
      if (k0 > 0) {
        dzc[r] = to_F<F>(vc[r] - __ldg(tr + ob - Q));
        dze[r] = to_F<F>(ve[r] - __ldg(tr + ob + 1 - Q));
        dzn[r] = to_F<F>(vn[r] - __ldg(tr + ob + P - Q));
      }
    }
    if (k0 > 0) {
      const long long op = L.at(i, j, k0 - 1);
      const F kd = ld(a.K, op);
      pe_below = kd + ld(a.K, op + 1);
      pn_below = kd + ld(a.K, op + P);
      F ct[10];
      top_coef(a, op, qx_cost, q_dyt_cost, cosu_s, cosu_c, ct);
#pragma unroll
      for (int r = 0; r < NTR; ++r) ft_prev[r] = top_flux(L, A[r].tr, op, ct);
    }
  };
  // offsets of a face's tensor coefficients: the four (p, r) components and the K_11 / K_22 factor
  const long long ai_off[4] = {0, a.sp, a.sr, a.sp + a.sr};
  const long long k_off[1] = {0};

  for (int k = kb; k < ke; ++k) {
    // double-buffered exchange: the barrier of level k+1 orders level k's
    // reads before level k+2's writes to the same buffer
    const int b = k & 1;
    const long long o = L.at(i, j, k);
    const F qz = ztab(0, k);
    F fe[NTR], fn[NTR], ft[NTR];
#pragma unroll
    for (int r = 0; r < NTR; ++r) fe[r] = fn[r] = ft[r] = 0.0;
    if (own && k >= kact) {
      if (k == kact) start_column(k);
      const bool up = k < Z - 1;
      if (kF32 && k + 1 < Z) {
        // split form: the next level's tensor coefficients and, two levels up, the tracers,
        // in L2 by then (1% on its flux kernel at 1 degree; nothing on the FP64 one's)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          prefetch_l2(a.Aez + o + Q + ai_off[c]);
          prefetch_l2(a.Anz + o + Q + ai_off[c]);
          prefetch_l2(a.Abx + o + Q + ai_off[c]);
          prefetch_l2(a.Aby + o + Q + ai_off[c]);
        }
        prefetch_l2(a.K11 + o + Q);
        prefetch_l2(a.K22 + o + Q);
        prefetch_l2(a.K + o + Q);
        if (k + 2 < Z) {
#pragma unroll
          for (int r = 0; r < NTR; ++r) prefetch_l2(A[r].tr + o + 2 * Q);
        }
      }
      double uc[NTR], ue[NTR], un[NTR], uw[NTR], us[NTR];  // level k+1
#pragma unroll
      for (int r = 0; r < NTR; ++r) {
        const double *tr = A[r].tr;
        if (up) {
          uc[r] = __ldg(tr + o + Q);
          ue[r] = __ldg(tr + o + 1 + Q);
          un[r] = __ldg(tr + o + P + Q);
          uw[r] = __ldg(tr + o - 1 + Q);
          us[r] = __ldg(tr + o - P + Q);
        } else {
          uc[r] = vc[r];
          ue[r] = ve[r];
          un[r] = vn[r];
          uw[r] = us[r] = 0.0;
        }
      }
      F ce[6], cn[6];
      const F kc = ld(a.K, o), pe = kc + ld(a.K, o + 1), pn = kc + ld(a.K, o + P);
      east_coef(a, o, face_diffloc(pe, pe_below, k, a.s1), inv_cost_dxu, qz, ce);
      north_coef(a, o, face_diffloc(pn, pn_below, k, a.s1), inv_dyu, qz, cn);
      pe_below = pe;
      pn_below = pn;
      F ct[10];
      if (up) top_coef(a, o, qx_cost, q_dyt_cost, cosu_s, cosu_c, ct);
#pragma unroll
      for (int r = 0; r < NTR; ++r) {
        // z differences above the own, east and north columns (0 on the top level)
        const F zc = to_F<F>(uc[r] - vc[r]), ze = to_F<F>(ue[r] - ve[r]), zn = to_F<F>(un[r] - vn[r]);
        // east face (diffusion.py:25-47), north face (:52-77)
        fe[r] = face_flux(ce, dzc[r], dze[r], zc, ze, he[r]);
        fn[r] = pm(cosu_c, face_flux(cn, dzc[r], dzn[r], zc, zn, hn[r]));
        // horizontal differences on level k+1
        const F hw1 = to_F<F>(uc[r] - uw[r]), he1 = to_F<F>(ue[r] - uc[r]);
        const F hs1 = to_F<F>(uc[r] - us[r]), hn1 = to_F<F>(un[r] - uc[r]);
        if (up) ft[r] = top_face_flux(ct, hw[r], hw1, he[r], he1, hs[r], hs1, hn[r], hn1);  // (diffusion.py:85-111)
        vc[r] = uc[r];
        ve[r] = ue[r];
        vn[r] = un[r];
        dzc[r] = zc;
        dze[r] = ze;
        dzn[r] = zn;
        hw[r] = hw1;
        hs[r] = hs1;
        he[r] = he1;
        hn[r] = hn1;
      }
    } else if (own && !a.tensor_from_pre) {
      // no mask bit on this column yet: faces with non-zero coefficients only
      if (any_nonzero(a.Aez, o, ai_off, 4) || any_nonzero(a.K11, o, k_off, 1)) {
        F ce[6];
        const F pe = ld(a.K, o) + ld(a.K, o + 1);
        const F peb = k >= 1 ? ld(a.K, o - Q) + ld(a.K, o + 1 - Q) : F(0);
        east_coef(a, o, face_diffloc(pe, peb, k, a.s1), inv_cost_dxu, qz, ce);
#pragma unroll
        for (int r = 0; r < NTR; ++r) fe[r] = east_flux(L, A[r].tr, o, k, ce);
      }
      if (any_nonzero(a.Anz, o, ai_off, 4) || any_nonzero(a.K22, o, k_off, 1)) {
        F cn[6];
        const F pn = ld(a.K, o) + ld(a.K, o + P);
        const F pnb = k >= 1 ? ld(a.K, o - Q) + ld(a.K, o + P - Q) : F(0);
        north_coef(a, o, face_diffloc(pn, pnb, k, a.s1), inv_dyu, qz, cn);
#pragma unroll
        for (int r = 0; r < NTR; ++r) fn[r] = north_flux(L, A[r].tr, o, k, cn, cosu_c);
      }
      if (k < Z - 1 && (any_nonzero(a.Abx, o, ai_off, 4) || any_nonzero(a.Aby, o, ai_off, 4))) {
        F ct[10];
        top_coef(a, o, qx_cost, q_dyt_cost, cosu_s, cosu_c, ct);
#pragma unroll
        for (int r = 0; r < NTR; ++r) ft[r] = top_flux(L, A[r].tr, o, ct);
      }
    }
    if (own) {
#pragma unroll
      for (int r = 0; r < NTR; ++r) {
        fe_s[b][r][ty][tx + 1] = fe[r];
        fn_s[b][r][ty + 1][tx] = fn[r];
      }
    }
    if (halo_n) {
      const long long oh = L.at(hi_n, j0 - 1, k);
      F cn[6];
      const F pn = ld(a.K, oh) + ld(a.K, oh + L.pitch);
      const F pnb = k >= 1 ? ld(a.K, oh - L.plane) + ld(a.K, oh + L.pitch - L.plane) : F(0);
      north_coef(a, oh, face_diffloc(pn, pnb, k, a.s1), h_inv_dyu, qz, cn);
#pragma unroll
      for (int r = 0; r < NTR; ++r) fn_s[b][r][0][lane] = north_flux(L, A[r].tr, oh, k, cn, h_cosu);
    }
    if (halo_e) {
      const long long oh = L.at(i0 - 1, hj_e, k);
      F ce[6];
      const F pe = ld(a.K, oh) + ld(a.K, oh + 1);
      const F peb = k >= 1 ? ld(a.K, oh - L.plane) + ld(a.K, oh + 1 - L.plane) : F(0);
      east_coef(a, oh, face_diffloc(pe, peb, k, a.s1), h_inv_cost_dxu, qz, ce);
#pragma unroll
      for (int r = 0; r < NTR; ++r) fe_s[b][r][lane][0] = east_flux(L, A[r].tr, oh, k, ce);
    }
    __syncthreads();
    const bool wetT = own && k >= kact && (__ldg(a.m + o) & VG_MASK_T);
    if (wetT) {  // maskT multiplies the divergence (diffusion.py:123-137)
#pragma unroll
      for (int r = 0; r < NTR; ++r) {
        const DiffArgs<F> &t = A[r];
        F e = pfma(fe[r] - fe_s[b][r][ty][tx], inv_fx, pm(fn[r] - fn_s[b][r][ty][tx], inv_fy));
        e = pfma(ft[r] - ft_prev[r], ztab(1, k), e);  // k = 0: ft_prev = 0 (diffusion.py:132-137)
        if (a.fuse_prepare) {
          // tr[taup1] = tr[tau] * 1 and dtracer_iso = 0 (thermodynamics.py:226-241, :427-429), then
          // the explicit update: the values the separate preparation and the update below give
          t.dtr_iso[o] = add_(F(0), e);
          t.trp[o] = fma(t.dt, to_D(e), __ldg(t.tr + o));
        } else {
          t.dtr_iso[o] = add_(t.dtr_iso[o], e);
          t.trp[o] = fma(t.dt, to_D(e), t.trp[o]);  // tr[taup1] += dt * dtr (diffusion.py:192)
        }
      }
    } else if (own && a.fuse_prepare) {  // no divergence: the prepared values (maskT = 0)
#pragma unroll
      for (int r = 0; r < NTR; ++r) {
        A[r].dtr_iso[o] = F(0);
        A[r].trp[o] = times_zero(__ldg(A[r].tr + o));
      }
    }
    if (own && a.fuse_prepare && a.P) a.P[o] = F(0);
    if (own) {
#pragma unroll
      for (int r = 0; r < NTR; ++r) {
        const DiffArgs<F> &t = A[r];
        ft_prev[r] = ft[r];
        if (t.save_fluxes) {
          t.fe[o] = fe[r];
          t.fn[o] = fn[r];
          t.ft[o] = ft[r];
        }
      }
    }
#pragma unroll
    for (int r = 0; r < NTR; ++r) {
      if (A[r].save_fluxes) {
        if (halo_n) A[r].fn[L.at(hi_n, j0 - 1, k)] = fn_s[b][r][0][lane];
        if (halo_e) A[r].fe[L.at(i0 - 1, hj_e, k)] = fe_s[b][r][lane][0];
      }
    }
  }
  // the tile's exchange buffers are reused by the next tile a persistent CTA takes
  __syncthreads();
}

// One domain: every resident CTA takes a share of the ntiles * Z
// tile-levels, tile-major, as one segment per tile it touches (a segment
// starting above level 0 pays the restart of a k-chunk): starts[c] ..
// starts[c+1] (weighted by the water on each tile-level, span_shares.cu) or,
// without starts, equal counts; the body ends with a barrier before its
// buffers are reused.
template <typename F, int TY, int NTR>
__global__ void __launch_bounds__(TX * TY, 16 / TY) flux_span_kernel(DiffArgs<F> a, DiffArgs<F> b, int ntx, int ntiles,
                                                                      const long long *__restrict__ starts) {
  extern __shared__ double zq_dzt[];
  const DiffArgs<F> A[2] = {a, b};
  const int Z = a.L.Z;
  const long long W = (long long)ntiles * Z;
  long long p = starts ? starts[blockIdx.x] : W * blockIdx.x / gridDim.x;
  const long long end = starts ? starts[blockIdx.x + 1] : W * (blockIdx.x + 1) / gridDim.x;
  while (p < end) {
    const int t = (int)(p / Z), kb = (int)(p % Z);
    const int ke = (int)min((long long)Z, end - (long long)t * Z);
    flux_div_body<F, TY, NTR>(A, zq_dzt, t % ntx, t / ntx, kb, ke);
    p = (long long)t * Z + ke;
  }
}

// Implicit solve of NRHS tracers sharing one matrix, one thread per column.
// The system (diffusion.py:154-164) is an M-matrix that is diagonally
// dominant by columns (|b_k| >= |a_{k+1}| + |c_{k-1}|), for which elimination
// without interchanges is backward stable; the Thomas sweep in reciprocal form
// keeps one division per level on the column's serial chain and none in the
// back substitution. The matrix entries use the reference's divisions; the
// factorisation is shared by the tracers. Shared memory holds c'_k and d'_k of
// each tracer, [k][thread].
// The solve of one column (i, j) whose water starts at level ks.
// FP32 <-> FP64 conversions of the implicit solve: hardware conversions,
// since this latency-bound kernel leaves the FP64 pipe mostly idle (the
// integer forms of to_F / to_D lengthen its serial chain)
__device__ __forceinline__ double cvt_d(double x) { return x; }
__device__ __forceinline__ double cvt_d(float x) { return (double)x; }
template <typename F>
__device__ __forceinline__ F cvt_f(double x) {
  return (F)x;
}

template <typename F, int NRHS>
__device__ __forceinline__ void implicit_column(const DiffArgs<F> &a, const DiffArgs<F> &b2, const double *dtdzw,
                                                const double *inv_dzt, double *cps, int cs, double *dps, int ds,
                                                int i, int j, int ks) {
  const Layout &L = a.L;
  const int Z = L.Z;
  const long long base = L.at2(i, j);
  double *trp[2] = {a.trp, b2.trp};
  F *dtr[2] = {a.dtr_iso, b2.dtr_iso};
  const double inv_dt = 1.0 / a.dt;

  // Loads run PF levels ahead of the serial chain (software pipelining): the
  // chain itself only waits for FP64 latency, not for global memory.
  constexpr int PF = 8;
  double qK[PF], qT[PF][NRHS];
#pragma unroll
  for (int u = 0; u < PF; ++u) {
    const int k = ks + u;
    const long long o = base + (long long)min(k, Z - 1) * L.plane;
    qK[u] = k < Z - 1 ? cvt_d(ld(a.K33, o)) : 0.0;
#pragma unroll
    for (int r = 0; r < NRHS; ++r) qT[u][r] = k < Z ? (double)trp[r][o] : 0.0;
  }
  // Thomas elimination of the system of diffusion.py:152-164 with one
  // reciprocal per level: the matrix entries use the per-level 1/dzt table
  double delta_prev = 0.0, cp = 0.0, dp[NRHS];
#pragma unroll
  for (int r = 0; r < NRHS; ++r) dp[r] = 0.0;
  for (int k0 = ks; k0 < Z; k0 += PF) {
#pragma unroll
    for (int u = 0; u < PF; ++u) {
      const int k = k0 + u;
      if (k < Z) {
        const double idzt = inv_dzt[k];
        const double delta = k < Z - 1 ? pm(dtdzw[k], qK[u]) : 0.0;
        double tr1[NRHS];
#pragma unroll
        for (int r = 0; r < NRHS; ++r) tr1[r] = qT[u][r];
        // refill this slot with level k + PF
        const int kn = k + PF;
        if (kn < Z) {
          const long long on = base + (long long)kn * L.plane;
          qK[u] = kn < Z - 1 ? cvt_d(ld(a.K33, on)) : 0.0;
#pragma unroll
          for (int r = 0; r < NRHS; ++r) qT[u][r] = (double)trp[r][on];
        }
        const double ak = k == ks ? 0.0 : pm(-delta_prev, idzt);  // a_tri, zero at the edge (operators.py:72)
        const double bk = pfma(k == ks ? delta : delta + delta_prev, idzt, 1.0);  // b_tri, b_tri_edge at ks
        const double ck = pm(-delta, idzt);                                      // c_tri (0 on the top level)
        const double den = recip_newton(pfma(-ak, cp, bk));  // pivot >= the diagonal's excess over 1
        cp = pm(ck, den);
        cps[(size_t)k * cs] = cp;
#pragma unroll
        for (int r = 0; r < NRHS; ++r) {
          dp[r] = pm(pfma(-ak, dp[r], tr1[r]), den);
          dps[((size_t)r * Z + k) * ds] = dp[r];
        }
        delta_prev = delta;
      }
    }
  }
  double x[NRHS];
#pragma unroll
  for (int r = 0; r < NRHS; ++r) x[r] = 0.0;
  const int nlev = Z - ks;
  for (int m0 = 0; m0 < nlev; m0 += PF) {
    // this group's old tracer values and partial tendencies, loaded together
    double t1[PF][NRHS], d1[PF][NRHS];
#pragma unroll
    for (int u = 0; u < PF; ++u) {
      const int k = Z - 1 - (m0 + u);
      if (k >= ks) {
        const long long o = base + (long long)k * L.plane;
#pragma unroll
        for (int r = 0; r < NRHS; ++r) {
          t1[u][r] = (double)trp[r][o];
          d1[u][r] = cvt_d(dtr[r][o]);
        }
      }
    }
#pragma unroll
    for (int u = 0; u < PF; ++u) {
      const int k = Z - 1 - (m0 + u);
      if (k >= ks) {
        const long long o = base + (long long)k * L.plane;
        const double c = cps[(size_t)k * cs];
#pragma unroll
        for (int r = 0; r < NRHS; ++r) {
          x[r] = pfma(-c, x[r], dps[((size_t)r * Z + k) * ds]);
          trp[r][o] = x[r];
          dtr[r][o] = cvt_f<F>(pfma(x[r] - t1[u][r], inv_dt, d1[u][r]));  // diffusion.py:204
        }
      }
    }
  }
}


// Columns [cb * blockDim, (cb + 1) * blockDim) of the interior of one domain.
template <typename F, int NRHS>
__device__ __forceinline__ void implicit_body(const DiffArgs<F> &a, const DiffArgs<F> &b2, double *smem, int cb) {
  const Layout &L = a.L;
  const int Z = L.Z;
  const int ncols_x = L.X - 4, ncols = ncols_x * (L.Y - 4);
  const int t = threadIdx.x, nb = blockDim.x;
  double *dtdzw = smem;
  double *inv_dzt = smem + Z;
  double *cps = smem + 2 * Z;
  double *dps = cps + (size_t)Z * nb;  // [r][k][thread]
  for (int k = t; k < Z; k += nb) {
    dtdzw[k] = rdiv(a.dt, a.g.dzw[k]);
    inv_dzt[k] = 1.0 / a.g.dzt[k];
  }
  __syncthreads();
  // with col_order, the deepest columns first: the lanes of a warp then walk
  // columns of similar length
  const int slot = cb * nb + t;
  const int col = a.col_order ? (slot < ncols ? __ldg(a.col_order + slot) : ncols) : slot;
  const int i = 2 + col % ncols_x;
  const int j = 2 + col / ncols_x;
  const int ks = (unsigned)col < (unsigned)ncols ? a.kbot[L.at2(i, j)] - 1 : -1;  // create_water_masks (utilities.py:38-48)
  if (ks >= 0 && ks < Z) implicit_column<F, NRHS>(a, b2, dtdzw, inv_dzt, cps + t, nb, dps + t, nb, i, j, ks);
  __syncthreads();  // dtdzw is refilled by the next block of columns a persistent CTA takes
}

template <typename F, int NRHS>
__global__ void __launch_bounds__(64) implicit_kernel(DiffArgs<F> a, DiffArgs<F> b2) {
  extern __shared__ double smem[];
  implicit_body<F, NRHS>(a, b2, smem, blockIdx.x);
}

// Temp and salt of a column on two neighbouring threads (lane 2c: a, lane
// 2c+1: b2): both form the shared factorisation (they write the same c'
// values to the column's slot) and each eliminates its own tracer, so twice
// as many warps hide the recurrence's latency for the same shared memory
// per column. The arithmetic of each tracer is that of implicit_kernel<F, 2>.
// The body of one CTA of the pair solve: column block cb of blockDim.x / 2
// columns. Also run by the batched ensemble's persistent CTAs.
template <typename F>
__device__ __forceinline__ void implicit_pair_body(const DiffArgs<F> &a, const DiffArgs<F> &b2, double *smem, int cb) {
  const Layout &L = a.L;
  const int Z = L.Z;
  const int ncols_x = L.X - 4, ncols = ncols_x * (L.Y - 4);
  const int t = threadIdx.x, nb = blockDim.x, nc = nb / 2, c = t >> 1, r = t & 1;
  double *dtdzw = smem;
  double *inv_dzt = smem + Z;
  double *cps = smem + 2 * Z;             // [k][column]
  double *dps = cps + (size_t)Z * nc;     // [k][thread]
  for (int k = t; k < Z; k += nb) {
    dtdzw[k] = rdiv(a.dt, a.g.dzw[k]);
    inv_dzt[k] = 1.0 / a.g.dzt[k];
  }
  __syncthreads();
  const int slot = cb * nc + c;
  const int col = a.col_order ? (slot < ncols ? __ldg(a.col_order + slot) : ncols) : slot;
  const int i = 2 + col % ncols_x;
  const int j = 2 + col / ncols_x;
  const int ks = (unsigned)col < (unsigned)ncols ? a.kbot[L.at2(i, j)] - 1 : -1;  // create_water_masks (utilities.py:38-48)
  const DiffArgs<F> &own = r ? b2 : a;
  if (ks >= 0 && ks < Z) implicit_column<F, 1>(own, own, dtdzw, inv_dzt, cps + c, nc, dps + t, nb, i, j, ks);
}

template <typename F>
__global__ void __launch_bounds__(128) implicit_pair_kernel(DiffArgs<F> a, DiffArgs<F> b2) {
  extern __shared__ double smem[];
  implicit_pair_body<F>(a, b2, smem, blockIdx.x);
}

// Energy branch (veros/core/isoneutral/diffusion.py:234-281 with
// veros/core/diffusion.py:9-62) for one tracer, or for temp then salt, which
// add into the same P_diss in that order. One thread per column (i, j),
// i in [1, X-2], j in [1, Y-2], walking the levels [k0, k0 + kc) of one chunk;
// the dissipation at k + 1, which the W-grid interpolation at k needs, and
// int_drhodX at k + 1 are carried to the next level. Divisions by the grid
// spacings are multiplications by reciprocals that each CTA forms once in
// shared memory (1/dxt of its columns, the 1/cost factors of its rows, and per
// level 1/dzw, -g/rho_0/dzw and dzw_pad/dzw). Every product and sum is rounded
// explicitly, so the one- and two-tracer launches give identical bits.
template <typename F>
struct EnergyColumn {
  bool fe0, fe1, fn0, fn1;  // saved east/north fluxes exist at i, i-1 / j, j-1
  F cx, cy;                 // 0.5 g / rho_0 / (dxt cost), ... / (dyt cost)
};

// Dissipation at T point o (diffusion.py:9-36); *I0 receives int_drhodX there.
template <typename F>
__device__ __forceinline__ F diss_col(const DiffArgs<F> &a, const EnergyColumn<F> &c, long long o, long long pitch,
                                      F *I0) {
  const F I = ld(a.idr, o);
  *I0 = I;
  const F fe0 = c.fe0 ? ld(a.fe, o) : F(0.0), fe1 = c.fe1 ? ld(a.fe, o - 1) : F(0.0);
  const F fn0 = c.fn0 ? ld(a.fn, o) : F(0.0), fn1 = c.fn1 ? ld(a.fn, o - pitch) : F(0.0);
  const F ex = pfma(ld(a.idr, o + 1) - I, fe0, pm(I - ld(a.idr, o - 1), fe1));
  const F ny = pfma(ld(a.idr, o + pitch) - I, fn0, pm(I - ld(a.idr, o - pitch), fn1));
  return pfma(ex, c.cx, pm(ny, c.cy));
}

constexpr int kEnergyTX = 32, kEnergyTY = 4, kEnergyMaxZ = 512;

template <typename F, int NTR>
__global__ void __launch_bounds__(kEnergyTX *kEnergyTY) energy_kernel(DiffArgs<F> a0, DiffArgs<F> a1, int kc) {
  __shared__ double inv_dxt[kEnergyTX], c_cost[kEnergyTY], c_dyt_cost[kEnergyTY];
  __shared__ F gidz[kEnergyMaxZ], idz_s[kEnergyMaxZ], ratio_s[kEnergyMaxZ];
  const Layout &L = a0.L;
  const int Z = L.Z;
  const int k0 = blockIdx.z * kc, k1 = min(Z, k0 + kc);
  const int i = 1 + blockIdx.x * kEnergyTX + threadIdx.x;
  const int j = 1 + blockIdx.y * kEnergyTY + threadIdx.y;
  {
    const int tid = threadIdx.y * kEnergyTX + threadIdx.x;
    const double c = 0.5 * a0.grav / a0.rho0;
    if (tid < kEnergyTX) {
      const int ii = 1 + blockIdx.x * kEnergyTX + tid;
      inv_dxt[tid] = ii < L.X - 1 ? 1.0 / a0.g.dxt[ii] : 0.0;
    } else if (tid < kEnergyTX + kEnergyTY) {
      const int r = tid - kEnergyTX, jj = 1 + blockIdx.y * kEnergyTY + r;
      const double cost = jj < L.Y - 1 ? a0.g.cost[jj] : 1.0;
      c_cost[r] = c / cost;
      c_dyt_cost[r] = jj < L.Y - 1 ? c / (a0.g.dyt[jj] * cost) : 0.0;
    }
    for (int t = tid; t < k1 - k0; t += kEnergyTX * kEnergyTY) {
      const int k = k0 + t;
      const double idz = 1.0 / a0.g.dzw[k];
      idz_s[t] = to_F<F>(idz);
      gidz[t] = to_F<F>(-a0.grav / a0.rho0 * idz);
      ratio_s[t] = to_F<F>(a0.g.dzw[k > 0 ? k - 1 : 0] / a0.g.dzw[k]);  // dzw_pad[k] / dzw[k] (diffusion.py:53-55)
    }
  }
  __syncthreads();
  if (i >= L.X - 1 || j >= L.Y - 1) return;
  const DiffArgs<F> *A[2] = {&a0, &a1};

  const int ks = a0.kbot[L.at2(i, j)] - 1;
  const bool land = ks >= 0;  // "land_mask" of create_water_masks: the column has water
  const bool inner = i >= 2 && i < L.X - 2 && j >= 2 && j < L.Y - 2;
  // flux_east exists on [1:-2, 2:-2] and flux_north on [2:-2, 1:-2]
  // (diffusion.py:25, :52); the reference reads flux_east[1:-1] and [:-2],
  // flux_north[:, 1:-1] and [:, :-2] (veros/core/diffusion.py:22-31), zero
  // outside those ranges. The halo columns i = 1, X-2 and rows j = 1, Y-2
  // only matter where kbot makes them water (a cyclic x boundary).
  EnergyColumn<F> col;
  col.fe0 = i < L.X - 2 && j >= 2 && j < L.Y - 2;  // flux_east[i, j]
  col.fe1 = i >= 2 && j >= 2 && j < L.Y - 2;       // flux_east[i-1, j]
  col.fn0 = i >= 2 && i < L.X - 2 && j < L.Y - 2;  // flux_north[i, j]
  col.fn1 = i >= 2 && i < L.X - 2 && j >= 2;       // flux_north[i, j-1]
  col.cx = to_F<F>(pm(c_cost[threadIdx.y], inv_dxt[threadIdx.x]));
  col.cy = to_F<F>(c_dyt_cost[threadIdx.y]);
  const F ratio = (land && ks >= k0 && ks < k1) ? ratio_s[ks - k0] : F(0.0);

  const long long pitch = L.pitch, plane = L.plane;
  long long o = L.at(i, j, k0);
  F d0[NTR], Ic[NTR];
#pragma unroll
  for (int t = 0; t < NTR; ++t) d0[t] = diss_col(*A[t], col, o, pitch, &Ic[t]);
  for (int k = k0; k < k1; ++k, o += plane) {
    const bool below = k < Z - 1;
    const bool mW = inner && below && (__ldg(a0.m + o) & VG_MASK_W);
    const F gz = gidz[k - k0], idz = idz_s[k - k0];
    F P = a0.P[o];
#pragma unroll
    for (int t = 0; t < NTR; ++t) {
      const DiffArgs<F> &a = *A[t];
      F d1 = F(0.0), In = F(0.0);
      F dw;
      if (below) {
        d1 = diss_col(a, col, o + plane, pitch, &In);
        const F h = pm(F(0.5), d0[t] + d1);
        dw = (land && k == ks) ? pfma(F(0.5), pm(d0[t], ratio), h) : ((land && k > ks) ? h : F(0.0));
      } else {
        dw = land ? d0[t] : F(0.0);
      }
      P = P + dw;
      // vertical-mixing term (diffusion.py:254-279); zero where maskW is:
      // P += (-g/rho_0 fxa) (flux_top + K_33 dtr/dzw), fxa = (I_k - I_k+1) / dzw
      if (mW) {
        const F g = pm(Ic[t] - In, gz);
        F term = ld(a.ft, o);
        if (a.iso) term = pfma(pm(ld(a.K33, o), to_F<F>(a.trp[o + plane] - a.trp[o])), idz, term);
        P = pfma(g, term, P);
      }
      d0[t] = d1;
      Ic[t] = In;
    }
    a0.P[o] = P;
  }
}

// Validates one tracer's arguments and fills its DiffArgs.
template <typename F, typename Ten, typename Tr>
inline int make_diff_args(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set, const Ten *ten, const F *K_field,
              const uint8_t *mask_bits, const int32_t *kbot, const Tr *tr, int skew, F *scratch3, DiffArgs<F> &a) {
  if (!grid_complete(grid) || !set || !ten || !K_field || !mask_bits || !kbot || !tr || !tr->tr_tau ||
      !tr->tr_taup1 || !tr->dtracer_iso || !ten->K_11 || !ten->K_22 || !ten->K_33 || !ten->Ai_ez ||
      !ten->Ai_nz || !ten->Ai_bx || !ten->Ai_by)
    return fail(VG_ERR_ARG, "isoneutral diffusion: NULL pointer argument");
  if (skew != 0 && skew != 1) return fail(VG_ERR_ARG, "skew must be 0 or 1");
  if (set->enable_conserve_energy && (!tr->int_drhodX_tau || !tr->P_diss))
    return fail(VG_ERR_ARG, "enable_conserve_energy needs int_drhodX_tau and P_diss");
  if (!(set->dt_tracer != 0.0)) return fail(VG_ERR_ARG, "dt_tracer must be non-zero");
  if (dom->Z > 512) return fail(VG_ERR_SHAPE, "Z=%d above the 512 levels supported", dom->Z);
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
  a.save_fluxes = set->enable_conserve_energy ? 1 : 0;
  const size_t fsz = (size_t)a.L.plane * a.L.Z;
  a.fe = scratch3;
  a.fn = scratch3 ? scratch3 + fsz : nullptr;
  a.ft = scratch3 ? scratch3 + 2 * fsz : nullptr;
  a.iso = skew ? 0 : 1;
  a.kchunk = 0;
  a.col_order = nullptr;
  a.fuse_prepare = 0;
  a.tensor_from_pre = 0;
  return VG_OK;
}

}  // namespace detail
}  // namespace vg
