// Isoneutral slopes and diffusion tensor (FP64), the work of
// veros/core/isoneutral/isoneutral.py:18-229.
//
// On GB300 the FP64 pipe (about 1 TFLOP/s) bounds this kernel, not HBM, so
// the design minimises FP64 instructions per cell:
//
// * 2.5-D tiling. A CTA owns a TX x TY tile of columns and walks k upward.
//   For every T point of the tile plus a one-cell ring it computes, once per
//   level, the quantities several faces share: drho/dT and drho/dS
//   (isoneutral.py:40-41), the east/north face gradients of T and S
//   (:64-95), and the reciprocals of the two clamped vertical density
//   gradients min(0, drho/dz) - epsln that every slope divides by (:121, :158,
//   :188, :207): one for the face below the point (kr = 0) and one above
//   (kr = 1). Two planes (k and k+1) live in shared memory.
// * Each slope is evaluated once. A slope belongs to a T point P, one of its
//   horizontal faces h (east, west, north, south) and one of its vertical
//   faces v (below, above): s = -(drdT(P) dT/dh + drdS(P) dS/dh) / R(P, v).
//   The reference evaluates it twice, in the term of face h (Ai_ez/Ai_nz,
//   K_11/K_22, :100-168) and in the term of face v (Ai_bx/Ai_by, K_33,
//   :173-224), with the same operands. Here each thread computes the eight
//   slopes and tapers of its own point per level and keeps them in
//   registers for its own faces; the taper and taper*slope of its west and
//   south slopes go to shared memory for the east/north faces of the
//   neighbouring point. A ring column and row of the tile add 2 slopes per
//   ring point. Slopes no face of the point uses (all their faces masked)
//   are skipped.
// * Grid divisions become multiplications by reciprocals computed once per
//   CTA; slope divisions become multiplications by the shared reciprocals.
// * The taper 0.5*(1+tanh(x)) (isoneutral.py:10-15) is a piecewise degree-4
//   Taylor polynomial about the points -4 + n/256 on [-4, 2] (taper_table.inc,
//   truncation error < 2e-15), the library tanh elsewhere, and an FP32 exp
//   below x = -10 where the taper is below 2e-9.
// * The two clamped reciprocals 1/(min(0, G) - epsln) per point use an FP32
//   reciprocal refined by two Newton-Raphson steps; min(0, .), max(.) and the
//   FP64 <-> FP32 conversions around it are integer operations.
// * Faces whose mask is zero skip the slope work and store the zeros the
//   reference's mask multiplication produces.
//
// Outputs are written only on the reference's sub-ranges (K_11[1:-2,2:-2],
// K_22[2:-2,1:-2], K_33[2:-2,2:-2,:-1], K_33[...,-1] = 0, Ai_* likewise); all
// other cells keep their contents.
#pragma once

#include "common.cuh"

namespace vg {
namespace detail {

#include "taper_table.inc"


constexpr double kEpsln = 1e-20;  // isoneutral.py:28
enum { Q_RT, Q_RS, Q_TX, Q_SX, Q_TY, Q_SY, Q_R0, Q_R1, NQ };

// Tile of TX = 32 (one warp along x) by TY columns; the point region adds a
// one-cell ring. TY (the columns per CTA) is chosen by the autotuner.
template <int TY_>
struct Tile {
  static constexpr int TX = 32, TY = TY_, NT = TX * TY;
  static constexpr int PX = TX + 2, PY = TY + 2, NP = PX * PY;
  static constexpr int kPtSlots = (NP + NT - 1) / NT;
};

// F is the type of the derived fields (K_iso in, K and Ai out) and of their
// arithmetic: double for the FP64 drop-in, float for the split form. The
// tracers stay FP64 in both: the vertical density gradient that every slope
// divides by is a difference of nearby tracer values, and FP32 storage alone
// would cost it ~1e-6 K of absolute accuracy.
template <typename F>
struct PreArgs {
  Layout L;
  Grid g;
  int eos_type;
  double slopec, inv_dslope, ksteep;
  const double *__restrict__ T;
  const double *__restrict__ S;
  const F *__restrict__ K;
  const uint8_t *__restrict__ m;
  F *K11, *K22, *K33, *Aez, *Anz, *Abx, *Aby;
  long long sp, sr;
  int kchunk;
  // optional (FP64, single domain): per point the 8 tapers, 8 slopes and the
  // 2 clamped reciprocals, fields SLOPE_T + n, SLOPE_S + n, SLOPE_R + v
  // slope_field doubles apart, for the adjoint
  double *slopes;
  long long slope_field;
  // 1 if T, S and the mask bytes allow 16-byte copies of their rows (aligned
  // bases, pitch and plane multiples of 16 elements): the split form then
  // stages its T/S/mask planes in shared memory (PreStage)
  int stage_ok;
};

// Whether the pre arguments allow the 16-byte row copies of the staged planes.
template <typename F>
inline int pre_stage_ok(const PreArgs<F> &a) {
  auto al = [](const void *p) { return ((uintptr_t)p & 15u) == 0; };
  return al(a.T) && al(a.S) && al(a.m) && a.L.pitch % 16 == 0 && a.L.plane % 16 == 0;
}
enum { SLOPE_T = 0, SLOPE_S = 8, SLOPE_R = 16, SLOPE_FIELDS = 18 };

// slope index h * 2 + v: h = east, west, north, south face; v = face below, above
enum { S_XE0, S_XE1, S_XW0, S_XW1, S_YN0, S_YN1, S_YS0, S_YS1, NS };
// published per point: taper and taper*slope of the west and south slopes
enum { PB_T_XW0, PB_T_XW1, PB_T_YS0, PB_T_YS1, PB_TS_XW0, PB_TS_XW1, PB_TS_YS0, PB_TS_YS1, NPB };
constexpr unsigned kMaskWBelow = 0x10;  // in the plane mask byte: W mask of the level below

// Staged planes of the split form: T, S (FP64) and the mask bytes of four
// consecutive levels (a ring, level l in slot l & 3) over rows j0-1 .. j0+PY-1
// and columns i0-1 .. i0+PX+1 (the plane points and their east / north
// neighbours), filled by cp.async two levels ahead of their use, so that a
// level's plane quantities read shared memory instead of waiting on global
// loads. The FP64 form has no shared memory to spare for it at two CTAs per SM.
template <bool kOn, int TY>
struct PreStage {};
template <int TY>
struct PreStage<true, TY> {
  static constexpr int ROWS = Tile<TY>::PY + 1, DW = 36, MW = 48;  // doubles / bytes per staged row
  double T[4][ROWS][DW];
  double S[4][ROWS][DW];
  unsigned char M[4][ROWS][MW];
};

// FP32 copies of the per-CTA grid tables the split form's arithmetic reads
// (the FP64 form reads the double tables themselves), converted once per CTA
// instead of once per point and level.
template <typename F, int TY>
struct SplitTables {};
template <int TY>
struct SplitTables<float, TY> {
  float inv_dxu_cost[Tile<TY>::NP], inv_dyu[Tile<TY>::PY];
  float dqx[2][Tile<TY>::PX], dqy[2][Tile<TY>::PY];
};

template <typename F, int TY>
struct Smem {
  static constexpr int PX = Tile<TY>::PX, PY = Tile<TY>::PY, NP = Tile<TY>::NP;
  static constexpr bool kStage = sizeof(F) == sizeof(float);
  __align__(16) PreStage<kStage, TY> st;
  F q[2][NQ][NP];  // per-point quantities; the split form keeps them FP32 (R computed in FP64)
  F pub[2][NPB][NP];
  double inv_dxu[PX], inv_dyu[PY], inv_cost[PY];
  double inv_dxu_cost[NP];  // 1 / (dxu cost) per plane point
  // K_33 weights of the top face's slopes: dxu(i-1+ip) / (4 dxt(i)) by thread column,
  // cosu(j-1+jp) dyu(j-1+jp) / (4 dyt(j) cost(j)) by thread row
  double dqx[2][PX], dqy[2][PY];
  SplitTables<F, TY> fv;
  uint8_t qm[2][NP];
  // wet-point ordering of the segment (see pre_tile_body): per plane point
  // the key (first level with a mask bit, counted from the segment's first
  // plane level), the plane points in key order, and the same for the own
  // points, whose key also covers their west and south neighbours
  short pkey[NP], plist[NP];
  short ukey[NP], vkey[NP];  // per plane point: first level with its U / V mask bit
  short okey[Tile<TY>::NT], olist[Tile<TY>::NT];
  unsigned slot0;  // %warpid of warp 0 (virtual_warp)
  // per level (dynamic tail): dzw, inv_dzw, 1/(4 dzt), eos constant; then
  // two (Z + 2)-entry int tables for the key histograms / running offsets;
  // in the split form then dzw, 1/(4 dzt) and the eos constant in FP32
};

template <typename F, int TY>
constexpr size_t pre_smem_bytes(int Z) {
  return sizeof(Smem<F, TY>) + 4 * (size_t)Z * sizeof(double) + 2 * ((size_t)Z + 2) * sizeof(int) +
         (sizeof(F) == sizeof(float) ? 3 * (size_t)Z * sizeof(float) : 0);
}

// Stable counting sort of n small keys (0 <= key < nkeys) by one warp:
// list[] receives the indices 0..n-1 in key order, equal keys in index
// order. off[] holds the exclusive prefix sums of the key histogram on entry
// and is advanced as the indices are placed. Lanes sharing a key within a
// chunk of 32 take consecutive slots after the group's running offset.
__device__ __forceinline__ void warp_stable_scatter(const short *key, int n, int *off, short *list, int lane) {
  for (int c0 = 0; c0 < n; c0 += 32) {
    const int idx = c0 + lane;
    const int kk = idx < n ? key[idx] : -1;
    const unsigned grp = __match_any_sync(0xffffffffu, kk);
    const int leader = __ffs(grp) - 1;
    const int rank = __popc(grp & ((1u << lane) - 1u));
    int base = (lane == leader && kk >= 0) ? off[kk] : 0;
    base = __shfl_sync(0xffffffffu, base, leader);
    if (kk >= 0) list[base + rank] = (short)idx;
    __syncwarp();
    if (lane == leader && kk >= 0) off[kk] = base + __popc(grp);
    __syncwarp();
  }
}

// In-place exclusive prefix sum of h[0..n) by one warp.
__device__ __forceinline__ void warp_exclusive_scan(int *h, int n, int lane) {
  int run = 0;
  for (int c0 = 0; c0 < n; c0 += 32) {
    const int v = c0 + lane < n ? h[c0 + lane] : 0;
    int x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, d);
      if (lane >= d) x += y;
    }
    if (c0 + lane < n) h[c0 + lane] = run + x - v;
    run += __shfl_sync(0xffffffffu, x, 31);
  }
}

template <typename F>
struct Slope {
  F t;  // taper
  F s;  // slope
};

// The table entry nearest to x is n = round(256 (x - X0)): x*256 + (1.5*2^52 -
// 256*X0) rounds to an integer (the ulp at 1.5*2^52 is 1), whose low word is n
// and whose high word is that of 1.5*2^52 for every n in the table (so
// infinities and NaN fail the test and take the tail path). Each table row
// ends with its centre X0 + n/256. sc = slopec / dslope.
static __device__ __forceinline__ double taper_of(double s, double sc, double inv_dslope) {
  constexpr double kMagic = 6755399441055744.0;  // 1.5 * 2^52
  const double x = fma(fabs(s), -inv_dslope, sc);
  const double y = fma(x, kTaperPerUnit, kMagic - kTaperX0 * kTaperPerUnit);
  const int n = __double2loint(y);
  if (__double2hiint(y) == 0x43380000 && (unsigned)n < (unsigned)kTaperN) {
    const double *c = kTaperCoef[n];
    const double b = x - __ldg(c + kTaperDeg + 1);
    double r = __ldg(c + 4);
    r = fma(r, b, __ldg(c + 3));
    r = fma(r, b, __ldg(c + 2));
    r = fma(r, b, __ldg(c + 1));
    return fma(r, b, __ldg(c + 0));
  }
  if (x < -10.0) return (double)expf(2.0f * (float)x);
  return 0.5 * (1.0 + tanh(x));
}

// 1/d for d = min(0, G) - epsln, i.e. d in (-inf, -1e-20]
static __device__ __forceinline__ double recip_neg(double d) { return recip_newton(d); }

// min(0, G) - epsln (isoneutral.py:121, :158, :188, :207) with the FP64
// subtraction only where it can change G: G >= +0 gives -epsln, and for
// |G| >= 2^-13 epsln = 1e-20 is below half an ulp of G, so G - epsln = G.
// Sign and exponent tests are integer operations.
static __device__ __forceinline__ double clamp_eps(double G) {
  const long long b = __double_as_longlong(G);
  if (b >= 0) return -kEpsln;
  return ((b >> 52) & 0x7FF) >= 1023 - 13 ? G : G - kEpsln;
}

// Split form: slope, taper argument and taper in FP32 (the slope's clamped
// denominator was formed in FP64); slopec_f, inv_dslope_f are FP32 copies.
static __device__ __forceinline__ float taper_of_split(float s, float slopec_f, float inv_dslope_f) {
  const float x = (slopec_f - fabsf(s)) * inv_dslope_f;
  return 0.5f * (1.0f + tanhf(x));
}

// The taper's constants in both precisions, formed once per CTA
struct TaperConsts {
  double sc, inv_dslope;       // FP64 path: slopec / dslope and 1 / dslope
  float slopec_f, inv_dslope_f;  // split form
};

template <typename F>
__device__ __forceinline__ F taper_t(F s, const TaperConsts &c);
template <>
__device__ __forceinline__ double taper_t<double>(double s, const TaperConsts &c) {
  return taper_of(s, c.sc, c.inv_dslope);
}
template <>
__device__ __forceinline__ float taper_t<float>(float s, const TaperConsts &c) {
  return taper_of_split(s, c.slopec_f, c.inv_dslope_f);
}

// max(K_iso_steep, x): FP64 by integer comparison, FP32 as is
__device__ __forceinline__ double max_t(double a, double b) { return dmax(a, b); }
__device__ __forceinline__ float max_t(float a, float b) { return fmaxf(a, b); }

__device__ __forceinline__ bool nonneg(double x) { return __double_as_longlong(x) >= 0; }
__device__ __forceinline__ bool nonneg(float x) { return __float_as_int(x) >= 0; }

// sum over kr, ip of dzw(kr) max(K_iso_steep, diffloc taper(kr, ip)) for K_11 / K_22
// (isoneutral.py:123-128, :160-165); t[0][*] = 0 on level 0. With K_iso_steep <= 0
// and diffloc >= 0 every max is its second argument, so diffloc factors out.
template <typename F>
__device__ __forceinline__ F face_sumz(const F t[2][2], const F dzwF[2], F diffloc, F ksteepF, bool lin_steep,
                                       int k) {
  if (lin_steep && nonneg(diffloc)) {
    F S = dzwF[1] * (t[1][0] + t[1][1]);
    if (k > 0) S = dzwF[0] * (t[0][0] + t[0][1]) + S;
    return diffloc * S;
  }
  F sumz = 0.0;
#pragma unroll
  for (int kr = 0; kr < 2; ++kr) {
    if (kr == 0 && k == 0) continue;
    sumz += dzwF[kr] * max_t(ksteepF, diffloc * t[kr][0]);
    sumz += dzwF[kr] * max_t(ksteepF, diffloc * t[kr][1]);
  }
  return sumz;
}

// One tile (bx, by) and levels [kb, ke) of one domain; the whole CTA takes part.
template <typename F, int TY>
__device__ __forceinline__ void pre_tile_body(const PreArgs<F> &a, unsigned char *smem_raw, int bx, int by, int kb,
                                              int ke) {
  using Sm = Smem<F, TY>;
  constexpr int TX = Tile<TY>::TX, NT = Tile<TY>::NT, PX = Tile<TY>::PX, PY = Tile<TY>::PY, NP = Tile<TY>::NP;
  constexpr int kPtSlots = Tile<TY>::kPtSlots;
  Sm &sm = *reinterpret_cast<Sm *>(smem_raw);
  double *zdzw = reinterpret_cast<double *>(smem_raw + sizeof(Sm));
  const Layout &L = a.L;
  const int Z = L.Z;
  double *zinv_dzw = zdzw + Z;
  double *zq_dzt = zinv_dzw + Z;
  double *zeos = zq_dzt + Z;
  // split form: dzw, 1/(4 dzt) and the eos constant per level in FP32 (after the two int tables)
  float *zf = reinterpret_cast<float *>(reinterpret_cast<int *>(zeos + Z) + 2 * (Z + 2));
  constexpr bool kF32 = sizeof(F) == sizeof(float);

  const int tid = threadIdx.x;
  const int warp = tid / 32, lane = tid % 32;
  const int i0 = 1 + bx * TX, j0 = 1 + by * TY;
  constexpr bool kStage = Sm::kStage;
  const bool stage = kStage && a.stage_ok;
  // the last plane compute_plane reads (its level + 1 below the top)
  const int pmax = min(min(ke, Z - 1) + 1, Z - 1);
  // cp.async of one level's T, S and mask rows into its ring slot (split form)
  auto issue_plane = [&](int lev) {
    if constexpr (kStage) {
      using St = PreStage<true, TY>;
      constexpr int ND = St::DW / 2, NM = St::MW / 16, PER_ROW = 2 * ND + NM;
      const int slot = lev & 3, xs = i0 - 1;  // xs = 32 bx: 16-byte aligned rows
      for (int c = tid; c < St::ROWS * PER_ROW; c += NT) {
        const int r = c / PER_ROW, q = c % PER_ROW, j = j0 - 1 + r;
        if (j >= L.Y) continue;
        if (q < 2 * ND) {
          const int x = xs + 2 * (q % ND);
          if (x + 1 >= L.pitch) continue;  // pitch is even: a pair never straddles it
          const double *src = (q < ND ? a.T : a.S) + L.at(x, j, lev);
          double *dst = q < ND ? &sm.st.T[slot][r][2 * (q % ND)] : &sm.st.S[slot][r][2 * (q % ND)];
          cp_async16(dst, src);
        } else {
          const int x = xs + 16 * (q - 2 * ND);
          if (x + 15 >= L.pitch) continue;  // pitch is a multiple of 16
          cp_async16(&sm.st.M[slot][r][16 * (q - 2 * ND)], a.m + L.at(x, j, lev));
        }
      }
    }
  };

  // the staged planes the prologue's compute_plane calls and the first loop level read
  const int lo_stage = max(kb - 1, 0);
  if (stage)
    for (int l = lo_stage; l <= min(kb + 2, pmax); ++l) issue_plane(l);

  // ---- per-CTA grid tables ------------------------------------------------
  for (int p = tid; p < PX; p += NT) {
    const int i = min(max(i0 - 1 + p, 0), L.X - 1);
    sm.inv_dxu[p] = 1.0 / a.g.dxu[i];
  }
  for (int p = tid; p < PY; p += NT) {
    const int j = min(max(j0 - 1 + p, 0), L.Y - 1);
    sm.inv_dyu[p] = 1.0 / a.g.dyu[j];
    sm.inv_cost[p] = 1.0 / a.g.cost[j];
    if constexpr (kF32) sm.fv.inv_dyu[p] = to_F<float>(sm.inv_dyu[p]);
  }
  for (int p = tid; p < TX; p += NT) {
    const int i = min(i0 + p, L.X - 1);
    const double q = 1.0 / (4.0 * a.g.dxt[i]);
    sm.dqx[0][p] = a.g.dxu[i - 1] * q;
    sm.dqx[1][p] = a.g.dxu[i] * q;
    if constexpr (kF32) {
      sm.fv.dqx[0][p] = to_F<float>(sm.dqx[0][p]);
      sm.fv.dqx[1][p] = to_F<float>(sm.dqx[1][p]);
    }
  }
  for (int p = tid; p < TY; p += NT) {
    const int j = min(j0 + p, L.Y - 1);
    const double q = 1.0 / (4.0 * a.g.dyt[j] * a.g.cost[j]);
    sm.dqy[0][p] = a.g.cosu[j - 1] * a.g.dyu[j - 1] * q;  // facty (isoneutral.py:202)
    sm.dqy[1][p] = a.g.cosu[j] * a.g.dyu[j] * q;
    if constexpr (kF32) {
      sm.fv.dqy[0][p] = to_F<float>(sm.dqy[0][p]);
      sm.fv.dqy[1][p] = to_F<float>(sm.dqy[1][p]);
    }
  }
  for (int k = tid; k < Z; k += NT) {
    zdzw[k] = a.g.dzw[k];
    zinv_dzw[k] = 1.0 / a.g.dzw[k];
    zq_dzt[k] = 1.0 / (4.0 * a.g.dzt[k]);
    // drho/dT = eos_c1 T + zeos[k]: type 3 -(betaTs (T - theta0) + betaT (1 - gammas grav zz rho0)) rho0
    // with zz = -|zt|; types 2, 4 -(betaT + 2 betaTs (T - theta0)) rho0; type 1 -betaT rho0
    if (a.eos_type == 3) {
      const double zz = -fabs(a.g.zt[k]) - 0.0;
      zeos[k] = (Eos::betaTs3 * Eos::theta0 - Eos::betaT * (1.0 - Eos::gammas * Eos::grav * zz * Eos::rho0)) *
                Eos::rho0;
    } else if (a.eos_type == 1) {
      zeos[k] = -Eos::betaT * Eos::rho0;
    } else {
      zeos[k] = (2.0 * Eos::betaTs24 * Eos::theta0 - Eos::betaT) * Eos::rho0;
    }
    if constexpr (kF32) {
      zf[k] = to_F<float>(zdzw[k]);
      zf[Z + k] = to_F<float>(zq_dzt[k]);
      zf[2 * Z + k] = to_F<float>(zeos[k]);
    }
  }

  // K_33 on the top level is zero on the whole plane (isoneutral.py:225)
  if (ke == Z) {
    for (int p = tid; p < (PX + 1) * (PY + 1); p += NT) {
      const int i = i0 - 1 + p % (PX + 1), j = j0 - 1 + p / (PX + 1);
      if (i < L.X && j < L.Y) a.K33[L.at(i, j, Z - 1)] = 0.0;
    }
  }
  __syncthreads();
  for (int p = tid; p < NP; p += NT) {
    sm.inv_dxu_cost[p] = sm.inv_dxu[p % PX] * sm.inv_cost[p / PX];
    if constexpr (kF32) sm.fv.inv_dxu_cost[p] = to_F<float>(sm.inv_dxu_cost[p]);
  }
  const double eos_c1 = a.eos_type == 3 ? -Eos::betaTs3 * Eos::rho0
                        : a.eos_type == 1 ? 0.0
                                          : -2.0 * Eos::betaTs24 * Eos::rho0;
  const F eos_c1F = to_F<F>(eos_c1);
  const double rS_wet_d = to_D(a.eos_type == 4 ? F(0.0) : F(Eos::betaS * Eos::rho0));  // drho/dS of a wet point
  // the F-typed per-level and per-point grid factors
  auto zeosF = [&](int k) -> F {
    if constexpr (kF32) return zf[2 * Z + k]; else return zeos[k];
  };
  auto zdzwF = [&](int k) -> F {
    if constexpr (kF32) return zf[k]; else return zdzw[k];
  };
  auto zqF_ = [&](int k) -> F {
    if constexpr (kF32) return zf[Z + k]; else return zq_dzt[k];
  };

  // ---- wet-point ordering of the segment -----------------------------------
  // An FP64 warp instruction holds the FP64 pipe for its whole warp, however
  // few of its lanes are active, and on a dry level a point's work reduces to
  // constants. So the threads take the points in the order of the level from
  // which on they carry work: a point's key is its first level in [lo, hi]
  // with a mask bit set (hi - lo + 1 if none); an own point's key is the least
  // of its own key and the first levels with the U mask bit of its west
  // neighbour and the V mask bit of its south neighbour (the faces it shares
  // with them, through which they read its west and south slopes). With the
  // masks of a Veros grid those faces are wet only where the point is, so an
  // own point's key is its first wet level. From its key on a point runs the full
  // computation on every level; before it, its plane quantities are those of
  // a point without mask bits (the constants filled in here) and it has no
  // faces to write but zeros. The arithmetic of every point is unchanged, so
  // results do not depend on the order. On each level the active points are a
  // prefix of the order, so whole warps of dry points skip the FP64 work.
  const int lo = max(kb - 1, 0), hi = min(ke, Z - 1), nkeys = hi - lo + 2;
  int *hist_p = reinterpret_cast<int *>(zeos + Z), *hist_o = hist_p + (Z + 2);
  {
    // plane quantities of a point without mask bits on this level and the one below
    const F rdry = to_F<F>(recip_neg(clamp_eps(0.0)));
    for (int n = tid; n < nkeys; n += NT) hist_p[n] = hist_o[n] = 0;
    for (int p = tid; p < NP; p += NT) {
#pragma unroll
      for (int b = 0; b < 2; ++b) {
        sm.q[b][Q_RT][p] = sm.q[b][Q_RS][p] = F(0);
        sm.q[b][Q_TX][p] = sm.q[b][Q_SX][p] = sm.q[b][Q_TY][p] = sm.q[b][Q_SY][p] = F(0);
        sm.q[b][Q_R0][p] = sm.q[b][Q_R1][p] = rdry;
        sm.qm[b][p] = 0;
      }
      const int i = i0 - 1 + p % PX, j = j0 - 1 + p / PX;
      int f = hi + 1, fu = hi + 1, fv = hi + 1;  // first level with any mask bit, with U, with V
      if (i < L.X && j < L.Y) {
        const uint8_t *mp = a.m + L.at(i, j, 0);
        for (int l0 = lo; l0 <= hi; l0 += 16) {
          unsigned v[16];
#pragma unroll
          for (int u = 0; u < 16; ++u) v[u] = l0 + u <= hi ? __ldg(mp + (long long)(l0 + u) * L.plane) : 0u;
          int cf = hi + 1, cu = hi + 1, cv = hi + 1;  // first of this chunk of levels
#pragma unroll
          for (int u = 15; u >= 0; --u) {
            if (v[u]) cf = l0 + u;
            if (v[u] & VG_MASK_U) cu = l0 + u;
            if (v[u] & VG_MASK_V) cv = l0 + u;
          }
          f = min(f, cf);
          fu = min(fu, cu);
          fv = min(fv, cv);
          if (f <= hi && fu <= hi && fv <= hi) break;
        }
      }
      sm.pkey[p] = (short)(f - lo);
      sm.ukey[p] = (short)(fu - lo);
      sm.vkey[p] = (short)(fv - lo);
    }
  }
  __syncthreads();
  {
    const int e = tid, pce = (e / TX + 1) * PX + e % TX + 1;
    const short k = min(sm.pkey[pce], min(sm.ukey[pce - 1], sm.vkey[pce - PX]));
    sm.okey[e] = k;
    atomicAdd(&hist_o[k], 1);
  }
  for (int p = tid; p < NP; p += NT) atomicAdd(&hist_p[sm.pkey[p]], 1);
  if (tid == 0) sm.slot0 = hw_warp_slot();
  __syncthreads();
  if (warp == 0) warp_exclusive_scan(hist_p, nkeys, lane);
  else if (warp == 1) warp_exclusive_scan(hist_o, nkeys, lane);
  __syncthreads();
  if (warp == 0) warp_stable_scatter(sm.pkey, NP, hist_p, sm.plist, lane);
  else if (warp == 1) warp_stable_scatter(sm.okey, NT, hist_o, sm.olist, lane);
  if (stage) cp_async_wait_all();  // the prologue's planes, visible after this barrier
  __syncthreads();
  // this thread's plane points (compute_plane) and own point (slopes, faces), with their keys;
  // the busiest entries go to virtual warp 0 (virtual_warp spreads co-resident CTAs' busy
  // warps over the sub-partitions)
  const int vt = virtual_warp(warp, NT / 32, sm.slot0) * 32 + lane;
  int pe[kPtSlots], pk[kPtSlots];
#pragma unroll
  // The plane points are taken from a rotated start: the wettest ones go to the virtual warps a
  // half (FP64, 4 of 8) or three quarters (split form, 3 of 4) of the CTA away from those holding
  // the wettest own points, so that on deep levels, where few warps carry work, a level's plane
  // quantities and the previous level's slopes and faces run on different warps side by side
  // instead of one after the other on the same warps. At 1 degree: FP64 pre 0.744 -> 0.705 ms
  // (rotations of 1, 2, 3, 5, 6, 7 warps: 0.737, 0.725, 0.712, 0.704, 0.709, 0.715), split pre
  // 0.346 -> 0.333 ms (1, 2 warps: 0.339, 0.337).
  constexpr int kRot = sizeof(F) == sizeof(double) ? 4 * 32 : 3 * 32;
  for (int s = 0; s < kPtSlots; ++s) {
    const int idx = (vt + kRot) % NT + s * NT;
    pe[s] = idx < NP ? sm.plist[idx] : -1;
    pk[s] = idx < NP ? sm.pkey[pe[s]] : 0x7fff;
  }
  const int oe = sm.olist[vt], ok = sm.okey[oe];
  const int tx = oe % TX, ty = oe / TX;

  // ---- per-point plane quantities ------------------------------------------
  double carryT[kPtSlots], carryS[kPtSlots];  // dT/dz, dS/dz of the previous level per point slot
  unsigned carryW[kPtSlots];                  // W mask of the previous level per point slot
#pragma unroll
  for (int s = 0; s < kPtSlots; ++s) {
    carryT[s] = carryS[s] = 0.0;
    carryW[s] = 0;
  }

  auto compute_plane = [&](int lev, int buf, bool store) {
#pragma unroll
    for (int s = 0; s < kPtSlots; ++s) {
      const int p = pe[s];
      if (p < 0) break;
      if (lev - lo < pk[s]) continue;  // dry so far: the prefilled constants, zero carries
      const int pi = p % PX, pj = p / PX;
      const int i = i0 - 1 + pi, j = j0 - 1 + pj;
      F rT = 0, rS = 0;
      double dTx = 0, dSx = 0, dTy = 0, dSy = 0, dTz = 0, dSz = 0;
      unsigned mk = 0;
      if (i < L.X && j < L.Y) {
        const long long o = L.at(i, j, lev);
        if constexpr (!kStage) {
          // the plane two levels up, which compute_plane(lev + 1) reads as its upper
          // neighbours: in L2 by then (the FP64 form loads T/S from global memory)
          if (store && lev + 2 < Z) {
            prefetch_l2(a.T + o + 2 * L.plane);
            prefetch_l2(a.S + o + 2 * L.plane);
          }
        }
        // T/S at the point, its east and north neighbours and the point above:
        // from the staged ring (split form, rows aligned) or global memory
        auto trc = [&](int which, int di, int dj, int dl) -> double {
          if constexpr (kStage) {
            if (stage) {
              const int sl = (lev + dl) & 3;
              return which ? sm.st.S[sl][pj + dj][pi + di] : sm.st.T[sl][pj + dj][pi + di];
            }
          }
          return __ldg((which ? a.S : a.T) + o + di + dj * L.pitch + dl * L.plane);
        };
        if constexpr (kStage) {
          mk = stage ? (unsigned)sm.st.M[lev & 3][pj][pi] : (unsigned)__ldg(a.m + o);
        } else {
          mk = __ldg(a.m + o);
        }
        const double Tc = trc(0, 0, 0, 0), Sc = trc(1, 0, 0, 0);
        if (mk & VG_MASK_T) {
          rT = to_F<F>(Tc) * eos_c1F + zeosF(lev);  // (isoneutral.py:40, get_rho.py:93-112)
          rS = a.eos_type == 4 ? F(0.0) : F(Eos::betaS * Eos::rho0);
        }
        // horizontal differences; their metric factors are applied in F below
        if ((mk & VG_MASK_U) && i < L.X - 1) {
          dTx = trc(0, 1, 0, 0) - Tc;
          dSx = trc(1, 1, 0, 0) - Sc;
        }
        if ((mk & VG_MASK_V) && j < L.Y - 1) {
          dTy = trc(0, 0, 1, 0) - Tc;
          dSy = trc(1, 0, 1, 0) - Sc;
        }
        if ((mk & VG_MASK_W) && lev < Z - 1) {
          dTz = (trc(0, 0, 0, 1) - Tc) * zinv_dzw[lev];
          dSz = (trc(1, 0, 0, 1) - Sc) * zinv_dzw[lev];
        }
        if (lev >= Z - 1) mk &= ~(unsigned)VG_MASK_W;  // no face above the top level
      }
      if (store) {
        // vertical density gradients in FP64 (exact products of the split form's FP32 values);
        // rS is 0 or the one constant of the equation of state
        const double rTd = to_D(rT), rSd = (mk & VG_MASK_T) ? rS_wet_d : 0.0;
        const double G0 = rTd * carryT[s] + rSd * carryS[s];  // face below (kr = 0)
        const double G1 = rTd * dTz + rSd * dSz;                   // face above (kr = 1)
        F(*q)[NP] = sm.q[buf];
        q[Q_RT][p] = rT;
        q[Q_RS][p] = rS;
        // face gradients (isoneutral.py:64-95): the FP64 difference times
        // 1/(dxu cost) or 1/dyu, the product in F (FP32 in the split form)
        F fx, fy;
        if constexpr (kF32) {
          fx = sm.fv.inv_dxu_cost[p];
          fy = sm.fv.inv_dyu[pj];
        } else {
          fx = sm.inv_dxu_cost[p];
          fy = sm.inv_dyu[pj];
        }
        q[Q_TX][p] = to_F<F>(dTx) * fx;
        q[Q_SX][p] = to_F<F>(dSx) * fx;
        q[Q_TY][p] = to_F<F>(dTy) * fy;
        q[Q_SY][p] = to_F<F>(dSy) * fy;
        q[Q_R0][p] = to_F<F>(recip_neg(clamp_eps(G0)));
        q[Q_R1][p] = to_F<F>(recip_neg(clamp_eps(G1)));
        sm.qm[buf][p] = (uint8_t)(mk | (carryW[s] ? kMaskWBelow : 0u));
      }
      carryT[s] = dTz;
      carryS[s] = dSz;
      carryW[s] = mk & VG_MASK_W;
    }
  };

  // slope (h, v) of plane point p: isoneutral.py:118-122, :155-159, :187-189, :205-207
  const TaperConsts tc{a.slopec * a.inv_dslope, a.inv_dslope, (float)a.slopec, (float)a.inv_dslope};
  // the numerator drdT dT/dh + drdS dS/dh, shared by the two slopes of face h
  auto numer_of = [&](const F(*q)[NP], int p, int h) -> F {
    const int pg = (h == 0 || h == 2) ? p : (h == 1 ? p - 1 : p - PX);
    const int qT = h < 2 ? Q_TX : Q_TY, qS = h < 2 ? Q_SX : Q_SY;
    return q[Q_RT][p] * q[qT][pg] + q[Q_RS][p] * q[qS][pg];
  };
  auto slope_of = [&](const F(*q)[NP], int p, F numer, int v, bool need) -> Slope<F> {
    if (!need) return Slope<F>{F(0), F(0)};
    const F s = -numer * q[v ? Q_R1 : Q_R0][p];
    return Slope<F>{taper_t<F>(s, tc), s};
  };

  const int pc = (ty + 1) * PX + (tx + 1);  // own point in the plane arrays
  // ring point whose west (east ring column) or south (north ring row) slopes this thread publishes:
  // the last TX + TY virtual threads, whose own points are the tile's driest, so that a level's
  // ring work does not lengthen the busiest warps' path to the barrier
  int pring = -1, hring = 0;
  {
    const int rt = vt - (NT - TX - TY);
    if (rt >= 0 && rt < TX) {
      pring = (TY + 1) * PX + rt + 1;
      hring = 3;
    } else if (rt >= TX) {
      pring = (rt - TX + 1) * PX + TX + 1;
      hring = 1;
    }
  }

  // the slopes of the ring points no tile owns (the last tile column / row of the domain)
  const bool ring_store = pring >= 0 && (hring == 1 ? bx == (L.X - 3 + TX - 1) / TX - 1
                                                    : by == (L.Y - 3 + TY - 1) / TY - 1);
  const int ring_i = i0 - 1 + (pring >= 0 ? pring % PX : 0), ring_j = j0 - 1 + (pring >= 0 ? pring / PX : 0);
  const bool own_in = i0 + tx < L.X && j0 + ty < L.Y;

  // the eight slopes of the own point at level lev; publishes its west/south slopes and the ring's
  auto slopes_level = [&](int lev, int b, Slope<F> *out) {
    const F(*q)[NP] = sm.q[b];
    const uint8_t *qm = sm.qm[b];
    F(*pb)[NP] = sm.pub[b];
    if (lev - lo < ok) {
      // no slope of the own point is needed yet, and no neighbour reads its published values
#pragma unroll
      for (int n = 0; n < NS; ++n) out[n] = Slope<F>{F(0), F(0)};
      if (a.slopes && lev < ke && own_in) {
        double *sl = a.slopes + L.at(i0 + tx, j0 + ty, lev);
        const long long F_ = a.slope_field;
#pragma unroll
        for (int n = 0; n < NS; ++n) {
          sl[(SLOPE_T + n) * F_] = 0.0;
          sl[(SLOPE_S + n) * F_] = 0.0;
        }
        sl[SLOPE_R * F_] = (double)q[Q_R0][pc];
        sl[(SLOPE_R + 1) * F_] = (double)q[Q_R1][pc];
      }
    } else {
    const unsigned m = qm[pc];
    const bool mH[4] = {(m & VG_MASK_U) != 0, (qm[pc - 1] & VG_MASK_U) != 0, (m & VG_MASK_V) != 0,
                        (qm[pc - PX] & VG_MASK_V) != 0};
    const bool mWv[2] = {(m & kMaskWBelow) != 0, (m & VG_MASK_W) != 0};
#pragma unroll
    for (int h = 0; h < 4; ++h) {
      const bool need0 = lev > 0 && (mH[h] || mWv[0]), need1 = mH[h] || mWv[1];
      const F numer = (need0 || need1) ? numer_of(q, pc, h) : F(0);
      out[h * 2] = slope_of(q, pc, numer, 0, need0);
      out[h * 2 + 1] = slope_of(q, pc, numer, 1, need1);
    }
    if (a.slopes && lev < ke && own_in) {
      double *sl = a.slopes + L.at(i0 + tx, j0 + ty, lev);
      const long long F_ = a.slope_field;
#pragma unroll
      for (int n = 0; n < NS; ++n) {
        sl[(SLOPE_T + n) * F_] = (double)out[n].t;
        sl[(SLOPE_S + n) * F_] = (double)out[n].s;
      }
      sl[SLOPE_R * F_] = (double)q[Q_R0][pc];
      sl[(SLOPE_R + 1) * F_] = (double)q[Q_R1][pc];
    }
#pragma unroll
    for (int v = 0; v < 2; ++v) {
      pb[PB_T_XW0 + v][pc] = out[S_XW0 + v].t;
      pb[PB_TS_XW0 + v][pc] = out[S_XW0 + v].t * F(out[S_XW0 + v].s);
      pb[PB_T_YS0 + v][pc] = out[S_YS0 + v].t;
      pb[PB_TS_YS0 + v][pc] = out[S_YS0 + v].t * F(out[S_YS0 + v].s);
    }
    }
    if (pring >= 0) {
      const bool mHr = hring == 1 ? (qm[pring - 1] & VG_MASK_U) != 0 : (qm[pring - PX] & VG_MASK_V) != 0;
      const int base_t = hring == 1 ? PB_T_XW0 : PB_T_YS0, base_ts = hring == 1 ? PB_TS_XW0 : PB_TS_YS0;
      const F numer = mHr ? numer_of(q, pring, hring) : F(0);
#pragma unroll
      for (int v = 0; v < 2; ++v) {
        const Slope<F> sl = slope_of(q, pring, numer, v, mHr && (v == 1 || lev > 0));
        pb[base_t + v][pring] = sl.t;
        pb[base_ts + v][pring] = sl.t * F(sl.s);
        if (a.slopes && lev < ke && ring_store && ring_i < L.X && ring_j < L.Y) {
          double *st = a.slopes + L.at(ring_i, ring_j, lev);
          const int n = hring * 2 + v;
          st[(SLOPE_T + n) * a.slope_field] = (double)sl.t;
          st[(SLOPE_S + n) * a.slope_field] = (double)sl.s;
          st[(SLOPE_R + v) * a.slope_field] = (double)q[v ? Q_R1 : Q_R0][pring];
        }
      }
    }
  };

  if (kb > 0) compute_plane(kb - 1, (kb - 1) & 1, false);  // only the carries
  compute_plane(kb, kb & 1, true);
  __syncthreads();
  // staged ring: plane kb+3 into the slot of plane kb-1, which nobody reads any more
  if (stage && kb + 3 <= pmax) issue_plane(kb + 3);
  Slope<F> cur[NS], nxt[NS];
#pragma unroll
  for (int n = 0; n < NS; ++n) nxt[n] = Slope<F>{F(0), F(0)};
  slopes_level(kb, kb & 1, cur);

  const int i = i0 + tx, j = j0 + ty;
  const bool lin_steep = a.ksteep <= 0.0;
  const F ksteepF = to_F<F>(a.ksteep);
  const bool east = i < L.X - 2 && j >= 2 && j < L.Y - 2;
  const bool north = i >= 2 && i < L.X - 2 && j < L.Y - 2;
  const bool top = i >= 2 && i < L.X - 2 && j >= 2 && j < L.Y - 2;

  for (int k = kb; k < ke; ++k) {
    if (k + 1 < Z) compute_plane(k + 1, (k + 1) & 1, true);
    // this thread's copies of plane k+3 (issued one level ago) have landed
    if (stage) cp_async_wait_all();
    // the own point's mask on level k, from the plane copy compute_plane(k) stored (zero before the
    // point's key, like the mask itself); read before this level's barrier, after which
    // compute_plane(k + 2) may rewrite the buffer. The face loads of K_iso then need no global
    // round trip for the mask first.
    const unsigned mk = (east || north || top) ? (unsigned)sm.qm[k & 1][pc] : 0u;
    // K_iso of the next level's faces, in L2 by then
    if (k + 1 < Z && (east || north || top) && k + 1 - lo >= ok) prefetch_l2(a.K + L.at(i, j, k + 1));
    // plane k+1 complete; the slopes of level k published; nobody still reads the buffers rewritten next;
    // the staged plane k+3 visible
    __syncthreads();
    // staged ring: plane k+4 into the slot of plane k, last read by compute_plane(k) and (k-1)
    if (stage && k + 4 <= pmax) issue_plane(k + 4);
    if (k + 1 < Z) slopes_level(k + 1, (k + 1) & 1, nxt);
    const F(*pb)[NP] = sm.pub[k & 1];
    const F(*pbn)[NP] = sm.pub[(k + 1) & 1];  // level k+1 (written only when k + 1 < Z; read only then)
    const long long o = L.at(i, j, k);
    // the face terms' grid factors in the derived-field type
    const F dzwF[2] = {zdzwF(k > 0 ? k - 1 : 0), zdzwF(k)}, qzF = zqF_(k);

    // east face: Ai_ez, K_11 (isoneutral.py:100-132); ip = 0 is this point, ip = 1 the east neighbour
    if (east) {
      F sumz = 0.0;
      if (mk & VG_MASK_U) {
        F diffloc;
        if (k >= 1)
          diffloc = F(0.25) * (__ldg(a.K + o) + __ldg(a.K + o - L.plane) + __ldg(a.K + o + 1) +
                               __ldg(a.K + o + 1 - L.plane));
        else
          diffloc = F(0.5) * (__ldg(a.K + o) + __ldg(a.K + o + 1));
        F t[2][2] = {{F(0), F(0)}, {F(0), F(0)}};  // [kr][ip]
#pragma unroll
        for (int kr = 0; kr < 2; ++kr) {
          if (kr == 0 && k == 0) continue;
          t[kr][0] = cur[S_XE0 + kr].t;
          t[kr][1] = pb[PB_T_XW0 + kr][pc + 1];
          a.Aez[o + kr * a.sr] = t[kr][0] * F(cur[S_XE0 + kr].s);
          a.Aez[o + a.sp + kr * a.sr] = pb[PB_TS_XW0 + kr][pc + 1];
        }
        sumz = face_sumz(t, dzwF, diffloc, ksteepF, lin_steep, k);
      } else {
#pragma unroll
        for (int kr = 0; kr < 2; ++kr) {
          if (kr == 0 && k == 0) continue;
          a.Aez[o + kr * a.sr] = 0.0;
          a.Aez[o + a.sp + kr * a.sr] = 0.0;
        }
      }
      a.K11[o] = sumz * qzF;
    }

    // north face: Ai_nz, K_22 (isoneutral.py:137-168); jp = 0 is this point, jp = 1 the north neighbour
    if (north) {
      F sumz = 0.0;
      if (mk & VG_MASK_V) {
        F diffloc;
        if (k >= 1)
          diffloc = F(0.25) * (__ldg(a.K + o) + __ldg(a.K + o - L.plane) + __ldg(a.K + o + L.pitch) +
                               __ldg(a.K + o + L.pitch - L.plane));
        else
          diffloc = F(0.5) * (__ldg(a.K + o) + __ldg(a.K + o + L.pitch));
        F t[2][2] = {{F(0), F(0)}, {F(0), F(0)}};
#pragma unroll
        for (int kr = 0; kr < 2; ++kr) {
          if (kr == 0 && k == 0) continue;
          t[kr][0] = cur[S_YN0 + kr].t;
          t[kr][1] = pb[PB_T_YS0 + kr][pc + PX];
          a.Anz[o + kr * a.sr] = t[kr][0] * F(cur[S_YN0 + kr].s);
          a.Anz[o + a.sp + kr * a.sr] = pb[PB_TS_YS0 + kr][pc + PX];
        }
        sumz = face_sumz(t, dzwF, diffloc, ksteepF, lin_steep, k);
      } else {
#pragma unroll
        for (int kr = 0; kr < 2; ++kr) {
          if (kr == 0 && k == 0) continue;
          a.Anz[o + kr * a.sr] = 0.0;
          a.Anz[o + a.sp + kr * a.sr] = 0.0;
        }
      }
      a.K22[o] = sumz * qzF;
    }

    // top face: Ai_bx, Ai_by, K_33 (isoneutral.py:173-224); kr = 0 is this point's upper slopes,
    // kr = 1 the lower slopes of the point above. K_33 = K_iso sum over the 8 slopes of
    // w (taper s) s, w the slope's dqx / dqy weight: K_iso factors out of the sums.
    if (top && k < Z - 1) {
      F k33 = 0.0;
      if (mk & VG_MASK_W) {
        F sx[2], sy[2];
#pragma unroll
        for (int ip = 0; ip < 2; ++ip) {
          // the west slopes' taper*s were published by slopes_level (levels k and k+1)
          const Slope<F> s0 = cur[ip ? S_XE1 : S_XW1], s1 = nxt[ip ? S_XE0 : S_XW0];
          const F a0 = ip ? s0.t * F(s0.s) : pb[PB_TS_XW1][pc], a1 = ip ? s1.t * F(s1.s) : pbn[PB_TS_XW0][pc];
          a.Abx[o + ip * a.sp] = a0;
          a.Abx[o + ip * a.sp + a.sr] = a1;
          // taper*s^2 as (taper*s)*s: reuses Ai and stays finite where an FP32 s^2
          // would overflow under a vanishing taper
          sx[ip] = a0 * F(s0.s) + a1 * F(s1.s);
        }
#pragma unroll
        for (int jp = 0; jp < 2; ++jp) {
          const Slope<F> s0 = cur[jp ? S_YN1 : S_YS1], s1 = nxt[jp ? S_YN0 : S_YS0];
          const F a0 = jp ? s0.t * F(s0.s) : pb[PB_TS_YS1][pc], a1 = jp ? s1.t * F(s1.s) : pbn[PB_TS_YS0][pc];
          a.Aby[o + jp * a.sp] = a0;
          a.Aby[o + jp * a.sp + a.sr] = a1;
          sy[jp] = a0 * F(s0.s) + a1 * F(s1.s);
        }
        F w;
        if constexpr (kF32)
          w = sm.fv.dqx[0][tx] * sx[0] + sm.fv.dqx[1][tx] * sx[1] + sm.fv.dqy[0][ty] * sy[0] +
              sm.fv.dqy[1][ty] * sy[1];
        else
          w = sm.dqx[0][tx] * sx[0] + sm.dqx[1][tx] * sx[1] + sm.dqy[0][ty] * sy[0] + sm.dqy[1][ty] * sy[1];
        k33 = __ldg(a.K + o) * w;
      } else {
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const long long oc = o + (c >> 1) * a.sp + (c & 1) * a.sr;
          a.Abx[oc] = 0.0;
          a.Aby[oc] = 0.0;
        }
      }
      a.K33[o] = k33;
    }
#pragma unroll
    for (int n = 0; n < NS; ++n) cur[n] = nxt[n];
  }
}

// Persistent form: the ntiles * Z tile-levels, tile-major, are cut into
// gridDim.x ranges, and CTA c walks range c as one segment per tile it
// touches (a segment starting above level 0 pays the restart of a k-chunk).
// The ranges are starts[c] .. starts[c+1] (shares weighted by the water on
// each tile-level, span_shares.cu) or, without starts, equal counts of
// tile-levels. With a whole number of tiles per SM rarely available, shares
// keep every SM busy to the end of the launch.
template <typename F, int TY>
__global__ void __launch_bounds__(32 * TY, 16 / TY) pre_span_kernel(PreArgs<F> a, int ntx, int ntiles,
                                                                     const long long *__restrict__ starts) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int Z = a.L.Z;
  const long long W = (long long)ntiles * Z;
  long long p = starts ? starts[blockIdx.x] : W * blockIdx.x / gridDim.x;
  const long long end = starts ? starts[blockIdx.x + 1] : W * (blockIdx.x + 1) / gridDim.x;
  while (p < end) {
    const int t = (int)(p / Z), kb = (int)(p % Z);
    const int ke = (int)min((long long)Z, end - (long long)t * Z);
    pre_tile_body<F, TY>(a, smem_raw, t % ntx, t / ntx, kb, ke);
    cp_async_wait_all();  // no staged copy of this segment may land in the next one's buffers
    __syncthreads();      // shared memory is rebuilt by the next segment
    p = (long long)t * Z + ke;
  }
}

}  // namespace detail

// The FP64 tensor of one domain plus the per-point slope fields of
// PreArgs::slopes (SLOPE_FIELDS fields of plane * Z doubles), for the adjoint.
int pre_f64_with_slopes(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set, const double *temp_tau,
                        const double *salt_tau, const double *K_iso, const uint8_t *mask_bits,
                        const VgTensorFields *out, double *slopes, void *stream);
}  // namespace vg
