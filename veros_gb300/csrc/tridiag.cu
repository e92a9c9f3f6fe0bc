// Column tridiagonal solves.
//
// * vg_solve_implicit_f64 / _f32: the drop-in for solve_implicit /
//   solve_tridiagonal (veros/core/utilities.py:51-59,
//   veros/core/operators.py:60-77) on float64 or float32 arrays. One thread
//   per column solves that column's water cells k = ks..nz-1 by Gaussian
//   elimination with partial pivoting in the operation order of LAPACK dgtsv,
//   which the reference calls (dgtsv.cuh); the factors stay in shared memory.
// * vg_tdma_cuda_{double,float}: same buffers/descriptor contract as the XLA
//   custom-call targets of veros/core/special/cuda_tdma_kernels.cu:81-111
//   (full-depth Thomas sweep, identity rows already folded in by the caller,
//   tdma_.py:63-66), but c' is kept in shared memory instead of a global
//   workspace and errors are reported instead of exiting.
#include <algorithm>
#include <cstring>

#include "common.cuh"
#include "dgtsv.cuh"

namespace vg {

namespace {

constexpr int kMaxNz = 200;

// Storage type T of the coefficients, right-hand sides and solution: double,
// or float for the reference's float32 runs, whose NumPy solve hands float32
// arrays to LAPACK dgtsv, which works on float64 copies, and stores the
// float64 solution into a float32 output (veros/core/operators.py:64, :75-76).
// The elimination below is always in double; a float solution is rounded
// once, on its store.
template <typename T>
struct TriArgs {
  int nsx, nsys, nz;
  long long sx, sy, sz;
  const T *a, *b, *c, *d, *b_edge, *d_edge;
  const uint8_t *water, *edge;
  T *out;
  int *bad;
};

// Row source of one generic column (b_edge/d_edge substituted at ks,
// utilities.py:53-57; a at the edge row is never read, operators.py:72).
// float entries widen to double exactly.
template <typename T>
struct GenSrc {
  const TriArgs<T> &p;
  long long base;
  int ks;
  __device__ long long at(int k) const { return base + p.sz * k; }
  __device__ double a(int k) const { return (double)p.a[at(k)]; }
  __device__ double b(int k) const { return (double)((k == ks && p.b_edge) ? p.b_edge[at(k)] : p.b[at(k)]); }
  __device__ double c(int k) const { return (double)p.c[at(k)]; }
  __device__ double d(int k) const { return (double)((k == ks && p.d_edge) ? p.d_edge[at(k)] : p.d[at(k)]); }
};

// One thread per column. Shared memory holds the eliminated diagonal of the
// CTA's columns, laid out [k][thread]; the eliminated right-hand side goes
// to the output when that is double (the back substitution overwrites it
// with the solution; the column stays in L2 between the sweeps), or to a
// second shared array [k][thread] when the output is float. With an
// interchange the column is re-solved from the inputs into the diagonal
// slots.
constexpr int kTriMaxThreads = 128;

template <typename T>
__global__ void __launch_bounds__(kTriMaxThreads) pivoting_solve_kernel(TriArgs<T> p) {
  extern __shared__ double sm[];
  __shared__ int ks_s[kTriMaxThreads], perm_s[kTriMaxThreads];
  const int t = threadIdx.x;
  const int nb = blockDim.x;
  const int nz = p.nz;
  auto base_of = [&](int s) { return p.sx * (long long)(s % p.nsx) + p.sy * (long long)(s / p.nsx); };

  // water/edge form check of the thread's own column (create_water_masks,
  // utilities.py:38-48) and the zero output of its rows k < ks
  {
    const int s = blockIdx.x * nb + t;
    int ks = -1;
    if (s < p.nsys) {
      const long long base = base_of(s);
      bool bad = false;
#pragma unroll 4
      for (int k = 0; k < nz; ++k) {
        const long long o = base + p.sz * k;
        const bool w = p.water[o] != 0, e = p.edge[o] != 0;
        if (ks < 0 && w) ks = k;
        if (w != (ks >= 0) || e != (ks == k)) bad = true;
      }
      if (bad && p.bad) atomicAdd(p.bad, 1);
      for (int k = 0; k < (ks < 0 ? nz : ks); ++k) p.out[base + p.sz * k] = T(0);
    }
    ks_s[t] = ks;
  }
  __syncthreads();
  // The CTA's columns ranked by their number of water rows (most first, ties
  // by position), so that the lanes of a warp solve systems of similar size.
  {
    const int n = ks_s[t] < 0 ? 0 : nz - ks_s[t];
    int rank = 0;
    for (int u = 0; u < nb; ++u) {
      const int m = ks_s[u] < 0 ? 0 : nz - ks_s[u];
      rank += (m > n) || (m == n && u < t);
    }
    perm_s[rank] = t;
  }
  __syncthreads();
  const int s = blockIdx.x * nb + perm_s[t];
  const int ks = ks_s[perm_s[t]];
  if (s >= p.nsys || ks < 0) return;
  const long long base = base_of(s);
  GenSrc<T> src{p, base, ks};
  double *Ds = sm + t;
  T *out = p.out + base;  // the solution
  // the eliminated right-hand side: in the output (double) or in shared memory (float)
  double *Bs;
  long long bstride;
  if constexpr (sizeof(T) == sizeof(double)) {
    Bs = reinterpret_cast<double *>(out);
    bstride = p.sz;
  } else {
    Bs = sm + (size_t)nb * nz + t;
    bstride = nb;
  }

  // Loads run PF levels ahead of the elimination's serial chain (software
  // pipelining); the arithmetic is dgtsv's, operation for operation.
  constexpr int PF = 8;
  double qa[PF], qb[PF], qc[PF], qd[PF];
#pragma unroll
  for (int u = 0; u < PF; ++u) {
    const int k = ks + 1 + u;
    qa[u] = k < nz ? src.a(k) : 0.0;
    qb[u] = k < nz ? (double)p.b[src.at(k)] : 0.0;
    qc[u] = k < nz - 1 ? src.c(k) : 0.0;
    qd[u] = k < nz ? (double)p.d[src.at(k)] : 0.0;
  }
  // elimination without interchange while dgtsv would take that branch
  bool interchange = false;
  double Dp = src.b(ks), Bp = src.d(ks), cp = ks < nz - 1 ? src.c(ks) : 0.0;
  Ds[(size_t)ks * nb] = Dp;
  Bs[bstride * ks] = Bp;
  for (int k0 = ks + 1; k0 < nz && !interchange; k0 += PF) {
#pragma unroll
    for (int u = 0; u < PF; ++u) {
      const int k = k0 + u;
      if (k < nz && !interchange) {
        const double dl = qa[u], bk = qb[u], ck = qc[u], dk = qd[u];
        const int kn = k + PF;
        if (kn < nz) {
          qa[u] = src.a(kn);
          qb[u] = (double)p.b[src.at(kn)];
          qc[u] = kn < nz - 1 ? src.c(kn) : 0.0;
          qd[u] = (double)p.d[src.at(kn)];
        }
        if (fabs(Dp) < fabs(dl)) {
          interchange = true;
        } else {
          const double fact = rdiv(dl, Dp);
          Dp = rsub(bk, rmul(fact, cp));
          Bp = rsub(dk, rmul(fact, Bp));
          cp = ck;
          Ds[(size_t)k * nb] = Dp;
          Bs[bstride * k] = Bp;
        }
      }
    }
  }
  if (interchange) {
    // the row sources are the inputs, which the output does not overlap
    dgtsv_slow_solve(src, ks, nz, Ds, nb);
    for (int k = ks; k < nz; ++k) out[p.sz * k] = (T)Ds[(size_t)k * nb];
    return;
  }
  double qcb[PF], qbs[PF];
#pragma unroll
  for (int u = 0; u < PF; ++u) {
    const int k = nz - 2 - u;
    qcb[u] = k >= ks ? src.c(k) : 0.0;
    qbs[u] = k >= ks ? Bs[bstride * k] : 0.0;
  }
  double x = rdiv(Bs[bstride * (nz - 1)], Ds[(size_t)(nz - 1) * nb]);
  out[p.sz * (nz - 1)] = (T)x;
  for (int k0 = nz - 2; k0 >= ks; k0 -= PF) {
#pragma unroll
    for (int u = 0; u < PF; ++u) {
      const int k = k0 - u;
      if (k >= ks) {
        const double ck = qcb[u], bk = qbs[u];
        if (k - PF >= ks) {
          qcb[u] = src.c(k - PF);
          qbs[u] = Bs[bstride * (k - PF)];
        }
        x = rdiv(rsub(bk, rmul(ck, x)), Ds[(size_t)k * nb]);
        out[p.sz * k] = (T)x;
      }
    }
  }
}

// Reciprocal of a pivot: the FP32 division in single precision; in double,
// recip_any (an FP32 seed refined by two Newton steps, within an ulp of the
// quotient) in place of the IEEE division, which takes tens of FP64
// instructions.
__device__ __forceinline__ float pivot_recip(float x) { return 1.0f / x; }
__device__ __forceinline__ double pivot_recip(double x) { return recip_any(x); }

// One thread per system; c' in shared memory [k][thread], d' in the output
// (overwritten by the solution in the back substitution). Both sweeps load PF
// levels ahead of their serial chain.
template <typename F>
__global__ void xla_thomas_kernel(const F *__restrict__ a, const F *__restrict__ b, const F *__restrict__ c,
                                  const F *__restrict__ d, F *__restrict__ out, int nsys, int depth) {
  extern __shared__ unsigned char sm_raw[];
  F *cp = reinterpret_cast<F *>(sm_raw);
  const int t = threadIdx.x, nb = blockDim.x;
  const int s = blockIdx.x * nb + t;
  if (s >= nsys) return;
  const long long n = nsys;
  constexpr int PF = 4;
  F qa[PF], qb[PF], qc[PF], qd[PF];
#pragma unroll
  for (int u = 0; u < PF; ++u) {
    const long long o = s + n * min(1 + u, depth - 1);
    qa[u] = a[o];
    qb[u] = b[o];
    qc[u] = c[o];
    qd[u] = d[o];
  }
  const F r0 = pivot_recip(b[s]);
  F cm = c[s] * r0;
  F dm = d[s] * r0;
  cp[t] = cm;
  out[s] = dm;
  for (int k0 = 1; k0 < depth; k0 += PF) {
#pragma unroll
    for (int u = 0; u < PF; ++u) {
      const int k = k0 + u;
      if (k < depth) {
        const F ak = qa[u], bk = qb[u], ck = qc[u], dk = qd[u];
        const int kn = k + PF;
        if (kn < depth) {
          const long long on = s + n * kn;
          qa[u] = a[on];
          qb[u] = b[on];
          qc[u] = c[on];
          qd[u] = d[on];
        }
        const F den = pivot_recip(bk - ak * cm);
        cm = ck * den;
        dm = (dk - ak * dm) * den;
        cp[(size_t)k * nb + t] = cm;
        out[s + n * k] = dm;
      }
    }
  }
  F qo[PF];
#pragma unroll
  for (int u = 0; u < PF; ++u) {
    const int k = depth - 2 - u;
    qo[u] = k >= 0 ? out[s + n * k] : F(0);
  }
  F x = dm;
  for (int k0 = depth - 2; k0 >= 0; k0 -= PF) {
#pragma unroll
    for (int u = 0; u < PF; ++u) {
      const int k = k0 - u;
      if (k >= 0) {
        const F ok = qo[u];
        if (k - PF >= 0) qo[u] = out[s + n * (k - PF)];
        x = ok - cp[(size_t)k * nb + t] * x;
        out[s + n * k] = x;
      }
    }
  }
}

struct TdmaDescriptor {
  int num_systems;
  int system_depth;
};

template <typename F>
void xla_tdma(void *stream, void **buffers, const char *opaque, size_t opaque_len, const char *name) {
  clear_error();
  if (opaque_len != sizeof(TdmaDescriptor) || !opaque || !buffers) {
    fail(VG_ERR_ARG, "%s: descriptor of %zu bytes, expected %zu", name, opaque_len, sizeof(TdmaDescriptor));
    return;
  }
  TdmaDescriptor desc;
  memcpy(&desc, opaque, sizeof(desc));
  if (desc.num_systems <= 0 || desc.system_depth <= 0 || desc.system_depth > 4096) {
    fail(VG_ERR_SHAPE, "%s: num_systems=%d system_depth=%d", name, desc.num_systems, desc.system_depth);
    return;
  }
  const F *a = static_cast<const F *>(buffers[0]);
  const F *b = static_cast<const F *>(buffers[1]);
  const F *c = static_cast<const F *>(buffers[2]);
  const F *d = static_cast<const F *>(buffers[3]);
  F *out = static_cast<F *>(buffers[4]);
  // one warp per CTA: the CTAs of a launch are spread evenly over the SMs
  const int nb = 32;
  const size_t smem = (size_t)nb * desc.system_depth * sizeof(F);
  if (smem > 200 * 1024) {
    fail(VG_ERR_SHAPE, "%s: system_depth %d too deep", name, desc.system_depth);
    return;
  }
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(xla_thomas_kernel<F>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) {
      fail(VG_ERR_LAUNCH, "%s: %s", name, cudaGetErrorString(e));
      return;
    }
  }
  xla_thomas_kernel<F><<<(desc.num_systems + nb - 1) / nb, nb, smem, as_stream(stream)>>>(a, b, c, d, out,
                                                                                        desc.num_systems,
                                                                                        desc.system_depth);
  check_launch(name);
}

template <typename T>
int solve_implicit(const char *name, int nsx, int nsy, int nz, long long s_x, long long s_y, long long s_z,
                   const T *a, const T *b, const T *c, const T *d, const uint8_t *water, const uint8_t *edge,
                   const T *b_edge, const T *d_edge, T *out, int *bad_columns, void *stream) {
  clear_error();
  if (nsx < 0 || nsy < 0 || nz < 1 || nz > kMaxNz)
    return fail(VG_ERR_SHAPE, "%s: nsx=%d nsy=%d nz=%d (1 <= nz <= %d)", name, nsx, nsy, nz, kMaxNz);
  if (!a || !b || !c || !d || !water || !edge || !out) return fail(VG_ERR_ARG, "%s: NULL pointer", name);
  const long long nsys = (long long)nsx * nsy;
  if (nsys == 0) return VG_OK;
  if (nsys > 0x7fffffffLL) return fail(VG_ERR_SHAPE, "%s: too many columns", name);
  {
    // the output holds intermediate values while the inputs are still read:
    // it may not overlap them (element offsets span [lo, hi] in every array)
    long long lo = 0, hi = 0;
    for (const long long span : {s_x * (nsx - 1), s_y * (nsy - 1), s_z * (nz - 1)}) (span < 0 ? lo : hi) += span;
    const long long es = (long long)sizeof(T);
    const char *o0 = reinterpret_cast<const char *>(out) + lo * es;
    const char *o1 = reinterpret_cast<const char *>(out) + (hi + 1) * es;
    auto overlaps = [&](const void *q, long long elem) {
      if (!q) return false;
      const char *q0 = static_cast<const char *>(q) + lo * elem;
      const char *q1 = static_cast<const char *>(q) + (hi + 1) * elem;
      return q0 < o1 && o0 < q1;
    };
    if (overlaps(a, es) || overlaps(b, es) || overlaps(c, es) || overlaps(d, es) || overlaps(b_edge, es) ||
        overlaps(d_edge, es) || overlaps(water, 1) || overlaps(edge, 1))
      return fail(VG_ERR_ARG, "%s: out overlaps an input", name);
  }
  TriArgs<T> p{nsx, (int)nsys, nz, s_x, s_y, s_z, a, b, c, d, b_edge, d_edge, water, edge, out, bad_columns};
  // shared doubles per column and level: the eliminated diagonal, and for a
  // float output also the eliminated right-hand side
  const size_t per = sizeof(T) == sizeof(double) ? 1 : 2;
  int nb = kTriMaxThreads;
  while (nb > 32 && (size_t)nb * nz * per * sizeof(double) > 100 * 1024) nb /= 2;
  const size_t smem = (size_t)nb * nz * per * sizeof(double);
  if (smem > 48 * 1024) {
    cudaError_t e =
        cudaFuncSetAttribute(pivoting_solve_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return fail(VG_ERR_LAUNCH, "%s: pivoting_solve_kernel smem: %s", name, cudaGetErrorString(e));
  }
  pivoting_solve_kernel<T><<<(unsigned)((nsys + nb - 1) / nb), nb, smem, as_stream(stream)>>>(p);
  return check_launch("pivoting_solve_kernel");
}

}  // namespace

}  // namespace vg

using namespace vg;

extern "C" int vg_solve_implicit_f64(int nsx, int nsy, int nz, long long s_x, long long s_y, long long s_z,
                                     const double *a, const double *b, const double *c, const double *d,
                                     const uint8_t *water, const uint8_t *edge, const double *b_edge,
                                     const double *d_edge, double *out, int *bad_columns, void *stream) {
  return solve_implicit<double>("vg_solve_implicit_f64", nsx, nsy, nz, s_x, s_y, s_z, a, b, c, d, water, edge,
                                b_edge, d_edge, out, bad_columns, stream);
}

extern "C" int vg_solve_implicit_f32(int nsx, int nsy, int nz, long long s_x, long long s_y, long long s_z,
                                     const float *a, const float *b, const float *c, const float *d,
                                     const uint8_t *water, const uint8_t *edge, const float *b_edge,
                                     const float *d_edge, float *out, int *bad_columns, void *stream) {
  return solve_implicit<float>("vg_solve_implicit_f32", nsx, nsy, nz, s_x, s_y, s_z, a, b, c, d, water, edge,
                               b_edge, d_edge, out, bad_columns, stream);
}

extern "C" void vg_tdma_cuda_double(void *stream, void **buffers, const char *opaque, size_t opaque_len) {
  xla_tdma<double>(stream, buffers, opaque, opaque_len, "vg_tdma_cuda_double");
}

extern "C" void vg_tdma_cuda_float(void *stream, void **buffers, const char *opaque, size_t opaque_len) {
  xla_tdma<float>(stream, buffers, opaque, opaque_len, "vg_tdma_cuda_float");
}
