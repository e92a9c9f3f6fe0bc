// Column tridiagonal solves.
//
// * vg_solve_implicit_f64: the drop-in for solve_implicit / solve_tridiagonal
//   (veros/core/utilities.py:51-59, veros/core/operators.py:60-77). One thread
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

struct TriArgs {
  int nsx, nsys, nz;
  long long sx, sy, sz;
  const double *a, *b, *c, *d, *b_edge, *d_edge;
  const uint8_t *water, *edge;
  double *out;
  int *bad;
};

// Row source of one generic column (b_edge/d_edge substituted at ks,
// utilities.py:53-57; a at the edge row is never read, operators.py:72).
struct GenSrc {
  const TriArgs &p;
  long long base;
  int ks;
  __device__ long long at(int k) const { return base + p.sz * k; }
  __device__ double a(int k) const { return p.a[at(k)]; }
  __device__ double b(int k) const { return (k == ks && p.b_edge) ? p.b_edge[at(k)] : p.b[at(k)]; }
  __device__ double c(int k) const { return p.c[at(k)]; }
  __device__ double d(int k) const { return (k == ks && p.d_edge) ? p.d_edge[at(k)] : p.d[at(k)]; }
};

// One thread per column. Shared memory holds the eliminated diagonal and
// right-hand side of the column, laid out [k][field][thread]; the solution
// reuses the diagonal slots.
__global__ void pivoting_solve_kernel(TriArgs p) {
  extern __shared__ double sm[];
  const int t = threadIdx.x;
  const int nb = blockDim.x;
  const int s = blockIdx.x * nb + t;
  if (s >= p.nsys) return;
  const long long base = p.sx * (long long)(s % p.nsx) + p.sy * (long long)(s / p.nsx);
  const int nz = p.nz;

  // water/edge form check (create_water_masks, utilities.py:38-48)
  int ks = -1;
  bool bad = false;
  for (int k = 0; k < nz; ++k) {
    const long long o = base + p.sz * k;
    const bool w = p.water[o] != 0, e = p.edge[o] != 0;
    if (ks < 0 && w) ks = k;
    if (w != (ks >= 0) || e != (ks == k)) bad = true;
  }
  if (bad && p.bad) atomicAdd(p.bad, 1);

  for (int k = 0; k < (ks < 0 ? nz : ks); ++k) p.out[base + p.sz * k] = 0.0;
  if (ks < 0) return;
  GenSrc src{p, base, ks};
  double *Ds = sm + t;
  double *Bs = sm + (size_t)nz * nb + t;

  // elimination without interchange while dgtsv would take that branch
  bool interchange = false;
  double Dp = src.b(ks), Bp = src.d(ks), cp = ks < nz - 1 ? src.c(ks) : 0.0;
  Ds[(size_t)ks * nb] = Dp;
  Bs[(size_t)ks * nb] = Bp;
  for (int k = ks + 1; k < nz && !interchange; ++k) {
    const double dl = src.a(k);
    if (fabs(Dp) < fabs(dl)) {
      interchange = true;
      break;
    }
    const double fact = rdiv(dl, Dp);
    Dp = rsub(src.b(k), rmul(fact, cp));
    Bp = rsub(src.d(k), rmul(fact, Bp));
    cp = k < nz - 1 ? src.c(k) : 0.0;
    Ds[(size_t)k * nb] = Dp;
    Bs[(size_t)k * nb] = Bp;
  }
  if (interchange) {
    dgtsv_slow_solve(src, ks, nz, Ds, nb);
  } else {
    double x = 0.0;
    for (int k = nz - 1; k >= ks; --k) {
      const double Dk = Ds[(size_t)k * nb], Bk = Bs[(size_t)k * nb];
      x = (k == nz - 1) ? rdiv(Bk, Dk) : rdiv(rsub(Bk, rmul(src.c(k), x)), Dk);
      Ds[(size_t)k * nb] = x;
    }
  }
  for (int k = ks; k < nz; ++k) p.out[base + p.sz * k] = Ds[(size_t)k * nb];
}

template <typename F>
__global__ void xla_thomas_kernel(const F *__restrict__ a, const F *__restrict__ b, const F *__restrict__ c,
                                  const F *__restrict__ d, F *__restrict__ out, int nsys, int depth) {
  extern __shared__ unsigned char sm_raw[];
  F *cp = reinterpret_cast<F *>(sm_raw);
  const int t = threadIdx.x, nb = blockDim.x;
  const int s = blockIdx.x * nb + t;
  if (s >= nsys) return;
  long long o = s;
  F cm = c[o] / b[o];
  F dm = d[o] / b[o];
  cp[t] = cm;
  out[o] = dm;
  for (int k = 1; k < depth; ++k) {
    o += nsys;
    const F ak = a[o];
    const F den = F(1) / (b[o] - ak * cm);
    cm = c[o] * den;
    dm = (d[o] - ak * dm) * den;
    cp[(size_t)k * nb + t] = cm;
    out[o] = dm;
  }
  F x = dm;
  for (int k = depth - 2; k >= 0; --k) {
    o -= nsys;
    x = out[o] - cp[(size_t)k * nb + t] * x;
    out[o] = x;
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
  int nb = 128;
  while (nb > 32 && (size_t)nb * desc.system_depth * sizeof(F) > 96 * 1024) nb /= 2;
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

}  // namespace

}  // namespace vg

using namespace vg;

extern "C" int vg_solve_implicit_f64(int nsx, int nsy, int nz, long long s_x, long long s_y, long long s_z,
                                     const double *a, const double *b, const double *c, const double *d,
                                     const uint8_t *water, const uint8_t *edge, const double *b_edge,
                                     const double *d_edge, double *out, int *bad_columns, void *stream) {
  clear_error();
  if (nsx < 0 || nsy < 0 || nz < 1 || nz > kMaxNz)
    return fail(VG_ERR_SHAPE, "vg_solve_implicit_f64: nsx=%d nsy=%d nz=%d (1 <= nz <= %d)", nsx, nsy, nz, kMaxNz);
  if (!a || !b || !c || !d || !water || !edge || !out) return fail(VG_ERR_ARG, "vg_solve_implicit_f64: NULL pointer");
  const long long nsys = (long long)nsx * nsy;
  if (nsys == 0) return VG_OK;
  if (nsys > 0x7fffffffLL) return fail(VG_ERR_SHAPE, "too many columns");
  TriArgs p{nsx, (int)nsys, nz, s_x, s_y, s_z, a, b, c, d, b_edge, d_edge, water, edge, out, bad_columns};
  int nb = 128;
  while (nb > 32 && (size_t)nb * nz * 2 * sizeof(double) > 100 * 1024) nb /= 2;
  const size_t smem = (size_t)nb * nz * 2 * sizeof(double);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(pivoting_solve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return fail(VG_ERR_LAUNCH, "pivoting_solve_kernel smem: %s", cudaGetErrorString(e));
  }
  pivoting_solve_kernel<<<(unsigned)((nsys + nb - 1) / nb), nb, smem, as_stream(stream)>>>(p);
  return check_launch("pivoting_solve_kernel");
}

extern "C" void vg_tdma_cuda_double(void *stream, void **buffers, const char *opaque, size_t opaque_len) {
  xla_tdma<double>(stream, buffers, opaque, opaque_len, "vg_tdma_cuda_double");
}

extern "C" void vg_tdma_cuda_float(void *stream, void **buffers, const char *opaque, size_t opaque_len) {
  xla_tdma<float>(stream, buffers, opaque, opaque_len, "vg_tdma_cuda_float");
}
