// Column tridiagonal solves.
//
// * vg_solve_implicit_f64: the drop-in for solve_implicit / solve_tridiagonal
//   (veros/core/utilities.py:51-59, veros/core/operators.py:60-77). One thread
//   per column solves that column's water cells k = ks..nz-1 by Gaussian
//   elimination with partial pivoting, the method of LAPACK dgtsv which the
//   reference calls; the factors stay in shared memory.
// * vg_tdma_cuda_{double,float}: same buffers/descriptor contract as the XLA
//   custom-call targets of veros/core/special/cuda_tdma_kernels.cu:81-111
//   (full-depth Thomas sweep, identity rows already folded in by the caller,
//   tdma_.py:63-66), but c' is kept in shared memory instead of a global
//   workspace and errors are reported instead of exiting.
#include <algorithm>
#include <cstring>

#include "common.cuh"

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

// Per row r of a column the shared memory holds the eliminated diagonal,
// first and second super-diagonals and right-hand side, laid out [r][field][thread].
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
    const bool w_exp = ks >= 0;
    const bool e_exp = ks == k;
    if (w != w_exp || e != e_exp) bad = true;
  }
  if (bad && p.bad) atomicAdd(p.bad, 1);

  for (int k = 0; k < nz; ++k) p.out[base + p.sz * k] = 0.0;
  if (ks < 0) return;
  const int n = nz - ks;

  auto D = [&](int r) -> double & { return sm[((size_t)r * 4 + 0) * nb + t]; };
  auto DU = [&](int r) -> double & { return sm[((size_t)r * 4 + 1) * nb + t]; };
  auto DU2 = [&](int r) -> double & { return sm[((size_t)r * 4 + 2) * nb + t]; };
  auto B = [&](int r) -> double & { return sm[((size_t)r * 4 + 3) * nb + t]; };

  // row r = 0 is the edge row: b_edge/d_edge substitution (utilities.py:53-57)
  {
    const long long o = base + p.sz * ks;
    double b0 = p.b_edge ? p.b_edge[o] : p.b[o];
    double d0 = p.d_edge ? p.d_edge[o] : p.d[o];
    D(0) = b0;
    B(0) = d0;
    DU(0) = n > 1 ? p.c[o] : 0.0;  // c[..., -1] = 0 cuts the top (operators.py:73)
  }
  for (int r = 0; r < n - 1; ++r) {
    const long long o1 = base + p.sz * (ks + r + 1);
    double dl = p.a[o1];
    double d_next = p.b[o1];
    double du_next = (r + 1 < n - 1) ? p.c[o1] : 0.0;
    double b_next = p.d[o1];
    const double dr = D(r);
    if (fabs(dr) >= fabs(dl)) {
      const double fact = dl / dr;
      d_next = d_next - fact * DU(r);
      b_next = b_next - fact * B(r);
      DU2(r) = 0.0;
    } else {
      const double fact = dr / dl;
      D(r) = dl;
      const double tmp = d_next;
      d_next = DU(r) - fact * tmp;
      DU2(r) = du_next;
      du_next = -fact * du_next;
      DU(r) = tmp;
      const double br = B(r);
      B(r) = b_next;
      b_next = br - fact * b_next;
    }
    D(r + 1) = d_next;
    DU(r + 1) = du_next;
    B(r + 1) = b_next;
  }
  // back substitution
  double x1 = B(n - 1) / D(n - 1), x2 = 0.0;
  p.out[base + p.sz * (ks + n - 1)] = x1;
  for (int r = n - 2; r >= 0; --r) {
    const double x = (B(r) - DU(r) * x1 - DU2(r) * x2) / D(r);
    p.out[base + p.sz * (ks + r)] = x;
    x2 = x1;
    x1 = x;
  }
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
  while (nb > 32 && (size_t)nb * nz * 4 * sizeof(double) > 100 * 1024) nb /= 2;
  const size_t smem = (size_t)nb * nz * 4 * sizeof(double);
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
