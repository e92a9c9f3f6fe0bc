// Status plumbing, domain validation and the mask-packing kernel.
#include <string.h>

#include "common.cuh"

namespace vg {

static thread_local char g_last_error[512] = "";

int fail(int code, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
  return code;
}

void clear_error() { g_last_error[0] = '\0'; }

int validate_domain(const VgDomain *dom) {
  if (!dom) return fail(VG_ERR_ARG, "domain is NULL");
  if (dom->X < 5 || dom->Y < 5 || dom->Z < 2)
    return fail(VG_ERR_SHAPE, "domain extents X=%d Y=%d Z=%d: need X>=5, Y>=5 (2 halo cells per side) and Z>=2",
                dom->X, dom->Y, dom->Z);
  if (dom->pitch < dom->X) return fail(VG_ERR_STRIDE, "pitch %lld < X %d", dom->pitch, dom->X);
  if (dom->plane < dom->pitch * dom->Y)
    return fail(VG_ERR_STRIDE, "plane %lld < pitch*Y %lld", dom->plane, dom->pitch * (long long)dom->Y);
  return VG_OK;
}

__global__ void pack_masks_kernel(Layout L, const uint8_t *__restrict__ mT, const uint8_t *__restrict__ mU,
                                  const uint8_t *__restrict__ mV, const uint8_t *__restrict__ mW,
                                  uint8_t *__restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int j = blockIdx.y;
  int k = blockIdx.z;
  if (i >= L.X) return;
  long long o = L.at(i, j, k);
  out[o] = (uint8_t)((mT[o] ? VG_MASK_T : 0u) | (mU[o] ? VG_MASK_U : 0u) | (mV[o] ? VG_MASK_V : 0u) |
                     (mW[o] ? VG_MASK_W : 0u));
}

// Fields between the reference's (X, Y, Z) C-order layout (z fastest, as a
// NumPy array of the state) and the canonical layout (x fastest, pitch and
// plane strides): per (field, four rows j) 32 x 32 tiles of (i, k) go through
// shared memory, so that both the reads and the writes run along their
// fastest index.
constexpr int kMaxLayoutFields = 8;
struct LayoutFields {
  const double *src[kMaxLayoutFields];
  double *dst[kMaxLayoutFields];
};

// j rows per CTA: four tiles' loads in flight before one barrier (1 degree,
// two fields to the canonical layout / four back: 48 / 81 us against 52 / 95
// with one row, 46 / 84 with two, 71 / 118 with eight)
constexpr int kLayoutRows = 4;

template <bool TO_CANONICAL>
__global__ void __launch_bounds__(256) layout_kernel(Layout L, LayoutFields f, int jblocks) {
  __shared__ double t[kLayoutRows][32][33];
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  const int j0 = (blockIdx.z % jblocks) * kLayoutRows, n = blockIdx.z / jblocks;
  const int i0 = blockIdx.y * 32, k0 = blockIdx.x * 32;
  const long long hstride_i = (long long)L.Y * L.Z;  // host layout: i * Y * Z + j * Z + k
  const double *src = f.src[n];
  double *dst = f.dst[n];
  if (TO_CANONICAL) {
#pragma unroll
    for (int jj = 0; jj < kLayoutRows; ++jj) {  // read along k
      const int j = j0 + jj;
      if (j >= L.Y) break;
      for (int r = ty; r < 32; r += 8) {
        const int i = i0 + r, k = k0 + tx;
        if (i < L.X && k < L.Z) t[jj][r][tx] = src[i * hstride_i + (long long)j * L.Z + k];
      }
    }
    __syncthreads();
#pragma unroll
    for (int jj = 0; jj < kLayoutRows; ++jj) {  // write along i
      const int j = j0 + jj;
      if (j >= L.Y) break;
      for (int r = ty; r < 32; r += 8) {
        const int i = i0 + tx, k = k0 + r;
        if (i < L.X && k < L.Z) dst[L.at(i, j, k)] = t[jj][tx][r];
      }
    }
  } else {
#pragma unroll
    for (int jj = 0; jj < kLayoutRows; ++jj) {  // read along i
      const int j = j0 + jj;
      if (j >= L.Y) break;
      for (int r = ty; r < 32; r += 8) {
        const int i = i0 + tx, k = k0 + r;
        if (i < L.X && k < L.Z) t[jj][tx][r] = src[L.at(i, j, k)];
      }
    }
    __syncthreads();
#pragma unroll
    for (int jj = 0; jj < kLayoutRows; ++jj) {  // write along k
      const int j = j0 + jj;
      if (j >= L.Y) break;
      for (int r = ty; r < 32; r += 8) {
        const int i = i0 + r, k = k0 + tx;
        if (i < L.X && k < L.Z) dst[i * hstride_i + (long long)j * L.Z + k] = t[jj][r][tx];
      }
    }
  }
}

template <bool TO_CANONICAL>
int convert_layout(const VgDomain *dom, int nfields, const double *const *src, double *const *dst, void *stream,
                   const char *name) {
  clear_error();
  int st = validate_domain(dom);
  if (st) return st;
  if (nfields < 1 || nfields > kMaxLayoutFields)
    return fail(VG_ERR_ARG, "%s: nfields=%d (1..%d)", name, nfields, kMaxLayoutFields);
  if (!src || !dst) return fail(VG_ERR_ARG, "%s: NULL pointer", name);
  LayoutFields f{};
  for (int n = 0; n < nfields; ++n) {
    if (!src[n] || !dst[n]) return fail(VG_ERR_ARG, "%s: NULL field pointer", name);
    f.src[n] = src[n];
    f.dst[n] = dst[n];
  }
  const Layout L = layout_of(dom);
  const int jblocks = (L.Y + kLayoutRows - 1) / kLayoutRows;
  if ((long long)jblocks * nfields > 65535) return fail(VG_ERR_SHAPE, "%s: Y * nfields too large", name);
  dim3 grid((L.Z + 31) / 32, (L.X + 31) / 32, jblocks * nfields);
  layout_kernel<TO_CANONICAL><<<grid, dim3(32, 8), 0, as_stream(stream)>>>(L, f, jblocks);
  return check_launch("layout_kernel");
}

}  // namespace vg

using namespace vg;

extern "C" int vg_layout_to_canonical_f64(const VgDomain *dom, int nfields, const double *const *src,
                                          double *const *dst, void *stream) {
  return convert_layout<true>(dom, nfields, src, dst, stream, "vg_layout_to_canonical_f64");
}

extern "C" int vg_layout_from_canonical_f64(const VgDomain *dom, int nfields, const double *const *src,
                                            double *const *dst, void *stream) {
  return convert_layout<false>(dom, nfields, src, dst, stream, "vg_layout_from_canonical_f64");
}

extern "C" const char *vg_last_error(void) { return g_last_error; }

extern "C" const char *vg_version(void) { return "veros_gb300 0.1 (sm_103a)"; }

extern "C" int vg_pack_masks(const VgDomain *dom, const uint8_t *maskT, const uint8_t *maskU, const uint8_t *maskV,
                             const uint8_t *maskW, uint8_t *mask_bits, void *stream) {
  clear_error();
  int st = validate_domain(dom);
  if (st) return st;
  if (!maskT || !maskU || !maskV || !maskW || !mask_bits) return fail(VG_ERR_ARG, "vg_pack_masks: NULL pointer");
  Layout L = layout_of(dom);
  dim3 block(128);
  dim3 grid((L.X + 127) / 128, L.Y, L.Z);
  pack_masks_kernel<<<grid, block, 0, as_stream(stream)>>>(L, maskT, maskU, maskV, maskW, mask_bits);
  return check_launch("pack_masks_kernel");
}
