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

}  // namespace vg

using namespace vg;

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
