// Launchers and C entry points of the tracer diffusion kernels (diffusion_kernels.cuh).
#include "diffusion_kernels.cuh"

using namespace vg;
using namespace vg::detail;

extern "C" size_t vg_isoneutral_diffusion_scratch_bytes(const VgDomain *dom) {
  if (!dom || dom->plane <= 0 || dom->Z <= 0) return 0;
  return 3 * (size_t)dom->plane * (size_t)dom->Z * sizeof(double);
}

namespace vg {
namespace {

// NTR = 2: temp and salt in one pass over the tensor (b: salt); NTR = 1: a alone
// Tiles of 32 x 8 columns in the FP64 form, 32 x 4 in the split form
// (flux_span_kernel): one CTA per tile on large domains, else every resident
// CTA with a share of the tile-levels. The split form's flux kernel is
// latency-bound at 128 registers a thread; on 4-warp tiles its level barriers
// wait for fewer warps (1 degree: 0.530 against 0.541 ms for the diffusion
// stage; more CTAs per SM by a tighter register budget spill and gain nothing).
template <typename F>
constexpr int flux_rows() {
  return sizeof(F) == sizeof(float) ? 4 : 8;
}

template <typename F, int NTR>
int flux_geometry(const Layout &L, int &nbx, int &nby, size_t &smem, int &nc, bool &per_tile) {
  constexpr int TY = flux_rows<F>();
  nbx = (L.X - 4 + TX - 1) / TX;
  nby = (L.Y - 4 + TY - 1) / TY;
  smem = flux_smem_bytes(L.Z);
  nc = span_ctas(flux_span_kernel<F, TY, NTR>, TX * TY, smem, nbx * nby, L.Z, 8, &per_tile);
  if (nc < 1) return fail(VG_ERR_LAUNCH, "flux_span_kernel: occupancy query failed");
  return VG_OK;
}

template <typename F, int NTR>
int launch_flux_div(DiffArgs<F> &a, DiffArgs<F> &b, cudaStream_t s, const long long *starts = nullptr,
                    int nstarts = 0) {
  constexpr int TY = flux_rows<F>();
  int nbx, nby, nc;
  size_t smem;
  bool per_tile;
  int st = flux_geometry<F, NTR>(a.L, nbx, nby, smem, nc, per_tile);
  if (st) return st;
  a.kchunk = b.kchunk = a.L.Z;
  // shares apply where the CTAs split the tile-levels (not one CTA per tile)
  const long long *sh = !per_tile && nstarts == nc ? starts : nullptr;
  flux_span_kernel<F, TY, NTR><<<nc, TX * TY, smem, s>>>(a, b, nbx, nbx * nby, sh);
  return check_launch("flux_span_kernel");
}

template <typename F, int NRHS>
int launch_implicit(const DiffArgs<F> &a, const DiffArgs<F> &b, cudaStream_t s) {
  const int ncols_x = a.L.X - 4, ncols = ncols_x * (a.L.Y - 4);
  // shared memory per CTA: the two per-level tables plus c' per column and d'
  // per thread; deep columns take fewer columns per CTA
  constexpr size_t kMaxSmem = 200 * 1024;
  if (NRHS == 2) {  // temp and salt of a column on two threads, up to 64 columns per CTA
    int nc = 64;
    while (nc > 8 && (2 + 3 * (size_t)nc) * a.L.Z * sizeof(double) > kMaxSmem) nc /= 2;
    const int nb = 2 * nc;
    const size_t smem = (2 + 3 * (size_t)nc) * a.L.Z * sizeof(double);
    if (smem > 48 * 1024) {
      cudaError_t e =
          cudaFuncSetAttribute(implicit_pair_kernel<F>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess)
        return fail(VG_ERR_LAUNCH, "implicit_pair_kernel smem %zu: %s", smem, cudaGetErrorString(e));
    }
    implicit_pair_kernel<F><<<(ncols + nc - 1) / nc, nb, smem, s>>>(a, b);
    return check_launch("implicit_pair_kernel");
  }
  int nb = 64;
  while (nb > 8 && (2 + (1 + NRHS) * (size_t)nb) * a.L.Z * sizeof(double) > kMaxSmem) nb /= 2;
  const size_t smem = (2 * (size_t)a.L.Z + (1 + NRHS) * (size_t)a.L.Z * nb) * sizeof(double);
  if (smem > 48 * 1024) {
    cudaError_t e =
        cudaFuncSetAttribute(implicit_kernel<F, NRHS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return fail(VG_ERR_LAUNCH, "implicit_kernel smem %zu: %s", smem, cudaGetErrorString(e));
  }
  implicit_kernel<F, NRHS><<<(ncols + nb - 1) / nb, nb, smem, s>>>(a, b);
  return check_launch("implicit_kernel");
}

// Levels per CTA of energy_kernel. The kernel is bound by the FP64 pipe,
// which an SM's resident CTAs share, so the cost of a chunking is the CTAs an
// SM receives times the levels per CTA, counting a chunk's extra dissipation
// evaluation at its top as half a level.
// The SM count is that of the current device, read on every call (an
// attribute query, no synchronisation): no state is shared between devices
// or host threads.
inline int energy_kchunk(int ctas_per_chunk, int Z) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                 cudaSuccess)
    sms = 1;
  sms = std::max(1, sms);
  int best = Z;
  double best_cost = 1e300;
  for (int nch = 1; nch <= std::min(Z, 64); ++nch) {
    const int kc = (Z + nch - 1) / nch, n = (Z + kc - 1) / kc;
    const long long ctas = (long long)ctas_per_chunk * n;
    const double cost = (double)((ctas + sms - 1) / sms) * (kc + 0.5);
    if (cost < best_cost) best_cost = cost, best = kc;
  }
  return best;
}

// One tracer, or temp and salt together when they add into the same P_diss.
template <typename F>
int launch_energy(const DiffArgs<F> &a, const DiffArgs<F> *b, cudaStream_t s) {
  if (a.L.Z > kEnergyMaxZ) return fail(VG_ERR_SHAPE, "energy_kernel: Z=%d above %d", a.L.Z, kEnergyMaxZ);
  dim3 block(kEnergyTX, kEnergyTY);
  const int gx = (a.L.X - 2 + kEnergyTX - 1) / kEnergyTX, gy = (a.L.Y - 2 + kEnergyTY - 1) / kEnergyTY;
  if (b && b->P == a.P) {
    const int kc = energy_kchunk(gx * gy, a.L.Z);
    energy_kernel<F, 2><<<dim3(gx, gy, (a.L.Z + kc - 1) / kc), block, 0, s>>>(a, *b, kc);
    return check_launch("energy_kernel");
  }
  const int kc = energy_kchunk(gx * gy, a.L.Z);
  energy_kernel<F, 1><<<dim3(gx, gy, (a.L.Z + kc - 1) / kc), block, 0, s>>>(a, a, kc);
  int st = check_launch("energy_kernel");
  if (st || !b) return st;
  energy_kernel<F, 1><<<dim3(gx, gy, (a.L.Z + kc - 1) / kc), block, 0, s>>>(*b, *b, kc);
  return check_launch("energy_kernel");
}

template <typename F, typename Ten, typename Tr>
int diffusion_one(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set, const Ten *ten,
                  const F *K_field, const uint8_t *mask_bits, const int32_t *kbot, const Tr *tr, int skew,
                  void *scratch, size_t scratch_bytes, void *stream) {
  clear_error();
  int st = validate_domain(dom);
  if (st) return st;
  const size_t need = vg_isoneutral_diffusion_scratch_bytes(dom);
  if (!scratch || scratch_bytes < need)
    return fail(VG_ERR_SCRATCH, "scratch of %zu bytes given, %zu needed", scratch_bytes, need);
  DiffArgs<F> a;
  if ((st = make_diff_args(dom, grid, set, ten, K_field, mask_bits, kbot, tr, skew, static_cast<F *>(scratch), a)))
    return st;
  cudaStream_t s = as_stream(stream);
  if ((st = launch_flux_div<F, 1>(a, a, s))) return st;
  if (a.iso && (st = launch_implicit<F, 1>(a, a, s))) return st;
  if (a.save_fluxes && (st = launch_energy<F>(a, nullptr, s))) return st;
  return VG_OK;
}

template <typename F, typename Ten, typename Tr>
int diffusion_pair(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set, const Ten *ten,
                   const F *K_iso, const uint8_t *mask_bits, const int32_t *kbot, const Tr *temp, const Tr *salt,
                   void *scratch, size_t scratch_bytes, void *stream, const int32_t *col_order = nullptr,
                   int fuse_prepare = 0, const long long *flux_starts = nullptr, int flux_nstarts = 0) {
  clear_error();
  int st = validate_domain(dom);
  if (st) return st;
  const size_t one = vg_isoneutral_diffusion_scratch_bytes(dom);
  if (!scratch || scratch_bytes < 2 * one)
    return fail(VG_ERR_SCRATCH, "scratch of %zu bytes given, %zu needed", scratch_bytes, 2 * one);
  DiffArgs<F> aT, aS;
  F *sc = static_cast<F *>(scratch);
  if ((st = make_diff_args(dom, grid, set, ten, K_iso, mask_bits, kbot, temp, 0, sc, aT))) return st;
  if ((st = make_diff_args(dom, grid, set, ten, K_iso, mask_bits, kbot, salt, 0, sc + one / sizeof(double), aS)))
    return st;
  aT.col_order = aS.col_order = col_order;
  aT.fuse_prepare = aS.fuse_prepare = fuse_prepare;
  aT.tensor_from_pre = aS.tensor_from_pre = fuse_prepare;  // the step's own tensor (stage 1)
  if (fuse_prepare && aT.P != aS.P)
    return fail(VG_ERR_ARG, "step diffusion: temp and salt must share P_diss_iso");
  cudaStream_t s = as_stream(stream);
  if ((st = launch_flux_div<F, 2>(aT, aS, s, flux_starts, flux_nstarts))) return st;
  if ((st = launch_implicit<F, 2>(aT, aS, s))) return st;
  if (aT.save_fluxes && (st = launch_energy<F>(aT, &aS, s))) return st;
  return VG_OK;
}

}  // namespace

int diffusion_pair_ordered_f64(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set,
                               const VgTensorFields *ten, const double *K_iso, const uint8_t *mask_bits,
                               const int32_t *kbot, const VgTracerArgs *temp, const VgTracerArgs *salt,
                               const int32_t *column_order, void *scratch, size_t scratch_bytes, void *stream,
                               int fuse_prepare, const long long *flux_starts, int flux_nstarts) {
  return diffusion_pair<double>(dom, grid, set, ten, K_iso, mask_bits, kbot, temp, salt, scratch, scratch_bytes,
                                stream, column_order, fuse_prepare, flux_starts, flux_nstarts);
}

int diffusion_pair_ordered_f32split(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set,
                                    const VgTensorFieldsF32 *ten, const float *K_iso, const uint8_t *mask_bits,
                                    const int32_t *kbot, const VgTracerArgsF32 *temp, const VgTracerArgsF32 *salt,
                                    const int32_t *column_order, void *scratch, size_t scratch_bytes,
                                    void *stream, int fuse_prepare, const long long *flux_starts,
                                    int flux_nstarts) {
  return diffusion_pair<float>(dom, grid, set, ten, K_iso, mask_bits, kbot, temp, salt, scratch, scratch_bytes,
                               stream, column_order, fuse_prepare, flux_starts, flux_nstarts);
}

// The temp+salt flux kernel's tiling on this device: tiles along x, tiles in
// all, and CTAs (as many as tiles where it runs one CTA per tile).
template <typename F>
int flux_span_plan(const VgDomain *dom, int *ntx, int *ntiles, int *nctas) {
  int nbx, nby, nc;
  size_t smem;
  bool per_tile;
  const int st = flux_geometry<F, 2>(layout_of(dom), nbx, nby, smem, nc, per_tile);
  if (st) return st;
  *ntx = nbx;
  *ntiles = nbx * nby;
  *nctas = per_tile ? 0 : nc;
  return VG_OK;
}
template int flux_span_plan<double>(const VgDomain *, int *, int *, int *);
template int flux_span_plan<float>(const VgDomain *, int *, int *, int *);

}  // namespace vg

extern "C" int vg_isoneutral_diffusion_f64(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set,
                                           const VgTensorFields *ten, const double *K_field,
                                           const uint8_t *mask_bits, const int32_t *kbot, const VgTracerArgs *tr,
                                           int skew, void *scratch, size_t scratch_bytes, void *stream) {
  return diffusion_one<double>(dom, grid, set, ten, K_field, mask_bits, kbot, tr, skew, scratch, scratch_bytes,
                               stream);
}

extern "C" int vg_isoneutral_diffusion_f32split(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set,
                                                const VgTensorFieldsF32 *ten, const float *K_field,
                                                const uint8_t *mask_bits, const int32_t *kbot,
                                                const VgTracerArgsF32 *tr, int skew, void *scratch,
                                                size_t scratch_bytes, void *stream) {
  return diffusion_one<float>(dom, grid, set, ten, K_field, mask_bits, kbot, tr, skew, scratch, scratch_bytes,
                              stream);
}

extern "C" size_t vg_isoneutral_diffusion_pair_scratch_bytes(const VgDomain *dom) {
  return 2 * vg_isoneutral_diffusion_scratch_bytes(dom);
}

extern "C" int vg_isoneutral_diffusion_pair_f64(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set,
                                                const VgTensorFields *ten, const double *K_iso,
                                                const uint8_t *mask_bits, const int32_t *kbot,
                                                const VgTracerArgs *temp, const VgTracerArgs *salt, void *scratch,
                                                size_t scratch_bytes, void *stream) {
  return diffusion_pair<double>(dom, grid, set, ten, K_iso, mask_bits, kbot, temp, salt, scratch, scratch_bytes,
                                stream);
}

extern "C" int vg_isoneutral_diffusion_pair_f32split(const VgDomain *dom, const VgGrid *grid,
                                                     const VgIsoSettings *set, const VgTensorFieldsF32 *ten,
                                                     const float *K_iso, const uint8_t *mask_bits,
                                                     const int32_t *kbot, const VgTracerArgsF32 *temp,
                                                     const VgTracerArgsF32 *salt, void *scratch,
                                                     size_t scratch_bytes, void *stream) {
  return diffusion_pair<float>(dom, grid, set, ten, K_iso, mask_bits, kbot, temp, salt, scratch, scratch_bytes,
                               stream);
}

// ---------------------------------------------------------------------------
// Scratch-free variant of vg_isoneutral_diffusion_f64.
//
// The diffusion needs a scratch triple of flux fields when the energy branch
// is on. Some callers cannot call cudaMalloc to provide it: an XLA custom-call
// or FFI handler (JAX reserves most of the GPU's memory for its own pool and
// the handler may only touch the buffers it is handed), or a host model that
// fixes all of its device memory at start-up and forbids allocation inside
// the time loop. For them this entry point keeps the scratch in a file-scope
// device array instead.
//
// * Limit: the array holds kNoAllocScratchBytes (32 MiB), enough for domains
//   with 3 * plane * Z * 8 bytes <= 32 MiB (for example 80 x 60 x 60 interior
//   cells); larger domains are rejected with VG_ERR_SCRATCH before anything is
//   enqueued. Every GPU that loads this library holds the array until the
//   process exits.
// * Set-up: the first call on a device (with that device current) looks up
//   the array's device address with cudaGetSymbolAddress and caches it per
//   device; make that first call before any stream capture. Host code must
//   never pass the array's name itself to a kernel: in host code it is only a
//   stand-in, not a device address. The cached address belongs to the
//   device's current context: after cudaDeviceReset (which unloads this
//   library's device code) call vg_isoneutral_diffusion_noalloc_reset before
//   the next call, so that the address is looked up again.
// * Sharing: every call uses the same array, which keeps the last call's
//   contents. Nothing in it has to start at zero (each call writes every
//   scratch cell it later reads), but calls that overlap on the GPU (on
//   different streams, or concurrently from several host threads) race on it.
// * No allocation: this function calls no cudaMalloc, cudaFree or allocating
//   library routine.
// ---------------------------------------------------------------------------
#include <mutex>

namespace vg {
namespace {
constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];
constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
void *g_noalloc_ptr[kMaxDevices] = {};
}  // namespace
}  // namespace vg

extern "C" size_t vg_isoneutral_diffusion_noalloc_capacity(void) { return vg::kNoAllocScratchBytes; }

extern "C" void vg_isoneutral_diffusion_noalloc_reset(void) {
  std::lock_guard<std::mutex> lock(vg::g_noalloc_mutex);
  for (void *&p : vg::g_noalloc_ptr) p = nullptr;
}

extern "C" int vg_isoneutral_diffusion_noalloc_f64(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set,
                                                   const VgTensorFields *ten, const double *K_field,
                                                   const uint8_t *mask_bits, const int32_t *kbot,
                                                   const VgTracerArgs *tr, int skew, void *stream) {
  clear_error();
  int st = validate_domain(dom);
  if (st) return st;
  const size_t need = vg_isoneutral_diffusion_scratch_bytes(dom);
  if (need > kNoAllocScratchBytes)
    return fail(VG_ERR_SCRATCH,
                "vg_isoneutral_diffusion_noalloc_f64: this domain needs %zu bytes of scratch but the static "
                "buffer holds %zu (32 MiB); use vg_isoneutral_diffusion_f64 with caller-provided scratch",
                need, kNoAllocScratchBytes);
  int device = -1;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return fail(VG_ERR_LAUNCH, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (device < 0 || device >= kMaxDevices) return fail(VG_ERR_ARG, "device index %d out of range", device);
  void *ptr = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[device]) {
      e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
      if (e != cudaSuccess)
        return fail(VG_ERR_LAUNCH, "cudaGetSymbolAddress(scratch) on device %d: %s", device, cudaGetErrorString(e));
      g_noalloc_ptr[device] = ptr;
    }
    ptr = g_noalloc_ptr[device];
  }
  return vg_isoneutral_diffusion_f64(dom, grid, set, ten, K_field, mask_bits, kbot, tr, skew, ptr,
                                     kNoAllocScratchBytes, stream);
}

extern "C" int vg_isoneutral_diffusion_pair_ordered_f64(const VgDomain *dom, const VgGrid *grid,
                                                        const VgIsoSettings *set, const VgTensorFields *ten,
                                                        const double *K_iso, const uint8_t *mask_bits,
                                                        const int32_t *kbot, const VgTracerArgs *temp,
                                                        const VgTracerArgs *salt, const int32_t *column_order,
                                                        void *scratch, size_t scratch_bytes, void *stream) {
  return diffusion_pair<double>(dom, grid, set, ten, K_iso, mask_bits, kbot, temp, salt, scratch, scratch_bytes,
                                stream, column_order);
}

extern "C" int vg_isoneutral_diffusion_pair_ordered_f32split(const VgDomain *dom, const VgGrid *grid,
                                                             const VgIsoSettings *set, const VgTensorFieldsF32 *ten,
                                                             const float *K_iso, const uint8_t *mask_bits,
                                                             const int32_t *kbot, const VgTracerArgsF32 *temp,
                                                             const VgTracerArgsF32 *salt,
                                                             const int32_t *column_order, void *scratch,
                                                             size_t scratch_bytes, void *stream) {
  return diffusion_pair<float>(dom, grid, set, ten, K_iso, mask_bits, kbot, temp, salt, scratch, scratch_bytes,
                               stream, column_order);
}
