// Work shares of the persistent pre and flux kernels of a step, weighted by
// the water on each tile-level.
//
// With equal counts of tile-levels per CTA, CTAs whose share holds dry tiles
// (land, polar caps, the deep levels of shallow columns) finish long before
// those holding wet ones: at 1 degree the FP64 pre kernel's CTAs ran 49 to
// 851 us (mean 689), the flux kernel's 259 to 732 us (mean 622). A CTA's time
// follows a + b * (busy warps) per tile-level, the busy warps of a level
// being ceil(wet points / 32) after the wet-point ordering; fitted to the
// per-CTA times of the equal shares (correlation 0.90 pre, 0.88 flux), a / b
// is about 1 for the FP64 pre kernel and 5 for the FP64 flux kernel. The
// shares cut the tile-major sequence of tile-levels where the running cost
// crosses each CTA's equal part of the total. Only the distribution of the
// work changes: every tile-level is computed by the same arithmetic, so the
// results are those of any other partition, bit for bit.
#include "common.cuh"

namespace vg {
namespace {

// cost[w] = a + ceil(wet T points / 32) of tile-level w, d if it has no wet
// T point (tile-major: tile
// w / Z, level w % Z); tiles of 32 x ty points from (i0s, j0s), ntx along x,
// points limited to i < xe, j < ye. One warp per tile-level.
__global__ void __launch_bounds__(256) tile_level_cost_kernel(Layout L, const uint8_t *__restrict__ m, int i0s,
                                                              int j0s, int xe, int ye, int ty, int ntx, long long W,
                                                              double a, double d, double *cost) {
  const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) / 32;
  const int lane = threadIdx.x & 31;
  if (w >= W) return;  // the lanes of a warp share w
  const int Z = L.Z;
  const int t = (int)(w / Z), k = (int)(w % Z);
  const int i = i0s + (t % ntx) * 32 + lane;
  int wet = 0;
  for (int r = 0; r < ty; ++r) {
    const int j = j0s + (t / ntx) * ty + r;
    const bool v = i < xe && j < ye && (__ldg(m + L.at(i, j, k)) & VG_MASK_T);
    wet += __popc(__ballot_sync(0xffffffffu, v));
  }
  if (lane == 0) cost[w] = wet ? a + (double)((wet + 31) / 32) : d;
}

// One CTA: cost[] becomes its exclusive prefix sums, then starts[c] is the
// first tile-level whose prefix reaches c / nc of the total (starts[0] = 0,
// starts[nc] = W).
__global__ void __launch_bounds__(1024) share_partition_kernel(double *cost, long long W, int nc,
                                                               long long *starts) {
  __shared__ double part[1024];
  __shared__ double total;
  const int t = threadIdx.x, nt = blockDim.x;
  const long long per = (W + nt - 1) / nt;
  const long long b = min(W, (long long)t * per), e = min(W, b + per);
  double s = 0.0;
  for (long long p = b; p < e; ++p) s += cost[p];
  part[t] = s;
  __syncthreads();
  if (t == 0) {
    double run = 0.0;
    for (int u = 0; u < nt; ++u) {
      const double v = part[u];
      part[u] = run;
      run += v;
    }
    total = run;
  }
  __syncthreads();
  double run = part[t];
  for (long long p = b; p < e; ++p) {
    const double v = cost[p];
    cost[p] = run;
    run += v;
  }
  __syncthreads();
  for (int c = t; c <= nc; c += nt) {
    if (c == 0 || c == nc) {
      starts[c] = c == 0 ? 0 : W;
      continue;
    }
    const double target = total * (double)c / (double)nc;
    long long lo = 0, hi = W;
    while (lo < hi) {
      const long long mid = (lo + hi) / 2;
      if (cost[mid] < target)
        lo = mid + 1;
      else
        hi = mid;
    }
    starts[c] = lo;
  }
}

// The cost of a tile-level in units of one busy warp's: a + busy warps if it
// holds water, d if not. The per-CTA fit of the header puts a near 1 (pre)
// and 5 (flux), but what the shares have to balance is measured CTA time,
// which a share of many dry tile-levels (a polar cap, the rim rows) also
// spends on segment restarts and on the dry levels' own stores; so the
// constants are the measured optimum at 1 degree, FP64 step in ms (CUDA
// events, 30 steps):
//   pre  a / d:  8 / 8 0.781,  8 / 1 0.743,  8 / 0.5 1.106,  8 / 2 0.755,
//                6 / 1 0.755, 10 / 1 0.806 (equal counts 0.850 before the
//                L2 prefetches)
//   flux a / d:  8 / 8 0.775, 12 / 6 0.759, 12 / 8 0.765, 10 / 8 0.764,
//                8 / 1 2.244, 8 / 12 0.789
// Below the optimum of d a share takes so many dry tile-levels that it
// becomes the longest (the flux kernel's dry tile-levels still prepare the
// new time level of their cells). With the pre kernel's rotated plane
// points: a / d = 8 / 1 0.704, 8 / 2 0.704, 6 / 1 0.706, 10 / 1 0.800,
// 12 / 1 0.888 ms; 8 / 2 keeps the ratio well below where the cliff starts. The split form's flux kernel gains nothing
// from shares (its fixed cost per level dominates) and takes equal counts;
// its pre kernel takes a = d = 16 (0.345 against 0.352 ms with d = 8).
constexpr double kPreFixedF64 = 8.0, kPreDryF64 = 2.0;
constexpr double kFluxFixedF64 = 12.0, kFluxDryF64 = 6.0;
constexpr double kPreFixedSplit = 16.0, kPreDrySplit = 16.0;

struct SharePlan {
  int n_pre, n_flux;  // CTAs with shares (0: the kernel runs one CTA per tile)
  int ntx_pre, ntx_flux, ntiles_pre, ntiles_flux;
};

template <typename F>
int share_plan(const VgDomain *dom, SharePlan &p) {
  int st = pre_span_plan<F>(dom, &p.ntx_pre, &p.ntiles_pre, &p.n_pre);
  if (st) return st;
  if ((st = flux_span_plan<F>(dom, &p.ntx_flux, &p.ntiles_flux, &p.n_flux))) return st;
  if (sizeof(F) == sizeof(float)) p.n_flux = 0;  // the split form's flux kernel: equal counts
  return VG_OK;
}

int plan_of(const VgDomain *dom, int precision, SharePlan &p) {
  clear_error();
  int st = validate_domain(dom);
  if (st) return st;
  if (precision == 0) return share_plan<double>(dom, p);
  if (precision == 1) return share_plan<float>(dom, p);
  return fail(VG_ERR_ARG, "precision %d: 0 (FP64) or 1 (split form)", precision);
}

}  // namespace
}  // namespace vg

using namespace vg;

extern "C" int vg_isoneutral_step_shares_size(const VgDomain *dom, int precision, int *n_pre, int *n_flux,
                                              size_t *scratch_bytes) {
  SharePlan p;
  int st = plan_of(dom, precision, p);
  if (st) return st;
  if (!n_pre || !n_flux || !scratch_bytes) return fail(VG_ERR_ARG, "vg_isoneutral_step_shares_size: NULL pointer");
  *n_pre = p.n_pre;
  *n_flux = p.n_flux;
  const long long W = (long long)std::max(p.ntiles_pre, p.ntiles_flux) * dom->Z;
  *scratch_bytes = (size_t)W * sizeof(double);
  return VG_OK;
}

extern "C" int vg_isoneutral_step_shares(const VgDomain *dom, int precision, const uint8_t *mask_bits,
                                         long long *pre_starts, long long *flux_starts, void *scratch,
                                         size_t scratch_bytes, void *stream) {
  SharePlan p;
  int st = plan_of(dom, precision, p);
  if (st) return st;
  if (!mask_bits || !scratch) return fail(VG_ERR_ARG, "vg_isoneutral_step_shares: NULL pointer");
  if ((p.n_pre && !pre_starts) || (p.n_flux && !flux_starts))
    return fail(VG_ERR_ARG, "vg_isoneutral_step_shares: NULL shares array where the plan has shares");
  const Layout L = layout_of(dom);
  const long long need = (long long)std::max(p.ntiles_pre, p.ntiles_flux) * L.Z * (long long)sizeof(double);
  if ((long long)scratch_bytes < need)
    return fail(VG_ERR_SCRATCH, "shares scratch of %zu bytes given, %lld needed", scratch_bytes, need);
  cudaStream_t s = as_stream(stream);
  double *cost = static_cast<double *>(scratch);
  const int ty = precision == 0 ? 8 : 4;
  struct Part {
    int n, ntx, ntiles, i0, xe_off;
    double a, d;
    long long *starts;
  } parts[2] = {{p.n_pre, p.ntx_pre, p.ntiles_pre, 1, 1, precision == 0 ? kPreFixedF64 : kPreFixedSplit,
                 precision == 0 ? kPreDryF64 : kPreDrySplit, pre_starts},
                {p.n_flux, p.ntx_flux, p.ntiles_flux, 2, 2, kFluxFixedF64, kFluxDryF64, flux_starts}};
  for (const Part &q : parts) {
    if (q.n == 0) continue;
    const long long W = (long long)q.ntiles * L.Z;
    const long long threads = W * 32;
    tile_level_cost_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(
        L, mask_bits, q.i0, q.i0, L.X - q.xe_off, L.Y - q.xe_off, ty, q.ntx, W, q.a, q.d, cost);
    if ((st = check_launch("tile_level_cost_kernel"))) return st;
    share_partition_kernel<<<1, 1024, 0, s>>>(cost, W, q.n, q.starts);
    if ((st = check_launch("share_partition_kernel"))) return st;
  }
  return VG_OK;
}
