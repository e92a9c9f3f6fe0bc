// Batched ensemble: one isoneutral step of many domains of uneven nx, ny, nz
// and kbot with one persistent launch per stage.
//
// The host builds, per stage, a work list of (member, tile) items sorted by
// descending cost; persistent CTAs (as many as fit on the 152 SMs) take items
// with an atomic counter, stage the member's arguments in shared memory and
// run the same tile bodies as the single-domain kernels (pre_kernels.cuh,
// diffusion_kernels.cuh). No CTA ever waits for another. The time-level
// rotation is handled by three argument tables, one per phase; a step is
// four launches plus one counter reset, so a rollout captures into a CUDA
// graph. As in the single-domain step, the prepare stage covers the two-cell
// rim and the flux stage prepares the interior cells it updates. Tile height (columns per CTA), k-chunk and solver CTA size are
// tuning parameters chosen by the caller (the Python autotuner).
//
// Why four launches and not one: every stage reads what the previous one
// wrote around each tile (pre reads the new tracer level of the neighbouring
// columns, the fluxes read the slopes and tensors of the tile's halo faces,
// the solve the explicit update of its column), so one persistent launch
// would need per-tile ready flags and spinning CTAs. Inside a CUDA graph a
// stage boundary costs a few microseconds against a step of tens of
// milliseconds, and each stage's work list is long enough (thousands of
// items over the resident CTAs) that its tail is short.
#include <algorithm>
#include <vector>

#include "diffusion_kernels.cuh"
#include "pre_kernels.cuh"

namespace vg {
namespace {

using namespace detail;

struct WorkItem {
  int member;
  // tile x, tile y, k-chunk (pre/flux); with equal shares: tile, first level,
  // end level (pre/flux); column block (solve); level (prepare)
  int a, b, c;
};

template <typename F>
struct MemberArgs {
  PreArgs<F> pre;
  DiffArgs<F> dT, dS;
};

// The prepare stage (new level, zeroed tendencies) of the two-cell rim of one
// level of one member; the flux stage prepares the interior cells
// (DiffArgs::fuse_prepare).
template <typename F>
__device__ __forceinline__ void prepare_body(const DiffArgs<F> &t, const DiffArgs<F> &s, const double *T0,
                                             const double *S0, int k) {
  const Layout &L = t.L;
  const int nrim = 4 * L.X + 4 * (L.Y - 4);
  for (int p = threadIdx.x; p < nrim; p += blockDim.x) {
    int i, j;
    if (p < 4 * L.X) {
      const int jr = p / L.X;
      i = p % L.X;
      j = jr < 2 ? jr : L.Y - 4 + jr;
    } else {
      const int q = p - 4 * L.X, c = q % 4;
      i = c < 2 ? c : L.X - 4 + c;
      j = 2 + q / 4;
    }
    const long long o = L.at(i, j, k);
    const double mT = (__ldg(t.m + o) & VG_MASK_T) ? 1.0 : 0.0;
    t.trp[o] = T0[o] * mT;
    s.trp[o] = S0[o] * mT;
    t.dtr_iso[o] = F(0.0);
    s.dtr_iso[o] = F(0.0);
  }
}

// Takes the next item; returns false when the list is exhausted (uniform across the CTA).
__device__ __forceinline__ bool next_item(int *counter, int nitems, const WorkItem *items, WorkItem &w) {
  __shared__ int slot;
  __syncthreads();  // the previous item's users of `slot` and of the staged arguments are done
  if (threadIdx.x == 0) slot = atomicAdd(counter, 1);
  __syncthreads();
  const int it = slot;
  if (it >= nitems) return false;
  w = items[it];
  return true;
}

// Cooperative copy of a trivially copyable struct into shared memory.
template <typename T>
__device__ __forceinline__ void stage(T *dst, const T *src) {
  static_assert(sizeof(T) % 8 == 0, "argument structs are 8-byte multiples");
  const unsigned long long *s = reinterpret_cast<const unsigned long long *>(src);
  unsigned long long *d = reinterpret_cast<unsigned long long *>(dst);
  for (int i = threadIdx.x; i < (int)(sizeof(T) / 8); i += blockDim.x) d[i] = s[i];
  __syncthreads();
}

template <typename F>
__global__ void __launch_bounds__(256) prepare_batched(const MemberArgs<F> *__restrict__ members,
                                                       const double *const *__restrict__ tau_levels,
                                                       const WorkItem *__restrict__ items, int nitems, int *counter) {
  __shared__ DiffArgs<F> t, s;
  WorkItem w;
  while (next_item(counter, nitems, items, w)) {
    stage(&t, &members[w.member].dT);
    stage(&s, &members[w.member].dS);
    prepare_body<F>(t, s, tau_levels[2 * w.member], tau_levels[2 * w.member + 1], w.c);
  }
}

template <typename F, int TY>
__global__ void __launch_bounds__(32 * TY, 16 / TY) pre_batched(const MemberArgs<F> *__restrict__ members,
                                                          const WorkItem *__restrict__ items, int nitems,
                                                          int *counter, int kchunk) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ PreArgs<F> a;
  WorkItem w;
  while (next_item(counter, nitems, items, w)) {
    stage(&a, &members[w.member].pre);
    if (threadIdx.x == 0) a.kchunk = kchunk > 0 ? min(kchunk, a.L.Z) : a.L.Z;
    __syncthreads();
    pre_tile_body<F, TY>(a, smem_raw, w.a, w.b, w.c * a.kchunk, min(a.L.Z, (w.c + 1) * a.kchunk));
    cp_async_wait_all();  // the staged planes of this item are complete before the next reuses them
  }
}

// Equal shares: CTA c runs the segments starts[c] .. starts[c+1]-1 (member,
// tile, first level, end level) in order, with no work counter.
template <typename F, int TY>
__global__ void __launch_bounds__(32 * TY, 16 / TY) pre_batched_shares(const MemberArgs<F> *__restrict__ members,
                                                                 const WorkItem *__restrict__ items,
                                                                 const int *__restrict__ starts) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ PreArgs<F> a;
  for (int it = starts[blockIdx.x]; it < starts[blockIdx.x + 1]; ++it) {
    const WorkItem w = items[it];
    __syncthreads();  // the previous segment is done with `a` and shared memory
    stage(&a, &members[w.member].pre);
    const int nbx = (a.L.X - 3 + 31) / 32;
    pre_tile_body<F, TY>(a, smem_raw, w.a % nbx, w.a / nbx, w.b, w.c);
    cp_async_wait_all();
  }
}

template <typename F, int TY>
__global__ void __launch_bounds__(32 * TY, 16 / TY) flux_batched(const MemberArgs<F> *__restrict__ members,
                                                           const WorkItem *__restrict__ items, int nitems,
                                                           int *counter, int kchunk) {
  extern __shared__ double zq_dzt[];
  __shared__ DiffArgs<F> a[2];  // temp, salt
  WorkItem w;
  while (next_item(counter, nitems, items, w)) {
    stage(&a[0], &members[w.member].dT);
    stage(&a[1], &members[w.member].dS);
    if (threadIdx.x == 0) a[0].kchunk = a[1].kchunk = kchunk > 0 ? min(kchunk, a[0].L.Z) : a[0].L.Z;
    __syncthreads();
    flux_div_body<F, TY, 2>(a, zq_dzt, w.a, w.b, w.c * a[0].kchunk, min(a[0].L.Z, (w.c + 1) * a[0].kchunk));
  }
}

template <typename F, int TY>
__global__ void __launch_bounds__(32 * TY, 16 / TY) flux_batched_shares(const MemberArgs<F> *__restrict__ members,
                                                                  const WorkItem *__restrict__ items,
                                                                  const int *__restrict__ starts) {
  extern __shared__ double zq_dzt[];
  __shared__ DiffArgs<F> a[2];
  for (int it = starts[blockIdx.x]; it < starts[blockIdx.x + 1]; ++it) {
    const WorkItem w = items[it];
    __syncthreads();
    stage(&a[0], &members[w.member].dT);
    stage(&a[1], &members[w.member].dS);
    const int nbx = (a[0].L.X - 4 + 31) / 32;
    flux_div_body<F, TY, 2>(a, zq_dzt, w.a % nbx, w.a / nbx, w.b, w.c);
  }
}

// temp and salt of a column on two threads (implicit_pair_body): a CTA of
// 2 x solve_threads threads solves one block of solve_threads columns per item
template <typename F>
__global__ void __launch_bounds__(128) implicit_batched(const MemberArgs<F> *__restrict__ members,
                                                        const WorkItem *__restrict__ items, int nitems,
                                                        int *counter) {
  extern __shared__ double smem[];
  __shared__ DiffArgs<F> t, s;
  WorkItem w;
  while (next_item(counter, nitems, items, w)) {
    stage(&t, &members[w.member].dT);
    stage(&s, &members[w.member].dS);
    implicit_pair_body<F>(t, s, smem, w.a);
  }
}

struct Tuning {
  int pre_rows, pre_kchunk, flux_rows, flux_kchunk, solve_threads;
};

struct EnsembleBase {
  virtual ~EnsembleBase() {}
  virtual int step(int phase, cudaStream_t s) = 0;
  virtual int tune(const Tuning &t) = 0;
};

template <typename F>
struct Ensemble : EnsembleBase {
  int n = 0, maxZ = 0;
  std::vector<Layout> layouts;
  MemberArgs<F> *d_args[3] = {nullptr, nullptr, nullptr};
  const double **d_tau[3] = {nullptr, nullptr, nullptr};
  WorkItem *d_prep = nullptr, *d_pre = nullptr, *d_flux = nullptr, *d_solve = nullptr;
  int n_prep = 0, n_pre = 0, n_flux = 0, n_solve = 0;
  int *d_pre_start = nullptr, *d_flux_start = nullptr;  // equal shares: first segment of each CTA
  int *d_counter = nullptr;
  Tuning tun{8, 0, 8, 0, 64};
  int grid_pre = 0, grid_flux = 0, grid_solve = 0, grid_prep = 0;
  size_t smem_pre = 0, smem_flux = 0, smem_solve = 0;

  ~Ensemble() override {
    for (int p = 0; p < 3; ++p) {
      cudaFree(d_args[p]);
      cudaFree(d_tau[p]);
    }
    cudaFree(d_prep);
    cudaFree(d_pre);
    cudaFree(d_flux);
    cudaFree(d_solve);
    cudaFree(d_pre_start);
    cudaFree(d_flux_start);
    cudaFree(d_counter);
  }

  template <typename T>
  static int upload(T **dst, const std::vector<T> &v) {
    cudaFree(*dst);
    *dst = nullptr;
    if (v.empty()) return VG_OK;
    cudaError_t e = cudaMalloc(dst, v.size() * sizeof(T));
    if (e == cudaSuccess) e = cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail(VG_ERR_LAUNCH, "ensemble work list: %s", cudaGetErrorString(e));
    return VG_OK;
  }

  // Equal shares: the members' tiles x levels, in list order, cut into ncta
  // equal ranges of tile-levels; each range becomes the segments (tile, first
  // level, end level) it covers. starts[c] is the first segment of CTA c.
  static void equal_shares(const std::vector<int> &order, const std::vector<int> &tiles,
                           const std::vector<Layout> &L, int ncta, std::vector<WorkItem> &seg,
                           std::vector<int> &starts) {
    long long W = 0;
    for (int m : order) W += (long long)tiles[m] * L[m].Z;
    starts.assign(ncta + 1, 0);
    size_t oi = 0;
    long long base = 0, p = 0;  // base: first tile-level of member order[oi]
    for (int c = 0; c < ncta; ++c) {
      starts[c] = (int)seg.size();
      const long long end = W * (c + 1) / ncta;
      while (p < end) {
        while (p >= base + (long long)tiles[order[oi]] * L[order[oi]].Z) {
          base += (long long)tiles[order[oi]] * L[order[oi]].Z;
          ++oi;
        }
        const int m = order[oi], Z = L[m].Z;
        const long long q = p - base;
        const int t = (int)(q / Z), kb = (int)(q % Z);
        const int ke = (int)std::min<long long>(Z, end - base - (long long)t * Z);
        seg.push_back({m, t, kb, ke});
        p = base + (long long)t * Z + ke;
      }
    }
    starts[ncta] = (int)seg.size();
  }

  // Work lists: largest members first, so the persistent CTAs finish together.
  int build_lists() {
    std::vector<int> order(n);
    for (int m = 0; m < n; ++m) order[m] = m;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
      return (long long)layouts[x].X * layouts[x].Y * layouts[x].Z > (long long)layouts[y].X * layouts[y].Y * layouts[y].Z;
    });
    std::vector<WorkItem> pre, flux, solve, prep;
    std::vector<int> pre_tiles(n), flux_tiles(n);
    for (int m : order) {
      const Layout &L = layouts[m];
      const int kc_pre = tun.pre_kchunk > 0 ? std::min(tun.pre_kchunk, L.Z) : L.Z;
      const int kc_flux = tun.flux_kchunk > 0 ? std::min(tun.flux_kchunk, L.Z) : L.Z;
      const int pbx = (L.X - 3 + 31) / 32, pby = (L.Y - 3 + tun.pre_rows - 1) / tun.pre_rows;
      const int pbz = (L.Z + kc_pre - 1) / kc_pre;
      pre_tiles[m] = pbx * pby;
      if (tun.pre_kchunk >= 0)
        for (int bz = 0; bz < pbz; ++bz)
          for (int by = 0; by < pby; ++by)
            for (int bx = 0; bx < pbx; ++bx) pre.push_back({m, bx, by, bz});
      const int fbx = (L.X - 4 + 31) / 32, fby = (L.Y - 4 + tun.flux_rows - 1) / tun.flux_rows;
      const int fbz = (L.Z + kc_flux - 1) / kc_flux;
      flux_tiles[m] = fbx * fby;
      if (tun.flux_kchunk >= 0)
        for (int bz = 0; bz < fbz; ++bz)  // temp and salt of a tile in one item
          for (int by = 0; by < fby; ++by)
            for (int bx = 0; bx < fbx; ++bx) flux.push_back({m, bx, by, bz});
      const int ncols = (L.X - 4) * (L.Y - 4);
      for (int cb = 0; cb < (ncols + tun.solve_threads - 1) / tun.solve_threads; ++cb) solve.push_back({m, cb, 0, 0});
      for (int k = 0; k < L.Z; ++k) prep.push_back({m, 0, 0, k});
    }
    std::vector<int> pre_start, flux_start;
    if (tun.pre_kchunk < 0) equal_shares(order, pre_tiles, layouts, grid_pre, pre, pre_start);
    if (tun.flux_kchunk < 0) equal_shares(order, flux_tiles, layouts, grid_flux, flux, flux_start);
    int st;
    if ((st = upload(&d_pre, pre)) || (st = upload(&d_flux, flux)) || (st = upload(&d_solve, solve)) ||
        (st = upload(&d_prep, prep)) || (st = upload(&d_pre_start, pre_start)) ||
        (st = upload(&d_flux_start, flux_start)))
      return st;
    n_pre = (int)pre.size();
    n_flux = (int)flux.size();
    n_solve = (int)solve.size();
    n_prep = (int)prep.size();
    return VG_OK;
  }

  template <typename K>
  static int occupancy_grid(K kernel, int threads, size_t smem, int &grid) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return fail(VG_ERR_LAUNCH, "ensemble smem %zu: %s", smem, cudaGetErrorString(e));
    }
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, smem);
    if (e != cudaSuccess || per < 1) return fail(VG_ERR_LAUNCH, "ensemble occupancy: %s", cudaGetErrorString(e));
    grid = sms * per;
    return VG_OK;
  }

  int tune(const Tuning &t) override {
    if ((t.pre_rows != 4 && t.pre_rows != 8) || (t.flux_rows != 4 && t.flux_rows != 8) ||
        (t.solve_threads != 32 && t.solve_threads != 64) || t.pre_kchunk < -1 || t.flux_kchunk < -1)
      return fail(VG_ERR_ARG, "tuning: rows must be 4 or 8, solve_threads 32 or 64, k-chunks >= -1");
    tun = t;
    int st;
    smem_pre = t.pre_rows == 4 ? pre_smem_bytes<F, 4>(maxZ) : pre_smem_bytes<F, 8>(maxZ);
    smem_flux = flux_smem_bytes(maxZ);
    smem_solve = (2 * (size_t)maxZ + 3 * (size_t)maxZ * t.solve_threads) * sizeof(double);
    const bool ps = t.pre_kchunk < 0, fs = t.flux_kchunk < 0;
    if (t.pre_rows == 4)
      st = ps ? occupancy_grid(pre_batched_shares<F, 4>, 128, smem_pre, grid_pre)
              : occupancy_grid(pre_batched<F, 4>, 128, smem_pre, grid_pre);
    else
      st = ps ? occupancy_grid(pre_batched_shares<F, 8>, 256, smem_pre, grid_pre)
              : occupancy_grid(pre_batched<F, 8>, 256, smem_pre, grid_pre);
    if (st) return st;
    if (t.flux_rows == 4)
      st = fs ? occupancy_grid(flux_batched_shares<F, 4>, 128, smem_flux, grid_flux)
              : occupancy_grid(flux_batched<F, 4>, 128, smem_flux, grid_flux);
    else
      st = fs ? occupancy_grid(flux_batched_shares<F, 8>, 256, smem_flux, grid_flux)
              : occupancy_grid(flux_batched<F, 8>, 256, smem_flux, grid_flux);
    if (st) return st;
    if ((st = occupancy_grid(implicit_batched<F>, 2 * t.solve_threads, smem_solve, grid_solve))) return st;
    if ((st = occupancy_grid(prepare_batched<F>, 256, 0, grid_prep))) return st;
    return build_lists();  // the equal shares are cut for the CTA counts above
  }

  int step(int phase, cudaStream_t s) override {
    if (phase < 0 || phase > 2) return fail(VG_ERR_ARG, "phase %d not in 0..2", phase);
    cudaError_t e = cudaMemsetAsync(d_counter, 0, 4 * sizeof(int), s);
    if (e != cudaSuccess) return fail(VG_ERR_LAUNCH, "ensemble counter reset: %s", cudaGetErrorString(e));
    const MemberArgs<F> *args = d_args[phase];
    int st;
    prepare_batched<F><<<std::min(grid_prep, n_prep), 256, 0, s>>>(args, d_tau[phase], d_prep, n_prep, d_counter);
    if ((st = check_launch("prepare_batched"))) return st;
    // equal shares: exactly the CTAs the shares were cut for
    const int gp = std::min(grid_pre, n_pre), gf = std::min(grid_flux, n_flux);
    if (d_pre_start) {
      if (tun.pre_rows == 4)
        pre_batched_shares<F, 4><<<grid_pre, 128, smem_pre, s>>>(args, d_pre, d_pre_start);
      else
        pre_batched_shares<F, 8><<<grid_pre, 256, smem_pre, s>>>(args, d_pre, d_pre_start);
    } else if (tun.pre_rows == 4) {
      pre_batched<F, 4><<<gp, 128, smem_pre, s>>>(args, d_pre, n_pre, d_counter + 1, tun.pre_kchunk);
    } else {
      pre_batched<F, 8><<<gp, 256, smem_pre, s>>>(args, d_pre, n_pre, d_counter + 1, tun.pre_kchunk);
    }
    if ((st = check_launch("pre_batched"))) return st;
    if (d_flux_start) {
      if (tun.flux_rows == 4)
        flux_batched_shares<F, 4><<<grid_flux, 128, smem_flux, s>>>(args, d_flux, d_flux_start);
      else
        flux_batched_shares<F, 8><<<grid_flux, 256, smem_flux, s>>>(args, d_flux, d_flux_start);
    } else if (tun.flux_rows == 4) {
      flux_batched<F, 4><<<gf, 128, smem_flux, s>>>(args, d_flux, n_flux, d_counter + 2, tun.flux_kchunk);
    } else {
      flux_batched<F, 8><<<gf, 256, smem_flux, s>>>(args, d_flux, n_flux, d_counter + 2, tun.flux_kchunk);
    }
    if ((st = check_launch("flux_batched"))) return st;
    implicit_batched<F><<<std::min(grid_solve, n_solve), 2 * tun.solve_threads, smem_solve, s>>>(
        args, d_solve, n_solve, d_counter + 3);
    return check_launch("implicit_batched");
  }
};

// Fills one member's argument tables for the three phases.
template <typename F, typename Fields, typename Ten, typename Tr>
int member_args(const VgDomain *dom, const VgGrid *grid, const VgIsoSettings *set, const Fields *phase,
                MemberArgs<F> *out, const double **tau) {
  int st = validate_domain(dom);
  if (st) return st;
  if (!grid_complete(grid) || !set) return fail(VG_ERR_ARG, "ensemble member: NULL grid or settings");
  if (set->enable_conserve_energy) return fail(VG_ERR_UNSUPPORTED, "ensemble: the energy branch is not batched");
  if (set->eq_of_state_type < 1 || set->eq_of_state_type > 4)
    return fail(VG_ERR_UNSUPPORTED, "eq_of_state_type %d not implemented (1-4 are)", set->eq_of_state_type);
  if (dom->Z > 512) return fail(VG_ERR_SHAPE, "Z=%d above the 512 levels supported", dom->Z);
  for (int p = 0; p < 3; ++p) {
    const Fields &f = phase[p];
    if (!f.temp_tau || !f.temp_taup1 || !f.salt_tau || !f.salt_taup1 || !f.K_iso || !f.mask_bits || !f.kbot ||
        !f.dtemp_iso || !f.dsalt_iso || !f.ten.K_11 || !f.ten.K_22 || !f.ten.K_33 || !f.ten.Ai_ez || !f.ten.Ai_nz ||
        !f.ten.Ai_bx || !f.ten.Ai_by)
      return fail(VG_ERR_ARG, "ensemble member: NULL field pointer (phase %d)", p);
    PreArgs<F> &a = out[p].pre;
    a.L = layout_of(dom);
    a.g = grid_of(grid);
    a.eos_type = set->eq_of_state_type;
    a.slopec = set->iso_slopec;
    a.inv_dslope = 1.0 / set->iso_dslope;
    a.ksteep = set->K_iso_steep;
    a.T = f.temp_tau;
    a.S = f.salt_tau;
    a.K = f.K_iso;
    a.m = f.mask_bits;
    a.K11 = f.ten.K_11;
    a.K22 = f.ten.K_22;
    a.K33 = f.ten.K_33;
    a.Aez = f.ten.Ai_ez;
    a.Anz = f.ten.Ai_nz;
    a.Abx = f.ten.Ai_bx;
    a.Aby = f.ten.Ai_by;
    a.sp = f.ten.ai_stride_p;
    a.sr = f.ten.ai_stride_r;
    a.kchunk = dom->Z;
    a.slopes = nullptr;
    a.slope_field = 0;
    a.stage_ok = pre_stage_ok(a);
    Tr trT{f.temp_tau, f.temp_taup1, f.dtemp_iso, nullptr, nullptr};
    Tr trS{f.salt_tau, f.salt_taup1, f.dsalt_iso, nullptr, nullptr};
    // the diffusion argument builder of diffusion_kernels.cuh; no scratch without the energy branch
    if ((st = make_diff_args<F>(dom, grid, set, &f.ten, f.K_iso, f.mask_bits, f.kbot, &trT, 0, nullptr, out[p].dT)) ||
        (st = make_diff_args<F>(dom, grid, set, &f.ten, f.K_iso, f.mask_bits, f.kbot, &trS, 0, nullptr, out[p].dS)))
      return st;
    out[p].dT.kchunk = out[p].dS.kchunk = dom->Z;
    out[p].dT.fuse_prepare = out[p].dS.fuse_prepare = 1;  // the flux stage prepares the interior
    out[p].dT.tensor_from_pre = out[p].dS.tensor_from_pre = 1;  // the step's own tensor
    out[p].dT.col_order = out[p].dS.col_order = f.column_order;  // optional per member
    tau[2 * p] = f.temp_tau;
    tau[2 * p + 1] = f.salt_tau;
  }
  return VG_OK;
}

template <typename F, typename Member, typename Fields, typename Ten, typename Tr>
int create(const Member *members, int n, const VgEnsembleTuning *t, void **handle) {
  clear_error();
  if (!members || n <= 0 || !handle) return fail(VG_ERR_ARG, "ensemble: no members");
  auto *E = new Ensemble<F>();
  E->n = n;
  std::vector<MemberArgs<F>> args[3];
  std::vector<const double *> tau[3];
  for (int p = 0; p < 3; ++p) {
    args[p].resize(n);
    tau[p].resize(2 * n);
  }
  for (int m = 0; m < n; ++m) {
    MemberArgs<F> tmp[3];
    const double *tp[6];
    int st = member_args<F, Fields, Ten, Tr>(&members[m].dom, &members[m].grid, &members[m].set, members[m].phase, tmp,
                                             tp);
    if (st) {
      delete E;
      return st;
    }
    for (int p = 0; p < 3; ++p) {
      args[p][m] = tmp[p];
      tau[p][2 * m] = tp[2 * p];
      tau[p][2 * m + 1] = tp[2 * p + 1];
    }
    E->layouts.push_back(layout_of(&members[m].dom));
    E->maxZ = std::max(E->maxZ, members[m].dom.Z);
  }
  cudaError_t e = cudaMalloc(&E->d_counter, 4 * sizeof(int));
  for (int p = 0; p < 3 && e == cudaSuccess; ++p) {
    e = cudaMalloc(&E->d_args[p], n * sizeof(MemberArgs<F>));
    if (e == cudaSuccess) e = cudaMemcpy(E->d_args[p], args[p].data(), n * sizeof(MemberArgs<F>), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&E->d_tau[p], 2 * n * sizeof(double *));
    if (e == cudaSuccess) e = cudaMemcpy(E->d_tau[p], tau[p].data(), 2 * n * sizeof(double *), cudaMemcpyHostToDevice);
  }
  if (e != cudaSuccess) {
    delete E;
    return fail(VG_ERR_LAUNCH, "ensemble tables: %s", cudaGetErrorString(e));
  }
  Tuning tun = t ? Tuning{t->pre_rows, t->pre_kchunk, t->flux_rows, t->flux_kchunk, t->solve_threads}
                 : Tuning{8, 0, 8, 0, 64};
  int st = E->tune(tun);
  if (st) {
    delete E;
    return st;
  }
  *handle = E;
  return VG_OK;
}

}  // namespace
}  // namespace vg

using namespace vg;

extern "C" int vg_ensemble_create_f64(const VgEnsembleMember *members, int n, const VgEnsembleTuning *tuning,
                                      void **handle) {
  return create<double, VgEnsembleMember, VgStepFields, VgTensorFields, VgTracerArgs>(members, n, tuning, handle);
}

extern "C" int vg_ensemble_create_f32split(const VgEnsembleMemberF32 *members, int n, const VgEnsembleTuning *tuning,
                                           void **handle) {
  return create<float, VgEnsembleMemberF32, VgStepFieldsF32, VgTensorFieldsF32, VgTracerArgsF32>(members, n, tuning,
                                                                                                handle);
}

extern "C" int vg_ensemble_tune(void *handle, const VgEnsembleTuning *t) {
  clear_error();
  if (!handle || !t) return fail(VG_ERR_ARG, "vg_ensemble_tune: NULL argument");
  return static_cast<EnsembleBase *>(handle)->tune(
      Tuning{t->pre_rows, t->pre_kchunk, t->flux_rows, t->flux_kchunk, t->solve_threads});
}

extern "C" int vg_ensemble_step(void *handle, int phase, void *stream) {
  clear_error();
  if (!handle) return fail(VG_ERR_ARG, "vg_ensemble_step: NULL handle");
  return static_cast<EnsembleBase *>(handle)->step(phase, as_stream(stream));
}

extern "C" int vg_ensemble_destroy(void *handle) {
  clear_error();
  delete static_cast<EnsembleBase *>(handle);
  return VG_OK;
}
