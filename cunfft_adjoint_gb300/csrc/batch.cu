// batch.cu -- batched accurate-mode adjoint NFFTs of many series of uneven
// length (cuna2_batch_*).
//
// A batch plan fixes, per series s, its sample count n_s, its output count
// nf_s (shared R and m), and its time origin/period (t0_s, T_s).  Samples of
// all series are concatenated in t and y, outputs in F (offsets are prefix
// sums).  One execution is a fixed set of work-list launches for the whole
// batch, independent of the number of series:
//
//   series with ng_s <= 2^15 (float) / 2^14 (double): k_bsmall, one CTA per
//     series (gridding in shared memory, FFT, epilogue), one launch per grid
//     size class, on a forked stream so they overlap the large series;
//   larger series: k_bcount / k_scan_tiles / k_bscatter (tile bucket sort over
//     one global tile space), k_bgrid (a CTA per tile of any series),
//     k_bcolpass / k_browpass (a CTA per column / row-pair block of any
//     series) -- each CTA reads its series' parameters from a descriptor table.
//
// With cuna2_batch_set_graph the launch sequence is captured once per
// argument set and replayed as one CUDA graph.
#include <limits.h>
#include <algorithm>
#include <map>
#include <mutex>
#include <vector>
#include "accurate_kernels.cuh"
#include "fftpass.cuh"

namespace cuna {
namespace {

template <typename T> struct BDesc {
  AccParams<T> e;
  PhaseMul pm;
  FftDev<T> f;
  int64_t s_off, n;  // samples [s_off, s_off + n) of t and y
  int64_t g_off;     // first real grid cell of this series in the batch grid
  int64_t f_off;     // first output of this series in F
  int tile0, ntiles;  // global tile range of a large series
};

struct Item {
  int s;     // series
  int a, b;  // sample range [a, b) (binning) or block index a (FFT passes)
  int r;     // binning: start of this block's row of the reservation table
};

constexpr int kBChunk = 2048;  // samples per binning CTA (512 threads x 4)

// Binning of the large series, in two launches with the reservations of
// binning.cuh: k_bcount histograms its block of samples per tile and reserves
// the block's range inside every touched tile (resv[it.r + u], relative to
// the tile's start); k_bscatter ranks the same samples with shared atomics
// and writes each record to offsets[tile] + reservation + rank.
template <typename T>
__global__ void __launch_bounds__(512) k_bcount(const double *__restrict__ t, const T *__restrict__ y,
                                                const BDesc<T> *__restrict__ D, const Item *__restrict__ items,
                                                int *__restrict__ counts, int *__restrict__ resv) {
  extern __shared__ int lc[];
  const Item it = items[blockIdx.x];
  const BDesc<T> d = D[it.s];
  for (int u = threadIdx.x; u < d.ntiles; u += blockDim.x) lc[u] = 0;
  __syncthreads();
  SampAcc<T> smp{t + d.s_off, y + d.s_off, d.n, d.pm, d.e};
  typename SampAcc<T>::Raw raw[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int i = it.a + threadIdx.x + k * blockDim.x;
    if (i < it.b) raw[k] = smp.load(i, false);
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int i = it.a + threadIdx.x + k * blockDim.x;
    if (i >= it.b) continue;
    Prep<typename SampAcc<T>::Rec> p;
    smp.prep(i, raw[k], p);
    for (int q = 0; q < p.nt; ++q) atomicAdd(&lc[p.t[q]], 1);
  }
  __syncthreads();
  for (int u = threadIdx.x; u < d.ntiles; u += blockDim.x)
    if (lc[u]) resv[it.r + u] = atomicAdd(&counts[d.tile0 + u], lc[u]);
}

template <typename T>
__global__ void __launch_bounds__(512) k_bscatter(const double *__restrict__ t, const T *__restrict__ y,
                                                  const BDesc<T> *__restrict__ D, const Item *__restrict__ items,
                                                  const int *__restrict__ offsets, const int *__restrict__ resv,
                                                  typename RecOf<T>::type *__restrict__ recs) {
  typedef typename RecOf<T>::type Rec;
  extern __shared__ int sh[];
  const Item it = items[blockIdx.x];
  const BDesc<T> d = D[it.s];
  int *lc = sh, *lbase = sh + d.ntiles;
  SampAcc<T> smp{t + d.s_off, y + d.s_off, d.n, d.pm, d.e};
  typename SampAcc<T>::Raw raw[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int i = it.a + threadIdx.x + k * blockDim.x;
    if (i < it.b) raw[k] = smp.load(i, true);
  }
  // entries of tiles this block does not touch are stale and never used
  for (int u = threadIdx.x; u < d.ntiles; u += blockDim.x) {
    lc[u] = 0;
    lbase[u] = offsets[d.tile0 + u] + resv[it.r + u];
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int i = it.a + threadIdx.x + k * blockDim.x;
    if (i >= it.b) continue;
    Prep<Rec> p;
    smp.prep(i, raw[k], p);
    for (int q = 0; q < p.nt; ++q) {
      const int u = p.t[q];
      recs[lbase[u] + atomicAdd(&lc[u], 1)] = p.rec;
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(kGridThreads, sizeof(T) == 4 ? 6 : 4) k_bgrid(
    const typename RecOf<T>::type *__restrict__ recs, const int *__restrict__ off, T *__restrict__ grid,
    const BDesc<T> *__restrict__ D, const int *__restrict__ tile_series) {
  const int gt = blockIdx.x;
  const BDesc<T> d = D[tile_series[gt]];
  grid_tile_fixed<T>(recs, off[gt], off[gt + 1], (gt - d.tile0) << d.e.logTL, grid + d.g_off, d.e, nullptr, 0, 0,
                     1, 0);
}

// The same tiles in gather form (grid_tile_body): CW = 8 cells per thread on
// 2048-cell tiles, else 4; MASKED as tail_free_gather decides.
template <typename T, int CW, bool MASKED>
__global__ void __launch_bounds__(kGridThreads, sizeof(T) == 4 ? 4 : 2) k_bgrid_gather(
    const typename RecOf<T>::type *__restrict__ recs, const int *__restrict__ off, T *__restrict__ grid,
    const BDesc<T> *__restrict__ D, const int *__restrict__ tile_series) {
  const int gt = blockIdx.x;
  const BDesc<T> d = D[tile_series[gt]];
  typedef const typename RecOf<T>::type *RecPtr;
  const RecPtr rp = recs;
  const T *no_wts = nullptr;
  grid_tile_body<T, CW, RecPtr, 1, MASKED>(rp, off[gt], off[gt + 1], (gt - d.tile0) << d.e.logTL, grid + d.g_off,
                                           d.e, no_wts, (int64_t)0, 0, 1, (int64_t)0);
}

template <typename T>
__global__ void __launch_bounds__(sizeof(T) == 4 ? 512 : 256) k_bcolpass(T *grid, const BDesc<T> *__restrict__ D,
                                                                         const Item *__restrict__ items) {
  typedef typename CxOf<T>::type C;
  const Item it = items[blockIdx.x];
  const BDesc<T> d = D[it.s];
  C *z = reinterpret_cast<C *>(grid + d.g_off);
  colpass_body<T>(z, z, d.f, it.a);
}

template <typename T>
__global__ void __launch_bounds__(sizeof(T) == 4 ? 512 : 256) k_browpass(const T *grid, const BDesc<T> *__restrict__ D,
                                                                         const Item *__restrict__ items,
                                                                         typename CxOf<T>::type *F) {
  typedef typename CxOf<T>::type C;
  const Item it = items[blockIdx.x];
  const BDesc<T> d = D[it.s];
  rowpass_acc_body<T>(reinterpret_cast<const C *>(grid + d.g_off), d.f, d.e, F + d.f_off, it.a);
}

// Four-step passes with compile-time geometry for one size class of large
// series: blockIdx.y indexes the class's series list.
template <typename T, int LOGL>
__global__ void __launch_bounds__(PassCfg<T>::THREADS) k_bct_colpass(T *grid, const BDesc<T> *__restrict__ D,
                                                                     const int *__restrict__ list) {
  typedef typename CxOf<T>::type C;
  const int s = list[blockIdx.y];
  C *z = reinterpret_cast<C *>(grid + D[s].g_off);
  ct_colpass_body<T, LOGL>(z, z, D[s].f, blockIdx.x);
}

template <typename T, int LOGL>
__global__ void __launch_bounds__(PassCfg<T>::THREADS) k_bct_rowpass(const T *grid, const BDesc<T> *__restrict__ D,
                                                                     const int *__restrict__ list,
                                                                     typename CxOf<T>::type *F) {
  typedef typename CxOf<T>::type C;
  const int s = list[blockIdx.y];
  ct_rowpass_body<T, LOGL>(reinterpret_cast<const C *>(grid + D[s].g_off), D[s].f, D[s].e, F + D[s].f_off,
                           blockIdx.x);
}

template <typename T, int LOGL>
int bct_at(T *grid, const BDesc<T> *D, const int *list, int cnt, typename CxOf<T>::type *F, cudaStream_t st) {
  constexpr int LOG1 = (LOGL + 1) / 2, LOG2 = LOGL / 2;
  constexpr int BA = PassCfg<T>::ELEMS >> LOG1;
  constexpr size_t smA = ct_colpass_smem<T, LOGL>(), smB = ct_rowpass_smem<T, LOGL>();
  static char attr;
  if (!setup_done(&attr)) {
    if (cudaFuncSetAttribute(k_bct_colpass<T, LOGL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smA) ||
        cudaFuncSetAttribute(k_bct_rowpass<T, LOGL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smB))
      return -1;
    mark_setup_done(&attr);
  }
  k_bct_colpass<T, LOGL><<<dim3((1 << LOG2) / BA, cnt), PassCfg<T>::THREADS, smA, st>>>(grid, D, list);
  if (cudaPeekAtLastError() != cudaSuccess) return -1;
  k_bct_rowpass<T, LOGL><<<dim3(ct_rowpass_ctas<T, LOGL>(), cnt), PassCfg<T>::THREADS, smB, st>>>(grid, D, list, F);
  if (cudaPeekAtLastError() != cudaSuccess) return -1;
  return 1;
}

// 1: launched, 0: no compiled instance for logL, -1: launch error
template <typename T>
int bct_passes(int logL, T *grid, const BDesc<T> *D, const int *list, int cnt, typename CxOf<T>::type *F,
               cudaStream_t st) {
#define CUNA_BCT(LG) \
  case LG: return bct_at<T, LG>(grid, D, list, cnt, F, st);
  if constexpr (sizeof(T) == 4) {
    switch (logL) { CUNA_BCT(15) CUNA_BCT(16) CUNA_BCT(17) CUNA_BCT(18) CUNA_BCT(19) CUNA_BCT(20) CUNA_BCT(21) CUNA_BCT(22) CUNA_BCT(23) CUNA_BCT(24) CUNA_BCT(25) }
  } else {
    switch (logL) { CUNA_BCT(14) CUNA_BCT(15) CUNA_BCT(16) CUNA_BCT(17) CUNA_BCT(18) CUNA_BCT(19) CUNA_BCT(20) CUNA_BCT(21) CUNA_BCT(22) CUNA_BCT(23) }
  }
#undef CUNA_BCT
  return 0;
}

template <typename T>
__global__ void __launch_bounds__(sizeof(T) == 4 ? 1024 : 512) k_bsmall(const double *__restrict__ t,
                                                                        const T *__restrict__ y,
                                                                        const BDesc<T> *__restrict__ D,
                                                                        const int *__restrict__ list,
                                                                        typename CxOf<T>::type *F) {
  const BDesc<T> d = D[list[blockIdx.x]];
  nfft_small_body<T>(t + d.s_off, y + d.s_off, d.n, d.pm, d.e, d.f, F + d.f_off);
}

template <typename T> AccParams<T> series_params(int64_t nf, int R, int m, double tau, int logTL) {
  AccParams<T> e;
  const int64_t ng = nf * R;
  e.ng = ng;
  e.nf = nf;
  e.K = nf / 2;
  e.m = m;
  e.logTL = logTL;
  e.ntiles = (int)(ng >> logTL);
  e.k1 = (T)(1.0 / (4.0 * tau * log(2.0)));
  e.k2 = (T)(1.0 / (2.0 * tau * log(2.0)));
  e.e3c = (T)(-1.0 / (4.0 * tau));
  e.c0 = (T)(0.5 / sqrt(4.0 * kPi * tau));
  e.c1 = (T)(4.0 * kPi * kPi * tau / ((double)ng * (double)ng));
  e.twk = (T)(2.0 / (double)ng);
  return e;
}

template <typename T> FftDev<T> geom_dev(const FftGeom &g) {
  typedef typename CxOf<T>::type C;
  FftDev<T> f;
  f.logL = g.logL;
  f.logL1 = g.logL1;
  f.logL2 = g.logL2;
  f.tw1 = (const C *)g.tw1;
  f.tw2 = (const C *)g.tw2;
  f.twlo = (const C *)g.twlo;
  f.twhi = (const C *)g.twhi;
  return f;
}

template <typename V> int upload(const std::vector<V> &h, void **d) {
  const size_t bytes = sizeof(V) * (h.empty() ? 1 : h.size());
  cudaError_t e = cudaMalloc(d, bytes);
  if (e != cudaSuccess) return fail(CUNA2_ERROR_ALLOC, "batch plan table of %zu bytes: %s", bytes, cudaGetErrorString(e));
  if (!h.empty()) {
    e = cudaMemcpy(*d, h.data(), sizeof(V) * h.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail_cuda(e, "cudaMemcpy(batch plan table)");
  }
  return CUNA2_SUCCESS;
}

}  // namespace
}  // namespace cuna

struct cuna2_batch_plan_st {
  int dtype, nseries;
  int m_max;  // the widest filter of the batch (shared-memory sizes, tile spans)
  std::vector<int> m_set;  // the batch's distinct filter widths
  // oversampling and filter half-width of each series (cuna2_batch_plan_create_ex)
  std::vector<int> R, m;
  bool tail_free = true;  // every series' Gaussian tail allows the unmasked gather
  // gridding schedule of the large series (cuna2_batch_set_schedule)
  int log_tile = 12;
  int grid_method = CUNA2_GRID_FIXED;
  int64_t n_total = 0, f_total = 0;
  std::vector<int64_t> n, nf;
  std::vector<double> t0, T;
  // large series
  int tiles_total = 0;
  int64_t large_samples = 0, grid_total = 0;
  int n_count_items = 0, n_col_items = 0, n_row_items = 0;
  size_t smem_col = 0, smem_row = 0, smem_bin = 0;
  int max_large_tiles = 0;
  // small series by grid size class (log2 of the packed length)
  std::vector<std::pair<int, int>> small_classes;  // (logL, count)
  std::vector<int> small_class_off;
  // large series by packed length (log2), for the compile-time FFT passes
  std::vector<std::pair<int, int>> fft_classes;  // (logL, count)
  std::vector<int> fft_class_off;
  bool fft_ct = false;  // every class has a compiled instance
  void *d_fft_list = nullptr;
  // device tables
  void *d_desc = nullptr, *d_count_items = nullptr, *d_tile_series = nullptr, *d_col_items = nullptr,
       *d_row_items = nullptr, *d_small_list = nullptr;
  void *host_desc = nullptr;  // host copy (plain memory) for time updates
  size_t desc_bytes = 0;
  // workspace
  void *ws = nullptr;
  int *counts = nullptr, *offsets = nullptr, *cursor = nullptr, *scan_totals = nullptr;
  int *resv = nullptr;  // reservation table of the binning, one row of ntiles per count block
  void *recs = nullptr, *grid = nullptr;
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  bool use_graph = false;
  cudaStream_t cap_stream = nullptr;
  struct GraphEntry {
    const void *t, *y, *F;
    cudaGraphExec_t exec;
  };
  std::vector<GraphEntry> graphs;
  std::mutex mu;
};

namespace cuna {
namespace {

template <typename T> int batch_build(cuna2_batch_plan_st *p) {
  typedef typename CxOf<T>::type C;
  typedef typename RecOf<T>::type Rec;
  const bool dbl = sizeof(T) == 8;
  const int single_log = dbl ? kSingleLogF64 : kSingleLogF32;
  const int elems = dbl ? kPassElemsF64 : kPassElemsF32;
  std::vector<BDesc<T>> desc(p->nseries);
  std::vector<Item> count_items, col_items, row_items;
  std::vector<int> tile_series;
  int64_t resv_total = 0;  // entries of the binning's reservation table
  std::map<int, std::vector<int>> small;  // logL -> series
  std::map<int, std::vector<int>> large;  // logL -> series
  int64_t s_off = 0, f_off = 0, g_off = 0;
  int tile0 = 0;
  for (int s = 0; s < p->nseries; ++s) {
    const int64_t nf = p->nf[s], ng = nf * p->R[s], L = ng / 2;
    const int logL = ilog2i(L);
    const bool is_small = logL <= single_log;
    const int logTL = std::min(ilog2i(ng), p->log_tile);
    BDesc<T> &d = desc[s];
    const double tau = (double)p->m[s] * p->R[s] / (4.0 * kPi * (p->R[s] - 0.5));
    d.e = series_params<T>(nf, p->R[s], p->m[s], tau, logTL);
    d.pm = phase_setup(p->t0[s], p->T[s]);
    FftGeom g;
    CUNA_TRY(fft_geometry(dbl, logL, &g));
    d.f = geom_dev<T>(g);
    d.s_off = s_off;
    d.n = p->n[s];
    d.f_off = f_off;
    d.g_off = -1;
    d.tile0 = 0;
    d.ntiles = 0;
    if (is_small) {
      small[logL].push_back(s);
    } else {
      d.g_off = g_off;
      d.tile0 = tile0;
      d.ntiles = (int)(ng >> logTL);
      if (d.ntiles > kBinSmemTiles)
        return fail(CUNA2_ERROR_UNSUPPORTED, "series %d: grid of %lld cells exceeds the batched tile limit", s,
                    (long long)ng);
      p->max_large_tiles = std::max(p->max_large_tiles, d.ntiles);
      for (int u = 0; u < d.ntiles; ++u) tile_series.push_back(s);
      for (int64_t a = 0; a < d.n; a += kBChunk) {
        count_items.push_back({s, (int)a, (int)std::min<int64_t>(d.n, a + kBChunk), (int)resv_total});
        resv_total += d.ntiles;
      }
      const int L1 = 1 << g.logL1, L2 = 1 << g.logL2;
      const int BA = elems / L1, BB = elems / L2, PB = BB / 2, npairs = L1 / 2 + 1;
      for (int cb = 0; cb < L2 / BA; ++cb) col_items.push_back({s, cb, 0, 0});
      for (int pb = 0; pb < (npairs + PB - 1) / PB; ++pb) row_items.push_back({s, pb, 0, 0});
      p->smem_col = std::max(p->smem_col, sizeof(C) * (size_t)BA * fft_pitch(L1, BA));
      p->smem_row = std::max(p->smem_row, sizeof(C) * (size_t)BB * fft_pitch(L2, BB));
      large[logL].push_back(s);
      tile0 += d.ntiles;
      g_off += ng;
      p->large_samples += d.n;
    }
    s_off += p->n[s];
    f_off += nf;
  }
  p->n_total = s_off;
  p->f_total = f_off;
  p->tiles_total = tile0;
  p->grid_total = g_off;
  p->n_count_items = (int)count_items.size();
  p->n_col_items = (int)col_items.size();
  p->n_row_items = (int)row_items.size();
  p->smem_bin = sizeof(int) * 2 * (size_t)std::max(1, p->max_large_tiles);
  std::vector<int> small_list;
  for (auto &kv : small) {
    p->small_classes.push_back({kv.first, (int)kv.second.size()});
    p->small_class_off.push_back((int)small_list.size());
    small_list.insert(small_list.end(), kv.second.begin(), kv.second.end());
  }
  std::vector<int> fft_list;
  p->fft_ct = true;
  const int lo = dbl ? 14 : 15, hi = dbl ? 23 : 25;
  for (auto &kv : large) {
    p->fft_classes.push_back({kv.first, (int)kv.second.size()});
    p->fft_class_off.push_back((int)fft_list.size());
    fft_list.insert(fft_list.end(), kv.second.begin(), kv.second.end());
    if (kv.first < lo || kv.first > hi || kv.second.size() > 65535) p->fft_ct = false;
  }
  CUNA_TRY(upload(fft_list, &p->d_fft_list));
  p->desc_bytes = sizeof(BDesc<T>) * desc.size();
  p->host_desc = malloc(p->desc_bytes ? p->desc_bytes : 1);
  if (!p->host_desc) return fail(CUNA2_ERROR_ALLOC, "host descriptor table");
  memcpy(p->host_desc, desc.data(), p->desc_bytes);
  CUNA_TRY(upload(desc, &p->d_desc));
  CUNA_TRY(upload(count_items, &p->d_count_items));
  CUNA_TRY(upload(tile_series, &p->d_tile_series));
  CUNA_TRY(upload(col_items, &p->d_col_items));
  CUNA_TRY(upload(row_items, &p->d_row_items));
  CUNA_TRY(upload(small_list, &p->d_small_list));
  if (resv_total > INT_MAX)
    return fail(CUNA2_ERROR_UNSUPPORTED, "batch too large: %lld binning reservations", (long long)resv_total);
  // workspace: counts | offsets | cursor | scan totals | reservations | records | grid
  const size_t nt = (size_t)std::max(1, p->tiles_total);
  const size_t o_off = align_up(sizeof(int) * nt), o_cur = o_off + align_up(sizeof(int) * (nt + 1));
  const size_t o_tot = o_cur + align_up(sizeof(int) * nt);
  const size_t o_rsv = o_tot + align_up(sizeof(int) * (nt / kScanChunk + 1));
  const size_t o_rec = o_rsv + align_up(sizeof(int) * (size_t)std::max<int64_t>(1, resv_total));
  const size_t o_grid = o_rec + align_up(sizeof(Rec) * 2 * (size_t)std::max<int64_t>(1, p->large_samples));
  const size_t bytes = o_grid + sizeof(T) * (size_t)std::max<int64_t>(1, p->grid_total);
  cudaError_t e = cudaMalloc(&p->ws, bytes);
  if (e != cudaSuccess) return fail(CUNA2_ERROR_ALLOC, "batch workspace of %zu bytes: %s", bytes, cudaGetErrorString(e));
  char *w = (char *)p->ws;
  p->counts = (int *)w;
  p->offsets = (int *)(w + o_off);
  p->cursor = (int *)(w + o_cur);
  p->scan_totals = (int *)(w + o_tot);
  p->resv = (int *)(w + o_rsv);
  p->recs = w + o_rec;
  p->grid = w + o_grid;
  CUNA_CK(cudaStreamCreateWithFlags(&p->side, cudaStreamNonBlocking));
  CUNA_CK(cudaEventCreateWithFlags(&p->ev_fork, cudaEventDisableTiming));
  CUNA_CK(cudaEventCreateWithFlags(&p->ev_join, cudaEventDisableTiming));
  return CUNA2_SUCCESS;
}

template <typename T>
int batch_run(cuna2_batch_plan_st *p, const double *t, const T *y, typename CxOf<T>::type *F, cudaStream_t st) {
  typedef typename CxOf<T>::type C;
  typedef typename RecOf<T>::type Rec;
  if ((p->n_total > 0 && (!t || !y)) || !F) return fail(CUNA2_ERROR_INVALID_VALUE, "NULL array");
  const BDesc<T> *D = (const BDesc<T> *)p->d_desc;
  static char attr;
  if (!setup_done(&attr)) {
    CUNA_CK(cudaFuncSetAttribute(k_bsmall<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024));
    CUNA_CK(cudaFuncSetAttribute(k_bgrid<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    CUNA_CK(cudaFuncSetAttribute(k_bgrid_gather<T, 8, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    CUNA_CK(cudaFuncSetAttribute(k_bgrid_gather<T, 8, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    CUNA_CK(cudaFuncSetAttribute(k_bgrid_gather<T, 4, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    CUNA_CK(cudaFuncSetAttribute(k_bgrid_gather<T, 4, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    CUNA_CK(cudaFuncSetAttribute(k_bcolpass<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    CUNA_CK(cudaFuncSetAttribute(k_browpass<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    mark_setup_done(&attr);
  }
  // small series on the side stream, overlapping the large-series pipeline
  if (!p->small_classes.empty()) {
    CUNA_CK(cudaEventRecord(p->ev_fork, st));
    CUNA_CK(cudaStreamWaitEvent(p->side, p->ev_fork, 0));
    for (size_t c = 0; c < p->small_classes.size(); ++c) {
      const int logL = p->small_classes[c].first, cnt = p->small_classes[c].second;
      const int L = 1 << logL;
      const size_t smem = sizeof(C) * (size_t)fft_pitch(L, 1) + sizeof(T) * (2 * p->m_max + 2);
      const int threads = std::max(32, std::min(1024, L / kFftE));
      k_bsmall<T><<<cnt, threads, smem, p->side>>>(t, y, D, (const int *)p->d_small_list + p->small_class_off[c], F);
      CUNA_CK(cudaGetLastError());
    }
    CUNA_CK(cudaEventRecord(p->ev_join, p->side));
  }
  if (p->tiles_total > 0) {
    const int ntl = p->tiles_total;
    CUNA_CK(cudaMemsetAsync(p->counts, 0, sizeof(int) * ntl, st));
    if (p->n_count_items > 0) {
      k_bcount<T><<<p->n_count_items, 512, p->smem_bin / 2, st>>>(t, y, D, (const Item *)p->d_count_items, p->counts,
                                                                 p->resv);
      CUNA_CK(cudaGetLastError());
    }
    if (ntl <= 2 * kScanChunk) {
      k_scan_tiles<<<1, 1024, 0, st>>>(p->counts, p->offsets, p->cursor, ntl);
    } else {
      const int nb = (ntl + kScanChunk - 1) / kScanChunk;
      int *totals = p->scan_totals;
      k_scan_blocks<<<nb, 1024, 0, st>>>(p->counts, p->offsets, totals, ntl);
      CUNA_CK(cudaGetLastError());
      k_scan_add<<<nb, 1024, 0, st>>>(p->offsets, totals, p->cursor, ntl, nb);
    }
    CUNA_CK(cudaGetLastError());
    if (p->n_count_items > 0) {
      k_bscatter<T><<<p->n_count_items, 512, p->smem_bin, st>>>(t, y, D, (const Item *)p->d_count_items, p->offsets,
                                                               p->resv, (Rec *)p->recs);
      CUNA_CK(cudaGetLastError());
    }
    const Rec *rc = (const Rec *)p->recs;
    const int *ts = (const int *)p->d_tile_series;
    if (p->grid_method == CUNA2_GRID_GATHER) {
      const size_t smg = (grid_smem_bytes<T>(p->log_tile, p->m_max) + 15) & ~(size_t)15;
      const bool free_ = sizeof(T) == 4 && p->tail_free && !masked_gather_forced();
      if (p->log_tile == 11) {
        if (free_) k_bgrid_gather<T, 8, false><<<ntl, kGridThreads, smg, st>>>(rc, p->offsets, (T *)p->grid, D, ts);
        else k_bgrid_gather<T, 8, true><<<ntl, kGridThreads, smg, st>>>(rc, p->offsets, (T *)p->grid, D, ts);
      } else {
        if (free_) k_bgrid_gather<T, 4, false><<<ntl, kGridThreads, smg, st>>>(rc, p->offsets, (T *)p->grid, D, ts);
        else k_bgrid_gather<T, 4, true><<<ntl, kGridThreads, smg, st>>>(rc, p->offsets, (T *)p->grid, D, ts);
      }
    } else {
      // the bucket table's length depends on m, not monotonically: the
      // largest over the batch's filter widths
      size_t smg = 0;
      for (int mw : p->m_set) smg = std::max(smg, grid_fixed_smem_bytes<T>(p->log_tile, mw));
      k_bgrid<T><<<ntl, kGridThreads, smg, st>>>(rc, p->offsets, (T *)p->grid, D, ts);
    }
    CUNA_CK(cudaGetLastError());
    if (p->fft_ct) {  // one column and one row launch per size class
      for (size_t c = 0; c < p->fft_classes.size(); ++c) {
        const int r = bct_passes<T>(p->fft_classes[c].first, (T *)p->grid, D,
                                    (const int *)p->d_fft_list + p->fft_class_off[c], p->fft_classes[c].second, F, st);
        if (r != 1) return fail_cuda(cudaGetLastError(), "batched FFT pass launch");
      }
    } else {
      const int threads = (sizeof(T) == 4 ? kPassElemsF32 : kPassElemsF64) / kFftE;
      k_bcolpass<T><<<p->n_col_items, threads, p->smem_col, st>>>((T *)p->grid, D, (const Item *)p->d_col_items);
      CUNA_CK(cudaGetLastError());
      k_browpass<T><<<p->n_row_items, threads, p->smem_row, st>>>((const T *)p->grid, D, (const Item *)p->d_row_items,
                                                                  F);
      CUNA_CK(cudaGetLastError());
    }
  }
  if (!p->small_classes.empty()) CUNA_CK(cudaStreamWaitEvent(st, p->ev_join, 0));
  return CUNA2_SUCCESS;
}

int batch_any(cuna2_batch_plan_st *p, const double *t, const void *y, void *F, cudaStream_t st) {
  if (p->dtype == CUNA2_F32) return batch_run<float>(p, t, (const float *)y, (float2 *)F, st);
  return batch_run<double>(p, t, (const double *)y, (double2 *)F, st);
}

int batch_graph(cuna2_batch_plan_st *p, const double *t, const void *y, void *F, cudaStream_t st) {
  for (auto &g : p->graphs)
    if (g.t == t && g.y == y && g.F == F) {
      CUNA_CK(cudaGraphLaunch(g.exec, st));
      return CUNA2_SUCCESS;
    }
  CUNA_TRY(batch_any(p, t, y, F, st));
  if (!p->cap_stream) CUNA_CK(cudaStreamCreateWithFlags(&p->cap_stream, cudaStreamNonBlocking));
  CUNA_CK(cudaStreamSynchronize(st));
  CUNA_CK(cudaStreamBeginCapture(p->cap_stream, cudaStreamCaptureModeThreadLocal));
  int s = batch_any(p, t, y, F, p->cap_stream);
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamEndCapture(p->cap_stream, &graph);
  if (s) return s;
  if (e != cudaSuccess) return fail_cuda(e, "cudaStreamEndCapture");
  cudaGraphExec_t exec = nullptr;
  e = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return fail_cuda(e, "cudaGraphInstantiate");
  if (p->graphs.size() >= 16) {
    cudaGraphExecDestroy(p->graphs.front().exec);
    p->graphs.erase(p->graphs.begin());
  }
  p->graphs.push_back({t, y, F, exec});
  return CUNA2_SUCCESS;
}

// Everything batch_build makes (tables, workspace, streams, graphs), so that
// it can build the plan again under another schedule.
void batch_release(cuna2_batch_plan_st *p) {
  for (auto &g : p->graphs) cudaGraphExecDestroy(g.exec);
  p->graphs.clear();
  if (p->cap_stream) cudaStreamDestroy(p->cap_stream);
  if (p->side) cudaStreamDestroy(p->side);
  if (p->ev_fork) cudaEventDestroy(p->ev_fork);
  if (p->ev_join) cudaEventDestroy(p->ev_join);
  p->cap_stream = p->side = nullptr;
  p->ev_fork = p->ev_join = nullptr;
  for (void **d : {&p->d_desc, &p->d_count_items, &p->d_tile_series, &p->d_col_items, &p->d_row_items,
                   &p->d_small_list, &p->d_fft_list, &p->ws}) {
    if (*d) cudaFree(*d);
    *d = nullptr;
  }
  free(p->host_desc);
  p->host_desc = nullptr;
  p->desc_bytes = 0;
  p->tiles_total = 0;
  p->large_samples = p->grid_total = 0;
  p->n_count_items = p->n_col_items = p->n_row_items = 0;
  p->smem_col = p->smem_row = p->smem_bin = 0;
  p->max_large_tiles = 0;
  p->small_classes.clear();
  p->small_class_off.clear();
  p->fft_classes.clear();
  p->fft_class_off.clear();
  p->fft_ct = false;
}

void batch_free(cuna2_batch_plan_st *p) {
  batch_release(p);
  delete p;
}

int batch_rebuild(cuna2_batch_plan_st *p) {
  CUNA_CK(cudaDeviceSynchronize());  // nothing may still use the old tables
  batch_release(p);
  return p->dtype == CUNA2_F32 ? batch_build<float>(p) : batch_build<double>(p);
}

template <typename T> void set_times_host(cuna2_batch_plan_st *p) {
  BDesc<T> *d = (BDesc<T> *)p->host_desc;
  for (int s = 0; s < p->nseries; ++s) d[s].pm = phase_setup(p->t0[s], p->T[s]);
}

}  // namespace
}  // namespace cuna

using namespace cuna;

extern "C" int cuna2_batch_plan_create_ex(cuna2_batch_plan *plan, int dtype, int nseries, const int64_t *n,
                                          const int64_t *nf, const int *R, const int *m, const double *t0,
                                          const double *T) {
  clear_error();
  if (!plan) return fail(CUNA2_ERROR_INVALID_VALUE, "plan pointer is NULL");
  *plan = nullptr;
  if (dtype != CUNA2_F32 && dtype != CUNA2_F64) return fail(CUNA2_ERROR_INVALID_VALUE, "dtype %d", dtype);
  if (nseries < 1 || !n || !nf || !R || !m)
    return fail(CUNA2_ERROR_INVALID_VALUE, "need nseries >= 1 and n, nf, R, m arrays");
  const int max_log = dtype == CUNA2_F32 ? 25 : 23;
  for (int s = 0; s < nseries; ++s) {
    if (R[s] < 2 || m[s] < 1 || m[s] > 16)
      return fail(CUNA2_ERROR_INVALID_VALUE, "series %d: need R >= 2 and 1 <= m <= 16 (R=%d m=%d)", s, R[s], m[s]);
    const int64_t ng = nf[s] * R[s], L = ng / 2;
    if (n[s] < 0 || n[s] > ((int64_t)1 << 30) || nf[s] < 2 || (nf[s] & 1) || (L & (L - 1)) || ng < 4 * m[s] ||
        ilog2i(L) > max_log)
      return fail(CUNA2_ERROR_INVALID_VALUE, "series %d: unsupported n=%lld nf=%lld (R*nf/2 must be a power of two)",
                  s, (long long)n[s], (long long)nf[s]);
    if (T && !(T[s] > 0)) return fail(CUNA2_ERROR_INVALID_VALUE, "series %d: T must be > 0", s);
  }
  cuna2_batch_plan_st *p = new cuna2_batch_plan_st();
  p->dtype = dtype;
  p->nseries = nseries;
  p->R.assign(R, R + nseries);
  p->m.assign(m, m + nseries);
  p->m_max = *std::max_element(m, m + nseries);
  p->m_set.assign(m, m + nseries);
  std::sort(p->m_set.begin(), p->m_set.end());
  p->m_set.erase(std::unique(p->m_set.begin(), p->m_set.end()), p->m_set.end());
  for (int s = 0; s < nseries; ++s)
    p->tail_free = p->tail_free && tail_free_gather(true, m[s], (double)m[s] * R[s] / (4.0 * kPi * (R[s] - 0.5)));
  p->n.assign(n, n + nseries);
  p->nf.assign(nf, nf + nseries);
  p->t0.assign(nseries, 0.0);
  p->T.assign(nseries, 1.0);
  if (t0) p->t0.assign(t0, t0 + nseries);
  if (T) p->T.assign(T, T + nseries);
  int st = dtype == CUNA2_F32 ? batch_build<float>(p) : batch_build<double>(p);
  if (st) {
    batch_free(p);
    return st;
  }
  *plan = p;
  return CUNA2_SUCCESS;
}

extern "C" int cuna2_batch_plan_create(cuna2_batch_plan *plan, int dtype, int nseries, const int64_t *n,
                                       const int64_t *nf, int R, int m, const double *t0, const double *T) {
  clear_error();
  if (!plan) return fail(CUNA2_ERROR_INVALID_VALUE, "plan pointer is NULL");
  *plan = nullptr;
  if (nseries < 1 || !n || !nf || R < 2 || m < 1 || m > 16)
    return fail(CUNA2_ERROR_INVALID_VALUE, "need nseries >= 1, n and nf arrays, R >= 2, 1 <= m <= 16");
  const std::vector<int> Rs(nseries, R), ms(nseries, m);
  return cuna2_batch_plan_create_ex(plan, dtype, nseries, n, nf, Rs.data(), ms.data(), t0, T);
}

extern "C" int cuna2_batch_get_filter(cuna2_batch_plan p, int *R, int *m) {
  clear_error();
  if (!p) return fail(CUNA2_ERROR_INVALID_VALUE, "NULL plan");
  for (int s = 0; s < p->nseries; ++s) {
    if (R) R[s] = p->R[s];
    if (m) m[s] = p->m[s];
  }
  return CUNA2_SUCCESS;
}

// Filter-width schedule of a batch.  The candidates for each size class
// (series of one output length nf) are R = 2, 4, 8 with the smallest m whose
// Gaussian error exp(-pi m sqrt(1 - 1/R)) reaches tol (clamped at the plan
// type's rounding).  Every class starts at R = 2; then, class by class (most
// samples first), R = 4 and 8 are tried with the other classes kept, each
// candidate batch autotuned over its gridding schedules on the caller's
// batch, and a class keeps the fastest.
extern "C" int cuna2_batch_plan_create_auto(cuna2_batch_plan *plan, int dtype, int nseries, const int64_t *n,
                                            const int64_t *nf, double tol, const double *t0, const double *T,
                                            const double *t, const void *y, void *F, cudaStream_t st, int *R_out,
                                            int *m_out) {
  clear_error();
  if (plan) *plan = nullptr;
  if (!plan || !n || !nf || nseries < 1 || !t || !y || !F || !(tol > 0) || !(tol < 1))
    return fail(CUNA2_ERROR_INVALID_VALUE, "invalid argument");
  if (dtype != CUNA2_F32 && dtype != CUNA2_F64) return fail(CUNA2_ERROR_INVALID_VALUE, "dtype %d", dtype);
  const double target = std::max(tol, dtype == CUNA2_F32 ? 1e-7 : 1e-15);
  auto width = [&](int R) {
    return std::max(2, (int)std::ceil(-std::log(target) / (kPi * std::sqrt(1.0 - 1.0 / R))));
  };
  // size classes by output length, most samples first
  std::map<int64_t, int64_t> cls_n;
  for (int s = 0; s < nseries; ++s) cls_n[nf[s]] += n[s];
  std::vector<std::pair<int64_t, int64_t>> classes(cls_n.begin(), cls_n.end());
  std::sort(classes.begin(), classes.end(), [](const std::pair<int64_t, int64_t> &a,
                                              const std::pair<int64_t, int64_t> &b) { return a.second > b.second; });
  std::map<int64_t, int> cls_R;
  for (auto &c : classes) cls_R[c.first] = 2;
  std::vector<int> Rs(nseries), ms(nseries);
  cuna2_batch_plan best = nullptr;
  float best_ms = 3.4e38f;
  int last = CUNA2_SUCCESS;
  // builds and times the batch with the classes' current R; keeps it when faster
  auto trial = [&](bool *kept) -> int {
    *kept = false;
    for (int s = 0; s < nseries; ++s) {
      Rs[s] = cls_R[nf[s]];
      ms[s] = width(Rs[s]);
      if (ms[s] > 16) return CUNA2_SUCCESS;  // not reachable at this R
    }
    cuna2_batch_plan c = nullptr;
    last = cuna2_batch_plan_create_ex(&c, dtype, nseries, n, nf, Rs.data(), ms.data(), t0, T);
    if (last != CUNA2_SUCCESS) return CUNA2_SUCCESS;  // e.g. a grid too large at this R
    float ms_c = 0.f;
    const int s = cuna2_batch_autotune(c, t, y, F, st, 3, &ms_c);
    if (s != CUNA2_SUCCESS) {
      cuna2_batch_plan_destroy(c);
      return s;
    }
    if (ms_c < best_ms) {
      if (best) cuna2_batch_plan_destroy(best);
      best = c;
      best_ms = ms_c;
      *kept = true;
    } else {
      cuna2_batch_plan_destroy(c);
    }
    return CUNA2_SUCCESS;
  };
  bool kept = false;
  int s = trial(&kept);
  for (size_t ci = 0; !s && ci < classes.size(); ++ci) {
    const int64_t key = classes[ci].first;
    int keepR = cls_R[key];
    for (int R = 4; !s && R <= 8; R *= 2) {
      cls_R[key] = R;
      s = trial(&kept);
      if (kept) keepR = R;
    }
    cls_R[key] = keepR;
  }
  if (s) {
    if (best) cuna2_batch_plan_destroy(best);
    return s;
  }
  if (!best) {
    if (last != CUNA2_SUCCESS) return last;  // the message of the last failed candidate stands
    return fail(CUNA2_ERROR_UNSUPPORTED, "no batch plan reaches tol=%g with m <= 16", tol);
  }
  clear_error();
  *plan = best;
  cuna2_batch_get_filter(best, R_out, m_out);
  return CUNA2_SUCCESS;
}

extern "C" int cuna2_batch_plan_destroy(cuna2_batch_plan p) {
  clear_error();
  if (p) batch_free(p);
  return CUNA2_SUCCESS;
}

extern "C" int cuna2_batch_set_times(cuna2_batch_plan p, const double *t0, const double *T) {
  clear_error();
  if (!p || !t0 || !T) return fail(CUNA2_ERROR_INVALID_VALUE, "invalid argument");
  std::lock_guard<std::mutex> lk(p->mu);
  for (int s = 0; s < p->nseries; ++s)
    if (!(T[s] > 0)) return fail(CUNA2_ERROR_INVALID_VALUE, "series %d: T must be > 0", s);
  p->t0.assign(t0, t0 + p->nseries);
  p->T.assign(T, T + p->nseries);
  if (p->dtype == CUNA2_F32) set_times_host<float>(p);
  else set_times_host<double>(p);
  CUNA_CK(cudaDeviceSynchronize());  // no execution may be reading the table
  CUNA_CK(cudaMemcpy(p->d_desc, p->host_desc, p->desc_bytes, cudaMemcpyHostToDevice));
  return CUNA2_SUCCESS;
}

extern "C" int cuna2_batch_info(cuna2_batch_plan p, int64_t *n_total, int64_t *nf_total) {
  clear_error();
  if (!p) return fail(CUNA2_ERROR_INVALID_VALUE, "NULL plan");
  if (n_total) *n_total = p->n_total;
  if (nf_total) *nf_total = p->f_total;
  return CUNA2_SUCCESS;
}

extern "C" int cuna2_batch_set_graph(cuna2_batch_plan p, int enable) {
  clear_error();
  if (!p) return fail(CUNA2_ERROR_INVALID_VALUE, "NULL plan");
  std::lock_guard<std::mutex> lk(p->mu);
  p->use_graph = enable != 0;
  return CUNA2_SUCCESS;
}

extern "C" int cuna2_batch_adjoint(cuna2_batch_plan p, const double *t, const void *y, void *F, cudaStream_t st) {
  clear_error();
  if (!p) return fail(CUNA2_ERROR_INVALID_VALUE, "NULL plan");
  std::lock_guard<std::mutex> lk(p->mu);
  return p->use_graph ? batch_graph(p, t, y, F, st) : batch_any(p, t, y, F, st);
}

extern "C" int cuna2_batch_set_schedule(cuna2_batch_plan p, int log_tile, int grid_method) {
  clear_error();
  if (!p) return fail(CUNA2_ERROR_INVALID_VALUE, "NULL plan");
  if (grid_method != CUNA2_GRID_GATHER && grid_method != CUNA2_GRID_FIXED)
    return fail(CUNA2_ERROR_INVALID_VALUE, "batched plans grid in gather or fixed-point form");
  if (log_tile < 10 || log_tile > (grid_method == CUNA2_GRID_FIXED ? 13 : 12))
    return fail(CUNA2_ERROR_INVALID_VALUE, "log_tile must be 10 to 13 (fixed point) or 10 to 12 (gather)");
  if (2 * p->m_max > (1 << log_tile)) return fail(CUNA2_ERROR_INVALID_VALUE, "tiles must span at least 2m cells");
  std::lock_guard<std::mutex> lk(p->mu);
  if (p->log_tile == log_tile && p->grid_method == grid_method) return CUNA2_SUCCESS;
  const int old_lt = p->log_tile, old_gm = p->grid_method;
  p->log_tile = log_tile;
  p->grid_method = grid_method;
  const int s = batch_rebuild(p);
  if (s) {  // put the previous schedule back
    p->log_tile = old_lt;
    p->grid_method = old_gm;
    batch_rebuild(p);
  }
  return s;
}

extern "C" int cuna2_batch_get_schedule(cuna2_batch_plan p, int *log_tile, int *grid_method) {
  clear_error();
  if (!p) return fail(CUNA2_ERROR_INVALID_VALUE, "NULL plan");
  if (log_tile) *log_tile = p->log_tile;
  if (grid_method) *grid_method = p->grid_method;
  return CUNA2_SUCCESS;
}

extern "C" int cuna2_batch_autotune(cuna2_batch_plan p, const double *t, const void *y, void *F, cudaStream_t st,
                                    int reps, float *best_ms) {
  clear_error();
  if (!p || reps < 1) return fail(CUNA2_ERROR_INVALID_VALUE, "invalid argument");
  bool graph;
  {
    std::lock_guard<std::mutex> lk(p->mu);
    graph = p->use_graph;
    p->use_graph = false;  // time eager executions; no graphs of trial schedules
  }
  // a buffer of twice the L2 size, overwritten before each timed run so the
  // inputs come from HBM
  int dev = 0, l2 = 0;
  CUNA_CK(cudaGetDevice(&dev));
  CUNA_CK(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev));
  void *flush = nullptr;
  if (cudaMalloc(&flush, 2 * (size_t)l2) != cudaSuccess) {
    cudaGetLastError();
    flush = nullptr;
  }
  cudaEvent_t e0, e1;
  CUNA_CK(cudaEventCreate(&e0));
  CUNA_CK(cudaEventCreate(&e1));
  float best = 1e30f;
  int best_lt = p->log_tile, best_gm = p->grid_method, status = CUNA2_SUCCESS;
  for (int gm : {CUNA2_GRID_FIXED, CUNA2_GRID_GATHER}) {
    for (int lt = 10; lt <= (gm == CUNA2_GRID_FIXED ? 13 : 12); ++lt) {
      if (2 * p->m_max > (1 << lt)) continue;
      if (cuna2_batch_set_schedule(p, lt, gm) != CUNA2_SUCCESS) continue;
      float ms = 1e30f;
      int s = cuna2_batch_adjoint(p, t, y, F, st);  // warm-up
      for (int r = 0; !s && r < reps; ++r) {
        if (flush) cudaMemsetAsync(flush, r & 0xff, 2 * (size_t)l2, st);
        cudaEventRecord(e0, st);
        s = cuna2_batch_adjoint(p, t, y, F, st);
        cudaEventRecord(e1, st);
        if (!s && cudaEventSynchronize(e1) == cudaSuccess) {
          float x = 0.f;
          cudaEventElapsedTime(&x, e0, e1);
          ms = std::min(ms, x);
        }
      }
      if (s) {
        status = s;
        break;
      }
      if (ms < best) {
        best = ms;
        best_lt = lt;
        best_gm = gm;
      }
    }
    if (status) break;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (flush) cudaFree(flush);
  const int s2 = cuna2_batch_set_schedule(p, best_lt, best_gm);
  {
    std::lock_guard<std::mutex> lk(p->mu);
    p->use_graph = graph;
  }
  if (status) return status;
  if (s2) return s2;
  if (best_ms) *best_ms = best;
  return CUNA2_SUCCESS;
}
