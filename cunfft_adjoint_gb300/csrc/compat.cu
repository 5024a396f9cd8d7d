// compat.cu -- the reference library's arithmetic on the GB300 pipeline.
//
// Compiled with --use_fast_math, the flag the reference builds with
// (Makefile:26), so expf/powf/sqrtf/division in the filter coefficients map to
// the same hardware approximations and the per-tap weights agree with the
// reference's GPU build bit for bit; only the summation order differs.
//
// Pipeline per call (all on the caller's stream, no host synchronisation):
//   k_bin_count / k_scan_tiles / k_bin_scatter  samples -> tile-sorted records
//   k_grid_compat     one CTA per (tile, resample): taps accumulated in shared
//                     memory in fixed point, flushed once with f_hat[c].x += acc[c]
//   FFT               in-place inverse FFT of ng points with the reference's
//                     deconvolution fused into the last pass
//                     (single CTA for ng <= 2^14 (f32) / 2^13 (f64), four-step
//                     otherwise; non power-of-two ng falls back to cuFFT +
//                     k_compat_normalize)
#include <cufft.h>
#include <limits.h>
#include <map>
#include <mutex>
#include <tuple>
#include <algorithm>
#include "binning.cuh"
#include "fft.cuh"
#include "fftpass_core.cuh"
#include "rng.cuh"
#include "runtime.h"

namespace cuna {
namespace {

#define CUNA_PI 3.14159265358979323846

template <typename T> struct FpOf;
template <> struct FpOf<float> { typedef cuna2_filter_properties_f32 type; };
template <> struct FpOf<double> { typedef cuna2_filter_properties_f64 type; };

constexpr int kCompatLogTL = 12;  // 4096-cell tiles
constexpr int kCompatMaxRf = 64;  // shared E3 table size

// ---------------------------------------------------------------------------
// filter precompute: set_gpu_filter_properties, src/gaussian_filter.cu:204-228
// ---------------------------------------------------------------------------
// Filter origin u = (int)(ng x - R_f) of src/gaussian_filter.cu:213, in the
// sample's own precision (nvcc contracts the product and the difference into
// one fused multiply-add, here as in the reference's build).
__device__ __forceinline__ int compat_origin(float x, int ng, int rf) { return (int)(ng * x - rf); }
__device__ __forceinline__ int compat_origin(double x, int ng, int rf) { return (int)(ng * x - rf); }

__global__ void k_compat_filter_f32(cuna2_filter_properties_f32 *f, const float *x, int ng, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    int u = compat_origin(x[i], ng, f->filter_radius);
    float eps = ng * x[i] - u;
    float eps2 = eps / f->b;
    f->E1[i] = expf(-eps * eps2) / sqrtf(CUNA_PI * f->b);
    f->E2[i] = expf(2 * eps2);
  } else if (i < n + f->filter_radius) {
    int m = i - n;
    f->E3[m] = expf(-m * m / f->b);
  }
}

__global__ void k_compat_filter_f64(cuna2_filter_properties_f64 *f, const double *x, int ng, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    int u = compat_origin(x[i], ng, f->filter_radius);
    double eps = ng * x[i] - u;
    double eps2 = eps / f->b;
    f->E1[i] = exp(-eps * eps2) / sqrt(CUNA_PI * f->b);
    f->E2[i] = exp(2 * eps2);
  } else if (i < n + f->filter_radius) {
    int m = i - n;
    f->E3[m] = exp(-m * m / f->b);
  }
}

// ---------------------------------------------------------------------------
// deconvolution factor of normalize / normalize_bootstrap,
// src/gaussian_filter.cu:278-302
// ---------------------------------------------------------------------------
__device__ __forceinline__ float compat_fac(int k, int ng, float b, float normfac) {
  float K = ((float)k) / ((float)ng);
  return normfac * expf(K * K * b * 0.25);
}
__device__ __forceinline__ double compat_fac(int k, int ng, double b, double normfac) {
  double K = ((double)k) / ((double)ng);
  return normfac * exp(K * K * b * 0.25);
}

__device__ __forceinline__ float cpow(float a, int m) { return powf(a, m); }
__device__ __forceinline__ double cpow(double a, int m) { return pow(a, m); }

// Reference cell j = (int)((x + 0.5) * (ng - 1)) (double arithmetic,
// src/gridding.cu:43,93) and the tap bounds of :53-58.  Returns false when the
// tap range is empty.  |j| beyond 2^30 is treated as empty: the reference's
// int arithmetic overflows there and writes out of bounds.
__device__ __forceinline__ bool compat_taps(double xd, int ng, int rf, bool clamp, int &j, int &ms,
                                            int &me) {
  j = (int)((xd + 0.5) * (ng - 1));
  if (clamp) {
    if (j >= ng) j = ng - 1;
    if (j < 0) j = 0;
  }
  if (j > (1 << 30) || j < -(1 << 30)) return false;
  ms = -rf + 1;
  me = rf;
  if (j + ms < 0) ms = -j;
  if (j + me > ng) me = ng - j;
  return ms < me;
}

// ---------------------------------------------------------------------------
// samplers for the binning kernels
// ---------------------------------------------------------------------------
template <typename T> __device__ __forceinline__ void set_val(RecF &r, float v) { r.p = __float_as_int(v); }
template <typename T> __device__ __forceinline__ void set_val(RecD &r, double v) { r.v = v; }

template <typename T, bool BOOT> struct SampCompat {
  typedef typename RecOf<T>::type Rec;
  typedef typename FpOf<T>::type FP;
  struct Raw {
    T x, y, E1, E2;
  };
  const T *x;
  const T *y;
  const FP *fp;
  int64_t n;
  int ng;
  __device__ __forceinline__ Raw load(int64_t i, bool with_value) const {
    Raw r;
    r.x = x[i];
    if (!BOOT && with_value) {
      r.y = y ? y[i] : (T)1.0;
      r.E1 = fp->E1[i];
      r.E2 = fp->E2[i];
    }
    return r;
  }
  __device__ __forceinline__ void prep(int64_t i, const Raw &r, Prep<Rec> &p) const {
    int j, ms, me;
    p.nt = 0;
    if (!compat_taps((double)r.x, ng, fp->filter_radius, !BOOT, j, ms, me)) return;
    const int t0 = (j + ms) >> kCompatLogTL, t1 = (j + me - 1) >> kCompatLogTL;
    p.t[0] = t0;
    p.t[1] = t1;
    p.nt = t0 == t1 ? 1 : 2;
    p.rec.cell = j;
    if (BOOT) {
      p.rec.p = (int)i;
    } else {
      p.rec.a = r.E1;
      p.rec.b = r.E2;
      set_val<T>(p.rec, r.y);
    }
  }
};

__device__ __forceinline__ float rec_val(const RecF &r) { return __int_as_float(r.p); }
__device__ __forceinline__ double rec_val(const RecD &r) { return r.v; }

// ---------------------------------------------------------------------------
// tiled gridding: fast_gridding / fast_gridding_bootstrap,
// src/gridding.cu:36-65,86-117.  Every tap weight is the reference's own
// expression val * (E1 * pow(E2, m) * E3[|m|]) (filter(),
// src/gaussian_filter.cu:264-273); only the summation differs: instead of
// float atomics into f_hat (order-dependent) each CTA sums its tile in
// fixed point with native shared integer atomics and adds the tile to f_hat
// once.  The tile's scale comes from a bound on every cell's sum: |val| <=
// Ymax over the tile's records, a weight is at most 1 / sqrt(pi b), and at
// most 2 hmax records reach one cell (hmax: the most records in a bucket of
// >= 2 rf cells).  The quantum is 2^-30 (float) / 2^-62 (double) of that
// bound, and the sums no longer depend on the order of the atomics.
// ---------------------------------------------------------------------------
template <typename T, bool BOOT>
__device__ __forceinline__ void compat_coefs(const typename RecOf<T>::type &rc, const T *E1g, const T *E2g,
                                             const T *y, int n, unsigned seed, int slab, T &E1, T &E2, T &val) {
  if (BOOT) {
    const int i = slab * n + rc.p;
    int d = rc.p;
    val = (T)1.0;
    if (y) {
      d = (int)boot_draw(seed, (unsigned)i, (unsigned)n);
      val = y[d];
    }
    E1 = E1g[d];
    E2 = E2g[d];
  } else {
    E1 = rc.a;
    E2 = rc.b;
    val = rec_val(rc);
  }
}

constexpr int kCompatThreads = 256;

template <typename T, bool BOOT>
__global__ void __launch_bounds__(kCompatThreads) k_grid_compat(const typename RecOf<T>::type *__restrict__ recs,
                                                                const int *__restrict__ off,
                                                                typename CxOf<T>::type *f_hat, int ng,
                                                                const typename FpOf<T>::type *fp,
                                                                const T *__restrict__ y, int n, unsigned seed) {
  typedef typename RecOf<T>::type Rec;
  typedef FixAccWide<T> FA;
  typedef typename FA::type A;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  A *acc = reinterpret_cast<A *>(smem_raw);
  T *e3 = reinterpret_cast<T *>(acc + (1 << kCompatLogTL));
  int *hist = reinterpret_cast<int *>(e3 + kCompatMaxRf);
  __shared__ float red[kCompatThreads / 32];
  __shared__ int redi[kCompatThreads / 32];
  __shared__ T scale_s;
  const int tile = blockIdx.x, slab = blockIdx.y;
  const int base = tile << kCompatLogTL;
  const int tl = min(1 << kCompatLogTL, ng - base);
  const int rf = fp->filter_radius;
  const T *E3g = fp->E3, *E1g = fp->E1, *E2g = fp->E2;
  // buckets of >= 2 rf cells: the records reaching one cell lie in two buckets
  int logBS = 4;
  while ((1 << logBS) < 2 * rf) ++logBS;
  const int NB = ((tl + 2 * rf) >> logBS) + 1;
  for (int c = threadIdx.x; c < tl; c += kCompatThreads) acc[c] = 0;
  for (int m = threadIdx.x; m < rf && m < kCompatMaxRf; m += kCompatThreads) e3[m] = E3g[m];
  for (int q = threadIdx.x; q < NB; q += kCompatThreads) hist[q] = 0;
  __syncthreads();
  const int r0 = off[tile], r1 = off[tile + 1];
  // bound pass: records per bucket and the largest |value| (NaN if any is not finite)
  float ym = 0.f;
  for (int r = r0 + threadIdx.x; r < r1; r += kCompatThreads) {
    const Rec rc = recs[r];
    atomicAdd(&hist[(rc.cell - base + rf) >> logBS], 1);
    T E1, E2, val;
    compat_coefs<T, BOOT>(rc, E1g, E2g, y, n, seed, slab, E1, E2, val);
    ym = isfinite(val) && !isnan(ym) ? fmaxf(ym, (float)fabs(val)) : __int_as_float(0x7fffffff);
  }
  __syncthreads();
  int hmax = 0;
  for (int q = threadIdx.x; q < NB; q += kCompatThreads) hmax = max(hmax, hist[q]);
  for (int o = 16; o > 0; o >>= 1) {
    hmax = max(hmax, __shfl_xor_sync(0xffffffffu, hmax, o));
    const float u = __shfl_xor_sync(0xffffffffu, ym, o);
    ym = (isnan(u) || isnan(ym)) ? __int_as_float(0x7fffffff) : fmaxf(ym, u);
  }
  if ((threadIdx.x & 31) == 0) {
    redi[threadIdx.x >> 5] = hmax;
    red[threadIdx.x >> 5] = ym;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int h = 0;
    float v = 0.f;
    bool bad = false;
    for (int w = 0; w < kCompatThreads / 32; ++w) {
      h = max(h, redi[w]);
      bad |= isnan(red[w]);
      v = fmaxf(v, red[w]);
    }
    // a tap weight E1 E2^m E3[|m|] = exp(-(eps - m)^2 / b) / sqrt(pi b) is at
    // most 1 / sqrt(pi b); 1% margin for the approximate exp and pow
    const T wmax = (T)1.01 / sqrt((T)CUNA_PI * fp->b);
    const T B = (T)v * wmax * (T)(2 * h);
    T sc = B > (T)0 ? FA::range / B : (T)0;
    if (isinf(sc)) sc = (T)0;
    scale_s = bad ? (T)NAN : sc;
  }
  __syncthreads();
  const T sc = scale_s;
  if (sc > (T)0) {
    for (int r = r0 + threadIdx.x; r < r1; r += kCompatThreads) {
      const Rec rc = recs[r];
      const int j = rc.cell;
      int ms = -rf + 1, me = rf;
      if (j + ms < 0) ms = -j;
      if (j + me > ng) me = ng - j;
      T E1, E2, val;
      compat_coefs<T, BOOT>(rc, E1g, E2g, y, n, seed, slab, E1, E2, val);
      const int lo = max(ms, base - j), hi = min(me, base + tl - j);
      for (int m = lo; m < hi; ++m) {
        const int mp = m < 0 ? -m : m;
        const T e3m = mp < kCompatMaxRf ? e3[mp] : E3g[mp];
        const T w = val * (E1 * cpow(E2, m) * e3m);
        FA::add(&acc[j + m - base], FA::to_fix(w * sc));
      }
    }
  }
  __syncthreads();
  typename CxOf<T>::type *out = f_hat + (int64_t)slab * ng + base;
  if (isnan(sc)) {  // a non-finite value: the tile is NaN, as the float sums would spread it
    for (int c = threadIdx.x; c < tl; c += kCompatThreads) out[c].x += (T)NAN;
    return;
  }
  const T inv = sc > (T)0 ? (T)1 / sc : (T)0;
  for (int c = threadIdx.x; c < tl; c += kCompatThreads) {
    const A v = acc[c];
    if (v != 0) out[c].x += (T)v * inv;
  }
}

template <typename T> constexpr size_t compat_grid_smem() {
  // accumulators, E3 table, bucket counts (buckets of >= 16 cells)
  return sizeof(typename FixAcc<T>::type) * (1 << kCompatLogTL) + sizeof(T) * kCompatMaxRf +
         sizeof(int) * (((1 << kCompatLogTL) + 2 * kCompatMaxRf) / 16 + 1);
}

// ---------------------------------------------------------------------------
// FFT with the reference deconvolution fused in
// ---------------------------------------------------------------------------
template <typename T> struct FacDst {
  typename CxOf<T>::type *p;
  int ng, logL1, r0, norm;
  T b, nf;
  __device__ __forceinline__ void store(int seq, int k2, typename CxOf<T>::type v) const {
    const int k = r0 + seq + (k2 << logL1);
    p[k] = norm ? cscale(v, compat_fac(k, ng, b, nf)) : v;
  }
};
template <typename T> struct RowSrc {
  const typename CxOf<T>::type *p;
  int logL2;
  __device__ __forceinline__ typename CxOf<T>::type load(int seq, int i) const {
    return p[((int64_t)seq << logL2) + i];
  }
};

template <typename T>
__global__ void __launch_bounds__(sizeof(T) == 4 ? 1024 : 512) k_fft_single_compat(typename CxOf<T>::type *data, FftDev<T> f,
                                                            const typename FpOf<T>::type *fp, int norm) {
  typedef typename CxOf<T>::type C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *s = reinterpret_cast<C *>(smem_raw);
  const int L = 1 << f.logL;
  C *d = data + (int64_t)blockIdx.x * L;
  // in place: every read of d precedes the first barrier, every write follows it
  RowSrc<T> src{d, 0};
  FacDst<T> dst{d, L, 0, 0, norm, fp->b, fp->normfac};
  fft_fused<T, true, false, false>(s, 0, f.logL, 0, f.tw1, src, dst);
}

template <typename T>
__global__ void __launch_bounds__(sizeof(T) == 4 ? 512 : 256) k_fft_rowpass_compat(const typename CxOf<T>::type *in,
                                                            typename CxOf<T>::type *out, FftDev<T> f,
                                                            const typename FpOf<T>::type *fp,
                                                            int64_t slab_stride, int norm) {
  typedef typename CxOf<T>::type C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *s = reinterpret_cast<C *>(smem_raw);
  const int logB = ilog2i((int64_t)blockDim.x * kFftE) - f.logL2;
  const int B = 1 << logB;
  const int pitch = fft_pitch(1 << f.logL2, B);
  const int r0 = blockIdx.x * B;
  RowSrc<T> src{in + blockIdx.y * slab_stride + ((int64_t)r0 << f.logL2), f.logL2};
  FacDst<T> dst{out + blockIdx.y * slab_stride, 1 << f.logL, f.logL1, r0, norm, fp->b, fp->normfac};
  // rows are read point-fastest (contiguous), outputs written row-fastest
  fft_fused<T, true, false, true>(s, pitch, f.logL2, logB, f.tw2, src, dst);
}

// Compile-time four-step passes of the compat transform: column pass from
// f_hat into scratch (twiddled), row pass from scratch back into f_hat in
// natural order with the reference normalisation fused in.
template <typename T, int LOGL>
__global__ void __launch_bounds__(PassCfg<T>::THREADS) k_ct_colpass_oop(const typename CxOf<T>::type *in,
                                                                        typename CxOf<T>::type *out, FftDev<T> f,
                                                                        int64_t slab_stride) {
  ct_colpass_body<T, LOGL>(in + blockIdx.y * slab_stride, out + blockIdx.y * slab_stride, f, blockIdx.x);
}

template <typename T, int LOG2> struct CtRowSrc {
  const typename CxOf<T>::type *p;  // first row of the block
  __device__ __forceinline__ typename CxOf<T>::type load(int seq, int j, int dr) const {
    return p[(seq << LOG2) + j + dr];
  }
};

template <typename T, int LOG1> struct CtFacDst {
  typename CxOf<T>::type *p;  // slab
  int ng, r0, norm;
  T b, nf;
  template <int R, int LOGNS>
  __device__ __forceinline__ void store(int seq, int idxD, typename CxOf<T>::type *v) const {
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int k = r0 + seq + ((idxD + (r << LOGNS)) << LOG1);
      p[k] = norm ? cscale(v[r], compat_fac(k, ng, b, nf)) : v[r];
    }
  }
};

template <typename T, int LOGL>
__global__ void __launch_bounds__(PassCfg<T>::THREADS) k_ct_rowpass_compat(const typename CxOf<T>::type *in,
                                                                           typename CxOf<T>::type *out, FftDev<T> f,
                                                                           const typename FpOf<T>::type *fp,
                                                                           int64_t slab_stride, int norm) {
  typedef typename CxOf<T>::type C;
  constexpr int LOG1 = (LOGL + 1) / 2, LOG2 = LOGL / 2;
  constexpr int LOGB = ilog2c(PassCfg<T>::ELEMS) - LOG2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *s = reinterpret_cast<C *>(smem_raw);
  const int r0 = blockIdx.x << LOGB;
  CtRowSrc<T, LOG2> src{in + blockIdx.y * slab_stride + ((int64_t)r0 << LOG2)};
  CtFacDst<T, LOG1> dst{out + blockIdx.y * slab_stride, 1 << LOGL, r0, norm, fp->b, fp->normfac};
  // rows are read point-fastest (contiguous), outputs written row-fastest
  ct_fft<T, LOG2, LOGB, true, false, true>(s, f.tw2, src, dst);
}

template <typename T, int LOGL>
int compat_ct_at(typename CxOf<T>::type *f_hat, typename CxOf<T>::type *scratch, const FftDev<T> &f,
                 const typename FpOf<T>::type *dfp, int nbs, bool norm, cudaStream_t st) {
  constexpr int LOG1 = (LOGL + 1) / 2, LOG2 = LOGL / 2;
  constexpr int BA = PassCfg<T>::ELEMS >> LOG1, BB = PassCfg<T>::ELEMS >> LOG2;
  constexpr size_t smA = ct_colpass_smem<T, LOGL>();
  constexpr size_t smB = sizeof(typename CxOf<T>::type) * (size_t)fft_pitch(1 << LOG2, BB) * BB;
  static char attr;
  if (!setup_done(&attr)) {
    if (cudaFuncSetAttribute(k_ct_colpass_oop<T, LOGL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smA) ||
        cudaFuncSetAttribute(k_ct_rowpass_compat<T, LOGL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smB))
      return -1;
    mark_setup_done(&attr);
  }
  const int64_t L = (int64_t)1 << LOGL;
  k_ct_colpass_oop<T, LOGL><<<dim3((1 << LOG2) / BA, nbs), PassCfg<T>::THREADS, smA, st>>>(f_hat, scratch, f, L);
  if (cudaPeekAtLastError() != cudaSuccess) return -1;
  k_ct_rowpass_compat<T, LOGL><<<dim3((1 << LOG1) / BB, nbs), PassCfg<T>::THREADS, smB, st>>>(scratch, f_hat, f, dfp,
                                                                                            L, norm ? 1 : 0);
  if (cudaPeekAtLastError() != cudaSuccess) return -1;
  return 1;
}

// 1: launched, 0: no compiled instance, -1: launch error
template <typename T>
int compat_ct(int logL, typename CxOf<T>::type *f_hat, typename CxOf<T>::type *scratch, const FftDev<T> &f,
              const typename FpOf<T>::type *dfp, int nbs, bool norm, cudaStream_t st) {
#define CUNA_CCT(LG) \
  case LG: return compat_ct_at<T, LG>(f_hat, scratch, f, dfp, nbs, norm, st);
  if constexpr (sizeof(T) == 4) {
    switch (logL) { CUNA_CCT(15) CUNA_CCT(16) CUNA_CCT(17) CUNA_CCT(18) CUNA_CCT(19) CUNA_CCT(20) CUNA_CCT(21) CUNA_CCT(22) CUNA_CCT(23) CUNA_CCT(24) CUNA_CCT(25) }
  } else {
    switch (logL) { CUNA_CCT(14) CUNA_CCT(15) CUNA_CCT(16) CUNA_CCT(17) CUNA_CCT(18) CUNA_CCT(19) CUNA_CCT(20) CUNA_CCT(21) CUNA_CCT(22) CUNA_CCT(23) }
  }
#undef CUNA_CCT
  return 0;
}

template <typename T>
__global__ void k_compat_normalize(typename CxOf<T>::type *f_hat, int ng, int64_t total,
                                   const typename FpOf<T>::type *fp) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < total) f_hat[i] = cscale(f_hat[i], compat_fac((int)(i % ng), ng, fp->b, fp->normfac));
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
template <typename T> FftDev<T> to_dev(const FftGeom &g) {
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

size_t align_up(size_t v) { return (v + 255) & ~(size_t)255; }

// cuFFT comparator plans for non power-of-two grids, cached per
// (device, stream, ng, batch, precision).
std::mutex g_cufft_mu;
std::map<std::tuple<int, cudaStream_t, int, int, int>, cufftHandle> *g_cufft =
    new std::map<std::tuple<int, cudaStream_t, int, int, int>, cufftHandle>();

template <typename T>
int cufft_inverse(typename CxOf<T>::type *data, int ng, int nbs, cudaStream_t st) {
  int dev = 0;
  CUNA_CK(cudaGetDevice(&dev));
  cufftHandle h;
  {
    std::lock_guard<std::mutex> lk(g_cufft_mu);
    auto key = std::make_tuple(dev, st, ng, nbs, (int)sizeof(T));
    auto it = g_cufft->find(key);
    if (it == g_cufft->end()) {
      int dims[1] = {ng};
      cufftResult r = cufftPlanMany(&h, 1, dims, nullptr, 1, ng, nullptr, 1, ng,
                                    sizeof(T) == 4 ? CUFFT_C2C : CUFFT_Z2Z, nbs);
      if (r != CUFFT_SUCCESS) return fail(CUNA2_ERROR_CUFFT, "cufftPlanMany failed (%d)", (int)r);
      if ((r = cufftSetStream(h, st)) != CUFFT_SUCCESS)
        return fail(CUNA2_ERROR_CUFFT, "cufftSetStream failed (%d)", (int)r);
      (*g_cufft)[key] = h;
    } else {
      h = it->second;
    }
  }
  cufftResult r;
  if (sizeof(T) == 4)
    r = cufftExecC2C(h, (cufftComplex *)data, (cufftComplex *)data, CUFFT_INVERSE);
  else
    r = cufftExecZ2Z(h, (cufftDoubleComplex *)data, (cufftDoubleComplex *)data, CUFFT_INVERSE);
  if (r != CUFFT_SUCCESS) return fail(CUNA2_ERROR_CUFFT, "cufftExec failed (%d)", (int)r);
  return CUNA2_SUCCESS;
}

template <typename T>
int compat_normalize(typename CxOf<T>::type *f_hat, int ng, int nbs, const typename FpOf<T>::type *dfp,
                     cudaStream_t st) {
  const int64_t total = (int64_t)ng * nbs;
  if (total == 0) return CUNA2_SUCCESS;
  k_compat_normalize<T><<<(unsigned)((total + 255) / 256), 256, 0, st>>>(f_hat, ng, total, dfp);
  CUNA_CK(cudaGetLastError());
  return CUNA2_SUCCESS;
}

// In-place inverse FFT of nbs slabs of ng points; `norm` fuses the reference
// deconvolution into the last pass.
template <typename T>
int compat_fft(typename CxOf<T>::type *f_hat, int ng, int nbs, const typename FpOf<T>::type *dfp,
               typename CxOf<T>::type *scratch, bool norm, cudaStream_t st) {
  typedef typename CxOf<T>::type C;
  const bool pow2 = (ng & (ng - 1)) == 0;
  const int logL = ilog2i(ng);
  // four-step limit: the column pass holds at least one column of L1 points
  const int max_log = sizeof(T) == 4 ? 26 : 24;
  if (!pow2 || logL > max_log) {
    CUNA_TRY(cufft_inverse<T>(f_hat, ng, nbs, st));
    return norm ? compat_normalize<T>(f_hat, ng, nbs, dfp, st) : CUNA2_SUCCESS;
  }
  FftGeom g;
  CUNA_TRY(fft_geometry(sizeof(T) == 8, logL, &g));
  FftDev<T> f = to_dev<T>(g);
  if (g.single) {
    const int L = 1 << logL;
    const int threads = max(32, L / kFftE);
    const size_t smem = sizeof(C) * (size_t)fft_pitch(L, 1);
    static char attr;
    if (!setup_done(&attr)) {
      CUNA_CK(cudaFuncSetAttribute(k_fft_single_compat<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   200 * 1024));
      mark_setup_done(&attr);
    }
    k_fft_single_compat<T><<<nbs, threads, smem, st>>>(f_hat, f, dfp, norm ? 1 : 0);
    CUNA_CK(cudaGetLastError());
    return CUNA2_SUCCESS;
  }
  {
    const int h = compat_ct<T>(logL, f_hat, scratch, f, dfp, nbs, norm, st);
    if (h < 0) return fail_cuda(cudaGetLastError(), "FFT pass launch");
    if (h == 1) return CUNA2_SUCCESS;
  }
  const int elems = sizeof(T) == 4 ? kPassElemsF32 : kPassElemsF64;
  const int threads = elems / kFftE;
  const int L1 = 1 << g.logL1, L2 = 1 << g.logL2;
  const int BA = elems / L1, BB = elems / L2;
  const size_t smemA = sizeof(C) * (size_t)BA * fft_pitch(L1, BA);
  const size_t smemB = sizeof(C) * (size_t)BB * fft_pitch(L2, BB);
  static char attr2;
  if (!setup_done(&attr2)) {
    CUNA_CK(cudaFuncSetAttribute(k_fft_colpass<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    CUNA_CK(cudaFuncSetAttribute(k_fft_rowpass_compat<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 200 * 1024));
    mark_setup_done(&attr2);
  }
  const int64_t L = (int64_t)ng;
  k_fft_colpass<T><<<dim3(L2 / BA, nbs), threads, smemA, st>>>(f_hat, scratch, f, L);
  CUNA_CK(cudaGetLastError());
  k_fft_rowpass_compat<T><<<dim3(L1 / BB, nbs), threads, smemB, st>>>(scratch, f_hat, f, dfp, L,
                                                                      norm ? 1 : 0);
  CUNA_CK(cudaGetLastError());
  return CUNA2_SUCCESS;
}

struct CompatWs {
  int *counts, *offsets, *cursor;
  int *resv;  // reservation table of the two-launch binning (up to kScanFuseTiles tiles)
  void *recs;
  void *scratch;
};

// blocks of the reserved binning for n samples on ntiles tiles (0: not used)
inline int compat_resv_blocks(int n, int ntiles) {
  if (n <= 0 || ntiles > kScanFuseTiles) return 0;
  const int64_t span = resv_span(n, ntiles, device_sm_count());
  return (int)((n + span - 1) / span);
}

template <typename T>
int compat_workspace(int n, int ng, int nbs, bool need_fft, cudaStream_t st, CompatWs *cw) {
  typedef typename CxOf<T>::type C;
  typedef typename RecOf<T>::type Rec;
  const int ntiles = (ng + (1 << kCompatLogTL) - 1) >> kCompatLogTL;
  const bool pow2 = (ng & (ng - 1)) == 0;
  const bool fourstep = need_fft && pow2 && ilog2i(ng) > (sizeof(T) == 4 ? kSingleLogF32 : kSingleLogF64) &&
                        ilog2i(ng) <= (sizeof(T) == 4 ? 26 : 24);
  const size_t o_off = align_up(sizeof(int) * ntiles), o_cur = o_off + align_up(sizeof(int) * (ntiles + 1));
  const size_t o_rsv = o_cur + align_up(sizeof(int) * ntiles);
  const size_t o_rec = o_rsv + align_up(sizeof(int) * (size_t)compat_resv_blocks(n, ntiles) * ntiles);
  const size_t o_fft = o_rec + align_up(sizeof(Rec) * 2 * (size_t)(n > 0 ? n : 1));
  const size_t bytes = o_fft + (fourstep ? sizeof(C) * (size_t)ng * nbs : 0);
  void *ws = nullptr;
  CUNA_TRY(stream_workspace(st, bytes, &ws));
  char *w = (char *)ws;
  cw->counts = (int *)w;
  cw->offsets = (int *)(w + o_off);
  cw->cursor = (int *)(w + o_cur);
  cw->resv = (int *)(w + o_rsv);
  cw->recs = w + o_rec;
  cw->scratch = fourstep ? (void *)(w + o_fft) : nullptr;
  return CUNA2_SUCCESS;
}

int check_args(int n, int ng, int nbs, const void *x, const void *f_hat, const void *dfp) {
  if (n < 0 || ng < 1 || nbs < 1 || !f_hat || !dfp || (n > 0 && !x))
    return fail(CUNA2_ERROR_INVALID_VALUE, "invalid argument (n=%d ng=%d nbs=%d)", n, ng, nbs);
  if ((int64_t)n * nbs > INT_MAX || (int64_t)ng * nbs > ((int64_t)1 << 40))
    return fail(CUNA2_ERROR_UNSUPPORTED, "n*nbs exceeds the reference's int index range");
  if (nbs > 65535) return fail(CUNA2_ERROR_UNSUPPORTED, "more than 65535 resamples per call");
  return CUNA2_SUCCESS;
}

// Binning: the bucket sort of the samples into 4096-cell tiles (records
// in cw.recs, tile t's records at [cw.offsets[t], cw.offsets[t+1])).
template <typename T>
int compat_bin(const T *x, const T *y, int n, int ng, const typename FpOf<T>::type *dfp, bool boot,
               const CompatWs &cw, cudaStream_t st) {
  typedef typename RecOf<T>::type Rec;
  const int ntiles = (ng + (1 << kCompatLogTL) - 1) >> kCompatLogTL;
  Rec *recs = (Rec *)cw.recs;
  SampCompat<T, false> sp{x, y, dfp, n, ng};
  SampCompat<T, true> sb{x, y, dfp, n, ng};
  const int sms = device_sm_count();
  const size_t smc = ntiles <= kBinSmemTiles ? sizeof(int) * ntiles : 0;
  const int gcount = (int)std::min<int64_t>((n + 4095) / 4096, 4 * sms);
  const int gscat = (int)((n + 512 * kScatterItems - 1) / (512 * kScatterItems));
  CUNA_CK(cudaMemsetAsync(cw.counts, 0, sizeof(int) * ntiles, st));
  const int nrb = compat_resv_blocks(n, ntiles);
  if (nrb > 0) {
    // count + reserve, then scan + scatter without global atomics (binning.cuh)
    const int64_t span = resv_span(n, ntiles, device_sm_count());
    const size_t sms3 = sizeof(int) * (3 * (size_t)ntiles + 1);
    static char attr;
    if (!setup_done(&attr)) {
      const int mx = (int)(sizeof(int) * (3 * kScanFuseTiles + 1));
      CUNA_CK(cudaFuncSetAttribute(k_bin_scatter_resv<SampCompat<T, false>>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
      CUNA_CK(cudaFuncSetAttribute(k_bin_scatter_resv<SampCompat<T, true>>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
      mark_setup_done(&attr);
    }
    if (boot) {
      k_bin_count_resv<<<nrb, 512, sizeof(int) * ntiles, st>>>(sb, cw.counts, cw.resv, ntiles, span);
      CUNA_CK(cudaGetLastError());
      k_bin_scatter_resv<<<nrb, 512, sms3, st>>>(sb, cw.counts, cw.resv, cw.offsets, recs, ntiles, span);
    } else {
      k_bin_count_resv<<<nrb, 512, sizeof(int) * ntiles, st>>>(sp, cw.counts, cw.resv, ntiles, span);
      CUNA_CK(cudaGetLastError());
      k_bin_scatter_resv<<<nrb, 512, sms3, st>>>(sp, cw.counts, cw.resv, cw.offsets, recs, ntiles, span);
    }
    CUNA_CK(cudaGetLastError());
  } else {
    if (boot) k_bin_count<<<gcount, 512, smc, st>>>(sb, cw.counts, ntiles);
    else k_bin_count<<<gcount, 512, smc, st>>>(sp, cw.counts, ntiles);
    CUNA_CK(cudaGetLastError());
    k_scan_tiles<<<1, 1024, 0, st>>>(cw.counts, cw.offsets, cw.cursor, ntiles);
    CUNA_CK(cudaGetLastError());
    if (boot) k_bin_scatter<<<gscat, 512, 2 * smc, st>>>(sb, cw.offsets, cw.cursor, recs, ntiles);
    else k_bin_scatter<<<gscat, 512, 2 * smc, st>>>(sp, cw.offsets, cw.cursor, recs, ntiles);
    CUNA_CK(cudaGetLastError());
  }
  return CUNA2_SUCCESS;
}

// Gridding stage: binning + tiled gridding, accumulating into f_hat.
template <typename T>
int compat_grid(const T *x, const T *y, typename CxOf<T>::type *f_hat, int n, int ng, int nbs,
                const typename FpOf<T>::type *dfp, unsigned seed, bool boot, const CompatWs &cw,
                cudaStream_t st) {
  typedef typename RecOf<T>::type Rec;
  if (n == 0) return CUNA2_SUCCESS;
  const int ntiles = (ng + (1 << kCompatLogTL) - 1) >> kCompatLogTL;
  CUNA_TRY(compat_bin<T>(x, y, n, ng, dfp, boot, cw, st));
  Rec *recs = (Rec *)cw.recs;
  const size_t smg = compat_grid_smem<T>();
  if (boot)
    k_grid_compat<T, true><<<dim3(ntiles, nbs), 256, smg, st>>>(recs, cw.offsets, f_hat, ng, dfp, y, n, seed);
  else
    k_grid_compat<T, false><<<dim3(ntiles, 1), 256, smg, st>>>(recs, cw.offsets, f_hat, ng, dfp, y, n, seed);
  CUNA_CK(cudaGetLastError());
  return CUNA2_SUCCESS;
}

template <typename T>
int compat_run(const T *x, const T *y, typename CxOf<T>::type *f_hat, int n, int ng, int nbs,
               const typename FpOf<T>::type *dfp, unsigned seed, bool boot, cudaStream_t st) {
  typedef typename CxOf<T>::type C;
  clear_error();
  CUNA_TRY(check_args(n, ng, boot ? nbs : 1, x, f_hat, dfp));
  if (!boot) nbs = 1;
  CompatWs cw;
  CUNA_TRY(compat_workspace<T>(n, ng, nbs, true, st, &cw));
  CUNA_TRY(compat_grid<T>(x, y, f_hat, n, ng, nbs, dfp, seed, boot, cw, st));
  return compat_fft<T>(f_hat, ng, nbs, dfp, (C *)cw.scratch, true, st);
}

template <typename T, typename FP>
int compat_filter(const T *x, int n, int ng, FP *h, FP *d, cudaStream_t st) {
  clear_error();
  if (n < 1 || ng < 1 || !h || !d || !x)
    return fail(CUNA2_ERROR_INVALID_VALUE, "invalid argument (n=%d ng=%d)", n, ng);
  const int rf = sizeof(T) == 4 ? 6 : 12;  // FILTER_RADIUS, src/gaussian_filter.cu:29-33
  // host part of generate_pinned_filter_properties, src/gaussian_filter.cu:54-57
  T R = ((T)ng) / n;
  h->b = 2 * R / (2 * R - 1) * (rf / CUNA_PI);
  h->filter_radius = rf;
  h->normfac = sqrt(2 * CUNA_PI);
  CUNA_CK(cudaMemcpyAsync(d, h, sizeof(FP), cudaMemcpyHostToDevice, st));
  const int nb = (n + rf + 255) / 256;
  if (sizeof(T) == 4)
    k_compat_filter_f32<<<nb, 256, 0, st>>>((cuna2_filter_properties_f32 *)d, (const float *)x, ng, n);
  else
    k_compat_filter_f64<<<nb, 256, 0, st>>>((cuna2_filter_properties_f64 *)d, (const double *)x, ng, n);
  CUNA_CK(cudaGetLastError());
  return CUNA2_SUCCESS;
}

}  // namespace
}  // namespace cuna

using namespace cuna;

extern "C" int cuna2_compat_filter_radius(int is_double) { return is_double ? 12 : 6; }

extern "C" int cuna2_compat_filter_f32(const float *x, int n, int ng, cuna2_filter_properties_f32 *h,
                                       cuna2_filter_properties_f32 *d, cudaStream_t st) {
  return compat_filter<float>(x, n, ng, h, d, st);
}
extern "C" int cuna2_compat_filter_f64(const double *x, int n, int ng, cuna2_filter_properties_f64 *h,
                                       cuna2_filter_properties_f64 *d, cudaStream_t st) {
  return compat_filter<double>(x, n, ng, h, d, st);
}
extern "C" int cuna2_compat_adjoint_f32(const float *x, const float *y, float2 *f_hat, int n, int ng,
                                        const cuna2_filter_properties_f32 *d, cudaStream_t st) {
  return compat_run<float>(x, y, f_hat, n, ng, 1, d, 0u, false, st);
}
extern "C" int cuna2_compat_adjoint_f64(const double *x, const double *y, double2 *f_hat, int n, int ng,
                                        const cuna2_filter_properties_f64 *d, cudaStream_t st) {
  return compat_run<double>(x, y, f_hat, n, ng, 1, d, 0u, false, st);
}
extern "C" int cuna2_compat_bootstrap_f32(const float *x, const float *y, float2 *f_hat, int n, int ng,
                                          int nbs, const cuna2_filter_properties_f32 *d, unsigned seed,
                                          cudaStream_t st) {
  return compat_run<float>(x, y, f_hat, n, ng, nbs, d, seed, true, st);
}
extern "C" int cuna2_compat_bootstrap_f64(const double *x, const double *y, double2 *f_hat, int n, int ng,
                                          int nbs, const cuna2_filter_properties_f64 *d, unsigned seed,
                                          cudaStream_t st) {
  return compat_run<double>(x, y, f_hat, n, ng, nbs, d, seed, true, st);
}

extern "C" int cuna2_compat_grid_f32(const float *x, const float *y, float2 *f_hat, int n, int ng,
                                     const cuna2_filter_properties_f32 *d, cudaStream_t st) {
  clear_error();
  CUNA_TRY(check_args(n, ng, 1, x, f_hat, d));
  CompatWs cw;
  CUNA_TRY(compat_workspace<float>(n, ng, 1, false, st, &cw));
  return compat_grid<float>(x, y, f_hat, n, ng, 1, d, 0u, false, cw, st);
}
extern "C" int cuna2_compat_grid_f64(const double *x, const double *y, double2 *f_hat, int n, int ng,
                                     const cuna2_filter_properties_f64 *d, cudaStream_t st) {
  clear_error();
  CUNA_TRY(check_args(n, ng, 1, x, f_hat, d));
  CompatWs cw;
  CUNA_TRY(compat_workspace<double>(n, ng, 1, false, st, &cw));
  return compat_grid<double>(x, y, f_hat, n, ng, 1, d, 0u, false, cw, st);
}
extern "C" int cuna2_compat_fft_f32(float2 *f_hat, int ng, int nbatch, const cuna2_filter_properties_f32 *d,
                                    int normalize, cudaStream_t st) {
  clear_error();
  CUNA_TRY(check_args(0, ng, nbatch, nullptr, f_hat, d));
  CompatWs cw;
  CUNA_TRY(compat_workspace<float>(0, ng, nbatch, true, st, &cw));
  return compat_fft<float>(f_hat, ng, nbatch, d, (float2 *)cw.scratch, normalize != 0, st);
}
extern "C" int cuna2_compat_fft_f64(double2 *f_hat, int ng, int nbatch, const cuna2_filter_properties_f64 *d,
                                    int normalize, cudaStream_t st) {
  clear_error();
  CUNA_TRY(check_args(0, ng, nbatch, nullptr, f_hat, d));
  CompatWs cw;
  CUNA_TRY(compat_workspace<double>(0, ng, nbatch, true, st, &cw));
  return compat_fft<double>(f_hat, ng, nbatch, d, (double2 *)cw.scratch, normalize != 0, st);
}
extern "C" int cuna2_compat_normalize_f32(float2 *f_hat, int ng, int nbatch,
                                          const cuna2_filter_properties_f32 *d, cudaStream_t st) {
  clear_error();
  CUNA_TRY(check_args(0, ng, nbatch, nullptr, f_hat, d));
  return compat_normalize<float>(f_hat, ng, nbatch, d, st);
}
extern "C" int cuna2_compat_normalize_f64(double2 *f_hat, int ng, int nbatch,
                                          const cuna2_filter_properties_f64 *d, cudaStream_t st) {
  clear_error();
  CUNA_TRY(check_args(0, ng, nbatch, nullptr, f_hat, d));
  return compat_normalize<double>(f_hat, ng, nbatch, d, st);
}

// ---------------------------------------------------------------------------
// Integer steps read back: per sample the cell j, the filter origin u and the
// tap range, the bootstrap draws, and the records of the binning, computed by
// the same device functions the transforms run (compat_taps, compat_origin,
// boot_draw, compat_bin).  Tests compare them with the oracle bit for bit;
// the transforms never call these.
// ---------------------------------------------------------------------------
namespace cuna {
namespace {

template <typename T>
__global__ void k_inspect_compat_taps(const T *x, int n, int ng, int rf, int clamp, int *cell, int *origin,
                                      int *tlo, int *thi) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const T xi = x[i];
  int j = 0, ms = 0, me = 0;
  const bool any = compat_taps((double)xi, ng, rf, clamp != 0, j, ms, me);
  if (cell) cell[i] = j;
  if (origin) origin[i] = compat_origin(xi, ng, rf);
  if (tlo) tlo[i] = any ? ms : 0;
  if (thi) thi[i] = any ? me : 0;
}

__global__ void k_inspect_draws(unsigned n, int64_t total, unsigned seed, int *d) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x)
    d[i] = (int)boot_draw(seed, (unsigned)i, n);
}

template <typename T>
int inspect_compat_taps(const T *x, int n, int ng, int clamp, int *cell, int *origin, int *tlo, int *thi,
                        cudaStream_t st) {
  clear_error();
  if (n < 0 || ng < 1 || (n > 0 && !x))
    return fail(CUNA2_ERROR_INVALID_VALUE, "invalid argument (n=%d ng=%d)", n, ng);
  if (n == 0) return CUNA2_SUCCESS;
  const int rf = sizeof(T) == 4 ? 6 : 12;
  k_inspect_compat_taps<T><<<(n + 255) / 256, 256, 0, st>>>(x, n, ng, rf, clamp, cell, origin, tlo, thi);
  CUNA_CK(cudaGetLastError());
  return CUNA2_SUCCESS;
}

template <typename T>
int inspect_compat_bins(const T *x, const T *y, int n, int ng, const typename FpOf<T>::type *dfp, int boot,
                        int *offsets, void *records, int max_records, int *nrecords, cudaStream_t st) {
  typedef typename RecOf<T>::type Rec;
  clear_error();
  CUNA_TRY(check_args(n, ng, 1, x, offsets, dfp));
  if (max_records < 0 || (max_records > 0 && !records))
    return fail(CUNA2_ERROR_INVALID_VALUE, "invalid record buffer (max_records=%d)", max_records);
  const int ntiles = (ng + (1 << kCompatLogTL) - 1) >> kCompatLogTL;
  int total = 0;
  if (n == 0) {
    CUNA_CK(cudaMemsetAsync(offsets, 0, sizeof(int) * (ntiles + 1), st));
  } else {
    CompatWs cw;
    CUNA_TRY(compat_workspace<T>(n, ng, 1, false, st, &cw));
    CUNA_TRY(compat_bin<T>(x, y, n, ng, dfp, boot != 0, cw, st));
    CUNA_CK(cudaMemcpyAsync(offsets, cw.offsets, sizeof(int) * (ntiles + 1), cudaMemcpyDeviceToDevice, st));
    CUNA_CK(cudaMemcpyAsync(&total, cw.offsets + ntiles, sizeof(int), cudaMemcpyDeviceToHost, st));
    CUNA_CK(cudaStreamSynchronize(st));
    if (total > max_records) {
      if (nrecords) *nrecords = total;
      return fail(CUNA2_ERROR_INVALID_VALUE, "%d records do not fit in max_records = %d", total, max_records);
    }
    if (total > 0)
      CUNA_CK(cudaMemcpyAsync(records, cw.recs, sizeof(Rec) * (size_t)total, cudaMemcpyDeviceToDevice, st));
  }
  if (nrecords) *nrecords = total;
  return CUNA2_SUCCESS;
}

}  // namespace
}  // namespace cuna

extern "C" int cuna2_inspect_compat_taps_f32(const float *x, int n, int ng, int clamp, int *cell, int *origin,
                                             int *tap_lo, int *tap_hi, cudaStream_t st) {
  return inspect_compat_taps<float>(x, n, ng, clamp, cell, origin, tap_lo, tap_hi, st);
}
extern "C" int cuna2_inspect_compat_taps_f64(const double *x, int n, int ng, int clamp, int *cell, int *origin,
                                             int *tap_lo, int *tap_hi, cudaStream_t st) {
  return inspect_compat_taps<double>(x, n, ng, clamp, cell, origin, tap_lo, tap_hi, st);
}
extern "C" int cuna2_inspect_bootstrap_draws(int n, int nbs, unsigned int seed, int *draw, cudaStream_t st) {
  clear_error();
  if (n < 1 || nbs < 1 || !draw || (int64_t)n * nbs > INT_MAX)
    return fail(CUNA2_ERROR_INVALID_VALUE, "invalid argument (n=%d nbs=%d)", n, nbs);
  const int64_t total = (int64_t)n * nbs;
  const int blocks = (int)std::min<int64_t>((total + 255) / 256, 8192);
  k_inspect_draws<<<blocks, 256, 0, st>>>((unsigned)n, total, seed, draw);
  CUNA_CK(cudaGetLastError());
  return CUNA2_SUCCESS;
}
extern "C" int cuna2_inspect_compat_bins_f32(const float *x, const float *y, int n, int ng,
                                             const cuna2_filter_properties_f32 *d, int boot, int *offsets,
                                             void *records, int max_records, int *nrecords, cudaStream_t st) {
  return inspect_compat_bins<float>(x, y, n, ng, d, boot, offsets, records, max_records, nrecords, st);
}
extern "C" int cuna2_inspect_compat_bins_f64(const double *x, const double *y, int n, int ng,
                                             const cuna2_filter_properties_f64 *d, int boot, int *offsets,
                                             void *records, int max_records, int *nrecords, cudaStream_t st) {
  return inspect_compat_bins<double>(x, y, n, ng, d, boot, offsets, records, max_records, nrecords, st);
}

// ---------------------------------------------------------------------------
// cuna2_compat_adjoint_noalloc_f32: cuna2_compat_adjoint_f32 for callers that
// cannot allocate device memory.
//
// Everything the transform needs beyond the caller's x, y, f_hat and filter
// lives in one statically sized device array that the library carries (every
// GPU that loads the library holds it until the process exits): the tile
// counters, the sorted sample records, the FFT scratch slab and the twiddle
// tables.  The entry point therefore never calls cudaMalloc / cudaFree or
// cuFFT.  Limits: n <= kNoAllocMaxN samples and a power-of-two grid of at
// most 2^kNoAllocMaxLogNg cells.
//
// The first call on a device sets that device up: it looks up the array's
// device address with cudaGetSymbolAddress (host code may not use the symbol
// itself as a pointer), fills the twiddle tables with a kernel and
// synchronises the caller's stream.  Make that first call before any stream
// capture.  All calls share the one array, which keeps the previous call's
// contents; the tile counters are cleared at the start of every call.  Calls
// that overlap on the GPU (different streams, or different host threads)
// race on the array: serialise them.
// ---------------------------------------------------------------------------
namespace cuna {
namespace {
constexpr int kNoAllocMaxN = 131072;
constexpr int kNoAllocMaxLogNg = 17;
constexpr size_t kNoAllocOffCounts = 0, kNoAllocOffOffsets = 256, kNoAllocOffCursor = 512;
constexpr size_t kNoAllocOffRecs = 1024;
constexpr size_t kNoAllocOffFft = kNoAllocOffRecs + sizeof(RecF) * 2 * (size_t)kNoAllocMaxN;
constexpr size_t kNoAllocOffTw = kNoAllocOffFft + sizeof(float2) * ((size_t)1 << kNoAllocMaxLogNg);
constexpr size_t kNoAllocTwEntries = 48 * 1024;  // all tables for logL = 0..17 (about 41K entries)
constexpr size_t kNoAllocBytes = kNoAllocOffTw + sizeof(float2) * kNoAllocTwEntries;
constexpr int kNoAllocMaxDevices = 64;
}  // namespace
}  // namespace cuna

static __device__ __align__(256) unsigned char cuna_noalloc_scratch[cuna::kNoAllocBytes];

namespace cuna {
namespace {

// exp(+2 pi i (q * step mod denom) / denom) for q < count, evaluated in double
__global__ void k_noalloc_twiddles(float2 *dst, int count, int step, int denom) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < count) {
    const long long num = ((long long)q * step) % denom;
    double s, c;
    sincospi(2.0 * (double)num / (double)denom, &s, &c);
    dst[q] = make_float2((float)c, (float)s);
  }
}

struct NoAllocDev {
  bool ready = false;
  unsigned char *base = nullptr;
  int sms = 1;
  FftDev<float> tab[kNoAllocMaxLogNg + 1];
};
std::mutex g_noalloc_mu;
NoAllocDev g_noalloc[kNoAllocMaxDevices];

int noalloc_table(float2 *tw, size_t &used, int count, int step, int denom, const float2 **out,
                  cudaStream_t st) {
  if (used + (size_t)count > kNoAllocTwEntries) return fail(CUNA2_ERROR_UNSUPPORTED, "twiddle region too small");
  float2 *dst = tw + used;
  k_noalloc_twiddles<<<(count + 255) / 256, 256, 0, st>>>(dst, count, step, denom);
  CUNA_CK(cudaGetLastError());
  used += (size_t)count;
  *out = dst;
  return CUNA2_SUCCESS;
}

// Once per device: device address of the array, twiddle tables, SM count.
int noalloc_setup(int dev, cudaStream_t st, NoAllocDev **out) {
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  NoAllocDev &d = g_noalloc[dev];
  if (!d.ready) {
    // set-up launches kernels and synchronises the stream, which a stream
    // capture cannot contain: refuse before touching anything
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    CUNA_CK(cudaStreamIsCapturing(st, &cs));
    if (cs != cudaStreamCaptureStatusNone)
      return fail(CUNA2_ERROR_UNSUPPORTED,
                  "no-allocation entry point: the first call on a device sets it up and must come before any "
                  "stream capture");
    void *p = nullptr;
    CUNA_CK(cudaGetSymbolAddress(&p, cuna_noalloc_scratch));
    d.base = (unsigned char *)p;
    CUNA_CK(cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev));
    float2 *tw = (float2 *)(d.base + kNoAllocOffTw);
    size_t used = 0;
    for (int logL = 0; logL <= kNoAllocMaxLogNg; ++logL) {
      FftDev<float> &f = d.tab[logL];
      const int L = 1 << logL;
      f.logL = logL;
      if (logL <= kSingleLogF32) {
        f.logL1 = logL;
        f.logL2 = 0;
      } else {
        f.logL1 = (logL + 1) / 2;
        f.logL2 = logL / 2;
      }
      const int L1 = 1 << f.logL1, L2 = 1 << f.logL2, nlo = L < 2048 ? L : 2048;
      CUNA_TRY(noalloc_table(tw, used, L1, 1, L1, &f.tw1, st));
      CUNA_TRY(noalloc_table(tw, used, L2, 1, L2, &f.tw2, st));
      if (logL > kSingleLogF32) {
        CUNA_TRY(noalloc_table(tw, used, nlo, 1, L, &f.twlo, st));
        CUNA_TRY(noalloc_table(tw, used, L / nlo, nlo, L, &f.twhi, st));
      } else {  // single-CTA lengths read tw1 only
        f.twlo = nullptr;
        f.twhi = nullptr;
      }
    }
    CUNA_CK(cudaFuncSetAttribute(k_fft_single_compat<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 200 * 1024));
    CUNA_CK(cudaFuncSetAttribute(k_fft_colpass<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    CUNA_CK(cudaFuncSetAttribute(k_fft_rowpass_compat<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 200 * 1024));
    CUNA_CK(cudaStreamSynchronize(st));
    d.ready = true;
  }
  *out = &d;
  return CUNA2_SUCCESS;
}

int compat_adjoint_noalloc(const float *x, const float *y, float2 *f_hat, int n, int ng,
                           const cuna2_filter_properties_f32 *dfp, cudaStream_t st) {
  clear_error();
  CUNA_TRY(check_args(n, ng, 1, x, f_hat, dfp));
  if (n > kNoAllocMaxN)
    return fail(CUNA2_ERROR_UNSUPPORTED, "no-allocation entry point: n = %d exceeds its maximum of %d samples",
                n, kNoAllocMaxN);
  if ((ng & (ng - 1)) != 0 || ilog2i(ng) > kNoAllocMaxLogNg)
    return fail(CUNA2_ERROR_UNSUPPORTED,
                "no-allocation entry point: ng = %d must be a power of two of at most %d", ng,
                1 << kNoAllocMaxLogNg);
  int dev = 0;
  CUNA_CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNoAllocMaxDevices) return fail(CUNA2_ERROR_UNSUPPORTED, "device index %d", dev);
  NoAllocDev *d = nullptr;
  CUNA_TRY(noalloc_setup(dev, st, &d));
  int *counts = (int *)(d->base + kNoAllocOffCounts);
  int *offsets = (int *)(d->base + kNoAllocOffOffsets);
  int *cursor = (int *)(d->base + kNoAllocOffCursor);
  RecF *recs = (RecF *)(d->base + kNoAllocOffRecs);
  float2 *scratch = (float2 *)(d->base + kNoAllocOffFft);
  const int ntiles = (ng + (1 << kCompatLogTL) - 1) >> kCompatLogTL;
  // the counters must start at zero; the rest is fully rewritten below
  CUNA_CK(cudaMemsetAsync(counts, 0, sizeof(int) * ntiles, st));
  if (n > 0) {
    SampCompat<float, false> sp{x, y, dfp, n, ng};
    const size_t smc = sizeof(int) * ntiles;
    const int gcount = (int)std::min<int64_t>((n + 4095) / 4096, 4 * d->sms);
    const int gscat = (int)((n + 512 * kScatterItems - 1) / (512 * kScatterItems));
    k_bin_count<<<gcount, 512, smc, st>>>(sp, counts, ntiles);
    CUNA_CK(cudaGetLastError());
    k_scan_tiles<<<1, 1024, 0, st>>>(counts, offsets, cursor, ntiles);
    CUNA_CK(cudaGetLastError());
    k_bin_scatter<<<gscat, 512, 2 * smc, st>>>(sp, offsets, cursor, recs, ntiles);
    CUNA_CK(cudaGetLastError());
    const size_t smg = compat_grid_smem<float>();
    k_grid_compat<float, false><<<dim3(ntiles, 1), 256, smg, st>>>(recs, offsets, f_hat, ng, dfp, y, n, 0u);
    CUNA_CK(cudaGetLastError());
  }
  const int logL = ilog2i(ng);
  const FftDev<float> &f = d->tab[logL];
  if (logL <= kSingleLogF32) {
    const int threads = std::max(32, ng / kFftE);
    const size_t smem = sizeof(float2) * (size_t)fft_pitch(ng, 1);
    k_fft_single_compat<float><<<1, threads, smem, st>>>(f_hat, f, dfp, 1);
    CUNA_CK(cudaGetLastError());
    return CUNA2_SUCCESS;
  }
  const int threads = kPassElemsF32 / kFftE;
  const int L1 = 1 << f.logL1, L2 = 1 << f.logL2;
  const int BA = kPassElemsF32 / L1, BB = kPassElemsF32 / L2;
  const size_t smemA = sizeof(float2) * (size_t)BA * fft_pitch(L1, BA);
  const size_t smemB = sizeof(float2) * (size_t)BB * fft_pitch(L2, BB);
  k_fft_colpass<float><<<dim3(L2 / BA, 1), threads, smemA, st>>>(f_hat, scratch, f, (int64_t)ng);
  CUNA_CK(cudaGetLastError());
  k_fft_rowpass_compat<float><<<dim3(L1 / BB, 1), threads, smemB, st>>>(scratch, f_hat, f, dfp, (int64_t)ng, 1);
  CUNA_CK(cudaGetLastError());
  return CUNA2_SUCCESS;
}

}  // namespace
}  // namespace cuna

extern "C" int cuna2_compat_adjoint_noalloc_f32(const float *x, const float *y, float2 *f_hat, int n, int ng,
                                                const cuna2_filter_properties_f32 *d, cudaStream_t st) {
  return compat_adjoint_noalloc(x, y, f_hat, n, ng, d, st);
}
