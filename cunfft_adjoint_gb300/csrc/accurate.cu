// accurate.cu -- accurate-mode adjoint NFFT (cuna2_plan_* / cuna2_adjoint).
//
//   F_k = sum_j y_j exp(+2 pi i k x_j),  x_j = (t_j - t0)/T - 1/2,
//   k = -nf/2 .. nf/2-1 stored at F[k + nf/2].
//
// Math: Gaussian gridding on a periodic grid of ng = R nf cells with kernel
// psi(d) = exp(-d^2 / (4 tau)), tau = m R / (4 pi (R - 1/2)) (Greengard & Lee
// 2004), taps d = -m+1..m around floor(s_j), s_j = (x_j + 1/2) ng.  The grid is
// real, so it is transformed as ng/2 packed complex points and unpacked in the
// last FFT pass, where the deconvolution 1/psi_hat(k), the (-1)^k phase of the
// x + 1/2 origin shift, output selection |k| <= nf/2 and Hermitian completion
// are fused in.
//
// Precision: s_j is reduced in 64-bit fixed point (phase.cuh); gridding, FFT
// and epilogue run in the plan's type.  Float plans use the fast Gaussian
// gridding factorisation y E1 E2^d E3[d] (E2^d by repeated multiplication).
//
// Kernels:
//   k_nfft_small<T>      ng <= 2^15 (f32) / 2^14 (f64): one CTA per transform,
//                        gridding straight into shared memory (no sort), FFT,
//                        epilogue -- a single launch.
//   binning (binning.cuh) + k_grid_acc + k_fft_colpass + k_fft_rowpass_acc for
//                        larger grids.
#include <math.h>
#include <algorithm>
#include <mutex>
#include <vector>
#include "binning.cuh"
#include "fft.cuh"
#include "phase.cuh"
#include "runtime.h"

namespace cuna {
namespace {

constexpr double kPi = 3.14159265358979323846;

__device__ __forceinline__ void sincospi_t(float a, float *s, float *c) { sincospif(a, s, c); }
__device__ __forceinline__ void sincospi_t(double a, double *s, double *c) { sincospi(a, s, c); }
__device__ __forceinline__ float exp_t(float a) { return expf(a); }
__device__ __forceinline__ double exp_t(double a) { return exp(a); }
__device__ __forceinline__ float exp2_t(float a) { return exp2f(a); }
__device__ __forceinline__ double exp2_t(double a) { return exp2(a); }

// Everything a kernel needs about the Gaussian and the output.
template <typename T> struct AccParams {
  int64_t ng, nf, K;  // K = nf / 2
  int m, logTL, ntiles;
  T k1, k2;           // E1 = 2^(-k1 f^2), E2 = 2^(k2 f)   (f = fractional cell)
  T e3c;              // E3[d] = exp(e3c d^2)
  T c0, c1;           // 0.5 / psi_hat(k) = c0 exp(c1 k^2)
  T twk;              // 2 / ng  (unpack twiddle angle / pi)
};

// fractional cell from the low word of S*ng
__device__ __forceinline__ float frac_of(uint64_t lo, float) { return (float)(lo >> 40) * 5.9604644775390625e-08f; }
__device__ __forceinline__ double frac_of(uint64_t lo, double) {
  return (double)(lo >> 11) * 1.1102230246251565e-16;
}

template <typename T>
__device__ __forceinline__ void reduce_sample(double t, const PhaseMul &pm, int64_t ng, int &cell, T &f) {
  const uint64_t S = phase_of(t, pm);
  if ((ng & (ng - 1)) == 0) {  // ng = 2^g: the top g bits are the cell
    const int g = 63 - __clzll((long long)ng);
    cell = g ? (int)(S >> (64 - g)) : 0;
    f = frac_of(S << g, (T)0);
  } else {
    cell = (int)umulhi64(S, (uint64_t)ng);
    f = frac_of(S * (uint64_t)ng, (T)0);
  }
}

// ---------------------------------------------------------------------------
// epilogue: real unpack + deconvolution + centring, one output k in [0, K]
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void acc_output(const AccParams<T> &e, int64_t k, typename CxOf<T>::type Zk,
                                           typename CxOf<T>::type Zmc, typename CxOf<T>::type *F) {
  typedef typename CxOf<T>::type C;
  const C A = cadd(Zk, Zmc);
  const C Bv = cmuli(csub(Zmc, Zk));
  T sn, cs;
  sincospi_t((T)k * e.twk, &sn, &cs);
  const C G2 = cadd(A, cmul(cmk(cs, sn), Bv));
  const T kf = (T)k;
  T sc = e.c0 * exp_t(e.c1 * kf * kf);
  if (k & 1) sc = -sc;
  const C Fk = cscale(G2, sc);
  if (k < e.K) F[e.K + k] = Fk;
  if (k >= 1) F[e.K - k] = cconj(Fk);
}

// ---------------------------------------------------------------------------
// single-CTA transform for small grids
// ---------------------------------------------------------------------------
__device__ __forceinline__ int real_slot(int c) { return 2 * pad16(c >> 1) + (c & 1); }

template <typename T>
__global__ void __launch_bounds__(sizeof(T) == 4 ? 1024 : 512) k_nfft_small(const double *__restrict__ t, const T *__restrict__ y,
                                                     int64_t n, PhaseMul pm, AccParams<T> e, FftDev<T> f,
                                                     typename CxOf<T>::type *F) {
  typedef typename CxOf<T>::type C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int L = 1 << f.logL;
  const int pitch = fft_pitch(L, 1);
  C *s = reinterpret_cast<C *>(smem_raw);
  T *sr = reinterpret_cast<T *>(smem_raw);
  T *e3 = reinterpret_cast<T *>(s + pitch);
  const int m = e.m, ng = (int)e.ng;
  for (int i = threadIdx.x; i < 2 * pitch; i += blockDim.x) sr[i] = (T)0;
  for (int d = threadIdx.x; d <= 2 * m; d += blockDim.x) e3[d] = exp_t(e.e3c * (T)((d - m) * (d - m)));
  __syncthreads();
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    int cell;
    T fr;
    reduce_sample<T>(t[i], pm, e.ng, cell, fr);
    const T E1 = exp2_t(-e.k1 * fr * fr), E2 = exp2_t(e.k2 * fr);
    const T w0 = y[i] * E1;
    T w = w0;
    for (int d = 0; d <= m; ++d) {
      int c = cell + d;
      if (c >= ng) c -= ng;
      atomicAdd(&sr[real_slot(c)], w * e3[d + m]);
      w *= E2;
    }
    const T E2i = (T)1 / E2;
    w = w0 * E2i;
    for (int d = -1; d > -m; --d) {
      int c = cell + d;
      if (c < 0) c += ng;
      atomicAdd(&sr[real_slot(c)], w * e3[d + m]);
      w *= E2i;
    }
  }
  __syncthreads();
  smem_fft<T>(s, pitch, f.logL, 1, f.tw1);
  for (int64_t k = threadIdx.x; k <= e.K; k += blockDim.x) {
    const C Zk = s[pad16((int)(k & (L - 1)))];
    const C Zm = cconj(s[pad16((int)((L - k) & (L - 1)))]);
    acc_output<T>(e, k, Zk, Zm, F);
  }
}

// ---------------------------------------------------------------------------
// binning sampler, tiled gridding, last FFT pass
// ---------------------------------------------------------------------------
// Sorted sample record of accurate mode: {cell, fractional cell, value}.
__device__ __forceinline__ void rec_set(RecF &r, int cell, float fr, float y) {
  r.cell = cell; r.a = fr; r.b = y; r.p = 0;
}
__device__ __forceinline__ void rec_set(RecD &r, int cell, double fr, double y) {
  r.cell = cell; r.p = 0; r.a = fr; r.b = y; r.v = 0.0;
}

template <typename T> struct SampAcc {
  typedef typename RecOf<T>::type Rec;
  struct Raw {
    double t;
    T y;
  };
  const double *t;
  const T *y;
  int64_t n;
  PhaseMul pm;
  AccParams<T> e;
  __device__ __forceinline__ Raw load(int64_t i, bool with_value) const {
    Raw r;
    r.t = t[i];
    if (with_value) r.y = y[i];
    return r;
  }
  __device__ __forceinline__ void prep(int64_t i, const Raw &r, Prep<Rec> &p) const {
    int cell;
    T fr;
    reduce_sample<T>(r.t, pm, e.ng, cell, fr);
    const int ng = (int)e.ng;
    int lo = cell - e.m + 1, hi = cell + e.m;
    if (lo < 0) lo += ng;
    if (hi >= ng) hi -= ng;
    const int t0 = lo >> e.logTL, t1 = hi >> e.logTL;
    p.t[0] = t0;
    p.t[1] = t1;
    p.nt = t0 == t1 ? 1 : 2;
    rec_set(p.rec, cell, fr, r.y);
  }
};

// ---------------------------------------------------------------------------
// Gridding, gather form.  One CTA owns tile [base, base + TL) of the grid and
// the records binned to it (its own samples plus the halo samples within m
// cells of its edges).  Per chunk of at most CAP records it counting-sorts
// them in shared memory by local slot lc = cell - base + m (integer atomics
// only), then every thread sums, for each of its cells c, the samples whose
// slot lies in [c - base, c - base + 2m): w = y exp(-(d - f)^2 / (4 tau)),
// d = c - cell.  Partial sums stay in registers across chunks and are written
// once, coalesced.  No floating-point atomics.
// ---------------------------------------------------------------------------
template <typename T> struct GridCfg;
template <> struct GridCfg<float> { static constexpr int CAP = 1024; };
template <> struct GridCfg<double> { static constexpr int CAP = 512; };
constexpr int kGridThreads = 256;
constexpr int kGridMaxCpt = 16;  // cells per thread: TL <= 4096

// 2^x with the hardware approximation (relative error < 2^-22 over the range
// used here; arguments are <= 0 and results below 2^-126 flush to zero, far
// beneath the 1e-6 accuracy of the float path).
__device__ __forceinline__ float ex2_fast(float x) {
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float gauss_w(float y, float dd, float k1) { return y * ex2_fast(-k1 * dd * dd); }
__device__ __forceinline__ double gauss_w(double y, double dd, double k1) { return y * exp2(-k1 * dd * dd); }

template <typename T> struct Pair;
template <> struct Pair<float> { typedef float2 type; };
template <> struct Pair<double> { typedef double2 type; };

template <typename T>
__global__ void __launch_bounds__(kGridThreads, sizeof(T) == 4 ? 4 : 2) k_grid_acc(const typename RecOf<T>::type *__restrict__ recs,
                                                           const int *__restrict__ off, T *__restrict__ grid,
                                                           AccParams<T> e) {
  typedef typename RecOf<T>::type Rec;
  constexpr int CAP = GridCfg<T>::CAP;
  constexpr int RPT = CAP / kGridThreads;  // records per thread per chunk
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int TL = 1 << e.logTL, m = e.m, W = TL + 2 * m;
  const int ng = (int)e.ng;
  typedef typename Pair<T>::type P2;
  int *start = reinterpret_cast<int *>(smem_raw);                 // W + 1 slots
  P2 *sfy = reinterpret_cast<P2 *>(smem_raw + sizeof(int) * ((W + 2 + 3) & ~3));  // (frac, y)
  short *slc = reinterpret_cast<short *>(sfy + CAP);
  // a single tile spanning the whole grid maps a record to up to two slots;
  // halve the chunk then so that placements never exceed CAP
  const int chunk = (TL + 2 * m > ng) ? CAP / 2 : CAP;
  __shared__ int wsum[kGridThreads / 32];
  const int tile = blockIdx.x, base = tile << e.logTL;
  const int cpt = (TL + kGridThreads - 1) / kGridThreads;
  T acc[kGridMaxCpt];
#pragma unroll
  for (int q = 0; q < kGridMaxCpt; ++q) acc[q] = (T)0;
  const int r0 = off[tile], r1 = off[tile + 1];
  for (int c0 = r0; c0 < r1; c0 += chunk) {
    const int cnt = min(chunk, r1 - c0);
    for (int i = threadIdx.x; i <= W; i += kGridThreads) start[i] = 0;
    __syncthreads();
    // load this thread's records; each maps to up to two slots (two only when
    // the tile wraps onto itself, i.e. a single tile spans the whole grid)
    Rec rc[RPT];
    int sl[RPT][2];
#pragma unroll
    for (int u = 0; u < RPT; ++u) {
      const int i = threadIdx.x + u * kGridThreads;
      if (i < cnt) rc[u] = recs[c0 + i];
    }
#pragma unroll
    for (int u = 0; u < RPT; ++u) {
      const int i = threadIdx.x + u * kGridThreads;
      sl[u][0] = sl[u][1] = -1;
      if (i < cnt) {
        int p0 = rc[u].cell - base;
        if (p0 < 0) p0 += ng;
        // slots p + m for every p = p0 + j*ng in [-m, TL + m), j in {-1, 0, 1}
        const int a = p0 - ng >= -m ? p0 - ng + m : -1;
        const int b = p0 < TL + m ? p0 + m : -1;
        const int c = p0 + ng < TL + m ? p0 + ng + m : -1;
        sl[u][0] = a >= 0 ? a : (b >= 0 ? b : c);
        sl[u][1] = a >= 0 ? (b >= 0 ? b : c) : (b >= 0 ? c : -1);
        if (sl[u][0] >= 0) atomicAdd(&start[sl[u][0]], 1);
        if (sl[u][1] >= 0) atomicAdd(&start[sl[u][1]], 1);
      }
    }
    __syncthreads();
    // exclusive scan of start[0..W]: slot lc occupies [start[lc], start[lc+1])
    {
      const int per = (W + 1 + kGridThreads - 1) / kGridThreads;
      const int b0 = min(threadIdx.x * per, W + 1), b1 = min(b0 + per, W + 1);
      int sum = 0;
      for (int i = b0; i < b1; ++i) sum += start[i];
      const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
      int v = sum;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
      }
      if (lane == 31) wsum[w] = v;
      __syncthreads();
      if (w == 0) {
        int t = lane < kGridThreads / 32 ? wsum[lane] : 0;
#pragma unroll
        for (int o = 1; o < kGridThreads / 32; o <<= 1) {
          const int u2 = __shfl_up_sync(0xffffffffu, t, o);
          if (lane >= o) t += u2;
        }
        if (lane < kGridThreads / 32) wsum[lane] = t;
      }
      __syncthreads();
      int run = v - sum + (w > 0 ? wsum[w - 1] : 0);
      for (int i = b0; i < b1; ++i) {
        const int c = start[i];
        start[i] = run;
        run += c;
      }
    }
    __syncthreads();
    // place: afterwards start[lc] is the END of slot lc (= old start[lc + 1])
#pragma unroll
    for (int u = 0; u < RPT; ++u) {
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const int lc = sl[u][q];
        if (lc < 0) continue;
        const int pos = atomicAdd(&start[lc], 1);
        P2 fy;
        fy.x = rc[u].a;
        fy.y = rc[u].b;
        sfy[pos] = fy;
        slc[pos] = (short)lc;
      }
    }
    __syncthreads();
    // gather: cell c_l (local) takes slots c_l .. c_l + 2m - 1
#pragma unroll
    for (int q = 0; q < kGridMaxCpt; ++q) {
      const int cl = threadIdx.x + q * kGridThreads;
      if (q >= cpt || cl >= TL) continue;
      const int rb = cl == 0 ? 0 : start[cl - 1];
      const int re = start[cl + 2 * m - 1];
      T a = (T)0;
      const int ctr = cl + m;
#pragma unroll 2
      for (int r = rb; r < re; ++r) {
        const P2 fy = sfy[r];
        const T dd = (T)(ctr - (int)slc[r]) - fy.x;
        a += gauss_w(fy.y, dd, e.k1);
      }
      acc[q] += a;
    }
    __syncthreads();
  }
  T *out = grid + base;
#pragma unroll
  for (int q = 0; q < kGridMaxCpt; ++q)
    if (q < cpt && threadIdx.x + q * kGridThreads < TL) out[threadIdx.x + q * kGridThreads] = acc[q];
}

template <typename T> size_t grid_smem_bytes(int logTL, int m) {
  const int W = (1 << logTL) + 2 * m;
  const size_t CAP = GridCfg<T>::CAP;
  return sizeof(int) * ((W + 2 + 3) & ~3) + sizeof(T) * 2 * CAP + sizeof(short) * CAP;
}

// Last four-step pass of the packed real transform: CTA owns row pairs
// (p, L1 - p), p in [p0, p0 + P), so both Z[k] and Z[L - k] are on chip.
template <typename T> struct PairRowSrc {
  const typename CxOf<T>::type *p;
  int logL2, L1, p0, npairs;
  __device__ __forceinline__ typename CxOf<T>::type load(int seq, int i) const {
    const int pp = p0 + (seq >> 1);
    const int row = (seq & 1) ? ((L1 - pp) & (L1 - 1)) : pp;
    return pp < npairs ? p[((int64_t)row << logL2) + i] : cmk((T)0, (T)0);
  }
};

template <typename T>
__global__ void __launch_bounds__(sizeof(T) == 4 ? 512 : 256) k_fft_rowpass_acc(const typename CxOf<T>::type *__restrict__ in,
                                                         FftDev<T> f, AccParams<T> e,
                                                         typename CxOf<T>::type *F) {
  typedef typename CxOf<T>::type C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *s = reinterpret_cast<C *>(smem_raw);
  const int L1 = 1 << f.logL1, L2 = 1 << f.logL2;
  const int logB = ilog2i((int64_t)blockDim.x * kFftE) - f.logL2;
  const int B = 1 << logB, logP = logB - 1, P = B >> 1;
  const int pitch = fft_pitch(L2, B);
  const int p0 = blockIdx.x * P, npairs = L1 / 2 + 1;
  const int tot = B << f.logL2;
  PairRowSrc<T> src{in, f.logL2, L1, p0, npairs};
  fft_fused<T, false, false, false>(s, pitch, f.logL2, logB, f.tw2, src, NoDst());
  for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
    const int i = idx & (P - 1), half = (idx >> logP) & 1, k2 = idx >> (logP + 1);
    const int p = p0 + i;
    if (p >= npairs) continue;
    const int rowA = p, rowB = (L1 - p) & (L1 - 1);
    if (half && rowA == rowB) continue;
    const int k1 = half ? rowB : rowA;
    const int64_t k = (int64_t)k1 + ((int64_t)k2 << f.logL1);
    if (k > e.K) continue;
    const int k2m = k1 == 0 ? ((L2 - k2) & (L2 - 1)) : (L2 - 1 - k2);
    const C Zk = s[(2 * i + half) * pitch + pad16(k2)];
    const C Zm = cconj(s[(2 * i + 1 - half) * pitch + pad16(k2m)]);
    acc_output<T>(e, k, Zk, Zm, F);
  }
}

// ---------------------------------------------------------------------------
// plan
// ---------------------------------------------------------------------------
size_t align_up(size_t v) { return (v + 255) & ~(size_t)255; }

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

}  // namespace
}  // namespace cuna

struct cuna2_plan_st {
  int dtype;
  int64_t nf, ng;
  int R, m;
  double tau;
  int logTL, ntiles;
  bool small;  // single-CTA fused path
  cuna::FftGeom geom;
  int device;
  std::mutex mu;
  void *ws = nullptr;
  size_t ws_bytes = 0;
  // device staging for cuna2_adjoint_host
  void *stage = nullptr;
  size_t stage_bytes = 0;
  // CUDA-graph replay of the launch sequence, keyed by the call arguments
  bool use_graph = false;
  cudaStream_t cap_stream = nullptr;
  struct GraphEntry {
    const void *t, *y, *F;
    int64_t n;
    double t0, T;
    cudaGraphExec_t exec;
  };
  std::vector<GraphEntry> graphs;
};

namespace cuna {
namespace {

template <typename T> AccParams<T> make_params(const cuna2_plan_st *p) {
  AccParams<T> e;
  e.ng = p->ng;
  e.nf = p->nf;
  e.K = p->nf / 2;
  e.m = p->m;
  e.logTL = p->logTL;
  e.ntiles = p->ntiles;
  const double tau = p->tau;
  e.k1 = (T)(1.0 / (4.0 * tau * log(2.0)));
  e.k2 = (T)(1.0 / (2.0 * tau * log(2.0)));
  e.e3c = (T)(-1.0 / (4.0 * tau));
  e.c0 = (T)(0.5 / sqrt(4.0 * kPi * tau));
  e.c1 = (T)(4.0 * kPi * kPi * tau / ((double)p->ng * (double)p->ng));
  e.twk = (T)(2.0 / (double)p->ng);
  return e;
}

int plan_workspace(cuna2_plan_st *p, size_t bytes, void **ws) {
  if (p->ws_bytes < bytes) {
    for (auto &g : p->graphs) cudaGraphExecDestroy(g.exec);  // they point at the old workspace
    p->graphs.clear();
    if (p->ws) {
      CUNA_CK(cudaDeviceSynchronize());
      CUNA_CK(cudaFree(p->ws));
      p->ws = nullptr;
      p->ws_bytes = 0;
    }
    size_t want = bytes + bytes / 4 + 4096;
    cudaError_t e = cudaMalloc(&p->ws, want);
    if (e != cudaSuccess) {
      p->ws = nullptr;
      return fail(CUNA2_ERROR_ALLOC, "plan workspace of %zu bytes: %s", want, cudaGetErrorString(e));
    }
    p->ws_bytes = want;
  }
  *ws = p->ws;
  return CUNA2_SUCCESS;
}

// Optional per-launch event marks (cuna2_plan_profile).
struct Prof {
  cudaEvent_t ev[16];
  const char *name[16];
  int n = 0;
};
inline void mark(Prof *pr, const char *name, cudaStream_t st) {
  if (pr && pr->n < 16) {
    pr->name[pr->n] = name;
    cudaEventRecord(pr->ev[pr->n++], st);
  }
}

template <typename T>
int adjoint_run(cuna2_plan_st *p, const double *t, const T *y, typename CxOf<T>::type *F, int64_t n,
                double t0, double T_, cudaStream_t st, Prof *pr = nullptr) {
  typedef typename CxOf<T>::type C;
  typedef typename RecOf<T>::type Rec;
  if (n < 0 || (n > 0 && (!t || !y)) || !F || !(T_ > 0) || !std::isfinite(T_) || !std::isfinite(t0))
    return fail(CUNA2_ERROR_INVALID_VALUE, "invalid argument (n=%lld T=%g)", (long long)n, T_);
  if (n > (int64_t)1 << 30) return fail(CUNA2_ERROR_UNSUPPORTED, "n > 2^30 samples per transform");
  const PhaseMul pm = phase_setup(t0, T_);
  const AccParams<T> e = make_params<T>(p);
  const FftDev<T> f = to_dev<T>(p->geom);
  const int L = 1 << p->geom.logL;
  if (p->small) {
    static bool attr = false;
    if (!attr) {
      CUNA_CK(cudaFuncSetAttribute(k_nfft_small<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024));
      attr = true;
    }
    const size_t smem = sizeof(C) * (size_t)fft_pitch(L, 1) + sizeof(T) * (2 * p->m + 2);
    const int threads = std::max(32, std::min(1024, L / kFftE));
    mark(pr, "start", st);
    k_nfft_small<T><<<1, threads, smem, st>>>(t, y, n, pm, e, f, F);
    CUNA_CK(cudaGetLastError());
    mark(pr, "nfft_small", st);
    return CUNA2_SUCCESS;
  }
  const int ntiles = p->ntiles;
  const size_t o_cnt = 0, o_off = align_up(sizeof(int) * ntiles), o_cur = o_off + align_up(sizeof(int) * (ntiles + 1));
  const size_t o_rec = o_cur + align_up(sizeof(int) * ntiles);
  const size_t o_grid = o_rec + align_up(sizeof(Rec) * 2 * (size_t)(n > 0 ? n : 1));
  const size_t bytes = o_grid + sizeof(T) * (size_t)p->ng;
  void *ws = nullptr;
  CUNA_TRY(plan_workspace(p, bytes, &ws));
  char *w = (char *)ws;
  int *counts = (int *)(w + o_cnt), *offsets = (int *)(w + o_off), *cursor = (int *)(w + o_cur);
  Rec *recs = (Rec *)(w + o_rec);
  T *grid = (T *)(w + o_grid);
  mark(pr, "start", st);
  CUNA_CK(cudaMemsetAsync(counts, 0, sizeof(int) * ntiles, st));
  if (n > 0) {
    SampAcc<T> smp{t, y, n, pm, e};
    const int sms = device_sm_count();
    const size_t smc = ntiles <= kBinSmemTiles ? sizeof(int) * ntiles : 0;
    const int gcount = (int)std::min<int64_t>((n + 4095) / 4096, 4 * sms);
    const int gscat = (int)((n + 512 * kScatterItems - 1) / (512 * kScatterItems));
    k_bin_count<<<gcount, 512, smc, st>>>(smp, counts, ntiles);
    CUNA_CK(cudaGetLastError());
    mark(pr, "bin_count", st);
    k_scan_tiles<<<1, 1024, 0, st>>>(counts, offsets, cursor, ntiles);
    CUNA_CK(cudaGetLastError());
    mark(pr, "scan_tiles", st);
    k_bin_scatter<<<gscat, 512, 2 * smc, st>>>(smp, offsets, cursor, recs, ntiles);
    CUNA_CK(cudaGetLastError());
    mark(pr, "bin_scatter", st);
  } else {
    k_scan_tiles<<<1, 1024, 0, st>>>(counts, offsets, cursor, ntiles);
    CUNA_CK(cudaGetLastError());
  }
  const size_t smg = grid_smem_bytes<T>(p->logTL, p->m);
  static bool attr3 = false;
  if (!attr3) {
    CUNA_CK(cudaFuncSetAttribute(k_grid_acc<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    attr3 = true;
  }
  k_grid_acc<T><<<ntiles, kGridThreads, smg, st>>>(recs, offsets, grid, e);
  CUNA_CK(cudaGetLastError());
  mark(pr, "grid", st);
  // packed complex view of the real grid
  C *z = reinterpret_cast<C *>(grid);
  const int elems = sizeof(T) == 4 ? kPassElemsF32 : kPassElemsF64;
  const int threads = elems / kFftE;
  const int L1 = 1 << p->geom.logL1, L2 = 1 << p->geom.logL2;
  const int BA = elems / L1, BB = elems / L2, PB = BB / 2;
  const size_t smemA = sizeof(C) * (size_t)BA * fft_pitch(L1, BA);
  const size_t smemB = sizeof(C) * (size_t)BB * fft_pitch(L2, BB);
  static bool attr2 = false;
  if (!attr2) {
    CUNA_CK(cudaFuncSetAttribute(k_fft_colpass<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    CUNA_CK(cudaFuncSetAttribute(k_fft_rowpass_acc<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    attr2 = true;
  }
  k_fft_colpass<T><<<dim3(L2 / BA, 1), threads, smemA, st>>>(z, z, f, (int64_t)L);
  CUNA_CK(cudaGetLastError());
  mark(pr, "fft_colpass", st);
  const int npairs = L1 / 2 + 1;
  k_fft_rowpass_acc<T><<<(npairs + PB - 1) / PB, threads, smemB, st>>>(z, f, e, F);
  CUNA_CK(cudaGetLastError());
  mark(pr, "fft_rowpass", st);
  return CUNA2_SUCCESS;
}

}  // namespace
}  // namespace cuna

using namespace cuna;

extern "C" int cuna2_plan_create(cuna2_plan *plan, int dtype, int64_t nf, int R, int m) {
  clear_error();
  if (!plan) return fail(CUNA2_ERROR_INVALID_VALUE, "plan pointer is NULL");
  *plan = nullptr;
  if (dtype != CUNA2_F32 && dtype != CUNA2_F64) return fail(CUNA2_ERROR_INVALID_VALUE, "dtype %d", dtype);
  if (nf < 2 || (nf & 1) || R < 2 || m < 1 || m > 16)
    return fail(CUNA2_ERROR_INVALID_VALUE, "need even nf >= 2, R >= 2, 1 <= m <= 16 (nf=%lld R=%d m=%d)",
                (long long)nf, R, m);
  const int64_t ng = nf * R, L = ng / 2;
  if (L & (L - 1)) return fail(CUNA2_ERROR_UNSUPPORTED, "R*nf/2 must be a power of two (R=%d nf=%lld)", R, (long long)nf);
  if (ng < 4 * m) return fail(CUNA2_ERROR_INVALID_VALUE, "grid of %lld cells is smaller than 4m", (long long)ng);
  const int logL = ilog2i(L);
  // the last pass pairs rows k1 and L1-k1, so it needs two rows per CTA
  const int max_log = dtype == CUNA2_F32 ? 25 : 23;
  if (logL > max_log) return fail(CUNA2_ERROR_UNSUPPORTED, "grid too large (R*nf = %lld)", (long long)ng);
  cuna2_plan_st *p = new cuna2_plan_st();
  p->dtype = dtype;
  p->nf = nf;
  p->ng = ng;
  p->R = R;
  p->m = m;
  p->tau = (double)m * R / (4.0 * kPi * (R - 0.5));
  p->small = logL <= (dtype == CUNA2_F32 ? kSingleLogF32 : kSingleLogF64);
  p->logTL = ng <= 8192 ? ilog2i(ng) : 12;
  p->ntiles = (int)(ng >> p->logTL);
  cudaGetDevice(&p->device);
  int st = fft_geometry(dtype == CUNA2_F64, logL, &p->geom);
  if (st) {
    delete p;
    return st;
  }
  *plan = p;
  return CUNA2_SUCCESS;
}

extern "C" int cuna2_plan_destroy(cuna2_plan p) {
  clear_error();
  if (!p) return CUNA2_SUCCESS;
  for (auto &g : p->graphs) cudaGraphExecDestroy(g.exec);
  if (p->cap_stream) cudaStreamDestroy(p->cap_stream);
  if (p->ws) cudaFree(p->ws);
  if (p->stage) cudaFree(p->stage);
  delete p;
  return CUNA2_SUCCESS;
}

extern "C" int cuna2_plan_info(cuna2_plan p, int64_t *ng, double *tau) {
  clear_error();
  if (!p) return fail(CUNA2_ERROR_INVALID_VALUE, "NULL plan");
  if (ng) *ng = p->ng;
  if (tau) *tau = p->tau;
  return CUNA2_SUCCESS;
}

namespace cuna {
namespace {
int run_graph(cuna2_plan p, const double *t, const void *y, void *F, int64_t n, double t0, double T,
              cudaStream_t st);
}
}  // namespace cuna

extern "C" int cuna2_adjoint(cuna2_plan p, const double *t, const void *y, void *F, int64_t n, double t0,
                             double T, cudaStream_t st) {
  clear_error();
  if (!p) return fail(CUNA2_ERROR_INVALID_VALUE, "NULL plan");
  std::lock_guard<std::mutex> lk(p->mu);
  if (p->use_graph) return run_graph(p, t, y, F, n, t0, T, st);
  if (p->dtype == CUNA2_F32)
    return adjoint_run<float>(p, t, (const float *)y, (float2 *)F, n, t0, T, st);
  return adjoint_run<double>(p, t, (const double *)y, (double2 *)F, n, t0, T, st);
}

namespace cuna {
namespace {
int run_any(cuna2_plan p, const double *t, const void *y, void *F, int64_t n, double t0, double T,
            cudaStream_t st, Prof *pr) {
  if (p->dtype == CUNA2_F32) return adjoint_run<float>(p, t, (const float *)y, (float2 *)F, n, t0, T, st, pr);
  return adjoint_run<double>(p, t, (const double *)y, (double2 *)F, n, t0, T, st, pr);
}

// Graph path: capture the launch sequence once per argument set on a private
// stream, then replay it on the caller's stream.
int run_graph(cuna2_plan p, const double *t, const void *y, void *F, int64_t n, double t0, double T,
              cudaStream_t st) {
  for (auto &g : p->graphs)
    if (g.t == t && g.y == y && g.F == F && g.n == n && g.t0 == t0 && g.T == T) {
      CUNA_CK(cudaGraphLaunch(g.exec, st));
      return CUNA2_SUCCESS;
    }
  // run once eagerly: sizes the workspace (allocation is not capturable) and
  // produces this call's result
  CUNA_TRY(run_any(p, t, y, F, n, t0, T, st, nullptr));
  if (!p->cap_stream) CUNA_CK(cudaStreamCreateWithFlags(&p->cap_stream, cudaStreamNonBlocking));
  CUNA_CK(cudaStreamSynchronize(st));
  CUNA_CK(cudaStreamBeginCapture(p->cap_stream, cudaStreamCaptureModeThreadLocal));
  int s = run_any(p, t, y, F, n, t0, T, p->cap_stream, nullptr);
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamEndCapture(p->cap_stream, &graph);
  if (s) return s;
  if (e != cudaSuccess) return fail_cuda(e, "cudaStreamEndCapture");
  cudaGraphExec_t exec = nullptr;
  e = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return fail_cuda(e, "cudaGraphInstantiate");
  if (p->graphs.size() >= 64) {
    cudaGraphExecDestroy(p->graphs.front().exec);
    p->graphs.erase(p->graphs.begin());
  }
  p->graphs.push_back({t, y, F, n, t0, T, exec});
  return CUNA2_SUCCESS;
}
}  // namespace
}  // namespace cuna

extern "C" int cuna2_plan_set_graph(cuna2_plan p, int enable) {
  clear_error();
  if (!p) return fail(CUNA2_ERROR_INVALID_VALUE, "NULL plan");
  std::lock_guard<std::mutex> lk(p->mu);
  p->use_graph = enable != 0;
  return CUNA2_SUCCESS;
}

extern "C" int cuna2_adjoint_host(cuna2_plan p, const double *t, const void *y, void *F, int64_t n, double t0,
                                  double T, cudaStream_t st) {
  clear_error();
  if (!p) return fail(CUNA2_ERROR_INVALID_VALUE, "NULL plan");
  if (n < 0 || (n > 0 && (!t || !y)) || !F) return fail(CUNA2_ERROR_INVALID_VALUE, "invalid argument");
  std::lock_guard<std::mutex> lk(p->mu);
  const size_t es = p->dtype == CUNA2_F32 ? 4 : 8;
  const size_t bt = align_up(8 * (size_t)(n > 0 ? n : 1)), by = align_up(es * (size_t)(n > 0 ? n : 1));
  const size_t bF = 2 * es * (size_t)p->nf;
  if (p->stage_bytes < bt + by + bF) {
    if (p->stage) {
      CUNA_CK(cudaDeviceSynchronize());
      CUNA_CK(cudaFree(p->stage));
      p->stage = nullptr;
      p->stage_bytes = 0;
    }
    cudaError_t e = cudaMalloc(&p->stage, bt + by + bF);
    if (e != cudaSuccess) return fail(CUNA2_ERROR_ALLOC, "staging buffers: %s", cudaGetErrorString(e));
    p->stage_bytes = bt + by + bF;
  }
  char *d = (char *)p->stage;
  double *td = (double *)d;
  void *yd = d + bt, *Fd = d + bt + by;
  if (n > 0) {
    CUNA_CK(cudaMemcpyAsync(td, t, 8 * (size_t)n, cudaMemcpyHostToDevice, st));
    CUNA_CK(cudaMemcpyAsync(yd, y, es * (size_t)n, cudaMemcpyHostToDevice, st));
  }
  CUNA_TRY(p->use_graph ? run_graph(p, td, yd, Fd, n, t0, T, st) : run_any(p, td, yd, Fd, n, t0, T, st, nullptr));
  CUNA_CK(cudaMemcpyAsync(F, Fd, bF, cudaMemcpyDeviceToHost, st));
  CUNA_CK(cudaStreamSynchronize(st));
  return CUNA2_SUCCESS;
}

extern "C" int cuna2_plan_profile(cuna2_plan p, const double *t, const void *y, void *F, int64_t n, double t0,
                                  double T, cudaStream_t st, float *stage_ms, const char **stage_names,
                                  int max_stages, int *nstages) {
  clear_error();
  if (!p || !stage_ms || !nstages) return fail(CUNA2_ERROR_INVALID_VALUE, "invalid argument");
  std::lock_guard<std::mutex> lk(p->mu);
  Prof pr;
  for (int i = 0; i < 16; ++i) CUNA_CK(cudaEventCreate(&pr.ev[i]));
  int s = run_any(p, t, y, F, n, t0, T, st, &pr);
  if (!s) {
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) s = fail_cuda(e, "cudaStreamSynchronize");
  }
  int k = 0;
  for (int i = 1; !s && i < pr.n && k < max_stages; ++i, ++k) {
    cudaEventElapsedTime(&stage_ms[k], pr.ev[i - 1], pr.ev[i]);
    if (stage_names) stage_names[k] = pr.name[i];
  }
  *nstages = k;
  for (int i = 0; i < 16; ++i) cudaEventDestroy(pr.ev[i]);
  return s;
}
