// accurate_kernels.cuh -- device code of accurate mode, shared by the
// single-series plans (accurate.cu) and the batched plans (batch.cu).
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
// are fused in.  The grid position is reduced in 64-bit fixed point
// (phase.cuh).
//
// Each kernel's work is a __device__ body taking the per-series parameters,
// so that the single-series kernels and the batched work-list kernels share
// it.
#pragma once
#include <math.h>
#include <algorithm>
#include <type_traits>
#include "binning.cuh"
#include "fft.cuh"
#include "phase.cuh"
#include "rng.cuh"
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
// (the float version converts a 32-bit integer: 64-bit integer to float
// conversions run on the narrow FP64 pipe of GB300)
__device__ __forceinline__ float frac_of(uint64_t lo, float) {
  return (float)(uint32_t)(lo >> 40) * 5.9604644775390625e-08f;
}
__device__ __forceinline__ double frac_of(uint64_t lo, double) {
  return (double)(lo >> 11) * 1.1102230246251565e-16;
}

// cell and fractional cell of the phase S = frac(x + 1/2) * 2^64
template <typename T>
__device__ __forceinline__ void cell_of_phase(uint64_t S, int64_t ng, int &cell, T &f) {
  if ((ng & (ng - 1)) == 0) {  // ng = 2^g: the top g bits are the cell
    const int g = 63 - __clzll((long long)ng);
    cell = g ? (int)(S >> (64 - g)) : 0;
    f = frac_of(S << g, (T)0);
  } else {
    cell = (int)umulhi64(S, (uint64_t)ng);
    f = frac_of(S * (uint64_t)ng, (T)0);
  }
}

template <typename T>
__device__ __forceinline__ void reduce_sample(double t, const PhaseMul &pm, int64_t ng, int &cell, T &f) {
  cell_of_phase<T>(phase_of(t, pm), ng, cell, f);
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
  const T kf = (T)(int)k;  // k <= nf/2 < 2^31; a 32-bit conversion
  sincospi_t(kf * e.twk, &sn, &cs);
  const C G2 = cadd(A, cmul(cmk(cs, sn), Bv));
  T sc = e.c0 * exp_t(e.c1 * kf * kf);
  if (k & 1) sc = -sc;
  const C Fk = cscale(G2, sc);
  if (k < e.K) F[e.K + k] = Fk;
  if (k >= 1) F[e.K - k] = cconj(Fk);
}

// The same with the unpack twiddle exp(2 pi i k / ng) supplied (from tables)
// and the deconvolution factor by exp2.
// (float-float plans: the unpack in float-float, the deconvolution factor and
// the output in double)
template <typename T>
__device__ __forceinline__ void acc_output_tw(const AccParams<typename AccOf<T>::type> &e, int64_t k,
                                              typename CxOf<T>::type Zk, typename CxOf<T>::type Zmc,
                                              typename MemOf<T>::type *F, typename CxOf<T>::type tw) {
  typedef typename CxOf<T>::type C;
  typedef typename AccOf<T>::type A;
  typedef typename MemOf<T>::type M;
  const C Ap = cadd(Zk, Zmc);
  const C Bv = cmuli(csub(Zmc, Zk));
  const C G2 = cadd(Ap, cmul(tw, Bv));
  M Fk;
  if constexpr (std::is_same<T, dfl>::value) {
    // the deconvolution factor in float-float too: only the final value is
    // rejoined in double
    const dfl kf((float)(int)k, 0.f);  // k <= nf / 2 <= 2^24: exact
    dfl sc = df_from_double(e.c0) * df_exp2(df_from_double(e.c1 * 1.4426950408889634) * kf * kf);
    if (k & 1) sc = -sc;
    Fk = cx_to_mem(cmk(G2.x * sc, G2.y * sc));
  } else {
    const A kf = (A)(int)k;
    A sc = e.c0 * exp2_t(e.c1 * (A)1.4426950408889634 * kf * kf);
    if (k & 1) sc = -sc;
    Fk = cscale(cx_to_mem(G2), sc);
  }
  if (k < e.K) F[e.K + k] = Fk;
  if (k >= 1) F[e.K - k] = cconj(Fk);
}

// ---------------------------------------------------------------------------
// single-CTA transform for small grids
// ---------------------------------------------------------------------------
__device__ __forceinline__ int real_slot(int c) { return 2 * pad16(c >> 1) + (c & 1); }

// Whole transform of one series in one CTA: gridding straight into shared
// memory (the grid is the packed complex FFT buffer), FFT, epilogue.
template <typename T>
__device__ __forceinline__ void nfft_small_body(const double *__restrict__ t, const T *__restrict__ y,
                                                int64_t n, const PhaseMul &pm, const AccParams<T> &e,
                                                const FftDev<T> &f, typename CxOf<T>::type *F) {
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

template <typename T>
__global__ void __launch_bounds__(sizeof(T) == 4 ? 1024 : 512) k_nfft_small(const double *__restrict__ t, const T *__restrict__ y,
                                                     int64_t n, PhaseMul pm, AccParams<T> e, FftDev<T> f,
                                                     typename CxOf<T>::type *F, const T *__restrict__ wts) {
  // one CTA per output slab: slab b grids wts[b*n + j] when wts is given
  // (bootstrap resample b), else y[j]
  if (wts) {
    y = wts + (int64_t)blockIdx.x * n;
    F += (int64_t)blockIdx.x * e.nf;
  }
  nfft_small_body<T>(t, y, n, pm, e, f, F);
}

// ---------------------------------------------------------------------------
// binning sampler, tiled gridding, last FFT pass
// ---------------------------------------------------------------------------
// Sorted sample record of accurate mode: {cell, fractional cell, value}.
__device__ __forceinline__ void rec_set(RecF &r, int cell, float fr, float y, int idx) {
  r.cell = cell; r.a = fr; r.b = y; r.p = idx;
}
__device__ __forceinline__ void rec_set(RecD &r, int cell, double fr, double y, int idx) {
  r.cell = cell; r.p = idx; r.a = fr; r.b = y; r.v = 0.0;
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
  uint64_t *sc = nullptr;  // optional: phases written here for SampAccS
  __device__ __forceinline__ Raw load(int64_t i, bool with_value) const {
    Raw r;
    r.t = t[i];
    if (with_value) r.y = y[i];
    return r;
  }
  __device__ __forceinline__ void prep(int64_t i, const Raw &r, Prep<Rec> &p) const {
    int cell;
    T fr;
    const uint64_t S = phase_of(r.t, pm);
    if (sc) sc[i] = S;
    cell_of_phase<T>(S, e.ng, cell, fr);
    const int ng = (int)e.ng;
    int lo = cell - e.m + 1, hi = cell + e.m;
    if (lo < 0) lo += ng;
    if (hi >= ng) hi -= ng;
    const int t0 = lo >> e.logTL, t1 = hi >> e.logTL;
    p.t[0] = t0;
    p.t[1] = t1;
    p.nt = t0 == t1 ? 1 : 2;
    rec_set(p.rec, cell, fr, r.y, (int)i);
  }
};

// Sampler over phases cached by a SampAcc pass (sc[i] = phase of t[i]): the
// scatter pass of the binning then skips the phase reduction.
template <typename T> struct SampAccS {
  typedef typename RecOf<T>::type Rec;
  struct Raw {
    uint64_t S;
    T y;
  };
  const uint64_t *sc;
  const T *y;
  int64_t n;
  AccParams<T> e;
  __device__ __forceinline__ Raw load(int64_t i, bool with_value) const {
    Raw r;
    r.S = __ldcg(reinterpret_cast<const unsigned long long *>(sc) + i);  // written by the count pass
    if (with_value) r.y = y[i];
    return r;
  }
  __device__ __forceinline__ void prep(int64_t i, const Raw &r, Prep<Rec> &p) const {
    int cell;
    T fr;
    cell_of_phase<T>(r.S, e.ng, cell, fr);
    const int ng = (int)e.ng;
    int lo = cell - e.m + 1, hi = cell + e.m;
    if (lo < 0) lo += ng;
    if (hi >= ng) hi -= ng;
    const int t0 = lo >> e.logTL, t1 = hi >> e.logTL;
    p.t[0] = t0;
    p.t[1] = t1;
    p.nt = t0 == t1 ? 1 : 2;
    rec_set(p.rec, cell, fr, r.y, (int)i);
  }
};

// ---------------------------------------------------------------------------
// Gridding, gather form.  One CTA owns tile [base, base + TL) of the grid and
// the records binned to it (its own samples plus the halo samples within m
// cells of its edges).  Per chunk of at most CAP records it counting-sorts
// them in shared memory by group of CW consecutive local slots (slot lc =
// cell - base + m; integer atomics only), then every thread sums, for each
// of its CW cells c, the records of the groups covering slots [c - base,
// c - base + 2m): w = y exp(-(d - f)^2 / (4 tau)), d = c - cell (records of
// those groups outside the window are masked, or, in the unmasked form, add
// their negligible tail).  Partial sums stay in registers across chunks and
// are written once, coalesced.  No floating-point atomics.
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

// a placed record in shared memory: fractional cell, value, slot
template <typename T> struct __align__(2 * sizeof(T) >= 16 ? 16 : 16) SRec {
  T f, y;
  int lc, pad;
};

// exp2 for the gridding weights: ex2.approx for float (relative error of a
// few ulp), the library exp2 for double
__device__ __forceinline__ float exp2_g(float x) { return ex2_fast(x); }
__device__ __forceinline__ double exp2_g(double x) { return exp2(x); }

// Weights y exp2(-k1 (x + i)^2) of one record for CW consecutive cells,
// i = 0..CW-1, by the fast Gaussian gridding factorisation (Greengard & Lee
// 2004) about the middle cell h = CW/2, xc = x + h:
//   y exp2(-k1 (xc + j)^2) = E Q^j c_j,  E = y exp2(-k1 xc^2),
//   Q = exp2(-2 k1 xc), c_j = exp2(-k1 j^2),
// three exp2 per record and cell group instead of CW.  Centring keeps E and
// the running products inside the float range for every m <= 16.
template <typename T, int CW> struct GaussCW {
  T c[CW / 2 + 1];
  __device__ explicit GaussCW(T k1) {
#pragma unroll
    for (int j = 0; j <= CW / 2; ++j) c[j] = exp2_g(-k1 * (T)(j * j));
  }
};
template <typename T, int CW>
__device__ __forceinline__ void gauss_cw(T y, T x, T k1, const GaussCW<T, CW> &g, T *w) {
  constexpr int H = CW / 2;
  const T xc = x + (T)H;
  const T E = y * exp2_g(-k1 * xc * xc);
  const T Q = exp2_g((T)(-2) * k1 * xc), Qi = exp2_g((T)2 * k1 * xc);
  w[H] = E;
  T u = E;
#pragma unroll
  for (int j = 1; j < CW - H; ++j) {
    u *= Q;
    w[H + j] = u * g.c[j];
  }
  u = E;
#pragma unroll
  for (int j = 1; j <= H; ++j) {
    u *= Qi;
    w[H - j] = u * g.c[j];
  }
}

// a[i] += y exp2(-k1 (x + i)^2) for the cells i a record in slot rel = lc - cl0
// reaches (0 <= rel - i < w2, w2 = 2m), by the centred factorisation of
// gauss_cw; the mask is applied before the last product so that each tap is
// one select and one fused multiply-add.
// MASKED == false adds the record to all CW cells: cells outside its taps
// lie more than m cells from it, where the Gaussian is below 2^(-k1 m^2) of
// its peak; the plan takes this form only where that bound is negligible
// (tail_free_gather), and then each tap is one product and one fused
// multiply-add.
template <typename T, int CW, bool MASKED = true>
__device__ __forceinline__ void gauss_acc(T y, T x, T k1, const GaussCW<T, CW> &g, int rel, int w2, T *a) {
  constexpr int H = CW / 2;
  const T xc = x + (T)H;
  const T E = y * exp2_g(-k1 * xc * xc);
  const T Q = exp2_g((T)(-2) * k1 * xc), Qi = exp2_g((T)2 * k1 * xc);
  if (MASKED) a[H] += (unsigned)(rel - H) < (unsigned)w2 ? E : (T)0;
  else a[H] += E;
  T u = E;
#pragma unroll
  for (int j = 1; j < CW - H; ++j) {
    u *= Q;
    if (MASKED) a[H + j] = fma((unsigned)(rel - H - j) < (unsigned)w2 ? u : (T)0, g.c[j], a[H + j]);
    else a[H + j] = fma(u, g.c[j], a[H + j]);
  }
  u = E;
#pragma unroll
  for (int j = 1; j <= H; ++j) {
    u *= Qi;
    if (MASKED) a[H - j] = fma((unsigned)(rel - H + j) < (unsigned)w2 ? u : (T)0, g.c[j], a[H - j]);
    else a[H - j] = fma(u, g.c[j], a[H - j]);
  }
}

__device__ __forceinline__ void store4(float *p, float a, float b, float c, float d) {
  *reinterpret_cast<float4 *>(p) = make_float4(a, b, c, d);
}
__device__ __forceinline__ void store4(double *p, double a, double b, double c, double d) {
  reinterpret_cast<double2 *>(p)[0] = make_double2(a, b);
  reinterpret_cast<double2 *>(p)[1] = make_double2(c, d);
}

// Slots (local cell + m) of a record whose cell is p0 cells right of the tile
// base, for every image p = p0 + j*ng (j in {-1, 0, 1}) in [-m, TL + m); the
// second slot exists only when one tile spans the whole periodic grid.
__device__ __forceinline__ void grid_slots(int p0, int ng, int TL, int m, int &s0, int &s1) {
  if (p0 < 0) p0 += ng;
  const int a = p0 - ng >= -m ? p0 - ng + m : -1;
  const int b = p0 < TL + m ? p0 + m : -1;
  const int c = p0 + ng < TL + m ? p0 + ng + m : -1;
  s0 = a >= 0 ? a : (b >= 0 ? b : c);
  s1 = a >= 0 ? (b >= 0 ? b : c) : (b >= 0 ? c : -1);
}

// One grid tile [base, base + 2^logTL) from records [r0, r1), for slabs
// [sbeg, send): slab s grids value wts[s*nvals + p] of sample p when wts is
// given (bootstrap), else the record's own value.
// CW consecutive cells per thread in the gather (4 or 8)
// SG > 1 (slab weights given, CW = 8 on 2048-cell tiles): SG slabs share each
// record's Gaussian, computed once per record visit and scaled by each slab's
// value from shared memory.
template <typename T, int CW, class Src, int SG = 1, bool MASKED = true>
__device__ __forceinline__ void grid_tile_body(const Src &recs, int r0, int r1,
                                               int base, T *__restrict__ grid, const AccParams<T> &e,
                                               const T *__restrict__ wts, int64_t nvals, int sbeg, int send,
                                               int64_t slab_stride) {
  typedef typename RecOf<T>::type Rec;
  constexpr int CAP = GridCfg<T>::CAP;
  // cells per thread: up to 16 in groups of 4 (TL <= 4096), or one group of
  // 8 (TL = 2048)
  constexpr int MAXC = CW == 8 ? 8 : kGridMaxCpt;
  constexpr int RPT = CAP / kGridThreads;  // records per thread per chunk
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int TL = 1 << e.logTL, m = e.m, W = TL + 2 * m;
  // records are counting-sorted into groups of CW consecutive slots (slot =
  // local cell + m), the unit of a thread's cell group: NG + 1 counters
  const int NG = (W + CW - 1) / CW;
  const int ng = (int)e.ng;
  int *start = reinterpret_cast<int *>(smem_raw);                                       // NG + 1 groups
  SRec<T> *srec = reinterpret_cast<SRec<T> *>(smem_raw + sizeof(int) * ((W + 2 + 3) & ~3));  // placed records
  int *sp = reinterpret_cast<int *>(srec + CAP);                                         // sample index
  T *yv = reinterpret_cast<T *>(sp + CAP);  // SG > 1: yv[s * CAP + r], value of slab s for placed record r
  static_assert(SG == 1 || CW == 8, "slab groups run with 8-cell groups on 2048-cell tiles");
  __shared__ int wsum[kGridThreads / 32];
  // a single tile spanning the whole grid maps a record to up to two slots;
  // halve the chunk then so that placements never exceed CAP
  const int chunk = (TL + 2 * m > ng) ? CAP / 2 : CAP;
  const int npass = (TL + kGridThreads * CW - 1) / (kGridThreads * CW);  // <= MAXC / CW
  const int nchunks = (r1 - r0 + chunk - 1) / chunk;
  const GaussCW<T, CW> gw(e.k1);
  // the records are sorted once for all slabs when they fit in one chunk
  for (int slab = sbeg; slab < send; slab += SG) {
    T acc[SG][MAXC];
#pragma unroll
    for (int g = 0; g < SG; ++g)
#pragma unroll
      for (int q = 0; q < MAXC; ++q) acc[g][q] = (T)0;
    for (int ck = 0; ck < nchunks; ++ck) {
      const int c0 = r0 + ck * chunk;
      const int cnt = min(chunk, r1 - c0);
      if (nchunks > 1 || slab == sbeg) {
        for (int i = threadIdx.x; i <= NG; i += kGridThreads) start[i] = 0;
        __syncthreads();
        // load this thread's records; each maps to up to two slots (two only
        // when the tile wraps onto itself, i.e. one tile spans the whole grid)
        Rec rc[RPT];
#pragma unroll
        for (int u = 0; u < RPT; ++u) {
          const int i = threadIdx.x + u * kGridThreads;
          if (i < cnt) rc[u] = recs[c0 + i];
        }
#pragma unroll
        for (int u = 0; u < RPT; ++u) {
          const int i = threadIdx.x + u * kGridThreads;
          if (i < cnt) {
            int s0, s1;
            grid_slots(rc[u].cell - base, ng, TL, m, s0, s1);
            if (s0 >= 0) atomicAdd(&start[s0 / CW], 1);
            if (s1 >= 0) atomicAdd(&start[s1 / CW], 1);
          }
        }
        __syncthreads();
        // exclusive scan of start[0..NG]: group g occupies [start[g], start[g+1])
        {
          const int per = (NG + 1 + kGridThreads - 1) / kGridThreads;
          const int b0 = min((int)threadIdx.x * per, NG + 1), b1 = min(b0 + per, NG + 1);
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
        // place: afterwards start[g] is the END of group g
#pragma unroll
        for (int u = 0; u < RPT; ++u) {
          const int i = threadIdx.x + u * kGridThreads;
          if (i >= cnt) continue;
          int sl[2];
          grid_slots(rc[u].cell - base, ng, TL, m, sl[0], sl[1]);
#pragma unroll
          for (int q = 0; q < 2; ++q) {
            const int lc = sl[q];
            if (lc < 0) continue;
            const int pos = atomicAdd(&start[lc / CW], 1);
            SRec<T> r;
            r.f = rc[u].a;
            r.y = rc[u].b;
            r.lc = lc;
            r.pad = __float_as_int((float)lc);  // the slot as a float (exact), for the unmasked gather
            srec[pos] = r;
            sp[pos] = rc[u].p;
          }
        }
        __syncthreads();
      }
      if (SG == 1 && wts) {  // this slab's values for the placed records
        const int placed = start[(W - 1) / CW];
        const T *ws = wts + (int64_t)slab * nvals;
        for (int i = threadIdx.x; i < placed; i += kGridThreads) srec[i].y = ws[sp[i]];
        __syncthreads();
      }
      if constexpr (SG > 1) {  // the group's values (0 past the last slab)
        const int placed = start[(W - 1) / CW];
#pragma unroll
        for (int g = 0; g < SG; ++g) {
          const T *ws = wts + (int64_t)(slab + g) * nvals;
          for (int i = threadIdx.x; i < placed; i += kGridThreads)
            yv[g * CAP + i] = slab + g < send ? ws[sp[i]] : (T)0;
        }
        __syncthreads();
      }
      // gather: the thread's cells cl0 .. cl0+CW-1 (local) take the records in
      // slots cl0 .. cl0 + CW - 1 + 2m - 1; record slot lc reaches cell c iff
      // 0 <= lc - c < 2m
#pragma unroll
      for (int q = 0; q < MAXC / CW; ++q) {
        const int cl0 = (threadIdx.x + q * kGridThreads) * CW;
        if (q >= npass || cl0 >= TL) continue;
        // the groups holding slots cl0 .. cl0 + CW + 2m - 2 (cl0 is a
        // multiple of CW; the last group may hold up to CW - 1 slots beyond
        // the window, whose records the masks drop or, unmasked, add below
        // 2^(-k1 m^2))
        const int g0 = cl0 / CW, g1 = (cl0 + CW + 2 * m - 2) / CW;
        const int rb = g0 == 0 ? 0 : start[g0 - 1];
        const int re = start[g1];
        // SG > 1 has one pass (CW = MAXC = 8) and accumulates into acc directly
        T a[1][CW];
#pragma unroll
        for (int i = 0; i < CW; ++i) a[0][i] = (T)0;
        const int ctr = cl0 + m, w2 = 2 * m;
        const float ctrf = (float)ctr;
        for (int r = rb; r < re; ++r) {
          const SRec<T> rr = srec[r];
          const int rel = rr.lc - cl0;  // lc - c for c = cl0
          // d - f for c = cl0; unmasked float tiles take the slot as a float
          // (a difference of small integers, exact) and skip the conversion
          T dd0;
          if constexpr (!MASKED && sizeof(T) == 4) dd0 = (ctrf - __int_as_float(rr.pad)) - rr.f;
          else dd0 = (T)(ctr - rr.lc) - rr.f;
          if constexpr (SG == 1) {
            gauss_acc<T, CW, MASKED>(rr.y, dd0, e.k1, gw, rel, w2, a[0]);
          } else {
            T w[CW];
            gauss_cw<T, CW>((T)1, dd0, e.k1, gw, w);
            if constexpr (MASKED) {
#pragma unroll
              for (int i = 0; i < CW; ++i) w[i] = (unsigned)(rel - i) < (unsigned)w2 ? w[i] : (T)0;
            }
#pragma unroll
            for (int g = 0; g < SG; ++g) {
              const T yg = yv[g * CAP + r];
#pragma unroll
              for (int i = 0; i < CW; ++i) acc[g][i] = fma(yg, w[i], acc[g][i]);
            }
          }
        }
        if constexpr (SG == 1) {
#pragma unroll
          for (int i = 0; i < CW; ++i) acc[0][CW * q + i] += a[0][i];
        }
      }
      __syncthreads();
    }
#pragma unroll
    for (int g = 0; g < SG; ++g) {
      if (slab + g >= send) break;
      T *out = grid + (int64_t)(slab + g) * slab_stride + base;
#pragma unroll
      for (int q = 0; q < MAXC / CW; ++q) {
        const int cl0 = (threadIdx.x + q * kGridThreads) * CW;
        // TL is a power of two >= CW (gather tiles have >= 512 cells or span
        // the grid, ng >= 4m >= 4 and CW = 4 there), so groups are whole
        if (q < npass && cl0 < TL) {
#pragma unroll
          for (int i = 0; i < CW; i += 4)
            store4(out + cl0 + i, acc[g][CW * q + i], acc[g][CW * q + i + 1], acc[g][CW * q + i + 2],
                   acc[g][CW * q + i + 3]);
        }
      }
    }
  }
}

// slab groups sharing each record's Gaussian (bootstrap resamples, channels)
template <typename T, bool MASKED = true>
__global__ void __launch_bounds__(kGridThreads, sizeof(T) == 4 ? 3 : 2) k_grid_acc_sg4(
    const typename RecOf<T>::type *recs, const int *off, T *grid, AccParams<T> e, const T *wts, int64_t nvals,
    int nslab, int group, int64_t slab_stride) {
  pdl_trigger();
  pdl_wait();  // records and offsets come from the binning
  const int tile = blockIdx.x;
  const int sbeg = blockIdx.y * group, send = min(nslab, sbeg + group);
  const CgSrc<typename RecOf<T>::type> rp{recs};
  const int r0 = __ldcg(off + tile), r1 = __ldcg(off + tile + 1);
  if constexpr (sizeof(T) == 4)
    grid_tile_body<T, 8, CgSrc<typename RecOf<T>::type>, 4, MASKED>(rp, r0, r1, tile << e.logTL, grid, e, wts, nvals,
                                                                     sbeg, send, slab_stride);
  else  // double plans keep one slab per pass (four accumulator sets do not fit)
    grid_tile_body<T, 8>(rp, r0, r1, tile << e.logTL, grid, e, wts, nvals, sbeg, send, slab_stride);
}

template <typename T, int CW, bool MASKED = true>
__global__ void __launch_bounds__(kGridThreads, sizeof(T) == 4 ? 4 : 2) k_grid_acc(
    const typename RecOf<T>::type *recs, const int *off, T *grid, AccParams<T> e, const T *wts, int64_t nvals,
    int nslab, int group, int64_t slab_stride) {
  pdl_trigger();
  pdl_wait();  // records and offsets come from the binning
  // a CTA per (tile, group of slabs)
  const int tile = blockIdx.x;
  const int sbeg = blockIdx.y * group, send = min(nslab, sbeg + group);
  const CgSrc<typename RecOf<T>::type> rp{recs};
  grid_tile_body<T, CW, CgSrc<typename RecOf<T>::type>, 1, MASKED>(rp, __ldcg(off + tile), __ldcg(off + tile + 1),
                                                                    tile << e.logTL, grid, e, wts, nvals, sbeg, send,
                                                                    slab_stride);
}

// Whether a float plan's gather may add each record to whole cell groups
// without the tap masks: every cell beyond a record's taps lies more than m
// cells from it, where the Gaussian exp(-d^2 / (4 tau)) is below
// exp(-m^2 / (4 tau)); below 1e-8 of the peak (under float rounding) the
// extra terms only bring the kernel closer to the untruncated Gaussian that
// the deconvolution divides by.  Double plans keep the masks.
inline bool tail_free_gather(bool is_float, int m, double tau) {
  return is_float && (double)m * m / (4.0 * tau) >= 18.43;  // exp(-18.43) = 1e-8
}

// Scatter form of the same tile gridding: the tile's cells accumulate in
// shared memory, one thread per (record, tap) pair adds its Gaussian weight
// with a shared-memory atomic, and the tile is flushed to HBM once, in cell
// order, with vector stores (no global atomics).  A block step covers
// floor(256 / 2m) records, thread t taking tap t mod 2m of record t / 2m, so
// every lane of a warp does useful work whatever the record density.  A tap
// lands in cell (cell + d) mod ng, kept when it falls in this tile; ng is a
// power of two.  Summation order within a cell follows the atomics.
template <typename T, class Src>
__device__ __forceinline__ void grid_tile_scatter(const Src &recs, int r0, int r1,
                                                  int base, T *__restrict__ grid, const AccParams<T> &e,
                                                  const T *__restrict__ wts, int64_t nvals, int sbeg, int send,
                                                  int64_t slab_stride) {
  typedef typename RecOf<T>::type Rec;
  constexpr int CAP = GridCfg<T>::CAP;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int TL = 1 << e.logTL, m = e.m, W2 = 2 * m;
  const int gmask = (int)e.ng - 1;
  T *acc = reinterpret_cast<T *>(smem_raw);                          // TL cells
  SRec<T> *srec = reinterpret_cast<SRec<T> *>(smem_raw + sizeof(T) * TL);  // CAP staged records
  int *sp = reinterpret_cast<int *>(srec + CAP);                       // sample index (weights)
  const int per = kGridThreads / W2;  // records per block step (W2 <= 32)
  const int rr = threadIdx.x / W2;
  const int d = (int)threadIdx.x - rr * W2 - m + 1;  // tap offset in [-m+1, m]
  const T dT = (T)d;
  const bool active = rr < per;
  const int nchunks = (r1 - r0 + CAP - 1) / CAP;
  for (int slab = sbeg; slab < send; ++slab) {
    for (int i = 4 * threadIdx.x; i < TL; i += 4 * kGridThreads) store4(acc + i, (T)0, (T)0, (T)0, (T)0);
    for (int ck = 0; ck < nchunks; ++ck) {
      const int c0 = r0 + ck * CAP;
      const int cnt = min(CAP, r1 - c0);
      if (nchunks > 1 || slab == sbeg) {
        for (int i = threadIdx.x; i < cnt; i += kGridThreads) {
          const Rec rc = recs[c0 + i];
          SRec<T> r;
          r.f = rc.a;
          r.y = rc.b;
          r.lc = rc.cell - base;
          r.pad = 0;
          srec[i] = r;
          sp[i] = rc.p;
        }
      }
      if (wts) {
        __syncthreads();
        const T *ws = wts + (int64_t)slab * nvals;
        for (int i = threadIdx.x; i < cnt; i += kGridThreads) srec[i].y = ws[sp[i]];
      }
      __syncthreads();
      if (active) {
        for (int r = rr; r < cnt; r += per) {
          const SRec<T> q = srec[r];
          const int lc = (q.lc + d) & gmask;
          const T w = gauss_w(q.y, dT - q.f, e.k1);
          if (lc < TL) atomicAdd(&acc[lc], w);
        }
      }
      __syncthreads();
    }
    // fixed-order flush; TL is a power of two >= 4, so groups of four are whole
    T *out = grid + (int64_t)slab * slab_stride + base;
    for (int i = 4 * threadIdx.x; i < TL; i += 4 * kGridThreads) store4(out + i, acc[i], acc[i + 1], acc[i + 2], acc[i + 3]);
    __syncthreads();
  }
}

template <typename T>
__global__ void __launch_bounds__(kGridThreads, sizeof(T) == 4 ? 6 : 3) k_grid_scatter(
    const typename RecOf<T>::type *recs, const int *off, T *grid, AccParams<T> e, const T *wts, int64_t nvals,
    int nslab, int group, int64_t slab_stride) {
  pdl_trigger();
  pdl_wait();  // records and offsets come from the binning
  const int tile = blockIdx.x;
  const int sbeg = blockIdx.y * group, send = min(nslab, sbeg + group);
  const CgSrc<typename RecOf<T>::type> rp{recs};
  grid_tile_scatter<T>(rp, __ldcg(off + tile), __ldcg(off + tile + 1), tile << e.logTL, grid, e, wts, nvals, sbeg,
                       send, slab_stride);
}

// Fixed-point form: one thread per record, all 2m taps from the fast Gaussian
// factorisation  y exp2(-k1 (d - f)^2) = [y exp2(-k1 f^2)] Q^d exp2(-k1 d^2),
// Q = exp2(2 k1 f)  (three exp2 per record, two multiplies per tap), each
// tap added into the shared tile as an integer with a native shared-memory
// integer atomic.  The tile's fixed-point scale comes from a bound on every
// cell's sum: |y| <= Ymax over the tile's records and at most 2 hmax records
// reach one cell, hmax the largest count of records in a bucket of
// max(2m, 16) consecutive cells (a cell's 2m-cell window meets two buckets);
// weights are <= 1.  With the sum bounded by 2^30 (float, int32 cells) or
// 2^50 (double, int64 cells, as two 32-bit words where hmax <= 2048) units,
// the quantum is 2^-30 (2^-50) of the
// bound.  Integer sums do not depend on the order of the atomics, so the grid
// is bit-reproducible run to run.  A non-finite value makes its tiles NaN.
// records [c0, c0 + cnt) -> srec (values from ws when given); returns the
// thread's max |value| (NaN once one is not finite)
template <typename T, class Src>
__device__ __forceinline__ float fixed_stage(const Src &recs, int c0, int cnt,
                                            int base, const T *__restrict__ ws, SRec<T> *srec) {
  float ym = 0.f;
#pragma unroll 1
  for (int i = threadIdx.x; i < cnt; i += kGridThreads) {
    const typename RecOf<T>::type rc = recs[c0 + i];
    SRec<T> r;
    r.f = rc.a;
    r.y = ws ? ws[rc.p] : rc.b;
    r.lc = rc.cell - base;
    r.pad = rc.p;
    srec[i] = r;
    ym = isfinite(r.y) && !isnan(ym) ? fmaxf(ym, (float)fabs(r.y)) : __int_as_float(0x7fffffff);
  }
  return ym;
}

// clear a fixed-point tile of TL cells (TL a multiple of 4, acc 16-byte
// aligned) with 16-byte stores
template <typename A> __device__ __forceinline__ void fixed_clear(A *acc, int TL) {
  int4 *v = reinterpret_cast<int4 *>(acc);
  const int nv = TL * (int)sizeof(A) / 16;
  for (int i = threadIdx.x; i < nv; i += kGridThreads) v[i] = make_int4(0, 0, 0, 0);
}
// cells [i, i + 4) of a fixed-point tile as values: 16-byte shared loads
__device__ __forceinline__ void fixed_load4(const int *acc, int i, float inv, float &a, float &b, float &c,
                                            float &d) {
  const int4 v = *reinterpret_cast<const int4 *>(acc + i);
  a = (float)v.x * inv;
  b = (float)v.y * inv;
  c = (float)v.z * inv;
  d = (float)v.w * inv;
}
__device__ __forceinline__ void fixed_load4(const long long *acc, int i, double inv, double &a, double &b,
                                            double &c, double &d) {
  const longlong2 u = *reinterpret_cast<const longlong2 *>(acc + i);
  const longlong2 v = *reinterpret_cast<const longlong2 *>(acc + i + 2);
  a = (double)u.x * inv;
  b = (double)u.y * inv;
  c = (double)v.x * inv;
  d = (double)v.y * inv;
}

// Double tiles in split form: each int64 tap v enters two 32-bit integer
// atomics instead of one 64-bit one (slower in shared memory: 212 against
// 179 us for a 2^22-cell float64 grid of 1e6 samples): hi[c] +=
// floor(v / 2^20) (signed) and lo[c] += v mod 2^20
// (unsigned), arrays of TL words each in the space of the int64 tile.  The
// cell's sum is hi * 2^20 + lo exactly when neither array overflows: a cell
// takes at most 2 hmax taps, so lo stays below 2 hmax 2^20 <= 2^32 for hmax
// <= 2048, and |hi| below 2^30 + 4 hmax (each |v| <= 2^50 / (2 hmax) + 1).
// The integer sums, hence the grid's bits, equal the int64 form's.
constexpr int kSplitBits = 20;
constexpr int kSplitMaxH = 2048;
template <typename T> struct FixAdd {  // one atomic in the tile's own type
  typename FixAcc<T>::type *acc;
  __device__ __forceinline__ void operator()(int c, typename FixAcc<T>::type v) const {
    FixAcc<T>::add(acc + c, v);
  }
};
struct SplitAdd {
  int *hi;
  unsigned *lo;
  __device__ __forceinline__ void operator()(int c, long long v) const {
    atomicAdd(lo + c, (unsigned)v & ((1u << kSplitBits) - 1u));
    atomicAdd(hi + c, (int)(v >> kSplitBits));
  }
};
// cells [i, i + 4) of a split tile as values: 16-byte shared loads
__device__ __forceinline__ void fixed_load4_split(const int *hi, const unsigned *lo, int i, double inv, double &a,
                                                  double &b, double &c, double &d) {
  const int4 h = *reinterpret_cast<const int4 *>(hi + i);
  const uint4 l = *reinterpret_cast<const uint4 *>(lo + i);
  constexpr long long U = 1ll << kSplitBits;
  a = (double)((long long)h.x * U + l.x) * inv;
  b = (double)((long long)h.y * U + l.y) * inv;
  c = (double)((long long)h.z * U + l.z) * inv;
  d = (double)((long long)h.w * U + l.w) * inv;
}

// Tap arithmetic of the fixed-point form: float plans in float; double plans
// in float-float on the FP32 pipe (about 48 bits, below the 2^-50 quantum's
// reach only where a tap is far below its tile's bound), the per-record
// factors E, Q, 1/Q and the 2m coefficients formed in double first.
template <typename T> struct TapOf { typedef T type; };
template <> struct TapOf<double> { typedef dfl type; };
__device__ __forceinline__ float tap_from(float v) { return v; }
__device__ __forceinline__ dfl tap_from(double v) { return df_from_double(v); }
__device__ __forceinline__ int tap_fix(float w) { return FixAcc<float>::to_fix(w); }
// round(hi + lo) for |hi + lo| <= 2^50, from the bit fields of hi: at or
// above 2^23 hi is an integer (its 24-bit significand shifted left) and lo,
// below half its ulp, rounds on its own; below 2^23 the float sum rounds.
__device__ __forceinline__ long long tap_fix(dfl w) {
  if (fabsf(w.hi) >= 8388608.0f) {
    const int b = __float_as_int(w.hi);
    const int sh = ((b >> 23) & 0xff) - 150;
    const long long mag = (long long)((b & 0x7fffff) | 0x800000) << sh;
    return (b < 0 ? -mag : mag) + (long long)__float2int_rn(w.lo);
  }
  return (long long)__float2int_rn(w.hi + w.lo);
}

// all 2m taps of the staged records srec[0, cnt) into the tile through add
// (add(c, v): integer v into local cell c), scaled by sc; cd holds the
// coefficients exp2(-k1 d^2) in the tap arithmetic's type
template <typename T, class Add>
__device__ __forceinline__ void fixed_taps(const SRec<T> *srec, int cnt, T sc, const AccParams<T> &e,
                                           const T *cd, const Add &add, int TL, int gmask) {
  typedef typename TapOf<T>::type W;
  const W *cw = reinterpret_cast<const W *>(cd);
  const int m = e.m;
  W k1w, k2w;  // the exponent constants in the tap arithmetic
  if constexpr (sizeof(T) == 8) {
    k1w = df_from_double(e.k1);
    k2w = df_from_double(e.k2);
  }
#pragma unroll 1
  for (int i = threadIdx.x; i < cnt; i += kGridThreads) {
    const SRec<T> q = srec[i];
    W Ew, Qw, Qiw;
    if constexpr (sizeof(T) == 8) {
      // E = y sc 2^(-k1 f^2), Q = 2^(k2 f), 1/Q in float-float: only the two
      // conversions from double use the FP64 pipe
      const dfl fw = df_from_double(q.f);
      Ew = df_from_double(q.y * sc) * df_exp2(-(k1w * fw * fw));
      Qw = df_exp2(k2w * fw);
      Qiw = df_rcp(Qw);
    } else {
      Ew = q.y * sc * exp2_g(-e.k1 * q.f * q.f);
      Qw = exp2_g(e.k2 * q.f);
      Qiw = exp2_g(-e.k2 * q.f);
    }
    const int p0 = q.lc;
    if (p0 - m + 1 >= 0 && p0 + m < TL) {  // every tap inside the tile
      W u = Ew;
#pragma unroll 4
      for (int d = 0; d <= m; ++d) {  // taps right of the cell, Q^d
        add(p0 + d, tap_fix(u * cw[d + m - 1]));
        u = u * Qw;
      }
      u = Ew * Qiw;
#pragma unroll 4
      for (int d = -1; d > -m; --d) {  // taps left of the cell
        add(p0 + d, tap_fix(u * cw[d + m - 1]));
        u = u * Qiw;
      }
    } else {  // near the tile edge: wrap, keep the taps inside the tile
      W u = Ew;
      for (int d = 0; d <= m; ++d) {
        const int lc = (p0 + d) & gmask;
        if (lc < TL) add(lc, tap_fix(u * cw[d + m - 1]));
        u = u * Qw;
      }
      u = Ew * Qiw;
      for (int d = -1; d > -m; --d) {
        const int lc = (p0 + d) & gmask;
        if (lc < TL) add(lc, tap_fix(u * cw[d + m - 1]));
        u = u * Qiw;
      }
    }
  }
}

// the tile's fixed-point scale from the per-warp maxima of |value| (NaN once
// one was not finite) and the largest bucket count hmax
template <typename T>
__device__ __forceinline__ T fixed_scale(const float *red, int hmax) {
  float y = 0.f;
  bool bad = false;
#pragma unroll
  for (int w = 0; w < kGridThreads / 32; ++w) {
    bad |= isnan(red[w]);
    y = fmaxf(y, red[w]);
  }
  // bound on any cell's |sum| in value units; the scale maps it to `range`
  const T B = (T)y * (T)(2 * hmax);
  T sc = B > (T)0 ? FixAcc<T>::range / B : (T)0;
  if (isinf(sc)) sc = (T)0;
  return bad ? (T)NAN : sc;
}

// the taps of srec[0, cnt) into the tile, in split form when asked (double)
template <typename T>
__device__ __forceinline__ void tile_taps(bool split, const SRec<T> *srec, int cnt, T sc, const AccParams<T> &e,
                                          const T *cd, typename FixAcc<T>::type *acc, int TL, int gmask) {
  if constexpr (sizeof(T) == 8) {
    if (split) {
      const SplitAdd add{reinterpret_cast<int *>(acc), reinterpret_cast<unsigned *>(acc) + TL};
      fixed_taps<T>(srec, cnt, sc, e, cd, add, TL, gmask);
      return;
    }
  }
  fixed_taps<T>(srec, cnt, sc, e, cd, FixAdd<T>{acc}, TL, gmask);
}

// fixed-order flush of the tile: out[i] = cell i * inv (inv = 1 / scale)
template <typename T>
__device__ __forceinline__ void tile_flush(bool split, const typename FixAcc<T>::type *acc, int TL, T inv,
                                           T *__restrict__ out) {
  if constexpr (sizeof(T) == 8) {
    if (split) {
      const int *hi = reinterpret_cast<const int *>(acc);
      const unsigned *lo = reinterpret_cast<const unsigned *>(acc) + TL;
      for (int i = 4 * threadIdx.x; i < TL; i += 4 * kGridThreads) {
        T a, b, c, d;
        fixed_load4_split(hi, lo, i, inv, a, b, c, d);
        store4(out + i, a, b, c, d);
      }
      return;
    }
  }
  for (int i = 4 * threadIdx.x; i < TL; i += 4 * kGridThreads) {
    T a, b, c, d;
    fixed_load4(acc, i, inv, a, b, c, d);
    store4(out + i, a, b, c, d);
  }
}

template <typename T, class Src>
__device__ __forceinline__ void grid_tile_fixed(const Src &recs, int r0, int r1,
                                                int base, T *__restrict__ grid, const AccParams<T> &e,
                                                const T *__restrict__ wts, int64_t nvals, int sbeg, int send,
                                                int64_t slab_stride) {
  typedef FixAcc<T> FA;
  typedef typename FA::type A;
  constexpr int CAP = GridCfg<T>::CAP;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ float red[kGridThreads / 32];
  __shared__ int redi[kGridThreads / 32];
  __shared__ T scale_s;
  const int TL = 1 << e.logTL, m = e.m;
  const int gmask = (int)e.ng - 1;
  int logBS = 4;
  while ((1 << logBS) < 2 * m) ++logBS;
  const int NB = ((TL + 2 * m) >> logBS) + 1;
  A *acc = reinterpret_cast<A *>(smem_raw);                                  // TL cells
  SRec<T> *srec = reinterpret_cast<SRec<T> *>(smem_raw + sizeof(A) * TL);    // CAP staged records
  T *cd = reinterpret_cast<T *>(srec + CAP);                                 // exp2(-k1 d^2), d = -m+1..m
  int *hist = reinterpret_cast<int *>(cd + 32);                              // NB buckets
  const int nchunks = (r1 - r0 + CAP - 1) / CAP;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int d = threadIdx.x; d < 2 * m; d += kGridThreads) {
    const T dd = (T)(d - m + 1);
    reinterpret_cast<typename TapOf<T>::type *>(cd)[d] = tap_from(exp2_g(-e.k1 * dd * dd));
  }
  // bucket histogram of the tile's records (slab independent); a record of
  // this tile lies in [base - m, base + TL + m) modulo ng
  for (int b = threadIdx.x; b < NB; b += kGridThreads) hist[b] = 0;
  if (!wts && sbeg + 1 == send && nchunks <= 1) {
    // One slab of the records' own values, one staging chunk: a single read
    // of the records stages them, builds the histogram and bounds |value|;
    // the largest bucket count is the largest count an atomic returned.
    // Three barriers per tile instead of six; same scale, same bits.
    constexpr int PER = CAP / kGridThreads;
    const int cnt = r1 - r0;
    fixed_clear(acc, TL);
    __syncthreads();
    typename RecOf<T>::type rc[PER];
#pragma unroll
    for (int k = 0; k < PER; ++k)
      if (threadIdx.x + k * kGridThreads < cnt) rc[k] = recs[r0 + threadIdx.x + k * kGridThreads];
    float ym = 0.f;
    int hm = 0;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      const int i = threadIdx.x + k * kGridThreads;
      if (i >= cnt) continue;
      SRec<T> r;
      r.f = rc[k].a;
      r.y = rc[k].b;
      r.lc = rc[k].cell - base;
      r.pad = rc[k].p;
      srec[i] = r;
      hm = max(hm, atomicAdd(&hist[((rc[k].cell - base + m) & gmask) >> logBS], 1) + 1);
      ym = isfinite(r.y) && !isnan(ym) ? fmaxf(ym, (float)fabs(r.y)) : __int_as_float(0x7fffffff);
    }
    for (int o = 16; o > 0; o >>= 1) {
      const float u = __shfl_xor_sync(0xffffffffu, ym, o);
      ym = (isnan(u) || isnan(ym)) ? __int_as_float(0x7fffffff) : fmaxf(ym, u);
      hm = max(hm, __shfl_xor_sync(0xffffffffu, hm, o));
    }
    if (lane == 0) {
      red[warp] = ym;
      redi[warp] = hm;
    }
    __syncthreads();
    int hmax = 0;
#pragma unroll
    for (int w = 0; w < kGridThreads / 32; ++w) hmax = max(hmax, redi[w]);
    const T sc = fixed_scale<T>(red, hmax);
    const bool split = sizeof(T) == 8 && hmax <= kSplitMaxH;
    if (sc > (T)0) tile_taps<T>(split, srec, cnt, sc, e, cd, acc, TL, gmask);
    __syncthreads();
    const T inv = sc > (T)0 ? (T)1 / sc : (sc == sc ? (T)0 : sc);
    tile_flush<T>(split, acc, TL, inv, grid + (int64_t)sbeg * slab_stride + base);
    return;
  }
  __syncthreads();
#pragma unroll 1
  for (int i = r0 + threadIdx.x; i < r1; i += kGridThreads)
    atomicAdd(&hist[((recs[i].cell - base + m) & gmask) >> logBS], 1);
  __syncthreads();
  int hmax = 0;
  for (int b = threadIdx.x; b < NB; b += kGridThreads) hmax = max(hmax, hist[b]);
  for (int o = 16; o > 0; o >>= 1) hmax = max(hmax, __shfl_xor_sync(0xffffffffu, hmax, o));
  if (lane == 0) redi[warp] = hmax;
  __syncthreads();
  hmax = 0;
#pragma unroll
  for (int w = 0; w < kGridThreads / 32; ++w) hmax = max(hmax, redi[w]);
  const bool split = sizeof(T) == 8 && hmax <= kSplitMaxH;
  for (int slab = sbeg; slab < send; ++slab) {
    const T *ws = wts ? wts + (int64_t)slab * nvals : nullptr;
    float ym = 0.f;
    if (slab > sbeg) __syncthreads();  // the previous slab's flush is done with acc and srec
    if (nchunks == 1) {
      ym = fixed_stage<T>(recs, r0, r1 - r0, base, ws, srec);
    } else {  // bound pass over all of the tile's records
#pragma unroll 1
      for (int i = r0 + threadIdx.x; i < r1; i += kGridThreads) {
        const T v = ws ? ws[recs[i].p] : recs[i].b;
        ym = isfinite(v) && !isnan(ym) ? fmaxf(ym, (float)fabs(v)) : __int_as_float(0x7fffffff);
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const float u = __shfl_xor_sync(0xffffffffu, ym, o);
      ym = (isnan(u) || isnan(ym)) ? __int_as_float(0x7fffffff) : fmaxf(ym, u);
    }
    if (lane == 0) red[warp] = ym;
    fixed_clear(acc, TL);
    __syncthreads();
    if (threadIdx.x == 0) scale_s = fixed_scale<T>(red, hmax);
    __syncthreads();
    const T sc = scale_s;
    for (int ck = 0; ck < nchunks; ++ck) {
      const int c0 = r0 + ck * CAP;
      const int cnt = min(CAP, r1 - c0);
      if (nchunks > 1) {
        if (ck > 0) __syncthreads();
        fixed_stage<T>(recs, c0, cnt, base, ws, srec);
        __syncthreads();
      }
      if (sc > (T)0) tile_taps<T>(split, srec, cnt, sc, e, cd, acc, TL, gmask);
    }
    __syncthreads();
    // fixed-order flush: cell = integer / scale
    const T inv = sc > (T)0 ? (T)1 / sc : (sc == sc ? (T)0 : sc);
    tile_flush<T>(split, acc, TL, inv, grid + (int64_t)slab * slab_stride + base);
  }
}

template <typename T>
__global__ void __launch_bounds__(kGridThreads, sizeof(T) == 4 ? 6 : 4) k_grid_fixed(
    const typename RecOf<T>::type *recs, const int *off, T *grid, AccParams<T> e, const T *wts, int64_t nvals,
    int nslab, int group, int64_t slab_stride) {
  pdl_trigger();
  pdl_wait();  // records and offsets come from the binning
  const int tile = blockIdx.x;
  const int sbeg = blockIdx.y * group, send = min(nslab, sbeg + group);
  const CgSrc<typename RecOf<T>::type> rp{recs};
  grid_tile_fixed<T>(rp, __ldcg(off + tile), __ldcg(off + tile + 1), tile << e.logTL, grid, e, wts, nvals, sbeg, send,
                     slab_stride);
}

template <typename T> size_t grid_fixed_smem_bytes(int logTL, int m) {
  int logBS = 4;
  while ((1 << logBS) < 2 * m) ++logBS;
  const size_t NB = ((((size_t)1 << logTL) + 2 * m) >> logBS) + 1;
  return sizeof(typename FixAcc<T>::type) * ((size_t)1 << logTL) + sizeof(SRec<T>) * (size_t)GridCfg<T>::CAP +
         sizeof(T) * 32 + sizeof(int) * NB;
}

// ---------------------------------------------------------------------------
// Tiles fed by the single-pass chunk-local binning (k_bin_local): a tile's
// records are nch runs, one per input chunk, located by loc[tile nch + c] =
// start | count << 16 within chunk c's region recs[c ch2 ..].
// ---------------------------------------------------------------------------
constexpr int kSegMaxChunks = 1024;

// element v of a tile's record list: binary search over the runs
template <typename T> struct SegSrc {
  typedef typename RecOf<T>::type Rec;
  const Rec *recs;
  const int *pre;   // shared, nch + 1: run c holds list elements [pre[c], pre[c+1])
  const int *base;  // shared, nch: record index of run c's first element
  int nch;
  __device__ __forceinline__ Rec operator[](int v) const {
    int lo = 0, hi = nch - 1;
    while (lo < hi) {  // last run with pre <= v (a non-empty one)
      const int mid = (lo + hi + 1) >> 1;
      if (pre[mid] <= v) lo = mid;
      else hi = mid - 1;
    }
    return recs[base[lo] + (v - pre[lo])];
  }
};

// CTA-wide: the runs of `tile` into shared memory sh (2 nch + 1 ints);
// returns the length of the tile's record list.  Ends with a barrier.
__device__ __forceinline__ int seg_setup(const int *__restrict__ loc, int tile, int nch, int ch2, int *sh) {
  int *pre = sh, *cnt = sh + nch + 1;
  const int *row = loc + (int64_t)tile * nch;
  for (int c = threadIdx.x; c < nch; c += blockDim.x) cnt[c] = (unsigned)row[c] >> 16;
  __syncthreads();
  cta_exclusive_scan(cnt, pre, nch);
  for (int c = threadIdx.x; c < nch; c += blockDim.x) cnt[c] = c * ch2 + (row[c] & 0xffff);  // now the run bases
  __syncthreads();
  return pre[nch];
}

#define CUNA_SEG_KERNEL(NAME, BODY, OCC32, OCC64)                                                              \
  template <typename T, int CW>                                                                               \
  __global__ void __launch_bounds__(kGridThreads, sizeof(T) == 4 ? OCC32 : OCC64) NAME(                        \
      const typename RecOf<T>::type *__restrict__ recs, const int *__restrict__ loc, int nch, int ch2,          \
      int seg_off, T *__restrict__ grid, AccParams<T> e, const T *__restrict__ wts, int64_t nvals, int nslab,    \
      int group, int64_t slab_stride) {                                                                         \
    extern __shared__ __align__(16) unsigned char smem_raw[];                                                   \
    int *sh = reinterpret_cast<int *>(smem_raw + seg_off);                                                      \
    const int tile = blockIdx.x;                                                                                \
    const int sbeg = blockIdx.y * group, send = min(nslab, sbeg + group);                                       \
    const int total = seg_setup(loc, tile, nch, ch2, sh);                                                       \
    const SegSrc<T> src{recs, sh, sh + nch + 1, nch};                                                           \
    BODY(src, 0, total, tile << e.logTL, grid, e, wts, nvals, sbeg, send, slab_stride);                          \
  }
CUNA_SEG_KERNEL(k_grid_acc_seg, (grid_tile_body<T, CW>), 4, 2)
CUNA_SEG_KERNEL(k_grid_scatter_seg, grid_tile_scatter<T>, 6, 3)
CUNA_SEG_KERNEL(k_grid_fixed_seg, grid_tile_fixed<T>, 6, 2)
#undef CUNA_SEG_KERNEL

template <typename T> size_t grid_scatter_smem_bytes(int logTL) {
  return sizeof(T) * ((size_t)1 << logTL) + (sizeof(SRec<T>) + sizeof(int)) * (size_t)GridCfg<T>::CAP;
}

template <typename T> size_t grid_smem_bytes(int logTL, int m, int sg = 1) {
  const int W = (1 << logTL) + 2 * m;
  const size_t CAP = GridCfg<T>::CAP;
  return sizeof(int) * ((W + 2 + 3) & ~3) + sizeof(SRec<T>) * CAP + sizeof(int) * CAP +
         (sg > 1 ? sizeof(T) * sg * CAP : 0);
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

// Last four-step pass of the packed real transform for row pairs (p, L1 - p),
// p in [p0, p0 + P): both Z[k] and Z[L - k] are on chip for the unpack.
template <typename T>
__device__ __forceinline__ void rowpass_acc_body(const typename CxOf<T>::type *__restrict__ in,
                                                 const FftDev<T> &f, const AccParams<T> &e,
                                                 typename CxOf<T>::type *F, int pblock) {
  typedef typename CxOf<T>::type C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *s = reinterpret_cast<C *>(smem_raw);
  const int L1 = 1 << f.logL1, L2 = 1 << f.logL2;
  const int logB = ilog2i((int64_t)blockDim.x * kFftE) - f.logL2;
  const int B = 1 << logB, logP = logB - 1, P = B >> 1;
  const int pitch = fft_pitch(L2, B);
  const int p0 = pblock * P, npairs = L1 / 2 + 1;
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

template <typename T>
__global__ void __launch_bounds__(sizeof(T) == 4 ? 512 : 256) k_fft_rowpass_acc(const typename CxOf<T>::type *__restrict__ in,
                                                         FftDev<T> f, AccParams<T> e,
                                                         typename CxOf<T>::type *F) {
  // slab blockIdx.y
  rowpass_acc_body<T>(in + ((int64_t)blockIdx.y << f.logL), f, e, F + (int64_t)blockIdx.y * e.nf, blockIdx.x);
}

// ---------------------------------------------------------------------------
// Backward (vector-Jacobian product) of the accurate transform.
//
// With g_k = dL/dRe F_k + i dL/dIm F_k for the stored outputs,
//   h_k = g_k (-1)^k / psi_hat(k),      R_c = Re sum_k h_k exp(-2 pi i k c / ng),
//   dL/dy_j = sum_d R_{b+d} psi(d - f),
//   dL/dt_j = (ng / T) y_j sum_d R_{b+d} (d - f) / (2 tau) psi(d - f),
// d = -m+1..m, b + f = s_j the grid position.  R is real: with the Hermitian
// part H_k = (h_k + conj(h_{-k})) / 2 of h, R = DFT_-(H) is computed as one
// complex DFT of length L = ng/2 of Zin[k] = E[k] + i O[k], E[k] = H_k +
// H_{k+L}, O[k] = (H_k - H_{k+L}) exp(-2 pi i k / ng), whose output is
// R[2n] + i R[2n+1].  DFT_- = conj(DFT_+(conj(.))); the conjugations are fused
// into the load and store functors of the (inverse-sign) FFT passes.
// ---------------------------------------------------------------------------
template <typename T> struct BwdSpec {
  const typename CxOf<T>::type *G;  // nf values, G[k + nf/2]
  int64_t ng, K;                     // K = nf / 2
  T c0b, c1;                         // 1/psi_hat(k) = c0b exp(c1 k^2)
  T twk;                             // 2 / ng
  // h_k for any integer k (taken mod ng), zero outside the output band
  __device__ __forceinline__ typename CxOf<T>::type h(int64_t k) const {
    k %= ng;
    if (k < 0) k += ng;
    if (k >= ng - K) k -= ng;  // to [-K, ng - K)
    if (k >= K || k < -K) return cmk((T)0, (T)0);
    const T kf = (T)(int)k;
    T sc = c0b * exp_t(c1 * kf * kf);
    if (k & 1) sc = -sc;
    return cscale(G[k + K], sc);
  }
  // conj(Zin[q]), q in [0, L)
  __device__ __forceinline__ typename CxOf<T>::type zin_conj(int64_t q) const {
    typedef typename CxOf<T>::type C;
    const int64_t L = ng / 2;
    const C hq = h(q), hmq = h(-q), hp = h(q + L), hmp = h(-q - L);
    const T half = (T)0.5;
    const C Hq = cscale(cadd(hq, cconj(hmq)), half);   // H_q
    const C Hp = cscale(cadd(hp, cconj(hmp)), half);   // H_{q+L}
    const C E = cadd(Hq, Hp);
    T sn, cs;
    sincospi_t((T)q * twk, &sn, &cs);
    const C O = cmul(csub(Hq, Hp), cmk(cs, -sn));      // (H_q - H_{q+L}) e^{-2 pi i q / ng}
    return cconj(cadd(E, cmuli(O)));
  }
};

// Per-series constants of a batch of backward passes (up to kBwdSeries
// series per launch, passed by value): the phase multiplier of x = (t - t0)/T
// and ng / T, the chain-rule factor of dL/dt.
constexpr int kBwdSeries = 256;
struct BwdSeries {
  PhaseMul pm[kBwdSeries];
  double tscale[kBwdSeries];
};

// interpolation of R at one sample: accumulates both gradient sums
template <typename T, class Rget>
__device__ __forceinline__ void bwd_sample(const Rget &R, int cell, T fr, int m, int ng, T k1, T inv2tau,
                                           T &sy, T &st) {
  sy = (T)0;
  st = (T)0;
  for (int d = -m + 1; d <= m; ++d) {
    int c = cell + d;
    if (c < 0) c += ng;
    else if (c >= ng) c -= ng;
    const T dd = (T)d - fr;
    const T w = R(c) * exp2_t(-k1 * dd * dd);
    sy += w;
    st += w * dd * inv2tau;
  }
}

// Single CTA per series: spectrum -> shared memory -> FFT -> interpolation at
// every sample.  CTA b handles series b of the batch (samples b*n.., upstream
// gradient b*nf..).
template <typename T>
__global__ void __launch_bounds__(sizeof(T) == 4 ? 1024 : 512) k_bwd_small(
    const double *__restrict__ t, const T *__restrict__ y, int64_t n, const __grid_constant__ BwdSeries ser,
    AccParams<T> e, BwdSpec<T> sp, FftDev<T> f, T *__restrict__ gy, double *__restrict__ gt) {
  typedef typename CxOf<T>::type C;
  const int b = blockIdx.x;
  const PhaseMul pm = ser.pm[b];
  const double tscale = ser.tscale[b];
  t += (int64_t)b * n;
  y += (int64_t)b * n;
  if (gy) gy += (int64_t)b * n;
  if (gt) gt += (int64_t)b * n;
  sp.G += (int64_t)b * 2 * sp.K;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int L = 1 << f.logL;
  const int pitch = fft_pitch(L, 1);
  C *s = reinterpret_cast<C *>(smem_raw);
  const T *sr = reinterpret_cast<const T *>(smem_raw);
  for (int q = threadIdx.x; q < L; q += blockDim.x) s[pad16(q)] = sp.zin_conj(q);
  __syncthreads();
  smem_fft<T>(s, pitch, f.logL, 1, f.tw1);
  // output z[nn] = conj(FFT result): R[2nn] = Re, R[2nn+1] = -Im
  auto R = [&](int c) -> T {
    const T v = sr[real_slot(c)];
    return (c & 1) ? -v : v;
  };
  const T inv2tau = (T)2.0 * e.e3c * (T)-1.0;  // 1 / (2 tau) = -2 e3c
  for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
    int cell;
    T fr;
    reduce_sample<T>(t[j], pm, e.ng, cell, fr);
    T a, b;
    bwd_sample<T>(R, cell, fr, e.m, (int)e.ng, e.k1, inv2tau, a, b);
    if (gy) gy[j] = a;
    if (gt) gt[j] = tscale * (double)y[j] * (double)b;
  }
}

// four-step pass A of the backward: columns of conj(Zin) computed from G on the fly
template <typename T> struct SpecColSrc {
  BwdSpec<T> sp;
  int L2, c0;
  __device__ __forceinline__ typename CxOf<T>::type load(int seq, int i) const {
    return sp.zin_conj((int64_t)i * L2 + c0 + seq);
  }
};

template <typename T>
__global__ void __launch_bounds__(sizeof(T) == 4 ? 512 : 256) k_bwd_colpass(BwdSpec<T> sp, typename CxOf<T>::type *z,
                                                                            FftDev<T> f) {
  typedef typename CxOf<T>::type C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *s = reinterpret_cast<C *>(smem_raw);
  sp.G += (int64_t)blockIdx.y * 2 * sp.K;  // series blockIdx.y of a batch
  z += (int64_t)blockIdx.y << f.logL;
  const int L2 = 1 << f.logL2;
  const int logB = ilog2i((int64_t)blockDim.x * kFftE) - f.logL1;
  const int B = 1 << logB;
  const int pitch = fft_pitch(1 << f.logL1, B);
  const int c0 = blockIdx.x * B;
  SpecColSrc<T> src{sp, L2, c0};
  ColDst<T> dst{z, L2, c0, f};
  fft_fused<T, true, true, true>(s, pitch, f.logL1, logB, f.tw1, src, dst);
}

// pass B: rows -> real field R (conjugated outputs, interleaved re/im)
template <typename T> struct ConjRealDst {
  typename CxOf<T>::type *r;  // R viewed as L complex values
  int logL1, r0;
  __device__ __forceinline__ void store(int seq, int k2, typename CxOf<T>::type v) const {
    r[r0 + seq + (k2 << logL1)] = cconj(v);
  }
};
template <typename T> struct PlainRowSrc {
  const typename CxOf<T>::type *p;
  int logL2;
  __device__ __forceinline__ typename CxOf<T>::type load(int seq, int i) const {
    return p[((int64_t)seq << logL2) + i];
  }
};

template <typename T>
__global__ void __launch_bounds__(sizeof(T) == 4 ? 512 : 256) k_bwd_rowpass(const typename CxOf<T>::type *z,
                                                                            typename CxOf<T>::type *r, FftDev<T> f) {
  typedef typename CxOf<T>::type C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *s = reinterpret_cast<C *>(smem_raw);
  z += (int64_t)blockIdx.y << f.logL;  // series blockIdx.y of a batch
  r += (int64_t)blockIdx.y << f.logL;
  const int logB = ilog2i((int64_t)blockDim.x * kFftE) - f.logL2;
  const int B = 1 << logB;
  const int pitch = fft_pitch(1 << f.logL2, B);
  const int r0 = blockIdx.x * B;
  PlainRowSrc<T> src{z + ((int64_t)r0 << f.logL2), f.logL2};
  ConjRealDst<T> dst{r, f.logL1, r0};
  fft_fused<T, true, false, true>(s, pitch, f.logL2, logB, f.tw2, src, dst);
}

// interpolation at samples j < n * nser of a batch: series s = j / n reads its
// own real field R + s * ng and constants ser.*[s]
template <typename T>
__global__ void __launch_bounds__(256) k_bwd_interp(const double *__restrict__ t, const T *__restrict__ y, int64_t n,
                                                    int nser, const __grid_constant__ BwdSeries ser, AccParams<T> e,
                                                    const T *__restrict__ R, T *__restrict__ gy,
                                                    double *__restrict__ gt) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n * nser) return;
  const int s = (int)(j / n);
  int cell;
  T fr;
  reduce_sample<T>(t[j], ser.pm[s], e.ng, cell, fr);
  const T inv2tau = (T)2.0 * e.e3c * (T)-1.0;
  const T *Rs = R + (int64_t)s * e.ng;
  auto Rg = [&](int c) -> T { return __ldg(&Rs[c]); };
  T a, b;
  bwd_sample<T>(Rg, cell, fr, e.m, (int)e.ng, e.k1, inv2tau, a, b);
  if (gy) gy[j] = a;
  if (gt) gt[j] = ser.tscale[s] * (double)y[j] * (double)b;
}

// ---------------------------------------------------------------------------
// bootstrap: resample b draws n indices d = xorshift32(wang_hash(seed + b*n +
// i)) % n with replacement; gridding resample b is gridding every original
// sample p with weight (number of times p was drawn) * y[p].
// ---------------------------------------------------------------------------
constexpr int kBootSmemN = 40960;  // int counters in shared memory (160 KB)

template <typename T>
__global__ void __launch_bounds__(1024) k_boot_weights(const T *__restrict__ y, int n, unsigned seed,
                                                       T *__restrict__ wts) {
  extern __shared__ int cnt[];
  const int b = blockIdx.x;
  T *w = wts + (int64_t)b * n;
  const unsigned s0 = seed + (unsigned)b * (unsigned)n;
  if (n <= kBootSmemN) {
    for (int p = threadIdx.x; p < n; p += blockDim.x) cnt[p] = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x)
      atomicAdd(&cnt[boot_draw(s0, (unsigned)i, (unsigned)n)], 1);
    __syncthreads();
    for (int p = threadIdx.x; p < n; p += blockDim.x) w[p] = (T)cnt[p] * y[p];
  } else {
    // w was zeroed; adding identical values y[d] is exact in any order
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const unsigned d = boot_draw(s0, (unsigned)i, (unsigned)n);
      atomicAdd(&w[d], y[d]);
    }
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

