/* cuna_oracle.c -- CPU oracle for the adjoint-NFFT path.  TEST INFRASTRUCTURE.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs may
 * load this library, and only to verify results or as the timed CPU baseline; the
 * product never routes through it.
 *
 * Contents
 *   1. compat_*   plain-C restatement of the reference library's arithmetic
 *                 (filter precompute, gridding, bootstrap gridding with its hash
 *                 RNG, deconvolution), float and double, each function citing
 *                 the reference file:line it follows.  Pinned against golden
 *                 vectors produced by running the reference's own sources
 *                 (oracle/build_ref.py, tests/golden/make_golden.py).
 *   2. fft_*      unnormalised complex DFT in double precision (the published
 *                 contract of cuFFT CUFFT_INVERSE, which the reference calls at
 *                 src/cuna_kernel.cu:87,172,214,270).
 *   3. accurate_* double-precision restatement of the accurate-mode algorithm
 *                 (periodic Gaussian gridding, Greengard & Lee 2004 kernel
 *                 width, deconvolution, centred output).
 *   4. ndft_*     FP64 direct adjoint NDFT F_k = sum_j y_j exp(+2 pi i k x_j),
 *                 the accuracy oracle.
 *   5. cpu_pipeline_* the reference pipeline (compat math) as a multi-threaded
 *                 CPU program: per-thread private grids + reduction, radix-2
 *                 FFT, deconvolution.  This is the timed CPU baseline.
 *   6. ndft_grad  FP64 direct-sum gradient through the adjoint NDFT.
 *   7. integer steps per sample: the compat cell, filter origin and tap
 *                 range, the bootstrap draws, and accurate mode's 64-bit
 *                 fixed-point phase, cell and fractional cell -- the values
 *                 the GPU must reproduce bit for bit.
 *
 * Build: gcc -O2 -fopenmp -fPIC -shared -ffp-contract=off (oracle/oracle.py).
 * -ffp-contract=off keeps float rounding identical on x86 and Arm; where the
 * reference's nvcc build contracts a*b-c into one fused multiply-add (the cell
 * offsets u and eps of src/gaussian_filter.cu:213-217) the restatement calls
 * fma/fmaf explicitly.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <limits.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ------------------------------------------------------------------------ */
/* helpers                                                                   */
/* ------------------------------------------------------------------------ */

/* C conversion (int)v of a double as the GPU performs it: truncation toward
 * zero, saturating at the int range.  A NaN double converts to INT_MIN
 * (measured on sm_103a for the code nvcc emits for (int) of a double). */
static int trunc_sat_int(double v) {
  if (v != v) return INT_MIN;
  if (v >= 2147483647.0) return INT_MAX;
  if (v <= -2147483648.0) return INT_MIN;
  return (int)v;
}

/* The same for a float source: saturating truncation, and a NaN float
 * converts to 0 (measured on sm_103a for (int) of a float). */
static int trunc_sat_int_f32(float v) {
  if (v != v) return 0;
  return trunc_sat_int((double)v);
}

/* wang_hash, src/gridding.cu:67-74 */
uint32_t cuna_oracle_wang_hash(uint32_t s) {
  s = (s ^ 61u) ^ (s >> 16);
  s *= 9u;
  s = s ^ (s >> 4);
  s *= 0x27d4eb2du;
  s = s ^ (s >> 15);
  return s;
}

/* rand_XORSHIFT, src/gridding.cu:76-82 */
uint32_t cuna_oracle_xorshift(uint32_t s) {
  s ^= (s << 13);
  s ^= (s >> 17);
  s ^= (s << 5);
  return s;
}

/* bootstrap draw d for global thread index i, src/gridding.cu:92-103 */
int cuna_oracle_bootstrap_draw(uint32_t seed, int i, int n) {
  return (int)(cuna_oracle_xorshift(cuna_oracle_wang_hash(seed + (uint32_t)i)) % (uint32_t)n);
}

/* cell j = (int)((x + 0.5) * (ng - 1)), evaluated in double because of the
 * 0.5 literal (src/gridding.cu:43, :93); `clamp` applies :44-45. */
int cuna_oracle_compat_cell(double x, int ng, int clamp) {
  int j = trunc_sat_int((x + 0.5) * (double)(ng - 1));
  if (clamp) {
    if (j >= ng) j = ng - 1;
    if (j < 0) j = 0;
  }
  return j;
}

/* ------------------------------------------------------------------------ */
/* 1. compat restatement, float (libcunaf) and double (libcunad)             */
/* ------------------------------------------------------------------------ */

/* filter radius: src/gaussian_filter.cu:29-33 */
#define RF_F32 6
#define RF_F64 12

/* generate_filter_properties host part, src/gaussian_filter.cu:125-134,
 * and set_gpu_filter_properties, src/gaussian_filter.cu:204-228 (float). */
void cuna_oracle_compat_filter_f32(const float *x, int n, int ng, float *b_out,
                                   float *normfac_out, int *rf_out, float *E1,
                                   float *E2, float *E3) {
  const int rf = RF_F32;
  float R = (float)ng / (float)n;                     /* ((dTyp) ng) / n    */
  float q = 2.0f * R / (2.0f * R - 1.0f);             /* float subexpression */
  float b = (float)((double)q * ((double)rf / M_PI)); /* * (FILTER_RADIUS/PI) */
  *b_out = b;
  *normfac_out = (float)sqrt(2.0 * M_PI);
  *rf_out = rf;
  const float ngf = (float)ng;
  for (int i = 0; i < n; ++i) {
    int u = (int)fmaf(ngf, x[i], -(float)rf);        /* Ngrid*x - radius   */
    float eps = fmaf(ngf, x[i], -(float)u);           /* Ngrid*x - u        */
    float eps2 = eps / b;
    E1[i] = expf(-eps * eps2) / sqrtf((float)(M_PI * (double)b));
    E2[i] = expf(2.0f * eps2);
  }
  for (int m = 0; m < rf; ++m) E3[m] = expf((float)(-m * m) / b);
}

void cuna_oracle_compat_filter_f64(const double *x, int n, int ng, double *b_out,
                                   double *normfac_out, int *rf_out, double *E1,
                                   double *E2, double *E3) {
  const int rf = RF_F64;
  double R = (double)ng / (double)n;
  double b = 2.0 * R / (2.0 * R - 1.0) * ((double)rf / M_PI);
  *b_out = b;
  *normfac_out = sqrt(2.0 * M_PI);
  *rf_out = rf;
  for (int i = 0; i < n; ++i) {
    int u = (int)fma((double)ng, x[i], -(double)rf);
    double eps = fma((double)ng, x[i], -(double)u);
    double eps2 = eps / b;
    E1[i] = exp(-eps * eps2) / sqrt(M_PI * b);
    E2[i] = exp(2.0 * eps2);
  }
  for (int m = 0; m < rf; ++m) E3[m] = exp((double)(-m * m) / b);
}

/* fast_gridding, src/gridding.cu:36-65, with filter() of
 * src/gaussian_filter.cu:264-273.  grid_re (double, length ng) accumulates
 * exactly in double; the reference accumulates in dTyp with atomics. */
void cuna_oracle_compat_grid_f32(const float *x, const float *y, int n, int ng,
                                 const float *E1, const float *E2, const float *E3,
                                 int rf, double *grid_re) {
  for (int i = 0; i < n; ++i) {
    int j = cuna_oracle_compat_cell((double)x[i], ng, 1);
    float val = y ? y[i] : 1.0f;
    int ms = -rf + 1, me = rf;
    if (j + ms < 0) ms = -j;
    if (j + me > ng) me = ng - j;
    for (int m = ms; m < me; ++m) {
      float w = E1[i] * powf(E2[i], (float)m) * E3[m < 0 ? -m : m];
      grid_re[j + m] += (double)(val * w);
    }
  }
}

void cuna_oracle_compat_grid_f64(const double *x, const double *y, int n, int ng,
                                 const double *E1, const double *E2, const double *E3,
                                 int rf, double *grid_re) {
  for (int i = 0; i < n; ++i) {
    int j = cuna_oracle_compat_cell(x[i], ng, 1);
    double val = y ? y[i] : 1.0;
    int ms = -rf + 1, me = rf;
    if (j + ms < 0) ms = -j;
    if (j + me > ng) me = ng - j;
    for (int m = ms; m < me; ++m) {
      double w = E1[i] * pow(E2[i], (double)m) * E3[m < 0 ? -m : m];
      grid_re[j + m] += val * w;
    }
  }
}

/* fast_gridding_bootstrap, src/gridding.cu:86-117: position from x[i % n],
 * value and filter coefficients from the drawn index d, no clamp of j,
 * slab (i / n) * ng.  grid_re has nbs * ng entries. */
void cuna_oracle_compat_grid_bootstrap_f32(const float *x, const float *y, int n, int ng,
                                           int nbs, const float *E1, const float *E2,
                                           const float *E3, int rf, uint32_t seed,
                                           double *grid_re) {
  for (int i = 0; i < n * nbs; ++i) {
    int d = i % n;
    int j = cuna_oracle_compat_cell((double)x[d], ng, 0);
    float val = 1.0f;
    if (y) {
      d = cuna_oracle_bootstrap_draw(seed, i, n);
      val = y[d];
    }
    int ms = -rf + 1, me = rf;
    if (j + ms < 0) ms = -j;
    if (j + me > ng) me = ng - j;
    int64_t off = (int64_t)(i / n) * ng;
    for (int m = ms; m < me; ++m) {
      float w = E1[d] * powf(E2[d], (float)m) * E3[m < 0 ? -m : m];
      grid_re[off + j + m] += (double)(val * w);
    }
  }
}

void cuna_oracle_compat_grid_bootstrap_f64(const double *x, const double *y, int n, int ng,
                                           int nbs, const double *E1, const double *E2,
                                           const double *E3, int rf, uint32_t seed,
                                           double *grid_re) {
  for (int i = 0; i < n * nbs; ++i) {
    int d = i % n;
    int j = cuna_oracle_compat_cell(x[d], ng, 0);
    double val = 1.0;
    if (y) {
      d = cuna_oracle_bootstrap_draw(seed, i, n);
      val = y[d];
    }
    int ms = -rf + 1, me = rf;
    if (j + ms < 0) ms = -j;
    if (j + me > ng) me = ng - j;
    int64_t off = (int64_t)(i / n) * ng;
    for (int m = ms; m < me; ++m) {
      double w = E1[d] * pow(E2[d], (double)m) * E3[m < 0 ? -m : m];
      grid_re[off + j + m] += val * w;
    }
  }
}

/* deconvolution factor of normalize / normalize_bootstrap,
 * src/gaussian_filter.cu:278-302: normfac * exp(K*K*b*0.25), K = k/ng. */
void cuna_oracle_compat_norm_f32(int ng, float b, float normfac, double *fac) {
  for (int k = 0; k < ng; ++k) {
    float K = (float)k / (float)ng;
    float e = expf((float)((double)(K * K * b) * 0.25));
    fac[k] = (double)(normfac * e);
  }
}

void cuna_oracle_compat_norm_f64(int ng, double b, double normfac, double *fac) {
  for (int k = 0; k < ng; ++k) {
    double K = (double)k / (double)ng;
    fac[k] = normfac * exp(K * K * b * 0.25);
  }
}

/* ------------------------------------------------------------------------ */
/* 2. unnormalised complex DFT (double), interleaved re/im                   */
/* ------------------------------------------------------------------------ */

/* In-place DFT of length n, sign +1 (CUFFT_INVERSE) or -1.  Iterative radix-2
 * for powers of two, direct O(n^2) sum with exact index reduction otherwise. */
void cuna_oracle_fft(double *a, int64_t n, int sign) {
  if (n <= 1) return;
  if ((n & (n - 1)) == 0) {
    for (int64_t i = 1, j = 0; i < n; ++i) {
      int64_t bit = n >> 1;
      for (; j & bit; bit >>= 1) j ^= bit;
      j ^= bit;
      if (i < j) {
        double t0 = a[2 * i], t1 = a[2 * i + 1];
        a[2 * i] = a[2 * j]; a[2 * i + 1] = a[2 * j + 1];
        a[2 * j] = t0; a[2 * j + 1] = t1;
      }
    }
    for (int64_t len = 2; len <= n; len <<= 1) {
      int64_t h = len / 2;
      for (int64_t k = 0; k < h; ++k) {
        double ang = sign * 2.0 * M_PI * (double)k / (double)len;
        double wr = cos(ang), wi = sin(ang);
        for (int64_t i = k; i < n; i += len) {
          double ur = a[2 * i], ui = a[2 * i + 1];
          double xr = a[2 * (i + h)], xi = a[2 * (i + h) + 1];
          double vr = xr * wr - xi * wi, vi = xr * wi + xi * wr;
          a[2 * i] = ur + vr; a[2 * i + 1] = ui + vi;
          a[2 * (i + h)] = ur - vr; a[2 * (i + h) + 1] = ui - vi;
        }
      }
    }
  } else {
    double *out = (double *)malloc(sizeof(double) * 2 * n);
    for (int64_t k = 0; k < n; ++k) {
      double sr = 0, si = 0;
      for (int64_t j = 0; j < n; ++j) {
        int64_t q = (j * k) % n;
        double ang = sign * 2.0 * M_PI * (double)q / (double)n;
        double c = cos(ang), s = sin(ang);
        sr += a[2 * j] * c - a[2 * j + 1] * s;
        si += a[2 * j] * s + a[2 * j + 1] * c;
      }
      out[2 * k] = sr; out[2 * k + 1] = si;
    }
    memcpy(a, out, sizeof(double) * 2 * n);
    free(out);
  }
}

/* ------------------------------------------------------------------------ */
/* 3. accurate mode (double restatement)                                     */
/* ------------------------------------------------------------------------ */

/* Gaussian kernel variance in grid cells^2 for half-width m and oversampling
 * R: tau = m R / (4 pi (R - 1/2)), Greengard & Lee, SIAM Rev. 46 (2004),
 * eq. 9 rewritten in units of the oversampled grid spacing. */
double cuna_oracle_accurate_tau(int m, double R) {
  return (double)m * R / (4.0 * M_PI * (R - 0.5));
}

/* Accurate adjoint NFFT in double:
 *   x_j = (t_j - t0)/T - 1/2,  F_k = sum_j y_j exp(+2 pi i k x_j),
 *   k = -nf/2 .. nf/2-1 stored at index k + nf/2 (interleaved re/im).
 * Periodic grid of ng = R*nf cells, taps d = -m+1..m around floor(s_j). */
void cuna_oracle_accurate_adjoint(const double *t, const double *y, int64_t n,
                                  double t0, double T, int64_t nf, int R, int m,
                                  double *F) {
  const int64_t ng = (int64_t)R * nf;
  const double tau = cuna_oracle_accurate_tau(m, (double)R);
  double *g = (double *)calloc((size_t)(2 * ng), sizeof(double));
  const double scale = (double)ng / T;
  for (int64_t j = 0; j < n; ++j) {
    double s = (t[j] - t0) * scale;
    double fb = floor(s);
    double frac = s - fb;
    int64_t b = (int64_t)fb % ng;
    if (b < 0) b += ng;
    for (int d = -m + 1; d <= m; ++d) {
      double dd = (double)d - frac;
      int64_t c = (b + d) % ng;
      if (c < 0) c += ng;
      g[2 * c] += y[j] * exp(-dd * dd / (4.0 * tau));
    }
  }
  cuna_oracle_fft(g, ng, +1);
  for (int64_t q = 0; q < nf; ++q) {
    int64_t k = q - nf / 2;
    int64_t c = (k % ng + ng) % ng;
    double kk = (double)k / (double)ng;
    double psi = sqrt(4.0 * M_PI * tau) * exp(-4.0 * M_PI * M_PI * tau * kk * kk);
    double sgn = (k & 1) ? -1.0 : 1.0;
    F[2 * q] = sgn * g[2 * c] / psi;
    F[2 * q + 1] = sgn * g[2 * c + 1] / psi;
  }
  free(g);
}

/* ------------------------------------------------------------------------ */
/* 4. FP64 direct adjoint NDFT                                               */
/* ------------------------------------------------------------------------ */

/* F[q] = sum_j y_j exp(+2 pi i k_q x_j), x_j = (t_j - t0)/T - 1/2, for an
 * arbitrary list of integer frequencies k_q.  y may be complex (yi != NULL).
 * The phase k*x is reduced to [-1/2, 1/2) before the sine/cosine. */
void cuna_oracle_ndft(const double *t, const double *yr, const double *yi, int64_t n,
                      double t0, double T, const int64_t *k, int64_t nk, double *F) {
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t q = 0; q < nk; ++q) {
    double sr = 0.0, si = 0.0, cr = 0.0, ci = 0.0; /* Kahan compensation */
    const double kq = (double)k[q];
    for (int64_t j = 0; j < n; ++j) {
      double x = (t[j] - t0) / T - 0.5;
      double ph = kq * x;
      ph -= nearbyint(ph);
      double c = cos(2.0 * M_PI * ph), s = sin(2.0 * M_PI * ph);
      double a = yr[j], bb = yi ? yi[j] : 0.0;
      double tr = a * c - bb * s - cr;
      double vr = sr + tr;
      cr = (vr - sr) - tr;
      sr = vr;
      double ti = a * s + bb * c - ci;
      double vi = si + ti;
      ci = (vi - si) - ti;
      si = vi;
    }
    F[2 * q] = sr;
    F[2 * q + 1] = si;
  }
}

/* ------------------------------------------------------------------------ */
/* 5. reference pipeline on the CPU (timed baseline), float, compat math     */
/* ------------------------------------------------------------------------ */

/* in-place radix-2 inverse FFT in float (interleaved), parallel butterflies */
static void fft_f32_inplace(float *a, int64_t n, const float *tw) {
  for (int64_t i = 1, j = 0; i < n; ++i) {
    int64_t bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) {
      float t0 = a[2 * i], t1 = a[2 * i + 1];
      a[2 * i] = a[2 * j]; a[2 * i + 1] = a[2 * j + 1];
      a[2 * j] = t0; a[2 * j + 1] = t1;
    }
  }
  for (int64_t len = 2; len <= n; len <<= 1) {
    const int64_t h = len / 2, step = n / len;
#pragma omp parallel for schedule(static)
    for (int64_t blk = 0; blk < n / len; ++blk) {
      int64_t i0 = blk * len;
      for (int64_t k = 0; k < h; ++k) {
        float wr = tw[2 * k * step], wi = tw[2 * k * step + 1];
        int64_t i = i0 + k;
        float ur = a[2 * i], ui = a[2 * i + 1];
        float xr = a[2 * (i + h)], xi = a[2 * (i + h) + 1];
        float vr = xr * wr - xi * wi, vi = xr * wi + xi * wr;
        a[2 * i] = ur + vr; a[2 * i + 1] = ui + vi;
        a[2 * (i + h)] = ur - vr; a[2 * (i + h) + 1] = ui - vi;
      }
    }
  }
}

/* Number of threads the CPU pipeline uses (OpenMP default team size). */
int cuna_oracle_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* One adjoint NFFT of the reference pipeline (float, compat math, R_f = 6):
 * filter precompute, gridding into per-thread private grids + reduction,
 * unnormalised inverse FFT, deconvolution.  Output f_hat: ng complex floats.
 * ng must be a power of two.  Scratch `work` holds nthreads*ng floats. */
void cuna_oracle_cpu_pipeline_f32(const float *x, const float *y, int n, int ng,
                                  float *f_hat, float *E1, float *E2, float *work,
                                  const float *tw) {
  const int rf = RF_F32;
  float R = (float)ng / (float)n;
  float q = 2.0f * R / (2.0f * R - 1.0f);
  const float b = (float)((double)q * ((double)rf / M_PI));
  const float normfac = (float)sqrt(2.0 * M_PI);
  float E3[RF_F32];
  for (int m = 0; m < rf; ++m) E3[m] = expf((float)(-m * m) / b);
  const float ngf = (float)ng;
#pragma omp parallel
  {
#ifdef _OPENMP
    const int tid = omp_get_thread_num(), nt = omp_get_num_threads();
#else
    const int tid = 0, nt = 1;
#endif
    float *priv = work + (size_t)tid * ng;
    memset(priv, 0, sizeof(float) * ng);
#pragma omp for schedule(static)
    for (int i = 0; i < n; ++i) {
      int u = (int)fmaf(ngf, x[i], -(float)rf);
      float eps = fmaf(ngf, x[i], -(float)u);
      float eps2 = eps / b;
      E1[i] = expf(-eps * eps2) / sqrtf((float)(M_PI * (double)b));
      E2[i] = expf(2.0f * eps2);
      int j = cuna_oracle_compat_cell((double)x[i], ng, 1);
      int ms = -rf + 1, me = rf;
      if (j + ms < 0) ms = -j;
      if (j + me > ng) me = ng - j;
      for (int m = ms; m < me; ++m)
        priv[j + m] += y[i] * (E1[i] * powf(E2[i], (float)m) * E3[m < 0 ? -m : m]);
    }
#pragma omp for schedule(static)
    for (int c = 0; c < ng; ++c) {
      float s = 0.0f;
      for (int t = 0; t < nt; ++t) s += work[(size_t)t * ng + c];
      f_hat[2 * c] = s;
      f_hat[2 * c + 1] = 0.0f;
    }
  }
  fft_f32_inplace(f_hat, ng, tw);
#pragma omp parallel for schedule(static)
  for (int k = 0; k < ng; ++k) {
    float K = (float)k / ngf;
    float fac = normfac * expf((float)((double)(K * K * b) * 0.25));
    f_hat[2 * k] *= fac;
    f_hat[2 * k + 1] *= fac;
  }
}

/* twiddles e^{+2 pi i k / n}, k < n/2, for cuna_oracle_cpu_pipeline_f32 */
void cuna_oracle_cpu_twiddles_f32(int64_t n, float *tw) {
  for (int64_t k = 0; k < n / 2; ++k) {
    double ang = 2.0 * M_PI * (double)k / (double)n;
    tw[2 * k] = (float)cos(ang);
    tw[2 * k + 1] = (float)sin(ang);
  }
}

/* ------------------------------------------------------------------------ */
/* 6. FP64 direct-sum gradient of a real loss through the adjoint NDFT       */
/* ------------------------------------------------------------------------ */

/* For F_q = sum_j y_j exp(+2 pi i k_q x_j), x_j = (t_j - t0)/T - 1/2, and a
 * real loss with g_q = dL/dRe F_q + i dL/dIm F_q (interleaved re/im):
 *   dL/dy_j = Re sum_q conj(g_q) exp(2 pi i k_q x_j)
 *   dL/dt_j = Re sum_q conj(g_q) y_j (2 pi i k_q / T) exp(2 pi i k_q x_j)  */
void cuna_oracle_ndft_grad(const double *t, const double *y, int64_t n, double t0, double T,
                           const int64_t *k, const double *g, int64_t nk, double *gy, double *gt) {
#pragma omp parallel for schedule(static)
  for (int64_t j = 0; j < n; ++j) {
    const double x = (t[j] - t0) / T - 0.5;
    double sy = 0.0, st = 0.0;
    for (int64_t q = 0; q < nk; ++q) {
      double ph = (double)k[q] * x;
      ph -= nearbyint(ph);
      const double c = cos(2.0 * M_PI * ph), s = sin(2.0 * M_PI * ph);
      const double gr = g[2 * q], gi = g[2 * q + 1];
      /* conj(g) e^{i phi} = (gr c + gi s) + i (gr s - gi c) */
      const double re = gr * c + gi * s, im = gr * s - gi * c;
      sy += re;
      st += -im * (double)k[q]; /* Re(i k (re + i im)) = -k im */
    }
    gy[j] = sy;
    gt[j] = y[j] * 2.0 * M_PI / T * st;
  }
}

/* ------------------------------------------------------------------------ */
/* 7. integer steps, per sample (checkers of the device's integer outputs)   */
/* ------------------------------------------------------------------------ */

/* Tap range [ms, me) of cell j, src/gridding.cu:53-58 / :105-110.  The
 * reference forms j + mend in int arithmetic, which overflows (and then
 * writes out of bounds) for |j| near 2^31; the drop-in library treats any
 * |j| > 2^30 as a sample without taps, and so does this restatement.  An
 * empty range is reported as (0, 0). */
static void compat_tap_range(int j, int ng, int rf, int *ms_out, int *me_out) {
  int ms = -rf + 1, me = rf;
  if (j > (1 << 30) || j < -(1 << 30)) {
    *ms_out = 0;
    *me_out = 0;
    return;
  }
  if (j + ms < 0) ms = -j;
  if (j + me > ng) me = ng - j;
  if (ms >= me) ms = me = 0;
  *ms_out = ms;
  *me_out = me;
}

/* Per sample i: cell j (src/gridding.cu:43-45, clamped when `clamp`, as
 * fast_gridding; unclamped as fast_gridding_bootstrap, :93-95), filter
 * origin u = (int)(ng*x - R_f) (src/gaussian_filter.cu:213; nvcc contracts
 * the product and difference into one fused multiply-add, so the restatement
 * rounds once) and the tap range [ms, me).  Any output may be NULL. */
void cuna_oracle_compat_taps_f32(const float *x, int n, int ng, int clamp, int *j_out, int *u_out,
                                 int *ms_out, int *me_out) {
  const int rf = RF_F32;
  for (int i = 0; i < n; ++i) {
    const int j = cuna_oracle_compat_cell((double)x[i], ng, clamp);
    int ms, me;
    compat_tap_range(j, ng, rf, &ms, &me);
    if (j_out) j_out[i] = j;
    if (u_out) u_out[i] = trunc_sat_int_f32(fmaf((float)ng, x[i], -(float)rf));
    if (ms_out) ms_out[i] = ms;
    if (me_out) me_out[i] = me;
  }
}

void cuna_oracle_compat_taps_f64(const double *x, int n, int ng, int clamp, int *j_out, int *u_out,
                                 int *ms_out, int *me_out) {
  const int rf = RF_F64;
  for (int i = 0; i < n; ++i) {
    const int j = cuna_oracle_compat_cell(x[i], ng, clamp);
    int ms, me;
    compat_tap_range(j, ng, rf, &ms, &me);
    if (j_out) j_out[i] = j;
    if (u_out) u_out[i] = trunc_sat_int(fma((double)ng, x[i], -(double)rf));
    if (ms_out) ms_out[i] = ms;
    if (me_out) me_out[i] = me;
  }
}

/* All draws of nbs resamples: d[i] for i < n*nbs, src/gridding.cu:101. */
void cuna_oracle_bootstrap_draws(uint32_t seed, int n, int nbs, int *d) {
  const int64_t total = (int64_t)n * nbs;
  for (int64_t i = 0; i < total; ++i)
    d[i] = (int)(cuna_oracle_xorshift(cuna_oracle_wang_hash(seed + (uint32_t)i)) % (uint32_t)n);
}

/* Accurate mode's grid-index reduction (no reference counterpart: the
 * reference takes x already scaled to [-1/2, 1/2]).  The phase of time t is
 * the unsigned 64-bit fixed-point number S = frac((t - t0)/T) 2^64, formed as
 * (t A - t0 A) mod 2^64 with A = 2^64/T held as a 64-bit significand mA and
 * a binary exponent eA, each product t*A truncated toward zero in magnitude
 * and negated in two's complement for negative t.  Then cell =
 * floor(S ng / 2^64) and the fractional cell is the low 64 bits of S ng.
 * Written from that definition with 128-bit integers. */
static uint64_t phase_times_ref(double t, uint64_t mA, int eA) {
  uint64_t u;
  memcpy(&u, &t, 8);
  const int ex = (int)((u >> 52) & 0x7FF);
  if (ex == 0x7FF) return 0;
  uint64_t mt = u & 0x000FFFFFFFFFFFFFull;
  int et;
  if (ex == 0) {
    et = -1074;
  } else {
    mt |= 0x0010000000000000ull;
    et = ex - 1075;
  }
  /* |t| A = mt mA 2^(et + eA), a product of up to 117 bits */
  const unsigned __int128 prod = (unsigned __int128)mt * mA;
  const int sh = et + eA;
  uint64_t r;
  if (sh >= 64) r = 0;                                  /* a multiple of 2^64 */
  else if (sh >= 0) r = (uint64_t)(prod << sh);         /* mod 2^64 */
  else if (sh > -128) r = (uint64_t)(prod >> (-sh));    /* truncation */
  else r = 0;
  return (u >> 63) ? (uint64_t)(0 - r) : r;
}

void cuna_oracle_phase_setup(double t0, double T, uint64_t *mA_out, int *eA_out, uint64_t *B_out) {
  uint64_t u;
  memcpy(&u, &T, 8);
  const int ex = (int)((u >> 52) & 0x7FF);
  uint64_t mT = u & 0x000FFFFFFFFFFFFFull;
  int eT;
  if (ex == 0) {
    eT = -1074;
    while (!(mT & 0x0010000000000000ull)) {
      mT <<= 1;
      --eT;
    }
  } else {
    mT |= 0x0010000000000000ull;
    eT = ex - 1075;
  }
  /* 2^64 / T = floor(2^116 / mT) 2^(64 - 116 - eT), the significand kept
   * below 2^64 */
  unsigned __int128 q = ((unsigned __int128)1 << 116) / mT;
  int eA = 64 - 116 - eT;
  if (q >> 64) {
    q >>= 1;
    eA += 1;
  }
  *mA_out = (uint64_t)q;
  *eA_out = eA;
  *B_out = phase_times_ref(t0, (uint64_t)q, eA);
}

/* Per sample: S, the cell, and the fractional cell as the float path stores
 * it (the top 24 bits of the low word, an exact 24-bit integer) and as the
 * double path stores it (the top 53 bits).  Any output may be NULL. */
void cuna_oracle_phases(const double *t, int64_t n, double t0, double T, int64_t ng, uint64_t *S_out,
                        int *cell_out, uint32_t *frac24_out, uint64_t *frac53_out) {
  uint64_t mA, B;
  int eA;
  cuna_oracle_phase_setup(t0, T, &mA, &eA, &B);
  for (int64_t i = 0; i < n; ++i) {
    const uint64_t S = phase_times_ref(t[i], mA, eA) - B;
    const unsigned __int128 p = (unsigned __int128)S * (uint64_t)ng;
    const uint64_t lo = (uint64_t)p;
    if (S_out) S_out[i] = S;
    if (cell_out) cell_out[i] = (int)(p >> 64);
    if (frac24_out) frac24_out[i] = (uint32_t)(lo >> 40);
    if (frac53_out) frac53_out[i] = lo >> 11;
  }
}
