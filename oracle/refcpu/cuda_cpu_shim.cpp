/* Host implementation of the stand-in CUDA runtime / cuFFT used to run the
 * reference library's own sources on the CPU (golden-vector generation only).
 * Compiled by oracle/build_ref.py together with the reference's
 * src/gridding.cu, src/gaussian_filter.cu, src/cuna_kernel.cu,
 * src/cufft_utils.cu, src/utils.cu and src/cuna.cpp, once with
 * -DDOUBLE_PRECISION and once without.
 *
 * It also exports a small extern "C" surface (refcpu_*) so that Python can
 * drive the reference entry points through ctypes.
 */
#include <vector>
#include <map>
#include <utility>
#include "cuda_runtime.h"
#include "cufft.h"

dim3 blockIdx, threadIdx, blockDim, gridDim;

cudaError_t cudaMalloc(void **p, size_t n) {
  *p = calloc(n ? n : 1, 1);
  return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
cudaError_t cudaFree(void *p) { free(p); return cudaSuccess; }
cudaError_t cudaMemcpy(void *d, const void *s, size_t n, cudaMemcpyKind) {
  memmove(d, s, n);
  return cudaSuccess;
}
cudaError_t cudaMemcpyAsync(void *d, const void *s, size_t n, cudaMemcpyKind k,
                            cudaStream_t) {
  return cudaMemcpy(d, s, n, k);
}
cudaError_t cudaMemset(void *d, int v, size_t n) { memset(d, v, n); return cudaSuccess; }
cudaError_t cudaDeviceSynchronize(void) { return cudaSuccess; }
cudaError_t cudaThreadSynchronize(void) { return cudaSuccess; }
cudaError_t cudaStreamSynchronize(cudaStream_t) { return cudaSuccess; }
cudaError_t cudaGetLastError(void) { return cudaSuccess; }
const char *cudaGetErrorString(cudaError_t) { return "cpu stand-in error"; }

float atomicAdd(float *a, float v) { float o = *a; *a = o + v; return o; }
#ifdef DOUBLE_PRECISION
double atomicAdd(double *a, double v) { double o = *a; *a = o + v; return o; }
#endif

/* ---- cuFFT stand-in: unnormalised complex DFT in double precision ---- */
struct CpuFftPlan { int nx, batch, dist; };
static std::map<int, CpuFftPlan> g_plans;
static int g_next_plan = 1;

struct cd { double re, im; };
static inline cd cmul(cd a, cd b) { return cd{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
static void dft_inplace(std::vector<cd> &a, int sign) {
  const size_t n = a.size();
  if (n == 0) return;
  if ((n & (n - 1)) == 0) {
    for (size_t i = 1, j = 0; i < n; ++i) {        /* bit reversal */
      size_t bit = n >> 1;
      for (; j & bit; bit >>= 1) j ^= bit;
      j ^= bit;
      if (i < j) std::swap(a[i], a[j]);
    }
    for (size_t len = 2; len <= n; len <<= 1) {     /* iterative radix-2 */
      for (size_t k = 0; k < len / 2; ++k) {
        double ang = sign * 2.0 * M_PI * (double)k / (double)len;
        cd w{cos(ang), sin(ang)};
        for (size_t i = k; i < n; i += len) {
          cd u = a[i], v = cmul(a[i + len / 2], w);
          a[i] = cd{u.re + v.re, u.im + v.im};
          a[i + len / 2] = cd{u.re - v.re, u.im - v.im};
        }
      }
    }
  } else {
    std::vector<cd> out(n);
    for (size_t k = 0; k < n; ++k) {
      cd s{0, 0};
      for (size_t j = 0; j < n; ++j) {
        size_t q = (j * k) % n;                   /* exact phase reduction */
        double ang = sign * 2.0 * M_PI * (double)q / (double)n;
        cd t = cmul(a[j], cd{cos(ang), sin(ang)});
        s.re += t.re;
        s.im += t.im;
      }
      out[k] = s;
    }
    a.swap(out);
  }
}

template <typename C>
static cufftResult exec_any(cufftHandle h, C *in, C *out, int dir) {
  auto it = g_plans.find(h);
  if (it == g_plans.end()) return CUFFT_INVALID_PLAN;
  const CpuFftPlan &p = it->second;
  std::vector<cd> buf(p.nx);
  for (int b = 0; b < p.batch; ++b) {
    C *src = in + (size_t)b * p.dist, *dst = out + (size_t)b * p.dist;
    for (int i = 0; i < p.nx; ++i) buf[i] = cd{(double)src[i].x, (double)src[i].y};
    dft_inplace(buf, dir == CUFFT_INVERSE ? +1 : -1);
    for (int i = 0; i < p.nx; ++i) {
      dst[i].x = (decltype(dst[i].x))buf[i].re;
      dst[i].y = (decltype(dst[i].y))buf[i].im;
    }
  }
  return CUFFT_SUCCESS;
}

cufftResult cufftPlan1d(cufftHandle *plan, int nx, cufftType, int batch) {
  if (nx <= 0 || batch <= 0) return CUFFT_INVALID_SIZE;
  *plan = g_next_plan++;
  g_plans[*plan] = CpuFftPlan{nx, batch, nx};
  return CUFFT_SUCCESS;
}
cufftResult cufftPlanMany(cufftHandle *plan, int rank, int *n, int *, int istride,
                          int idist, int *, int ostride, int odist, cufftType,
                          int batch) {
  if (rank != 1 || istride != 1 || ostride != 1 || idist != odist) return CUFFT_INVALID_VALUE;
  *plan = g_next_plan++;
  g_plans[*plan] = CpuFftPlan{n[0], batch, idist};
  return CUFFT_SUCCESS;
}
cufftResult cufftSetStream(cufftHandle, cudaStream_t) { return CUFFT_SUCCESS; }
cufftResult cufftExecC2C(cufftHandle h, cufftComplex *i, cufftComplex *o, int d) {
  return exec_any(h, i, o, d);
}
cufftResult cufftExecZ2Z(cufftHandle h, cufftDoubleComplex *i, cufftDoubleComplex *o, int d) {
  return exec_any(h, i, o, d);
}
cufftResult cufftDestroy(cufftHandle h) { g_plans.erase(h); return CUFFT_SUCCESS; }

/* ---- ctypes surface ---- */
#include "cuna.h"
#include "cuna_filter.h"
#include "cuna_gridding.h"

/* defined in the reference's src/cuna_kernel.cu:237 (9 arguments; the header
 * inc/cuna.h:55 declares an 8-argument overload that nothing defines). */
void cunfft_adjoint_raw_async_bootstrap(const dTyp *x, const dTyp *f_data, Complex *f_hat,
                                        const int n, const int ng, const int nbs,
                                        const filter_properties *gpu_fprops,
                                        cudaStream_t stream, const unsigned int seed);

/* copyResultsToCPU, src/cuna_kernel.cu:120-134 (no header declares it) */
void copyResultsToCPU(plan *p);

extern "C" {
int refcpu_dtype_size(void) { return (int)sizeof(dTyp); }

/* generate_filter_properties (src/gaussian_filter.cu:104) and copy it out */
void refcpu_filter_properties(const dTyp *x, int n, int ng, dTyp *b, dTyp *normfac,
                              int *rf, dTyp *E1, dTyp *E2, dTyp *E3) {
  filter_properties *h, *d;
  generate_filter_properties(x, n, ng, &h, &d);
  *b = h->b; *normfac = h->normfac; *rf = h->filter_radius;
  memcpy(E1, h->E1, sizeof(dTyp) * n);
  memcpy(E2, h->E2, sizeof(dTyp) * n);
  memcpy(E3, h->E3, sizeof(dTyp) * h->filter_radius);
  free_filter_properties(d, h);
}

/* fast_gridding (src/gridding.cu:36) alone, launched like performGridding */
void refcpu_fast_gridding(const dTyp *x, const dTyp *y, Complex *f_hat, int n, int ng) {
  filter_properties *h, *d;
  generate_filter_properties(x, n, ng, &h, &d);
  int nblocks = (n + BLOCK_SIZE - 1) / BLOCK_SIZE;
  CUNA_CPU_LAUNCH(nblocks, BLOCK_SIZE, fast_gridding, y, f_hat, x, ng, n, d);
  free_filter_properties(d, h);
}

/* fast_gridding_bootstrap (src/gridding.cu:86) alone */
void refcpu_fast_gridding_bootstrap(const dTyp *x, const dTyp *y, Complex *f_hat, int n,
                                    int ng, int nbs, unsigned seed) {
  filter_properties *h, *d;
  generate_filter_properties(x, n, ng, &h, &d);
  int nblocks = (n * nbs + BLOCK_SIZE - 1) / BLOCK_SIZE;
  CUNA_CPU_LAUNCH(nblocks, BLOCK_SIZE, fast_gridding_bootstrap, y, f_hat, x, ng, n, nbs, d, seed);
  free_filter_properties(d, h);
}

/* cunfft_adjoint_raw (src/cuna_kernel.cu:149) with its filter setup */
void refcpu_adjoint_raw(const dTyp *x, const dTyp *y, Complex *f_hat, int n, int ng) {
  filter_properties *h, *d;
  generate_filter_properties(x, n, ng, &h, &d);
  cunfft_adjoint_raw(x, y, f_hat, n, ng, d);
  free_filter_properties(d, h);
}

/* cunfft_adjoint_raw_async (src/cuna_kernel.cu:188) */
void refcpu_adjoint_raw_async(const dTyp *x, const dTyp *y, Complex *f_hat, int n, int ng) {
  filter_properties *h, *d;
  generate_filter_properties(x, n, ng, &h, &d);
  cunfft_adjoint_raw_async(x, y, f_hat, n, ng, d, (cudaStream_t)0);
  free_filter_properties(d, h);
}

/* init_plan (src/utils.cu:95-178) and cunfft_adjoint_from_plan
 * (src/cuna_kernel.cu:137-145); the results are read back with
 * copyResultsToCPU because from_plan never copies (its flag test at
 * src/cuna_kernel.cu:142 is always false).  f_hat_win is filled when flags
 * ask for the window function. */
void refcpu_plan_adjoint(const dTyp *x, const dTyp *y, int n, int ng, unsigned flags, Complex *f_hat,
                         Complex *f_hat_win) {
  plan *p = (plan *)malloc(sizeof(plan));
  init_plan(p, x, y, n, ng, flags);
  cunfft_adjoint_from_plan(p);
  copyResultsToCPU(p);
  memcpy(f_hat, p->f_hat, sizeof(Complex) * ng);
  if ((flags & CALCULATE_WINDOW_FUNCTION) && f_hat_win) memcpy(f_hat_win, p->f_hat_win, sizeof(Complex) * ng);
  free_plan(p);
}

/* cunfft_adjoint_raw_async_bootstrap (src/cuna_kernel.cu:237) */
void refcpu_adjoint_bootstrap(const dTyp *x, const dTyp *y, Complex *f_hat, int n, int ng,
                              int nbs, unsigned seed) {
  filter_properties *h, *d;
  generate_filter_properties(x, n, ng, &h, &d);
  cunfft_adjoint_raw_async_bootstrap(x, y, f_hat, n, ng, nbs, d, (cudaStream_t)0, seed);
  free_filter_properties(d, h);
}
}
