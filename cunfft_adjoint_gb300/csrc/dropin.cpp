// dropin.cpp -- the CUNA v1.3 API (include/cuna.h, cuna_filter.h,
// cuna_utils.h) over the GB300 core library.  Compiled twice: without
// DOUBLE_PRECISION into libcunaf.so and with it into libcunad.so, exporting
// the same C++ linkage names as the reference's two libraries.
//
// Error behaviour follows the reference: a failing CUDA or library call
// prints a message and terminates the process (reference
// inc/cuna_typedefs.h:80-89, src/cufft_utils.cu:78-83).  The extern "C"
// cuna2_* functions underneath return status codes instead.
#include <string.h>
#include <time.h>
#include "../../include/cuna.h"
#include "../../include/cuna2.h"
#include "../../include/cuna_filter.h"
#include "../../include/cuna_utils.h"
#include "../../include/cufft_utils.h"

#ifdef DOUBLE_PRECISION
#define CUNA2_FN(name) cuna2_##name##_f64
typedef cuna2_filter_properties_f64 fp2_t;
static const int kFilterRadius = 12;
#else
#define CUNA2_FN(name) cuna2_##name##_f32
typedef cuna2_filter_properties_f32 fp2_t;
static const int kFilterRadius = 6;
#endif

static_assert(sizeof(filter_properties) == sizeof(fp2_t), "filter_properties layout");
static_assert(sizeof(plan) == 96, "plan layout");

static void cuna_check(int status, const char *where) {
  if (status != CUNA2_SUCCESS) {
    fprintf(stderr, "CUNA ERROR in %s: %s (%s)\n", where, cuna2_last_error(), cuna2_status_string(status));
    exit(status);
  }
}

static const fp2_t *as2(const filter_properties *f) { return reinterpret_cast<const fp2_t *>(f); }
static fp2_t *as2(filter_properties *f) { return reinterpret_cast<fp2_t *>(f); }

// ---------------------------------------------------------------------------
// filter setup
// ---------------------------------------------------------------------------
void generate_pinned_filter_properties(const dTyp *x, const int n, const int ng, filter_properties *h_fprops,
                                       filter_properties *d_fprops, cudaStream_t stream) {
  cuna_check(CUNA2_FN(compat_filter)(x, n, ng, as2(h_fprops), as2(d_fprops), stream),
             "generate_pinned_filter_properties");
}

void generate_filter_properties(const dTyp *x, const int n, const int ng, filter_properties **fprops_host,
                                filter_properties **fprops_device) {
  filter_properties *h = (filter_properties *)malloc(sizeof(filter_properties));
  if (!h) {
    fprintf(stderr, "CUNA ERROR: out of host memory\n");
    exit(EXIT_FAILURE);
  }
  memset(h, 0, sizeof *h);
  checkCudaErrors(cudaMalloc((void **)fprops_device, sizeof(filter_properties)));
  checkCudaErrors(cudaMalloc((void **)&h->E1, sizeof(dTyp) * (n > 0 ? n : 1)));
  checkCudaErrors(cudaMalloc((void **)&h->E2, sizeof(dTyp) * (n > 0 ? n : 1)));
  checkCudaErrors(cudaMalloc((void **)&h->E3, sizeof(dTyp) * kFilterRadius));
  *fprops_host = h;
  cuna_check(CUNA2_FN(compat_filter)(x, n, ng, as2(h), as2(*fprops_device), (cudaStream_t)0),
             "generate_filter_properties");
  checkCudaErrors(cudaDeviceSynchronize());
}

void set_filter_properties(plan *p) {
  p->filter_radius = kFilterRadius;
  generate_filter_properties(p->g_x_data, p->Ndata, p->Ngrid, &p->fprops_host, &p->fprops_device);
}

void free_filter_properties(filter_properties *d_fp, filter_properties *fp) {
  checkCudaErrors(cudaFree(fp->E1));
  checkCudaErrors(cudaFree(fp->E2));
  checkCudaErrors(cudaFree(fp->E3));
  checkCudaErrors(cudaFree(d_fp));
  free(fp);
}

// ---------------------------------------------------------------------------
// transforms
// ---------------------------------------------------------------------------
void cunfft_adjoint_raw(const dTyp *x, const dTyp *f_data, Complex *f_hat, const int n, const int ng,
                        const filter_properties *gpu_fprops) {
  cuna_check(CUNA2_FN(compat_adjoint)(x, f_data, f_hat, n, ng, as2(gpu_fprops), (cudaStream_t)0),
             "cunfft_adjoint_raw");
}

void cunfft_adjoint_raw_async(const dTyp *x, const dTyp *f_data, Complex *f_hat, const int n, const int ng,
                              const filter_properties *gpu_fprops, cudaStream_t stream) {
  cuna_check(CUNA2_FN(compat_adjoint)(x, f_data, f_hat, n, ng, as2(gpu_fprops), stream),
             "cunfft_adjoint_raw_async");
}

void cunfft_adjoint_raw_async_bootstrap(const dTyp *x, const dTyp *f_data, Complex *f_hat, const int n,
                                        const int ng, const int nbs, const filter_properties *gpu_fprops,
                                        cudaStream_t stream, const unsigned int seed) {
  cuna_check(CUNA2_FN(compat_bootstrap)(x, f_data, f_hat, n, ng, nbs, as2(gpu_fprops), seed, stream),
             "cunfft_adjoint_raw_async_bootstrap");
}

void cunfft_adjoint_raw_async_bootstrap(const dTyp *x, const dTyp *f_data, Complex *f_hat, const int n,
                                        const int ng, const int nbs, const filter_properties *gpu_fprops,
                                        cudaStream_t stream) {
  cunfft_adjoint_raw_async_bootstrap(x, f_data, f_hat, n, ng, nbs, gpu_fprops, stream, 0u);
}

// ---------------------------------------------------------------------------
// plans
// ---------------------------------------------------------------------------
void init_plan(plan *p, const dTyp *x, const dTyp *f, int Ndata, int Ngrid, unsigned int plan_flags) {
  memset(p, 0, sizeof *p);
  p->Ndata = Ndata;
  p->Ngrid = Ngrid;
  p->flags = plan_flags;
  p->x_data = (dTyp *)malloc(sizeof(dTyp) * (Ndata > 0 ? Ndata : 1));
  p->f_data = f ? (dTyp *)malloc(sizeof(dTyp) * (Ndata > 0 ? Ndata : 1)) : NULL;
  p->f_hat = (Complex *)malloc(sizeof(Complex) * Ngrid);
  if (!p->x_data || !p->f_hat || (f && !p->f_data)) {
    fprintf(stderr, "CUNA ERROR: out of host memory\n");
    exit(EXIT_FAILURE);
  }
  memcpy(p->x_data, x, sizeof(dTyp) * Ndata);
  if (f)
    memcpy(p->f_data, f, sizeof(dTyp) * Ndata);
  else  // the reference prints this and continues with undefined values; here f == NULL grids y = 1
    fprintf(stderr, "you passed a NULL pointer to init_plan.\n");
  checkCudaErrors(cudaMalloc((void **)&p->g_x_data, sizeof(dTyp) * (Ndata > 0 ? Ndata : 1)));
  checkCudaErrors(cudaMalloc((void **)&p->g_f_hat, sizeof(Complex) * Ngrid));
  checkCudaErrors(cudaMemset(p->g_f_hat, 0, sizeof(Complex) * Ngrid));
  if (f) {
    checkCudaErrors(cudaMalloc((void **)&p->g_f_data, sizeof(dTyp) * (Ndata > 0 ? Ndata : 1)));
    checkCudaErrors(cudaMemcpy(p->g_f_data, p->f_data, sizeof(dTyp) * Ndata, cudaMemcpyHostToDevice));
  }
  if (p->flags & CALCULATE_WINDOW_FUNCTION) {
    p->f_hat_win = (Complex *)malloc(sizeof(Complex) * Ngrid);
    checkCudaErrors(cudaMalloc((void **)&p->g_f_hat_win, sizeof(Complex) * Ngrid));
    checkCudaErrors(cudaMemset(p->g_f_hat_win, 0, sizeof(Complex) * Ngrid));
  }
  checkCudaErrors(cudaMemcpy(p->g_x_data, p->x_data, sizeof(dTyp) * Ndata, cudaMemcpyHostToDevice));
  checkCudaErrors(cudaDeviceSynchronize());
  set_filter_properties(p);
}

void free_plan(plan *p) {
  free(p->f_hat);
  free(p->x_data);
  free(p->f_data);
  free_filter_properties(p->fprops_device, p->fprops_host);
  checkCudaErrors(cudaFree(p->g_f_hat));
  checkCudaErrors(cudaFree(p->g_f_data));
  checkCudaErrors(cudaFree(p->g_x_data));
  if (p->flags & CALCULATE_WINDOW_FUNCTION) {
    checkCudaErrors(cudaFree(p->g_f_hat_win));
    free(p->f_hat_win);
  }
  free(p);
}

void performGridding(plan *p) {
  cuna_check(CUNA2_FN(compat_grid)(p->g_x_data, p->g_f_data, p->g_f_hat, p->Ndata, p->Ngrid,
                                   as2(p->fprops_device), (cudaStream_t)0),
             "performGridding");
  if (p->flags & CALCULATE_WINDOW_FUNCTION)
    cuna_check(CUNA2_FN(compat_grid)(p->g_x_data, NULL, p->g_f_hat_win, p->Ndata, p->Ngrid,
                                     as2(p->fprops_device), (cudaStream_t)0),
               "performGridding(window)");
}

void performFFTs(plan *p) {
  cuna_check(CUNA2_FN(compat_fft)(p->g_f_hat, p->Ngrid, 1, as2(p->fprops_device), 0, (cudaStream_t)0),
             "performFFTs");
  if (p->flags & CALCULATE_WINDOW_FUNCTION)
    cuna_check(CUNA2_FN(compat_fft)(p->g_f_hat_win, p->Ngrid, 1, as2(p->fprops_device), 0, (cudaStream_t)0),
               "performFFTs(window)");
}

void normalizeResults(plan *p) {
  cuna_check(CUNA2_FN(compat_normalize)(p->g_f_hat, p->Ngrid, 1, as2(p->fprops_device), (cudaStream_t)0),
             "normalizeResults");
  if (p->flags & CALCULATE_WINDOW_FUNCTION)
    cuna_check(CUNA2_FN(compat_normalize)(p->g_f_hat_win, p->Ngrid, 1, as2(p->fprops_device), (cudaStream_t)0),
               "normalizeResults(window)");
}

void copyResultsToCPU(plan *p) {
  checkCudaErrors(cudaMemcpy(p->f_hat, p->g_f_hat, sizeof(Complex) * p->Ngrid, cudaMemcpyDeviceToHost));
  if (p->flags & CALCULATE_WINDOW_FUNCTION)
    checkCudaErrors(cudaMemcpy(p->f_hat_win, p->g_f_hat_win, sizeof(Complex) * p->Ngrid, cudaMemcpyDeviceToHost));
}

// Gridding, FFT and deconvolution as one fused pipeline; the results are
// copied back unless DONT_TRANSFER_TO_CPU is set (the reference's test of
// that flag is always false, src/cuna_kernel.cu:142, so it never copies).
void cunfft_adjoint_from_plan(plan *p) {
  cuna_check(CUNA2_FN(compat_adjoint)(p->g_x_data, p->g_f_data, p->g_f_hat, p->Ndata, p->Ngrid,
                                      as2(p->fprops_device), (cudaStream_t)0),
             "cunfft_adjoint_from_plan");
  if (p->flags & CALCULATE_WINDOW_FUNCTION)
    cuna_check(CUNA2_FN(compat_adjoint)(p->g_x_data, NULL, p->g_f_hat_win, p->Ndata, p->Ngrid,
                                        as2(p->fprops_device), (cudaStream_t)0),
               "cunfft_adjoint_from_plan(window)");
  if (!(p->flags & DONT_TRANSFER_TO_CPU)) copyResultsToCPU(p);
}

void cunfft_adjoint(const dTyp *x, const dTyp *f, cTyp *fft, int n, int ng, unsigned int flags) {
  plan *p = (plan *)malloc(sizeof(plan));
  if (!p) {
    fprintf(stderr, "CUNA ERROR: out of host memory\n");
    exit(EXIT_FAILURE);
  }
  init_plan(p, x, f, n, ng, flags & ~(unsigned)DONT_TRANSFER_TO_CPU);
  cunfft_adjoint_from_plan(p);
  for (int i = 0; i < ng; ++i) {
    dTyp *o = reinterpret_cast<dTyp *>(&fft[i]);
    o[0] = p->f_hat[i].x;
    o[1] = p->f_hat[i].y;
  }
  free_plan(p);
}

// ---------------------------------------------------------------------------
// utilities
// ---------------------------------------------------------------------------
void launchDummyKernel() { checkCudaErrors(cudaFree(0)); }

unsigned int nextPowerOfTwo(unsigned int v) {
  v--;
  v |= v >> 1;
  v |= v >> 2;
  v |= v >> 4;
  v |= v >> 8;
  v |= v >> 16;
  return v + 1;
}

dTyp seconds(clock_t dt) { return ((dTyp)dt) / ((dTyp)CLOCKS_PER_SEC); }

// scale_x, src/utils.cu:84-93, with the reference's exact arithmetic: the
// loop subtracts the CURRENT x[0], which its first pass has already turned
// into -1/2, so x[0] becomes -1/2 and every later element becomes
// (x[i] + 1/2) / (x[size-1] - x[0]) - 1/2 with the range taken before the
// loop.  Callers who wanted [-1/2, 1/2] get it only when x[0] == -1/2 on
// entry; accurate mode (cuna2_plan_*) takes t0 and T instead and needs no
// rescaling.  The expressions keep the reference's types (a double
// reciprocal stored in dTyp, the 0.5 subtracted in double) and this file is
// compiled without floating-point contraction, so the bits match the
// reference's on every host.  size < 1 returns (the reference reads x[-1]).
void scale_x(dTyp *x, int size) {
  if (size < 1) return;
  dTyp invrange = 1. / (x[size - 1] - x[0]);
  for (int i = 0; i < size; i++) {
    x[i] -= x[0];
    x[i] *= invrange;
    x[i] -= 0.5;
  }
}

void printComplex(Complex *a, int N, FILE *out) {
  for (int i = 0; i < N; i++) fprintf(out, "%-5d %-10.3e %-10.3e\n", i, a[i].x, a[i].y);
}
void printReal(dTyp *a, int N, FILE *out) {
  for (int i = 0; i < N; i++) fprintf(out, "%-5d %-10.3e\n", i, a[i]);
}
void printComplex_d(Complex *a, int N, FILE *out) {
  Complex *h = (Complex *)malloc(sizeof(Complex) * N);
  checkCudaErrors(cudaMemcpy(h, a, sizeof(Complex) * N, cudaMemcpyDeviceToHost));
  printComplex(h, N, out);
  free(h);
}
void printReal_d(dTyp *a, int N, FILE *out) {
  dTyp *h = (dTyp *)malloc(sizeof(dTyp) * N);
  checkCudaErrors(cudaMemcpy(h, a, sizeof(dTyp) * N, cudaMemcpyDeviceToHost));
  printReal(h, N, out);
  free(h);
}
void print_plan(plan *p) {
  fprintf(stderr, "PLAN: \n\tp->Ngrid = %d\n\tp->Ndata = %d\n", p->Ngrid, p->Ndata);
  fprintf(stderr, "  plan->x_data\n");
  printReal(p->x_data, p->Ndata, stderr);
  fprintf(stderr, "  plan->g_f_hat\n");
  printComplex_d(p->g_f_hat, p->Ngrid, stderr);
}

char *cufftParseError(cufftResult_t r) {
  static char msg[64];
  switch (r) {
    case CUFFT_SUCCESS: return (char *)"The cuFFT operation was successful.";
    case CUFFT_INVALID_PLAN: return (char *)"cuFFT was passed an invalid plan handle.";
    case CUFFT_ALLOC_FAILED: return (char *)"cuFFT failed to allocate GPU or CPU memory.";
    case CUFFT_INVALID_VALUE: return (char *)"User specified an invalid pointer or parameter.";
    case CUFFT_INTERNAL_ERROR: return (char *)"Driver or internal cuFFT library error.";
    case CUFFT_EXEC_FAILED: return (char *)"Failed to execute an FFT on the GPU.";
    case CUFFT_SETUP_FAILED: return (char *)"The cuFFT library failed to initialize.";
    case CUFFT_INVALID_SIZE: return (char *)"User specified an invalid transform size.";
    case CUFFT_INVALID_DEVICE: return (char *)"Execution of a plan was on different GPU than plan creation.";
    case CUFFT_NO_WORKSPACE: return (char *)"No workspace has been provided prior to plan execution.";
    default:
      snprintf(msg, sizeof msg, "unknown cuFFT status %d", (int)r);
      return msg;
  }
}

void checkCufftError(cufftResult_t r) {
  if (r == CUFFT_SUCCESS) return;
  fprintf(stderr, "cuFFT ERROR: %s\n", cufftParseError(r));
  exit(r);
}
