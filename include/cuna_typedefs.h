/* cuna_typedefs.h -- types of the CUNA-compatible drop-in API.
 *
 * Same names, layouts and precision switch as the reference's
 * inc/cuna_typedefs.h (johnh2o2/cunfft_adjoint v1.3): build against
 * libcunad.so with -DDOUBLE_PRECISION, against libcunaf.so without it.
 * Struct layouts are part of the ABI: filter_properties is 40 bytes (float)
 * / 48 bytes (double) with E1 at offset 16 / 24; plan is 96 bytes.
 */
#ifndef CUNA_TYPEDEFS_H
#define CUNA_TYPEDEFS_H

#include <stdio.h>
#include <stdlib.h>
#include <vector_types.h>
#include <cuda_runtime.h>
#include <cufft.h>

#ifdef DOUBLE_PRECISION
#define dTyp double
#define cTyp double _Complex
#define Complex cufftDoubleComplex
#else
#define dTyp float
#define cTyp float _Complex
#define Complex cufftComplex
#endif

#ifndef PI
#define PI 3.14159265358979323846
#endif

/* Report a CUDA error and terminate, as the reference library does
 * (reference inc/cuna_typedefs.h:80-89). */
#define checkCudaErrors(ans) cuna_gpu_assert((ans), __FILE__, __LINE__)
static inline void cuna_gpu_assert(cudaError_t code, const char *file, int line) {
  if (code != cudaSuccess) {
    fprintf(stderr, "CUDA ERROR %-24s L[%-5d]: %s\n", file, line, cudaGetErrorString(code));
    exit(code);
  }
}

/* Gaussian filter description; E1/E2 (n values) and E3 (filter_radius
 * values) are device arrays. */
typedef struct {
  dTyp b, normfac;
  int filter_radius;
  dTyp *E1;
  dTyp *E2;
  dTyp *E3;
} filter_properties;

/* Behaviour flags of init_plan / cunfft_adjoint. */
typedef enum {
  NO_FLAGS = 0x01,
  OUTPUT_INTERMEDIATE = 0x02,
  CALCULATE_WINDOW_FUNCTION = 0x04,
  DONT_TRANSFER_TO_CPU = 0x08,
  PRINT_TIMING = 0x10
} FLAGS;

/* Host/device state of one transform (init_plan / free_plan). */
typedef struct {
  dTyp *x_data, *f_data;          /* host copies of the inputs            */
  Complex *f_hat, *f_hat_win;     /* host results (f_hat_win: window fn)  */
  Complex *g_f_hat, *g_f_hat_win; /* device results                       */
  dTyp *g_x_data, *g_f_data;      /* device inputs                        */
  unsigned int flags;
  int Ndata, Ngrid, filter_radius;
  filter_properties *fprops_host, *fprops_device;
} plan;

void free_plan(plan *p);
void init_plan(plan *p, const dTyp *x, const dTyp *f, int Ndata, int Ngrid, unsigned int plan_flags);

#endif
