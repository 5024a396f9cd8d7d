/* Host-only stand-in for <cufft.h> (reference-on-CPU build only).
 *
 * cuFFT (CUDA 13.0, libcufft 12.0.0.61) is a closed third-party dependency of
 * the reference that is not part of its source tree.  Its published contract
 * for the calls the reference makes (src/cuna_kernel.cu:82-99,169-178,208-220,
 * 261-276) is restated here: a 1-D complex DFT of length nx, batch `batch`
 * with element distance idist, X[k] = sum_n x[n] exp(s*2*pi*i*n*k/nx) with
 * s = +1 for CUFFT_INVERSE and -1 for CUFFT_FORWARD, unnormalised, in place
 * allowed.  The stand-in evaluates it in double precision (radix-2 for powers
 * of two, direct sum otherwise) and rounds to the transform's element type.
 */
#ifndef CUNA_REFCPU_CUFFT_H
#define CUNA_REFCPU_CUFFT_H
#include "cuda_runtime.h"
typedef float2 cufftComplex;
typedef double2 cufftDoubleComplex;
typedef float cufftReal;
typedef double cufftDoubleReal;
typedef int cufftHandle;
typedef enum cufftResult_t {
  CUFFT_SUCCESS = 0x0,
  CUFFT_INVALID_PLAN = 0x1,
  CUFFT_ALLOC_FAILED = 0x2,
  CUFFT_INVALID_TYPE = 0x3,
  CUFFT_INVALID_VALUE = 0x4,
  CUFFT_INTERNAL_ERROR = 0x5,
  CUFFT_EXEC_FAILED = 0x6,
  CUFFT_SETUP_FAILED = 0x7,
  CUFFT_INVALID_SIZE = 0x8,
  CUFFT_UNALIGNED_DATA = 0x9,
  CUFFT_INCOMPLETE_PARAMETER_LIST = 0xA,
  CUFFT_INVALID_DEVICE = 0xB,
  CUFFT_PARSE_ERROR = 0xC,
  CUFFT_NO_WORKSPACE = 0xD
} cufftResult;
typedef enum cufftType_t { CUFFT_C2C = 0x29, CUFFT_Z2Z = 0x69 } cufftType;
#define CUFFT_FORWARD -1
#define CUFFT_INVERSE 1
cufftResult cufftPlan1d(cufftHandle *plan, int nx, cufftType type, int batch);
cufftResult cufftPlanMany(cufftHandle *plan, int rank, int *n, int *inembed,
                          int istride, int idist, int *onembed, int ostride,
                          int odist, cufftType type, int batch);
cufftResult cufftSetStream(cufftHandle plan, cudaStream_t stream);
cufftResult cufftExecC2C(cufftHandle plan, cufftComplex *idata,
                         cufftComplex *odata, int direction);
cufftResult cufftExecZ2Z(cufftHandle plan, cufftDoubleComplex *idata,
                         cufftDoubleComplex *odata, int direction);
cufftResult cufftDestroy(cufftHandle plan);
#endif
