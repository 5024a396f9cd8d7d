/* Host-only stand-in for <cuda_runtime.h>, used ONLY to compile the reference
 * library's own sources on the CPU so that its outputs can serve as golden
 * vectors for the oracle.  Test infrastructure: nothing in the product links it.
 *
 * Device memory is host memory, a kernel launch is a sequential loop over
 * (block, thread) (see CUNA_CPU_LAUNCH), atomics are plain read-modify-writes.
 * This is exact for the reference kernels, which use neither shared memory nor
 * barriers (gridding.cu:36-117, gaussian_filter.cu:204-302).
 */
#ifndef CUNA_REFCPU_CUDA_RUNTIME_H
#define CUNA_REFCPU_CUDA_RUNTIME_H
#include <stdlib.h>
#include <stdio.h>
#include <string.h>
#include <math.h>
#include <time.h>
#include "vector_types.h"

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline

typedef enum cudaError_enum_cpu {
  cudaSuccess = 0,
  cudaErrorMemoryAllocation = 2,
  cudaErrorInvalidValue = 1
} cudaError_t;

typedef enum {
  cudaMemcpyHostToHost = 0,
  cudaMemcpyHostToDevice = 1,
  cudaMemcpyDeviceToHost = 2,
  cudaMemcpyDeviceToDevice = 3,
  cudaMemcpyDefault = 4
} cudaMemcpyKind;

struct CUstream_st;
typedef struct CUstream_st *cudaStream_t;

extern dim3 blockIdx, threadIdx, blockDim, gridDim;

cudaError_t cudaMalloc(void **p, size_t n);
cudaError_t cudaFree(void *p);
cudaError_t cudaMemcpy(void *d, const void *s, size_t n, cudaMemcpyKind k);
cudaError_t cudaMemcpyAsync(void *d, const void *s, size_t n, cudaMemcpyKind k,
                            cudaStream_t st = 0);
cudaError_t cudaMemset(void *d, int v, size_t n);
cudaError_t cudaDeviceSynchronize(void);
cudaError_t cudaThreadSynchronize(void);
cudaError_t cudaStreamSynchronize(cudaStream_t s);
cudaError_t cudaGetLastError(void);
const char *cudaGetErrorString(cudaError_t e);

float atomicAdd(float *addr, float v);
/* the double overload is declared by the reference's own cuna_utils.h */

/* Sequential emulation of kern<<<grid, block, ...>>>(args).  The recipe in
 * oracle/build_ref.py rewrites every launch in the reference sources into
 * CUNA_CPU_LAUNCH(grid, block, kern, args...). */
#define CUNA_CPU_LAUNCH(grid_, block_, kern_, ...)                               \
  do {                                                                         \
    dim3 cuna_g_((unsigned)(grid_)), cuna_b_((unsigned)(block_));              \
    gridDim = cuna_g_;                                                         \
    blockDim = cuna_b_;                                                        \
    for (unsigned cuna_bx_ = 0; cuna_bx_ < cuna_g_.x; ++cuna_bx_)              \
      for (unsigned cuna_tx_ = 0; cuna_tx_ < cuna_b_.x; ++cuna_tx_) {          \
        blockIdx = dim3(cuna_bx_);                                             \
        threadIdx = dim3(cuna_tx_);                                            \
        kern_(__VA_ARGS__);                                                    \
      }                                                                        \
  } while (0)

#endif
