/* Force-included when the reference library's own sources are compiled with
 * today's CUDA toolkit (oracle/build_ref_cuda.py).  Test infrastructure: it
 * maps three names the reference uses that CUDA 13 no longer provides, and
 * changes nothing else.
 *   cudaThreadSynchronize            removed from the runtime; the same call
 *                                    is cudaDeviceSynchronize
 *                                    (src/cuna_kernel.cu:175)
 *   CUFFT_INCOMPLETE_PARAMETER_LIST,  removed from cufftResult; the
 *   CUFFT_PARSE_ERROR                reference only names them in its error
 *                                    strings (src/cufft_utils.cu:60,66), so
 *                                    they get values no call returns */
#pragma once
#define cudaThreadSynchronize cudaDeviceSynchronize
#define CUFFT_INCOMPLETE_PARAMETER_LIST ((cufftResult_t)0x7F01)
#define CUFFT_PARSE_ERROR ((cufftResult_t)0x7F02)
