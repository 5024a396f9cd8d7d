/* cufft_utils.h -- cuFFT status helpers of the CUNA-compatible API (drop-in
 * for the reference library's inc/cufft_utils.h). */
#ifndef CUFFT_UTILS_H
#define CUFFT_UTILS_H
#include <cufft.h>
/* Text for a cuFFT status (static storage; the reference returns a leaked
 * malloc'ed buffer).  Replaces src/cufft_utils.cu:27-70. */
char *cufftParseError(cufftResult_t r);
/* Print and exit on a failing cuFFT status.  Replaces src/cufft_utils.cu:72-77. */
void checkCufftError(cufftResult_t r);
#endif
