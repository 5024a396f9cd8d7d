/* cuna_utils.h -- CUNA-compatible host utilities (drop-in for the host part
 * of the reference library's inc/cuna_utils.h). */
#ifndef CUNA_UTILS_H
#define CUNA_UTILS_H
#include <time.h>
#include "cuna_typedefs.h"

/* Launch an empty kernel (context warm-up).  Replaces src/utils.cu:67-75. */
void launchDummyKernel();
/* Smallest power of two >= v.  Replaces src/utils.cu:55-65. */
unsigned int nextPowerOfTwo(unsigned int v);
/* clock() ticks to seconds.  Replaces src/utils.cu:78-82. */
dTyp seconds(clock_t dt);
/* Map increasing x in place to [-1/2, 1/2]: (x - x0)/(x_last - x0) - 1/2.
 * Replaces src/utils.cu:84-93. */
void scale_x(dTyp *x, int size);
/* Printing helpers.  Replace src/utils.cu:180-245. */
void print_plan(plan *p);
void printComplex_d(Complex *a, int N, FILE *out);
void printReal_d(dTyp *a, int N, FILE *out);
void printComplex(Complex *a, int N, FILE *out);
void printReal(dTyp *a, int N, FILE *out);
#endif
