/* Host-only stand-in for <cuComplex.h> (reference-on-CPU build only). */
#ifndef CUNA_REFCPU_CUCOMPLEX_H
#define CUNA_REFCPU_CUCOMPLEX_H
#include "vector_types.h"
typedef float2 cuFloatComplex;
typedef cuFloatComplex cuComplex;
typedef double2 cuDoubleComplex;
#endif
