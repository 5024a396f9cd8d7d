/* Host-only stand-in for <cuda.h> (reference-on-CPU build only). */
#include "cuda_runtime.h"
