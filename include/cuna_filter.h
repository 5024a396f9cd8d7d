/* cuna_filter.h -- CUNA-compatible Gaussian filter setup (drop-in for the
 * reference library's inc/cuna_filter.h). */
#ifndef CUNA_FILTER_H
#define CUNA_FILTER_H
#include "cuna_typedefs.h"

/* Allocate and fill a plan's filter.  Replaces src/gaussian_filter.cu:168-177. */
void set_filter_properties(plan *p);

/* Caller-allocated variant on `stream`: fills h_fprops->{b, normfac,
 * filter_radius}, copies it to d_fprops and computes E1/E2/E3 into the device
 * arrays whose pointers h_fprops holds.  Replaces src/gaussian_filter.cu:43-66. */
void generate_pinned_filter_properties(const dTyp *x, const int n, const int ng,
                                       filter_properties *h_fprops, filter_properties *d_fprops,
                                       cudaStream_t stream);

/* Allocate host and device filter descriptions for the device positions x
 * and compute them (synchronous).  Replaces src/gaussian_filter.cu:102-164. */
void generate_filter_properties(const dTyp *x, const int n, const int ng,
                                filter_properties **fprops_host, filter_properties **fprops_device);

/* Free what generate_filter_properties allocated.  Replaces
 * src/gaussian_filter.cu:180-190. */
void free_filter_properties(filter_properties *d_fp, filter_properties *fp);
#endif
