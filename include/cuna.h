/* cuna.h -- CUNA-compatible adjoint NFFT entry points (drop-in for the
 * reference library's inc/cuna.h; link libcunaf.so or libcunad.so).
 *
 * Each declaration below replaces the reference function of the same name and
 * signature; the symbols have the same C++ linkage names.
 */
#ifndef CUNA_H
#define CUNA_H
#include "cuna_typedefs.h"

/* Host arrays in, host array out (ng complex values).  Replaces
 * src/cuna.cpp:38-49; unlike the reference, results are copied back. */
void cunfft_adjoint(const dTyp *x, const dTyp *f, cTyp *fft, int n, int ng, unsigned int flags);

/* Run a plan made by init_plan.  Replaces src/cuna_kernel.cu:137-145. */
void cunfft_adjoint_from_plan(plan *p);

/* Device arrays, default stream; f_hat accumulates (zero it first).
 * Replaces src/cuna_kernel.cu:148-183. */
void cunfft_adjoint_raw(const dTyp *x, const dTyp *f_data, Complex *f_hat, const int n,
                        const int ng, const filter_properties *gpu_fprops);

/* Same on `stream`.  Replaces src/cuna_kernel.cu:186-232. */
void cunfft_adjoint_raw_async(const dTyp *x, const dTyp *f_data, Complex *f_hat, const int n,
                              const int ng, const filter_properties *gpu_fprops,
                              cudaStream_t stream);

/* nbs bootstrap resamples into f_hat[nbs][ng].  The reference defines the
 * seeded form (src/cuna_kernel.cu:236-289) but its header declares the form
 * without seed (inc/cuna.h:55-56), which it never defines; both are provided
 * here, the unseeded one using seed 0. */
void cunfft_adjoint_raw_async_bootstrap(const dTyp *x, const dTyp *f_data, Complex *f_hat,
                                        const int n, const int ng, const int nbs,
                                        const filter_properties *gpu_fprops, cudaStream_t stream);
void cunfft_adjoint_raw_async_bootstrap(const dTyp *x, const dTyp *f_data, Complex *f_hat,
                                        const int n, const int ng, const int nbs,
                                        const filter_properties *gpu_fprops, cudaStream_t stream,
                                        const unsigned int seed);

/* Pipeline stages of a plan (reference src/cuna_kernel.cu:52-134). */
void performGridding(plan *p);
void performFFTs(plan *p);
void normalizeResults(plan *p);
void copyResultsToCPU(plan *p);
#endif
