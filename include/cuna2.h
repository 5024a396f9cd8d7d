/* cuna2.h -- extern "C" interface of the GB300 adjoint-NFFT library
 * (libcuna_gb300.so).  Plain pointers and sizes only; every array argument is
 * CUDA device memory unless stated otherwise; every function returns a status
 * code (CUNA2_SUCCESS == 0) instead of exiting the process.
 *
 * Two families:
 *
 *  - cuna2_compat_*: the reference library's arithmetic (CUNA v1.3), the
 *    C-ABI form of the reference entry points.  The drop-in libraries
 *    libcunaf.so / libcunad.so (include/cuna.h) are thin wrappers over these.
 *
 *  - cuna2_plan_* / cuna2_adjoint*: accurate mode.  Samples at times t_j with
 *    values y_j are mapped to x_j = (t_j - t0)/T - 1/2 and the library returns
 *        F_k = sum_j y_j exp(+2 pi i k x_j),   k = -nf/2 .. nf/2 - 1,
 *    stored at F[k + nf/2], accurate to about 1e-6 relative (float32 plans)
 *    against a direct double-precision sum.  The grid-index reduction of t_j
 *    is done in 64-bit fixed point, so long baselines keep full phase
 *    accuracy.
 */
#ifndef CUNA2_H
#define CUNA2_H

#include <stddef.h>
#include <stdint.h>
#include <cuda_runtime.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------------- */
/* status                                                                  */
/* ---------------------------------------------------------------------- */
enum {
  CUNA2_SUCCESS = 0,
  CUNA2_ERROR_INVALID_VALUE = 1, /* bad size, NULL pointer, bad plan       */
  CUNA2_ERROR_CUDA = 2,          /* a CUDA runtime call failed              */
  CUNA2_ERROR_UNSUPPORTED = 3,   /* size/configuration this library rejects */
  CUNA2_ERROR_ALLOC = 4,         /* device or host allocation failed        */
  CUNA2_ERROR_CUFFT = 5          /* the cuFFT comparator path failed        */
};

/* Message for the last failing call made by this thread ("" if none). */
const char *cuna2_last_error(void);
/* Name of a status code. */
const char *cuna2_status_string(int status);
/* Library version string. */
const char *cuna2_version(void);
/* Number of bounded device waits (TMA copy completions) that ran out since
   the process started; 0 in normal operation.  A kernel whose wait runs out
   counts it here and leaves its output unwritten instead of waiting on. */
long long cuna2_wait_timeouts(void);

/* ---------------------------------------------------------------------- */
/* compat mode: the reference library's arithmetic                         */
/* ---------------------------------------------------------------------- */

/* Same memory layout as the reference's filter_properties
 * (inc/cuna_typedefs.h:92-108) in its float build (40 bytes) and double build
 * (48 bytes).  E1/E2 hold n values, E3 holds filter_radius values; all three
 * are device pointers. */
typedef struct {
  float b, normfac;
  int filter_radius;
  float *E1, *E2, *E3;
} cuna2_filter_properties_f32;

typedef struct {
  double b, normfac;
  int filter_radius;
  double *E1, *E2, *E3;
} cuna2_filter_properties_f64;

/* Fill h_fprops->{b, normfac, filter_radius}, copy *h_fprops to d_fprops and
 * compute E1/E2/E3 on `stream`.  The caller allocates d_fprops (device) and
 * the E1 (n), E2 (n), E3 (filter_radius) device arrays whose pointers it
 * stores in h_fprops.  filter_radius is 6 (f32) or 12 (f64).
 * Replaces generate_pinned_filter_properties, src/gaussian_filter.cu:43-66. */
int cuna2_compat_filter_f32(const float *x, int n, int ng,
                            cuna2_filter_properties_f32 *h_fprops,
                            cuna2_filter_properties_f32 *d_fprops, cudaStream_t stream);
int cuna2_compat_filter_f64(const double *x, int n, int ng,
                            cuna2_filter_properties_f64 *h_fprops,
                            cuna2_filter_properties_f64 *d_fprops, cudaStream_t stream);

/* Radius the compat filter uses: 6 for float, 12 for double. */
int cuna2_compat_filter_radius(int is_double);

/* Gridding -> in-place unnormalised inverse FFT -> deconvolution on `stream`.
 * f_hat (ng complex values) ACCUMULATES the gridded samples, exactly as the
 * reference: zero it first for a plain transform.  f_data == NULL grids
 * y_j = 1 (the window function).
 * Replaces cunfft_adjoint_raw_async, src/cuna_kernel.cu:188-232. */
int cuna2_compat_adjoint_f32(const float *x, const float *f_data, float2 *f_hat, int n,
                             int ng, const cuna2_filter_properties_f32 *d_fprops,
                             cudaStream_t stream);
int cuna2_compat_adjoint_f64(const double *x, const double *f_data, double2 *f_hat, int n,
                             int ng, const cuna2_filter_properties_f64 *d_fprops,
                             cudaStream_t stream);

/* nbs bootstrap resamples into f_hat[nbs][ng] (accumulating), same draw
 * stream as the reference (wang_hash then xorshift32 of seed + i).
 * Replaces cunfft_adjoint_raw_async_bootstrap, src/cuna_kernel.cu:236-289. */
int cuna2_compat_bootstrap_f32(const float *x, const float *f_data, float2 *f_hat, int n,
                               int ng, int nbs, const cuna2_filter_properties_f32 *d_fprops,
                               unsigned int seed, cudaStream_t stream);
int cuna2_compat_bootstrap_f64(const double *x, const double *f_data, double2 *f_hat, int n,
                               int ng, int nbs, const cuna2_filter_properties_f64 *d_fprops,
                               unsigned int seed, cudaStream_t stream);

/* The three stages of cuna2_compat_adjoint_* separately (the reference's
 * performGridding / performFFTs / normalizeResults, src/cuna_kernel.cu:52-117):
 * gridding only (accumulating), the unnormalised in-place inverse FFT of
 * nbatch slabs of ng points (normalize != 0 fuses the deconvolution in), and
 * the deconvolution alone. */
int cuna2_compat_grid_f32(const float *x, const float *f_data, float2 *f_hat, int n, int ng,
                          const cuna2_filter_properties_f32 *d_fprops, cudaStream_t stream);
int cuna2_compat_grid_f64(const double *x, const double *f_data, double2 *f_hat, int n, int ng,
                          const cuna2_filter_properties_f64 *d_fprops, cudaStream_t stream);
int cuna2_compat_fft_f32(float2 *f_hat, int ng, int nbatch, const cuna2_filter_properties_f32 *d_fprops,
                         int normalize, cudaStream_t stream);
int cuna2_compat_fft_f64(double2 *f_hat, int ng, int nbatch, const cuna2_filter_properties_f64 *d_fprops,
                         int normalize, cudaStream_t stream);
int cuna2_compat_normalize_f32(float2 *f_hat, int ng, int nbatch,
                               const cuna2_filter_properties_f32 *d_fprops, cudaStream_t stream);
int cuna2_compat_normalize_f64(double2 *f_hat, int ng, int nbatch,
                               const cuna2_filter_properties_f64 *d_fprops, cudaStream_t stream);

/* cuna2_compat_adjoint_f32 for callers that cannot allocate device memory.
 * No counterpart in the reference library.
 *
 * Some callers must not call cudaMalloc once they are running: real-time or
 * latency-critical loops (cudaFree synchronises the whole device), processes
 * whose device memory belongs to a framework's caching allocator, and plugin
 * hosts whose contract forbids a plugin from allocating.  This entry point
 * allocates nothing: its scratch (tile counters, sorted sample records, FFT
 * scratch, twiddle tables) is one statically sized device array of about
 * 5.6 MB that every GPU loading the library holds until the process exits.
 * The caller still passes x, f_data, f_hat and d_fprops, with the same
 * meaning as cuna2_compat_adjoint_f32.
 *
 * Limits: n <= 131072 samples; ng a power of two <= 131072.  Larger sizes
 * return CUNA2_ERROR_UNSUPPORTED with a message and touch nothing.
 * The first call on a device sets it up (looks up the array's device address,
 * fills the twiddle tables, synchronises `stream`): make it before any stream
 * capture.  Every call shares the array and keeps the previous call's
 * contents; the counters are cleared per call.  Calls that overlap on the GPU
 * race on the array, so serialise them. */
int cuna2_compat_adjoint_noalloc_f32(const float *x, const float *f_data, float2 *f_hat, int n,
                                     int ng, const cuna2_filter_properties_f32 *d_fprops,
                                     cudaStream_t stream);

/* ---------------------------------------------------------------------- */
/* accurate mode                                                           */
/* ---------------------------------------------------------------------- */
enum { CUNA2_F32 = 0, CUNA2_F64 = 1 };

typedef struct cuna2_plan_st *cuna2_plan;

/* Plan for nf output frequencies (even, >= 2), oversampling R (>= 2) and
 * Gaussian half-width m (2..16 grid cells) in precision dtype.  The grid has
 * ng = R * nf cells.  Allocates twiddle tables on the current device. */
int cuna2_plan_create(cuna2_plan *plan, int dtype, int64_t nf, int R, int m);
int cuna2_plan_destroy(cuna2_plan plan);
/* Grid size ng and the kernel variance tau (grid cells^2) the plan uses. */
int cuna2_plan_info(cuna2_plan plan, int64_t *ng, double *tau);

/* One adjoint NFFT: t (n doubles), y (n floats for CUNA2_F32 plans, doubles
 * for CUNA2_F64), F (nf complex values of the plan's precision).  t0 and T
 * define x_j = (t_j - t0)/T - 1/2; values outside [t0, t0 + T) wrap
 * periodically.  Stream-ordered; the plan's workspace grows on demand (the
 * first call with a larger n allocates, so make it before any stream
 * capture). */
int cuna2_adjoint(cuna2_plan plan, const double *t, const void *y, void *F, int64_t n,
                  double t0, double T, cudaStream_t stream);

/* Bootstrap: nbs resamples of (t, y) drawn with replacement, resample b
 * taking samples d = xorshift32(wang_hash(seed + b*n + i)) % n, i < n (the
 * reference's draw stream, src/gridding.cu:67-82,101), each transformed like
 * cuna2_adjoint into F[b*nf .. (b+1)*nf).  The positions are binned once per
 * call; each resample grids the original samples weighted by their draw
 * multiplicity.  Requires nbs <= 65535 and nbs*n < 2^31. */
int cuna2_adjoint_bootstrap(cuna2_plan plan, const double *t, const void *y, void *F, int64_t n,
                            int nbs, unsigned int seed, double t0, double T, cudaStream_t stream);

/* nchan value channels at the same sample times (y holds nchan rows of n
 * values, F receives nchan rows of nf outputs), transformed together: one
 * binning pass and one gridding launch shared by all channels, then one
 * slab-batched FFT.  A channel of ones gives the window function.
 * 1 <= nchan <= 65535. */
int cuna2_adjoint_multi(cuna2_plan plan, const double *t, const void *y, void *F, int64_t n,
                        int nchan, double t0, double T, cudaStream_t stream);

/* Generalised (floating-mean) Lomb-Scargle periodogram of (t, y) with
 * optional uncertainties dy (NULL: equal weights) at frequencies
 * f_k = (k + 1) df, k < nfreq, written to power (nfreq values of dtype).
 * Built on one two-channel adjoint NFFT (weighted centred values and
 * weights) with period 1/df, Nf the smallest power of two > 4 nfreq,
 * oversampling R and half-width m.  Plans are cached per (device, size). */
int cuna2_lomb_scargle(int dtype, const double *t, const void *y, const void *dy, int64_t n,
                       int64_t nfreq, double df, double t0, int R, int m, void *power,
                       cudaStream_t stream);

/* Vector-Jacobian product of cuna2_adjoint for a real loss L(F): given
 * G[k + nf/2] = dL/dRe F_k + i dL/dIm F_k (nf complex values of the plan's
 * precision), writes dL/dy_j (n values of the plan's precision) to grad_y and
 * dL/dt_j (n doubles) to grad_t; either may be NULL.  Uses the same Gaussian
 * kernel: one FFT of the deconvolved spectrum to a real field on the grid,
 * then per sample the kernel and its derivative interpolate it.  Nothing of
 * the forward pass is stored or needed besides t and y. */
int cuna2_adjoint_backward(cuna2_plan plan, const double *t, const void *y, const void *G,
                           void *grad_y, double *grad_t, int64_t n, double t0, double T,
                           cudaStream_t stream);

/* cuna2_adjoint_backward for nseries series of n samples each on one plan
 * (the training form: a batch of light curves per step).  Series s has times
 * t[s*n .. (s+1)*n), values y[...], upstream gradient G[s*nf .. (s+1)*nf),
 * its own t0[s] and T[s] (host arrays), and receives grad_y[s*n ..] and
 * grad_t[s*n ..] (either may be NULL).  One launch per stage covers up to 256
 * series; the plan's backward workspace grows to two packed complex grids
 * per series of such a group.  No counterpart in the reference library. */
int cuna2_adjoint_backward_batch(cuna2_plan plan, const double *t, const void *y, const void *G, void *grad_y,
                                 double *grad_t, int64_t n, int nseries, const double *t0, const double *T,
                                 cudaStream_t stream);

/* Same transform with HOST arrays (pinned or pageable): copies t and y to
 * plan-owned device staging buffers, runs on `stream`, copies F back and
 * synchronises the stream before returning. */
int cuna2_adjoint_host(cuna2_plan plan, const double *t, const void *y, void *F, int64_t n,
                       double t0, double T, cudaStream_t stream);

/* The same without the final synchronisation: copies in, transform and copy
 * out are only enqueued on `stream`, so a caller that streams many series
 * through two plans on two streams overlaps one series' transfers with the
 * other's transform (the replacement, with host arrays, for the reference's
 * cunfft_adjoint_raw_async, src/cuna_kernel.cu:181-223).  t, y and F must be
 * pinned and stay untouched until the stream reaches the end of the call;
 * one plan must not be used on two streams at once (its staging and
 * workspace are shared). */
int cuna2_adjoint_host_async(cuna2_plan plan, const double *t, const void *y, void *F, int64_t n,
                             double t0, double T, cudaStream_t stream);

/* enable != 0: cuna2_adjoint, cuna2_adjoint_host, cuna2_adjoint_bootstrap
 * and cuna2_adjoint_multi capture their launch sequence into a CUDA graph the
 * first time they see an argument set (pointers, n, t0, T, and the resample
 * count and seed or the channel count) and replay it afterwards (up to 64
 * cached sets, the oldest dropped first).  The capture is taken on a private
 * stream; the caller's stream only sees graph launches. */
int cuna2_plan_set_graph(cuna2_plan plan, int enable);

/* Per-launch durations of one transform: the launch sequence is captured with
 * an event after every launch into a CUDA graph, launches serialised, and the
 * graph is replayed once on `stream` (writing F), so each timestamp is taken
 * on the device.  The first call on a plan, or one with more samples than
 * before, runs the transform once eagerly beforehand to size the workspace.
 * Returns the duration of
 * each launch in milliseconds (stage_ms[0..*nstages)) and, if stage_names is
 * non-NULL, a static name for each; the last entry, "event_gap", is the time
 * between two event nodes with nothing between them, which every other
 * entry includes once.  Synchronises `stream`. */
int cuna2_plan_profile(cuna2_plan plan, const double *t, const void *y, void *F, int64_t n,
                       double t0, double T, cudaStream_t stream, float *stage_ms,
                       const char **stage_names, int max_stages, int *nstages);

/* The gridding kernel's own launch time: one transform of (t, y) into F in
 * which the gridding launch (idempotent on the binned records) runs `reps`
 * times back to back between two CUDA events on `stream`; *ms_per_launch
 * receives the mean.  Tiled plans only (CUNA2_ERROR_UNSUPPORTED otherwise).
 * Synchronises `stream`. */
int cuna2_plan_time_grid(cuna2_plan plan, const double *t, const void *y, void *F, int64_t n, double t0,
                         double T, int reps, cudaStream_t stream, float *ms_per_launch);

/* Gridding schedule.  The grid is cut into tiles of 2^log_tile cells, one CTA
 * per tile staging it in shared memory and writing it to HBM once.  Forms:
 *   CUNA2_GRID_GATHER   the tile's records are counting-sorted by cell in
 *                       shared memory and each thread sums four consecutive
 *                       cells over its window of records (log_tile <= 12);
 *   CUNA2_GRID_SCATTER  one thread per (record, tap) adds its Gaussian weight
 *                       into the shared tile with an atomic (log_tile <= 13);
 *   CUNA2_GRID_FIXED    one thread per record computes all 2m taps from the
 *                       factorised Gaussian and adds them as fixed-point
 *                       integers (int32 cells for float plans, int64 for
 *                       double) scaled to a per-tile bound on the cell sums,
 *                       so the grid is bit-reproducible (log_tile <= 13).
 * All compute the same sums to rounding.  With more than one tile,
 * 2^log_tile >= 2m.
 * New plans start at (11, CUNA2_GRID_GATHER) for float and (12,
 * CUNA2_GRID_FIXED) for double (a grid of at most 8192 cells is one tile).  Changing the
 * schedule drops the plan's cached graphs.  No counterpart in the reference
 * (its gridding kernel, src/gridding.cu:36-65, has a fixed launch shape). */
enum { CUNA2_GRID_GATHER = 0, CUNA2_GRID_SCATTER = 1, CUNA2_GRID_FIXED = 2 };
int cuna2_plan_set_schedule(cuna2_plan plan, int log_tile, int grid_method);
int cuna2_plan_get_schedule(cuna2_plan plan, int *log_tile, int *grid_method);

/* Filter-width schedule: creates the plan for nf outputs that reaches a
 * relative error target `tol` fastest on the caller's data.  For each
 * oversampling R in {2, 4, 8} it takes the smallest half-width m with
 * exp(-pi m sqrt(1 - 1/R)) <= tol (the Gaussian kernel's error; clamped at
 * 1e-7 for float plans), autotunes that plan on (t, y) (writing F, nf
 * values) and keeps the fastest; R_out / m_out (may be NULL) receive the
 * choice.  The reference fixes its filter width (R_f 6 / 12). */
int cuna2_plan_create_auto(cuna2_plan *plan, int dtype, int64_t nf, double tol, const double *t,
                           const void *y, void *F, int64_t n, double t0, double T, cudaStream_t stream,
                           int *R_out, int *m_out);

/* Bucket sort in front of the tiled gridding:
 *   CUNA2_BIN_GLOBAL  count pass, then one pass that scans the tile counts and
 *                     scatters the records into one tile-ordered array;
 *   CUNA2_BIN_LOCAL   one pass: each CTA sorts a chunk of samples by tile in
 *                     shared memory and writes runs; the gridding reads a
 *                     tile's records as one run per chunk (used when at most
 *                     4096 tiles and 1024 chunks of <= 16384 samples; else
 *                     the global form runs).
 * New plans use CUNA2_BIN_GLOBAL.  Changing it drops cached graphs. */
enum { CUNA2_BIN_GLOBAL = 0, CUNA2_BIN_LOCAL = 1 };
int cuna2_plan_set_binning(cuna2_plan plan, int mode);
int cuna2_plan_get_binning(cuna2_plan plan, int *mode);

/* Autotuner: runs the transform of (t, y) into F under every admissible
 * schedule (both binning forms, every gridding form, log_tile in 9..13 below
 * the whole grid), reps timed runs each (CUDA events on `stream`, minimum
 * taken, with a buffer of twice the L2 size overwritten before each run so
 * the inputs come from HBM), and keeps the fastest; best_ms (may be NULL)
 * receives its time.  Allocates and frees that buffer; synchronises
 * `stream`.  Plans small enough for the single-CTA path have nothing to tune
 * and keep their schedule. */
int cuna2_plan_autotune(cuna2_plan plan, const double *t, const void *y, void *F, int64_t n,
                        double t0, double T, cudaStream_t stream, int reps, float *best_ms);

/* ---------------------------------------------------------------------- */
/* batched accurate mode: many series of uneven length                     */
/* ---------------------------------------------------------------------- */
typedef struct cuna2_batch_plan_st *cuna2_batch_plan;

/* Plan for nseries series: series s has n[s] samples and nf[s] outputs
 * (R*nf[s]/2 a power of two), all sharing R and m; t0/T (host arrays, may be
 * NULL for 0 and 1) give x = (t - t0[s])/T[s] - 1/2.  The samples of all
 * series are concatenated in t and y (series s at offset n[0]+..+n[s-1]) and
 * so are the outputs in F.  Builds the work tables and allocates the whole
 * workspace up front. */
int cuna2_batch_plan_create(cuna2_batch_plan *plan, int dtype, int nseries, const int64_t *n,
                            const int64_t *nf, int R, int m, const double *t0, const double *T);
/* A batch plan with its own oversampling R[s] and filter half-width m[s] per
 * series (host arrays of nseries ints; R[s] * nf[s] / 2 a power of two,
 * 1 <= m[s] <= 16); otherwise as cuna2_batch_plan_create, which is this with
 * one R and m for every series. */
int cuna2_batch_plan_create_ex(cuna2_batch_plan *plan, int dtype, int nseries, const int64_t *n,
                               const int64_t *nf, const int *R, const int *m, const double *t0,
                               const double *T);
/* R[s] and m[s] of every series (host arrays of nseries ints; either may be
 * NULL). */
int cuna2_batch_get_filter(cuna2_batch_plan plan, int *R, int *m);
/* Filter-width schedule of a batch, per size class (the series of one output
 * length nf): candidates R = 2, 4, 8 with the smallest m whose Gaussian error
 * exp(-pi m sqrt(1 - 1/R)) <= tol (tol clamped at 1e-7 for float plans).  All
 * classes start at R = 2; then, class by class (most samples first), R = 4
 * and 8 are tried with the other classes kept, each candidate batch autotuned
 * by cuna2_batch_autotune on (t, y) (writing F), and a class keeps the
 * fastest.  R_out / m_out (host arrays of nseries ints, may be NULL) receive
 * the choice.  No counterpart in the reference, whose filter width is fixed
 * and whose batched API was never finished (src/cuna_kernel.cu:302-358). */
int cuna2_batch_plan_create_auto(cuna2_batch_plan *plan, int dtype, int nseries, const int64_t *n,
                                 const int64_t *nf, double tol, const double *t0, const double *T,
                                 const double *t, const void *y, void *F, cudaStream_t stream, int *R_out,
                                 int *m_out);
int cuna2_batch_plan_destroy(cuna2_batch_plan plan);
/* Replace every series' t0/T (host arrays; synchronises the device). */
int cuna2_batch_set_times(cuna2_batch_plan plan, const double *t0, const double *T);
/* Total samples and total outputs of the batch. */
int cuna2_batch_info(cuna2_batch_plan plan, int64_t *n_total, int64_t *nf_total);
/* enable != 0: capture the batch's launch sequence into a CUDA graph per
 * (t, y, F) and replay it. */
int cuna2_batch_set_graph(cuna2_batch_plan plan, int enable);
/* All transforms of the batch, stream-ordered. */
int cuna2_batch_adjoint(cuna2_batch_plan plan, const double *t, const void *y, void *F,
                        cudaStream_t stream);

/* Gridding schedule of the batch's large series (grids above the one-CTA
 * size): tiles of 2^log_tile cells in CUNA2_GRID_FIXED form (log_tile 10 to
 * 13; bit-reproducible, the default, with 4096-cell tiles) or
 * CUNA2_GRID_GATHER form (log_tile 10 to 12).  Changing it rebuilds the plan's tables and workspace (synchronises
 * the device, drops cached graphs). */
int cuna2_batch_set_schedule(cuna2_batch_plan plan, int log_tile, int grid_method);
int cuna2_batch_get_schedule(cuna2_batch_plan plan, int *log_tile, int *grid_method);

/* Autotuner of a batched plan: runs the batch of (t, y) into F under every
 * admissible schedule (fixed point with log_tile 10..13, gather with
 * 10..12), reps timed runs each
 * (CUDA events on `stream`, minimum taken, a buffer of twice the L2 size
 * overwritten before each run so the inputs come from HBM), and keeps the
 * fastest; best_ms (may be NULL) receives its time.  Allocates and frees that
 * buffer; synchronises the device.  No counterpart in the reference, whose
 * batched API was never finished (src/cuna_kernel.cu:302-358). */
int cuna2_batch_autotune(cuna2_batch_plan plan, const double *t, const void *y, void *F, cudaStream_t stream,
                         int reps, float *best_ms);

/* ---------------------------------------------------------------------- */
/* integer steps read back (tests and diagnostics, not a transform path)   */
/* ---------------------------------------------------------------------- */
/* Each of these runs the same device functions as the transforms and writes
 * what they computed, so that callers can compare the integer steps with a
 * CPU restatement bit for bit.  Output arrays are device memory; any per-
 * sample output may be NULL. */

/* Compat mode, per sample i < n (x as for cuna2_compat_adjoint_*):
 *   cell[i]    j = (int)((x_i + 1/2)(ng - 1)), evaluated in double, clamped
 *              to [0, ng) when clamp != 0 (fast_gridding, src/gridding.cu:
 *              43-45) and left unclamped otherwise (fast_gridding_bootstrap,
 *              src/gridding.cu:93-95);
 *   origin[i]  u = (int)(ng x_i - R_f) of the filter coefficients
 *              (set_gpu_filter_properties, src/gaussian_filter.cu:213);
 *   tap_lo[i], tap_hi[i]  the taps m in [tap_lo, tap_hi) that reach the
 *              grid (src/gridding.cu:53-58); (0, 0) when none does, which
 *              includes |j| > 2^30, where the reference's int arithmetic
 *              overflows. */
int cuna2_inspect_compat_taps_f32(const float *x, int n, int ng, int clamp, int *cell, int *origin,
                                  int *tap_lo, int *tap_hi, cudaStream_t stream);
int cuna2_inspect_compat_taps_f64(const double *x, int n, int ng, int clamp, int *cell, int *origin,
                                  int *tap_lo, int *tap_hi, cudaStream_t stream);

/* The bootstrap draw stream of both modes: draw[b*n + i] = xorshift32(
 * wang_hash(seed + b*n + i)) % n for resample b < nbs and draw i < n
 * (src/gridding.cu:67-82,101).  n*nbs <= INT_MAX. */
int cuna2_inspect_bootstrap_draws(int n, int nbs, unsigned int seed, int *draw, cudaStream_t stream);

/* The bucket sort in front of compat gridding, as cuna2_compat_adjoint_*
 * (boot == 0) or cuna2_compat_bootstrap_* (boot != 0) runs it: each sample
 * is binned into every 4096-cell tile its taps reach.  offsets (ngt + 1 ints,
 * ngt = ceil(ng / 4096)) delimit tile t's records [offsets[t], offsets[t+1]);
 * records receives them (at most max_records) and *nrecords their number
 * (a host int).  Record layout, float (16 bytes): {int cell; float E1;
 * float E2; int value_bits} (boot == 0) or {int cell; int -, -; int sample}
 * (boot != 0); double (32 bytes): {int cell; int sample; double E1, E2,
 * value}, the sample index set only when boot != 0.  Within a tile the
 * records form a set: their order depends on scheduling and on nothing the
 * results depend on.  Synchronises `stream`. */
int cuna2_inspect_compat_bins_f32(const float *x, const float *y, int n, int ng,
                                  const cuna2_filter_properties_f32 *d_fprops, int boot, int *offsets,
                                  void *records, int max_records, int *nrecords, cudaStream_t stream);
int cuna2_inspect_compat_bins_f64(const double *x, const double *y, int n, int ng,
                                  const cuna2_filter_properties_f64 *d_fprops, int boot, int *offsets,
                                  void *records, int max_records, int *nrecords, cudaStream_t stream);

/* Accurate mode's grid-index reduction per sample: phase[i] = frac((t_i -
 * t0)/T) 2^64 as an unsigned 64-bit fixed-point number ((t_i A - t0 A) mod
 * 2^64, A = 2^64/T to 64 significant bits, each product truncated) and
 * cell[i] = floor(phase[i] ng / 2^64), for a grid of ng <= 2^30 cells. */
int cuna2_inspect_phases(const double *t, int64_t n, double t0, double T, int64_t ng, uint64_t *phase,
                         int *cell, cudaStream_t stream);

/* The plan's own binning of (t, y) as cuna2_adjoint runs it (tiled plans
 * with the global binning form; other plans return CUNA2_ERROR_UNSUPPORTED):
 * offsets (ntiles + 1 ints, ntiles = ng / 2^log_tile of the plan's
 * schedule), the records (at most max_records) and *nrecords (host).  Each
 * sample gives a record in every tile that its taps cell-m+1 .. cell+m (mod
 * ng) reach.  Record layout, float plans (16 bytes): {int cell; float frac;
 * float y; int sample}, frac the fractional cell (the top 24 bits of the low
 * word of phase*ng, scaled by 2^-24); double plans (32 bytes): {int cell; int
 * sample; double frac (top 53 bits, scaled by 2^-53); double y; double 0}.
 * Within a tile the records form a set.  Synchronises `stream`. */
int cuna2_plan_inspect_bins(cuna2_plan plan, const double *t, const void *y, int64_t n, double t0, double T,
                            int *offsets, void *records, int64_t max_records, int64_t *nrecords,
                            cudaStream_t stream);

#ifdef __cplusplus
}
#endif
#endif /* CUNA2_H */
