// runtime.h -- host-side runtime shared by the compat and accurate paths:
// error reporting, per-(device, stream) workspaces, cached FFT twiddle tables,
// and launch-shape constants.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>
#include "../../include/cuna2.h"

namespace cuna {

// Record `status` with a printf-style message for cuna2_last_error(); returns
// status so call sites can `return fail(...)`.
int fail(int status, const char *fmt, ...);
// CUDA error -> CUNA2_ERROR_CUDA with the call text.
int fail_cuda(cudaError_t e, const char *what);
void clear_error();

#define CUNA_CK(call)                                   \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return fail_cuda(e_, #call); \
  } while (0)
#define CUNA_TRY(expr)           \
  do {                           \
    int s_ = (expr);             \
    if (s_ != CUNA2_SUCCESS) return s_; \
  } while (0)

// Scratch memory for one (current device, stream): grows on demand, never
// shrinks, freed at process exit.  Calls on different streams get different
// buffers, so concurrent streams do not race.  Growing synchronises the device.
int stream_workspace(cudaStream_t stream, size_t bytes, void **ptr);

// Number of SMs of the current device.
int device_sm_count();

// FFT geometry for a complex length L = 2^logL.  Single-CTA transforms use
// logL1 = logL and logL2 = 0.
struct FftGeom {
  int logL, logL1, logL2;
  bool single;
  const void *tw1, *tw2, *twlo, *twhi;
};
// Largest single-CTA length (log2) and the per-CTA element budget of the
// four-step passes for each precision.
constexpr int kSingleLogF32 = 14;  // 16384 complex64 = 128 KB + padding
constexpr int kSingleLogF64 = 13;  // 8192 complex128
constexpr int kPassElemsF32 = 8192;
constexpr int kPassElemsF64 = 4096;
constexpr int kMaxLogL = 26;

// Geometry and device twiddle tables (computed in double precision on the
// host, rounded once to the element type, cached per device).  `min_rows`
// forces the row pass to hold at least that many rows (2 for the real-input
// unpack, which pairs rows k1 and L1-k1).
// split: force the four-step L1 x L2 factorisation even where one CTA could
// hold the whole transform (multi-CTA passes for a single small transform)
int fft_geometry(bool is_double, int logL, FftGeom *g, bool split = false);
// The four-step geometry of a float-float transform of length 2^logL: the
// same tables as the double one, each entry a float-float complex.
int fft_geometry_df(int logL, FftGeom *g);

// One-time per-device setup (kernel attributes): setup_done(key) tells whether
// `key` has been marked on the current device, mark_setup_done(key) marks it.
// Thread-safe; two threads may both run an idempotent setup before it is
// marked.
bool setup_done(const void *key);
void mark_setup_done(const void *key);

// Device pointer (host-mapped) of the counter of bounded waits that ran out;
// nullptr when mapped host memory is unavailable (TMA kernels are then not
// used).
int *wait_timeout_counter();
// The TMA column pass is used when the environment sets CUNA2_TMA=1.  It
// gives bit-identical spectra; measured on GB300 it ties the load/store
// column pass where the grid is L2-resident and is slower (101 against 88 us
// for 1024 grids of 2^15 points) where the pass streams from HBM, because a
// CTA can start its transform only once all its boxes have landed.
bool tma_enabled();
// CUNA2_GATHER_MASKS=1: float plans keep the tap masks in the gather even
// where the Gaussian's tail allows the unmasked form (for comparisons)
bool masked_gather_forced();
// CUNA2_F64_PASSES=1: double plans run their four-step passes in FP64
// arithmetic instead of float-float (for comparisons)
bool fp64_passes_forced();
// Tiled 3D tensor map (CUtensorMap, 128 bytes at `map`) over float32 data at
// `base`: dims {d0, d1, d2} (d0 innermost), byte strides {s1, s2} of
// dimensions 1 and 2, box {b0, b1, 1}.  Returns false when the CUDA driver entry
// point is missing or the encoding is rejected.
bool encode_tmap_f32_3d(void *map, const void *base, uint64_t d0, uint64_t d1, uint64_t d2, uint64_t s1,
                        uint64_t s2, uint32_t b0, uint32_t b1);

}  // namespace cuna
