// phase.cuh -- grid-index reduction of sample times in 64-bit fixed point.
//
// Accurate mode needs, per sample, the grid position s = ((t - t0)/T mod 1)*ng
// split into an integer cell and a fraction.  Done in FP64 that costs several
// double-precision operations per sample, which run at a small fraction of the
// FP32 rate on GB300.  Instead the phase is formed as an unsigned 64-bit
// fixed-point number
//       S = frac((t - t0)/T) * 2^64 = (t*A - t0*A) mod 2^64,   A = 2^64/T,
// with integer multiplies only: t's 53-bit significand times a 64-bit
// significand of A, shifted by the sum of exponents and truncated mod 2^64.
// Then cell = floor(S*ng / 2^64) (the high word of a 64x64 product) and the
// fraction is the low word.  Resolution is 2^-64 of the period, finer than
// FP64's, and the result is exact in the sense of truncation for any t.
//
// The same functions run on the host, which computes t0*A the identical way so
// that t == t0 maps to phase 0 exactly.
#pragma once
#include <stdint.h>
#include <math.h>
#include <string.h>

#if defined(__CUDACC__)
#define CUNA_HD __host__ __device__ __forceinline__
#else
#define CUNA_HD inline
#endif

namespace cuna {

CUNA_HD uint64_t umulhi64(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * (unsigned __int128)b) >> 64);
#endif
}

CUNA_HD uint64_t dbits(double v) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(v);
#else
  uint64_t u;
  memcpy(&u, &v, 8);
  return u;
#endif
}

// Multiplier A = 2^64 / T as mA * 2^eA with mA in [2^63, 2^64).
struct PhaseMul {
  uint64_t mA;
  int eA;
  uint64_t B;  // t0 * A mod 2^64, filled by phase_setup
};

// t * A mod 2^64 (truncated toward zero in magnitude, two's complement sign).
CUNA_HD uint64_t phase_times(double t, const PhaseMul &pm) {
  const uint64_t u = dbits(t);
  const int ex = (int)((u >> 52) & 0x7FF);
  if (ex == 0x7FF) return 0;  // inf / nan: defined but meaningless
  uint64_t mt = u & 0x000FFFFFFFFFFFFFull;
  int et;
  if (ex == 0) {
    et = -1074;
  } else {
    mt |= 0x0010000000000000ull;
    et = ex - 1075;
  }
  const uint64_t lo = mt * pm.mA;
  const uint64_t hi = umulhi64(mt, pm.mA);
  const int sh = et + pm.eA;
  uint64_t r;
  if (sh >= 64) r = 0;
  else if (sh >= 0) r = lo << sh;
  else if (sh > -64) r = (lo >> (-sh)) | (hi << (64 + sh));
  else if (sh > -128) r = hi >> (-sh - 64);
  else r = 0;
  return (u >> 63) ? (uint64_t)(0 - r) : r;
}

// Host: constants for x = (t - t0)/T.  T must be finite and > 0.
inline PhaseMul phase_setup(double t0, double T) {
  PhaseMul pm;
  uint64_t u;
  memcpy(&u, &T, 8);
  int ex = (int)((u >> 52) & 0x7FF);
  uint64_t mT = u & 0x000FFFFFFFFFFFFFull;
  int eT;
  if (ex == 0) {  // subnormal T: normalise
    eT = -1074;
    while (!(mT & 0x0010000000000000ull)) { mT <<= 1; --eT; }
  } else {
    mT |= 0x0010000000000000ull;
    eT = ex - 1075;
  }
  // 2^64 / T = (2^116 / mT) * 2^(64 - 116 - eT)
  unsigned __int128 num = (unsigned __int128)1 << 116;
  unsigned __int128 q = num / mT;
  int eA = 64 - 116 - eT;
  if (q >> 64) {  // mT == 2^52 exactly: 2^64 does not fit, halve
    q >>= 1;
    eA += 1;
  }
  pm.mA = (uint64_t)q;
  pm.eA = eA;
  pm.B = 0;
  pm.B = phase_times(t0, pm);
  return pm;
}

// frac((t - t0)/T) * 2^64
CUNA_HD uint64_t phase_of(double t, const PhaseMul &pm) { return phase_times(t, pm) - pm.B; }

}  // namespace cuna
