// common.cuh -- complex helpers, records and small utilities shared by the
// binning, gridding and FFT kernels of the GB300 adjoint-NFFT library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace cuna {

// Float-float ("double-float") scalar: an unevaluated sum hi + lo of two
// floats, |lo| at most about ulp(hi) (results of + and * are renormalised to
// half an ulp; pairs split from a double by df_from_double are not), about
// 48 significant bits.  The float64 plan's FFT passes and fixed-point taps
// compute in it on the FP32 pipe (GB300's FP64 rate is a small fraction of
// its FP32 rate) and keep double in memory.  Sums by Knuth's two-sum,
// products by an FMA-exact product (Dekker's method with fma), both
// renormalised by a fast two-sum (Dekker 1971; Hida, Li, Bailey 2001).
struct dfl {
  float hi, lo;
  dfl() = default;
  __host__ __device__ constexpr dfl(float h, float l) : hi(h), lo(l) {}
  // from a double constant or value: the nearest float and the remainder
  __host__ __device__ constexpr dfl(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
};
__host__ __device__ __forceinline__ dfl df_fast_two_sum(float a, float b) {
  const float s = a + b;
  return dfl(s, b - (s - a));
}
__host__ __device__ __forceinline__ dfl operator+(dfl a, dfl b) {
  const float s = a.hi + b.hi;
  const float v = s - a.hi;
  float e = (a.hi - (s - v)) + (b.hi - v);
  e += a.lo + b.lo;
  return df_fast_two_sum(s, e);
}
__host__ __device__ __forceinline__ dfl operator-(dfl a) { return dfl(-a.hi, -a.lo); }
__host__ __device__ __forceinline__ dfl operator-(dfl a, dfl b) { return a + (-b); }
__host__ __device__ __forceinline__ dfl operator*(dfl a, dfl b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return df_fast_two_sum(p, e);
}
__host__ __device__ __forceinline__ double df_to_double(dfl a) { return (double)a.hi + (double)a.lo; }
// double -> float-float from the bit fields, integer and FP32 operations only:
// hi keeps the top 24 significant bits (truncated, same sign and exponent),
// lo the remaining 29-bit integer times 2^(e - 52), rounded to a float; hi +
// lo is d to 2^-47 relative.  Zero, values outside the float range and
// non-finite values take the FP64 conversions.
__device__ __forceinline__ dfl df_from_double(double d) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(d);
  const int ex = (int)((u >> 52) & 0x7ff);
  const int fe = ex - 1023 + 127;
  if (fe <= 0 || fe >= 255) {
    const float h = __double2float_rn(d);
    return dfl(h, __double2float_rn(d - (double)h));
  }
  const unsigned sign = (unsigned)(u >> 63) << 31;
  const unsigned long long mant = u & 0xFFFFFFFFFFFFFull;
  const float hi = __int_as_float((int)(sign | ((unsigned)fe << 23) | (unsigned)(mant >> 29)));
  const float lo = ldexpf(__int2float_rn((int)(mant & 0x1FFFFFFFull)), ex - 1075);
  return dfl(hi, sign ? -lo : lo);
}
// 2^(j/64), j = 0..63, as float-float pairs (hi, lo): the value to 1.5e-15
// relative (2^-49), from 200-bit arithmetic
__device__ const float2 kDfExp2Tab[64] = {
    {0x1p+0f, 0.0f}, {0x1.02c9a4p+0f, -0x1.887fap-28f}, {0x1.059b0ep+0f, -0x1.9d4f52p-25f}, {0x1.087452p+0f, -0x1.e2990ep-26f},
    {0x1.0b5586p+0f, 0x1.9f3122p-25f}, {0x1.0e3ec4p+0f, -0x1.a585ccp-25f}, {0x1.11301ep+0f, -0x1.fdb496p-25f}, {0x1.1429aap+0f, 0x1.d525bcp-25f},
    {0x1.172b84p+0f, -0x1.c15742p-27f}, {0x1.1a35bep+0f, 0x1.6df96ep-25f}, {0x1.1d4874p+0f, -0x1.d2e8cap-25f}, {0x1.2063b8p+0f, 0x1.0c519ap-25f},
    {0x1.2387a6p+0f, 0x1.ceac48p-25f}, {0x1.26b456p+0f, 0x1.789f38p-26f}, {0x1.29e9ep+0f, -0x1.5c0424p-25f}, {0x1.2d285ap+0f, 0x1.b900c2p-26f},
    {0x1.306fep+0f, 0x1.4636e2p-25f}, {0x1.33c08cp+0f, -0x1.b37d2p-25f}, {0x1.371a74p+0f, -0x1.18aac6p-25f}, {0x1.3a7db4p+0f, -0x1.634c02p-25f},
    {0x1.3dea64p+0f, 0x1.824684p-25f}, {0x1.4160a2p+0f, 0x1.f72e2ap-28f}, {0x1.44e086p+0f, 0x1.8624b4p-30f}, {0x1.486a2cp+0f, -0x1.47d866p-25f},
    {0x1.4bfdaep+0f, -0x1.593abcp-25f}, {0x1.4f9b28p+0f, -0x1.2c5a6cp-25f}, {0x1.5342b6p+0f, -0x1.2c561p-25f}, {0x1.56f474p+0f, -0x1.295b04p-25f},
    {0x1.5ab07ep+0f, -0x1.5bd5ecp-27f}, {0x1.5e76f2p+0f, -0x1.4a5bd6p-25f}, {0x1.6247ecp+0f, -0x1.f8b55p-25f}, {0x1.662388p+0f, 0x1.2a9112p-27f},
    {0x1.6a09e6p+0f, 0x1.9fcef4p-26f}, {0x1.6dfb24p+0f, -0x1.cd72e8p-27f}, {0x1.71f75ep+0f, 0x1.1d8beep-25f}, {0x1.75feb6p+0f, -0x1.37b306p-25f},
    {0x1.7a1148p+0f, -0x1.829fdp-25f}, {0x1.7e2f34p+0f, -0x1.261634p-25f}, {0x1.82589ap+0f, -0x1.accc7cp-26f}, {0x1.868d9ap+0f, -0x1.2edb44p-26f},
    {0x1.8ace54p+0f, 0x1.15506ep-27f}, {0x1.8f1aeap+0f, -0x1.baa232p-26f}, {0x1.93737cp+0f, -0x1.e64744p-25f}, {0x1.97d82ap+0f, -0x1.0d8d84p-31f},
    {0x1.9c4918p+0f, 0x1.51f848p-27f}, {0x1.a0c668p+0f, -0x1.2886a6p-26f}, {0x1.a5503cp+0f, -0x1.b83b54p-25f}, {0x1.a9e6b6p+0f, -0x1.50c048p-25f},
    {0x1.ae89fap+0f, -0x1.a94b14p-26f}, {0x1.b33a2cp+0f, -0x1.ec3a82p-26f}, {0x1.b7f77p+0f, -0x1.a09438p-25f}, {0x1.bcc1eap+0f, -0x1.f687c6p-25f},
    {0x1.c199bep+0f, -0x1.3d56b2p-27f}, {0x1.c67f12p+0f, 0x1.cafa2ap-25f}, {0x1.cb720ep+0f, -0x1.8837ccp-27f}, {0x1.d072d4p+0f, 0x1.40f13p-25f},
    {0x1.d5818ep+0f, -0x1.822dbcp-27f}, {0x1.da9e6p+0f, 0x1.ed9942p-27f}, {0x1.dfc974p+0f, -0x1.908c94p-25f}, {0x1.e502eep+0f, 0x1.e2cffep-26f},
    {0x1.ea4afap+0f, 0x1.52486cp-27f}, {0x1.efa1bep+0f, 0x1.cc2b44p-25f}, {0x1.f50766p+0f, -0x1.246ebp-26f}, {0x1.fa7c18p+0f, 0x1.9e90d8p-28f},
};
// 2^x for |x| < 100 in float-float, table-driven (Tang 1989): x = n + j/64
// + r with k = 64 n + j = rint(64 x), |r| <= 1/128 (r = x - k/64 exactly
// in its high part); 2^(j/64) = t from the table; 2^r - 1 = e^z - 1,
// z = r ln 2, |z| < 0.0055, as z + z^2 s with s = 1/2 + z/6 + z^2/24 +
// z^3/120 (truncation below 4e-17; the z/6 term in float-float, the rest in
// float); 2^(j/64 + r) as t + t (2^r - 1), whose product is below 0.006 of
// the sum; then the exact scaling by 2^n.  Relative error below 7e-15
// (about 2^-47), checked against 120-bit arithmetic over |x| < 100.
__device__ __forceinline__ dfl df_exp2(dfl x) {
  const float kf = rintf(x.hi * 64.0f);
  const int k = (int)kf;
  const dfl r = x - dfl(kf * 0.015625f, 0.f);
  const dfl z = r * dfl(0.69314718055994530942);
  const dfl c6 = z * dfl(1.0 / 6.0);
  const float u2 = (z.hi * z.hi) * fmaf(z.hi, 1.0f / 120.0f, 1.0f / 24.0f);
  dfl s = df_fast_two_sum(0.5f, c6.hi);
  s = df_fast_two_sum(s.hi, s.lo + (c6.lo + u2));
  const dfl em1 = z + (z * z) * s;
  const float2 tt = __ldg(&kDfExp2Tab[k & 63]);
  const dfl t(tt.x, tt.y);
  const dfl v = t + t * em1;
  const float sc = __int_as_float((127 + (k >> 6)) << 23);  // 2^n, |n| <= 100
  return dfl(v.hi * sc, v.lo * sc);
}
// 1/a: the float reciprocal of a.hi refined by one Newton step in float-float
__device__ __forceinline__ dfl df_rcp(dfl a) {
  const dfl r0(__frcp_rn(a.hi), 0.f);
  const dfl e = dfl(1.0f, 0.f) - a * r0;
  return r0 + r0 * e;
}
struct __align__(16) dcx {
  dfl x, y;
};

template <typename T> struct CxOf;
template <> struct CxOf<float> { typedef float2 type; };
template <> struct CxOf<double> { typedef double2 type; };
template <> struct CxOf<dfl> { typedef dcx type; };
// the element type a complex array of the plan type is stored as in memory
// (the float-float passes read and write double)
template <typename T> struct MemOf { typedef typename CxOf<T>::type type; };
template <> struct MemOf<dfl> { typedef double2 type; };
// the scalar the plan's epilogue parameters are kept in
template <typename T> struct AccOf { typedef T type; };
template <> struct AccOf<dfl> { typedef double type; };

__host__ __device__ __forceinline__ float2 cmk(float a, float b) { return make_float2(a, b); }
__host__ __device__ __forceinline__ double2 cmk(double a, double b) { return make_double2(a, b); }
__host__ __device__ __forceinline__ dcx cmk(dfl a, dfl b) {
  dcx c;
  c.x = a;
  c.y = b;
  return c;
}

// memory <-> computation forms of a complex value, and read-only twiddle loads
template <typename C, typename M> __device__ __forceinline__ C cx_load(M v) { return v; }
template <> __device__ __forceinline__ dcx cx_load<dcx, double2>(double2 v) {
  return cmk(df_from_double(v.x), df_from_double(v.y));
}
__device__ __forceinline__ float2 cx_to_mem(float2 v) { return v; }
__device__ __forceinline__ double2 cx_to_mem(double2 v) { return v; }
__device__ __forceinline__ double2 cx_to_mem(dcx v) { return make_double2(df_to_double(v.x), df_to_double(v.y)); }
__device__ __forceinline__ float2 ldtw(const float2 *p) { return __ldg(p); }
__device__ __forceinline__ double2 ldtw(const double2 *p) { return __ldg(p); }
__device__ __forceinline__ dcx ldtw(const dcx *p) {
  const float4 v = __ldg(reinterpret_cast<const float4 *>(p));
  return cmk(dfl(v.x, v.y), dfl(v.z, v.w));
}

template <typename C> __host__ __device__ __forceinline__ C cadd(C a, C b) { return cmk(a.x + b.x, a.y + b.y); }
template <typename C> __host__ __device__ __forceinline__ C csub(C a, C b) { return cmk(a.x - b.x, a.y - b.y); }
template <typename C> __host__ __device__ __forceinline__ C cmul(C a, C b) {
  return cmk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
template <typename C> __host__ __device__ __forceinline__ C cmulc(C a, C b) {
  return cmk(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
template <typename C> __host__ __device__ __forceinline__ C cconj(C a) { return cmk(a.x, -a.y); }
// i * a
template <typename C> __host__ __device__ __forceinline__ C cmuli(C a) { return cmk(-a.y, a.x); }
template <typename C, typename T> __host__ __device__ __forceinline__ C cscale(C a, T s) {
  return cmk(a.x * s, a.y * s);
}

// Sorted sample record of the float path: 16 bytes, one vector load.
//   cell : grid cell the taps are anchored on (accurate: floor(s) mod ng;
//          compat: the reference's j)
//   a, b : per-sample filter factors (accurate: y*E1, E2; compat: E1, E2)
//   p    : value (compat, as float bits) or original sample index (bootstrap)
struct __align__(16) RecF {
  int cell;
  float a, b;
  int p;
};
// Double path: 32 bytes.
struct __align__(16) RecD {
  int cell;
  int p;
  double a, b;
  double v;
};
template <typename T> struct RecOf;
template <> struct RecOf<float> { typedef RecF type; };
template <> struct RecOf<double> { typedef RecD type; };

// Records read through L2 only (ld.global.cg), for kernels that start before
// the kernel writing the records has finished (dependent launch): no L1 line
// filled before the grid-completion wait can serve them.
template <typename R> struct CgSrc {
  const R *p;
  __device__ __forceinline__ R operator[](int64_t i) const {
    static_assert(sizeof(R) % 16 == 0, "records are whole 16-byte vectors");
    R r;
    const int4 *s = reinterpret_cast<const int4 *>(p + i);
    int4 *d = reinterpret_cast<int4 *>(&r);
#pragma unroll
    for (int q = 0; q < (int)(sizeof(R) / 16); ++q) d[q] = __ldcg(s + q);
    return r;
  }
};

__host__ __device__ __forceinline__ int ilog2i(int64_t v) {
  int r = 0;
  while ((int64_t(1) << (r + 1)) <= v) ++r;
  return r;
}

// Programmatic dependent launch.  A kernel launched with programmatic stream
// serialization may start while its predecessor in the stream is finishing:
// pdl_trigger() lets the successor launch once every CTA of this grid has
// called it, and pdl_wait() blocks until the predecessor grid has completed
// and its memory is visible (a hardware grid-completion wait; it returns at
// once when the kernel was launched without the attribute).  Every read of a
// predecessor's output must follow pdl_wait() and be an ordinary (coherent)
// load: no __ldg on it and no __restrict__ parameter in the kernel (from
// restrict-qualified outputs the compiler may infer that the other inputs are
// read-only and read them through the non-coherent path).  Non-coherent loads
// assume the data does not change while the kernel runs, and here the kernel
// starts before its predecessors have finished writing (measured: a row pass
// reading the column pass's output through const __restrict__ returned a
// wrong spectrum whenever it ran one CTA per SM).
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Launch with programmatic stream serialization: the kernel may start while
// its predecessor finishes and waits for it with pdl_wait() (common.cuh).
bool pdl_enabled();  // runtime.cu: false when the environment sets CUNA2_PDL=0
void pdl_suppress(bool off);  // runtime.cu: this thread launches without it while `off`

template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, Args... args) {
  if (!pdl_enabled()) {
    k<<<grid, block, smem, st>>>(static_cast<KArgs>(args)...);
    return cudaGetLastError();
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k, static_cast<KArgs>(args)...);
}

// Fixed-point accumulation in shared memory: a value w (already scaled so
// that every cell's sum stays within `range`) is rounded to an integer and
// added with a native shared-memory integer atomic; integer sums do not
// depend on the order of the atomics.  Double cells round by adding
// 1.5 * 2^52 (the integer lands in the low mantissa bits; exact round to
// nearest for |w| < 2^51), one FP64 add that the multiply before it fuses
// into, instead of a conversion on the FP64 pipe (gridding of the large
// float64 workload 354 -> 299 us); hence the 2^50 range, a quantum of 2^-50
// of each tile's bound.
template <typename T> struct FixAcc;
template <> struct FixAcc<float> {
  typedef int type;
  static constexpr float range = 1073741824.0f;  // 2^30
  __device__ static int to_fix(float w) { return __float2int_rn(w); }
  __device__ static void add(int *a, int v) { atomicAdd(a, v); }
};
// The drop-in's tile sums (reference arithmetic) keep the widest double
// range, 2^62 with a conversion per value: their target is the reference's
// own FP64 result (6e-16 relative on GB300), not a kernel error.
template <typename T> struct FixAccWide : FixAcc<T> {};
template <> struct FixAccWide<double> {
  typedef long long type;
  static constexpr double range = 4611686018427387904.0;  // 2^62
  __device__ static long long to_fix(double w) { return __double2ll_rn(w); }
  __device__ static void add(long long *a, long long v) {
    atomicAdd(reinterpret_cast<unsigned long long *>(a), (unsigned long long)v);
  }
};
template <> struct FixAcc<double> {
  typedef long long type;
  static constexpr double range = 1125899906842624.0;  // 2^50
  __device__ static long long to_fix(double w) {
    return __double_as_longlong(w + 6755399441055744.0) - 0x4338000000000000ll;
  }
  __device__ static void add(long long *a, long long v) {
    atomicAdd(reinterpret_cast<unsigned long long *>(a), (unsigned long long)v);
  }
};

}  // namespace cuna
