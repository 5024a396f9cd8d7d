// fft.cuh -- hand-written inverse (e^{+2 pi i nk/L}) complex FFT for sm_103a.
//
// A transform of length L = 2^p runs either in one CTA (L <= the single-CTA
// limit: the whole sequence lives in shared memory) or as a four-step
// transform L = L1 * L2 in two passes over global memory:
//   pass A (columns): for each n2, FFT over n1 of x[n1*L2 + n2], multiply by
//                     W_L^{n2 k1}, store in place at k1*L2 + n2;
//   pass B (rows):    for each k1, FFT over n2 of row k1, result X[k1 + L1 k2]
//                     goes through a fused epilogue (deconvolution, output
//                     selection, real-input unpacking, frequency shift).
// Inside a CTA each sequence is transformed by Stockham autosort stages of
// radix 16 (plus one leading radix 2/4/8 stage): every thread holds E = 16
// values in registers per stage, so a stage is read-all / barrier / write-all
// on a single shared buffer.  Shared indices are padded (i + i/16) so that
// the strided writes of the first stage are bank-conflict free.
//
// Everything here has internal linkage (anonymous namespace) because the
// compat translation unit is compiled with the reference's --use_fast_math
// while the accurate one is not.
#pragma once
#include "common.cuh"

namespace cuna {
namespace {

constexpr int kFftE = 16;  // complex values per thread per stage

__device__ __forceinline__ int pad16(int i) { return i + (i >> 4); }

// Shared-memory pitch (in complex elements) of one sequence of length L when
// `nseq` sequences are stored side by side: at least L + L/16, and congruent
// to 16/nseq (mod 16) so that the column-wise global<->shared copies of the
// four-step passes spread over all banks.
__host__ __device__ constexpr int fft_pitch(int L, int nseq) {
  int base = L + (L >> 4) + 1;
  int want = nseq >= 16 ? 1 : 16 / (nseq > 0 ? nseq : 1);
  int r = base & 15;
  return base + ((want - r) & 15);
}

// ---- radix butterflies, inverse sign, natural order in and out ----
template <typename C> __device__ __forceinline__ void bf4(C &a0, C &a1, C &a2, C &a3) {
  C t0 = cadd(a0, a2), t1 = csub(a0, a2), t2 = cadd(a1, a3), t3 = cmuli(csub(a1, a3));
  a0 = cadd(t0, t2);
  a2 = csub(t0, t2);
  a1 = cadd(t1, t3);
  a3 = csub(t1, t3);
}

template <typename C> __device__ __forceinline__ void dft2(C *v) {
  C a = v[0];
  v[0] = cadd(a, v[1]);
  v[1] = csub(a, v[1]);
}
template <typename C> __device__ __forceinline__ void dft4(C *v) { bf4(v[0], v[1], v[2], v[3]); }

template <typename C> __device__ __forceinline__ void dft8(C *v) {
  typedef decltype(v[0].x) T;
  const T c = (T)0.70710678118654752440;
  C e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
  C o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
  bf4(e0, e1, e2, e3);
  bf4(o0, o1, o2, o3);
  C t1 = cmk((o1.x - o1.y) * c, (o1.x + o1.y) * c);   // W8^1 o1
  C t2 = cmuli(o2);                                    // W8^2 o2
  C t3 = cmk(-(o3.x + o3.y) * c, (o3.x - o3.y) * c);  // W8^3 o3
  v[0] = cadd(e0, o0); v[4] = csub(e0, o0);
  v[1] = cadd(e1, t1); v[5] = csub(e1, t1);
  v[2] = cadd(e2, t2); v[6] = csub(e2, t2);
  v[3] = cadd(e3, t3); v[7] = csub(e3, t3);
}

template <typename C> __device__ __forceinline__ void dft16(C *v) {
  typedef decltype(v[0].x) T;
  const T c1 = (T)0.92387953251128675613, s1 = (T)0.38268343236508977173;
  const T h = (T)0.70710678118654752440;
  // 16 = 4 x 4: columns n2, A[n2][k1] lands at v[n2 + 4 k1]
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) bf4(v[n2], v[n2 + 4], v[n2 + 8], v[n2 + 12]);
  // twiddles W16^{n2 k1}
  v[5] = cmul(v[5], cmk(c1, s1));     // n2=1,k1=1: W^1
  v[9] = cmul(v[9], cmk(h, h));       // n2=1,k1=2: W^2
  v[13] = cmul(v[13], cmk(s1, c1));   // n2=1,k1=3: W^3
  v[6] = cmul(v[6], cmk(h, h));       // n2=2,k1=1: W^2
  v[10] = cmuli(v[10]);               // n2=2,k1=2: W^4
  v[14] = cmul(v[14], cmk(-h, h));    // n2=2,k1=3: W^6
  v[7] = cmul(v[7], cmk(s1, c1));     // n2=3,k1=1: W^3
  v[11] = cmul(v[11], cmk(-h, h));    // n2=3,k1=2: W^6
  v[15] = cmul(v[15], cmk(-c1, -s1)); // n2=3,k1=3: W^9
  // rows k1: DFT over n2, X[k1 + 4 k2] lands at v[4 k1 + k2]
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) bf4(v[4 * k1], v[4 * k1 + 1], v[4 * k1 + 2], v[4 * k1 + 3]);
  C t[16];
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1)
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) t[k1 + 4 * k2] = v[4 * k1 + k2];
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = t[i];
}

template <int R, typename C> __device__ __forceinline__ void dftR(C *v) {
  if (R == 2) dft2(v);
  else if (R == 4) dft4(v);
  else if (R == 8) dft8(v);
  else dft16(v);
}

// One Stockham stage of radix R over nseq sequences of length 2^logL stored
// at s[seq*pitch + pad16(i)].  Ns = 2^logNs is the length already
// transformed.  tw[q] = exp(+2 pi i q / L).
template <typename T, int R>
__device__ __forceinline__ void fft_stage(typename CxOf<T>::type *s, int pitch, int logL,
                                          int logNs, int total_bf,
                                          const typename CxOf<T>::type *__restrict__ tw) {
  typedef typename CxOf<T>::type C;
  constexpr int LOGR = (R == 2) ? 1 : (R == 4) ? 2 : (R == 8) ? 3 : 4;
  constexpr int NB = kFftE / R;
  const int logLR = logL - LOGR;
  const int maskLR = (1 << logLR) - 1;
  const int maskNs = (1 << logNs) - 1;
  const int twsh = logL - logNs - LOGR;
  C v[NB][R];
#pragma unroll
  for (int u = 0; u < NB; ++u) {
    const int g = threadIdx.x + u * blockDim.x;
    if (g < total_bf) {
      const int seq = g >> logLR, j = g & maskLR;
      const C *base = s + seq * pitch;
#pragma unroll
      for (int r = 0; r < R; ++r) v[u][r] = base[pad16(j + (r << logLR))];
      if (logNs > 0) {
        const int k = j & maskNs;
#pragma unroll
        for (int r = 1; r < R; ++r) v[u][r] = cmul(v[u][r], ldtw(&tw[(r * k) << twsh]));
      }
      dftR<R>(v[u]);
    }
  }
  __syncthreads();
#pragma unroll
  for (int u = 0; u < NB; ++u) {
    const int g = threadIdx.x + u * blockDim.x;
    if (g < total_bf) {
      const int seq = g >> logLR, j = g & maskLR;
      C *base = s + seq * pitch;
      const int k = j & maskNs;
      const int idxD = ((j >> logNs) << (logNs + LOGR)) + k;
#pragma unroll
      for (int r = 0; r < R; ++r) base[pad16(idxD + (r << logNs))] = v[u][r];
    }
  }
  __syncthreads();
}

// Inverse FFT of nseq sequences of length 2^logL held in shared memory.  All
// threads of the block must call it; blockDim.x * kFftE >= nseq * L.
template <typename T>
__device__ void smem_fft(typename CxOf<T>::type *s, int pitch, int logL, int nseq,
                         const typename CxOf<T>::type *__restrict__ tw) {
  if (logL == 0) return;
  int r0 = logL & 3;
  if (r0 == 0) r0 = 4;
  const int total = nseq << logL;
  switch (r0) {
    case 1: fft_stage<T, 2>(s, pitch, logL, 0, total >> 1, tw); break;
    case 2: fft_stage<T, 4>(s, pitch, logL, 0, total >> 2, tw); break;
    case 3: fft_stage<T, 8>(s, pitch, logL, 0, total >> 3, tw); break;
    default: fft_stage<T, 16>(s, pitch, logL, 0, total >> 4, tw); break;
  }
  for (int logNs = r0; logNs < logL; logNs += 4)
    fft_stage<T, 16>(s, pitch, logL, logNs, total >> 4, tw);
}

// ---------------------------------------------------------------------------
// Stockham FFT whose first stage reads its inputs straight from global memory
// and whose last stage writes straight to global memory (through functors),
// so a pass touches shared memory only between stages.
//   Src: __device__ C load(int seq, int i)           input element i of seq
//   Dst: __device__ void store(int seq, int k, C v)   output element k of seq
// Each stage picks its own mapping of butterflies to threads: "seq fastest"
// (consecutive threads take consecutive sequences, i.e. consecutive columns
// of a row-major array) or "j fastest" (consecutive points of one sequence),
// so that the global side of the first and last stage is coalesced.
// ---------------------------------------------------------------------------
template <typename T, int R, bool IN_G, bool OUT_G, bool SEQ_FAST, class Src, class Dst>
__device__ __forceinline__ void fstage(typename CxOf<T>::type *s, int pitch, int logL, int logNs,
                                       int logNseq, const typename CxOf<T>::type *__restrict__ tw,
                                       const Src &src, const Dst &dst) {
  typedef typename CxOf<T>::type C;
  constexpr int LOGR = (R == 2) ? 1 : (R == 4) ? 2 : (R == 8) ? 3 : 4;
  constexpr int NB = kFftE / R;
  const int logLR = logL - LOGR;
  const int total = 1 << (logNseq + logLR);
  const int maskNs = (1 << logNs) - 1;
  const int twsh = logL - logNs - LOGR;
  C v[NB][R];
#pragma unroll
  for (int u = 0; u < NB; ++u) {
    const int g = threadIdx.x + u * blockDim.x;
    if (g < total) {
      const int seq = SEQ_FAST ? (g & ((1 << logNseq) - 1)) : (g >> logLR);
      const int j = SEQ_FAST ? (g >> logNseq) : (g & ((1 << logLR) - 1));
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int i = j + (r << logLR);
        v[u][r] = IN_G ? src.load(seq, i) : s[seq * pitch + pad16(i)];
      }
      if (logNs > 0) {
        const int k = j & maskNs;
#pragma unroll
        for (int r = 1; r < R; ++r) v[u][r] = cmul(v[u][r], ldtw(&tw[(r * k) << twsh]));
      }
      dftR<R>(v[u]);
    }
  }
  if (!IN_G && !OUT_G) __syncthreads();
#pragma unroll
  for (int u = 0; u < NB; ++u) {
    const int g = threadIdx.x + u * blockDim.x;
    if (g < total) {
      const int seq = SEQ_FAST ? (g & ((1 << logNseq) - 1)) : (g >> logLR);
      const int j = SEQ_FAST ? (g >> logNseq) : (g & ((1 << logLR) - 1));
      const int idxD = ((j >> logNs) << (logNs + LOGR)) + (j & maskNs);
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int k = idxD + (r << logNs);
        if (OUT_G) dst.store(seq, k, v[u][r]);
        else s[seq * pitch + pad16(k)] = v[u][r];
      }
    }
  }
  if (!OUT_G) __syncthreads();
}

template <typename T, int R, bool IN_G, bool OUT_G, bool FIRST_SEQ_FAST, bool LAST_SEQ_FAST, class Src, class Dst>
__device__ __forceinline__ void fstage_sel(typename CxOf<T>::type *s, int pitch, int logL, int logNs,
                                           int logNseq, const typename CxOf<T>::type *tw, const Src &src,
                                           const Dst &dst) {
  // first stages follow the load mapping, the last one the store mapping
  if (OUT_G) fstage<T, R, IN_G, OUT_G, LAST_SEQ_FAST>(s, pitch, logL, logNs, logNseq, tw, src, dst);
  else fstage<T, R, IN_G, OUT_G, FIRST_SEQ_FAST>(s, pitch, logL, logNs, logNseq, tw, src, dst);
}

// Full transform: Src -> [stages] -> Dst when TO_GLOBAL, or Src -> [stages] ->
// shared memory (s[seq*pitch + pad16(k)], followed by a barrier) otherwise.
template <typename T, bool TO_GLOBAL, bool FIRST_SEQ_FAST, bool LAST_SEQ_FAST, class Src, class Dst>
__device__ void fft_fused(typename CxOf<T>::type *s, int pitch, int logL, int logNseq,
                          const typename CxOf<T>::type *__restrict__ tw, const Src &src, const Dst &dst) {
  int r0 = logL & 3;
  if (r0 == 0) r0 = 4;
  const bool single = r0 == logL;  // one stage only
#define CUNA_FIRST(RR)                                                                          \
  if (single) {                                                                                 \
    fstage_sel<T, RR, true, TO_GLOBAL, FIRST_SEQ_FAST, LAST_SEQ_FAST>(s, pitch, logL, 0, logNseq, tw, src, dst); \
    return;                                                                                     \
  }                                                                                             \
  fstage_sel<T, RR, true, false, FIRST_SEQ_FAST, LAST_SEQ_FAST>(s, pitch, logL, 0, logNseq, tw, src, dst);
  switch (r0) {
    case 1: { CUNA_FIRST(2) break; }
    case 2: { CUNA_FIRST(4) break; }
    case 3: { CUNA_FIRST(8) break; }
    default: { CUNA_FIRST(16) break; }
  }
#undef CUNA_FIRST
  int logNs = r0;
  for (; logNs + 4 < logL; logNs += 4)
    fstage_sel<T, 16, false, false, FIRST_SEQ_FAST, LAST_SEQ_FAST>(s, pitch, logL, logNs, logNseq, tw, src, dst);
  fstage_sel<T, 16, false, TO_GLOBAL, FIRST_SEQ_FAST, LAST_SEQ_FAST>(s, pitch, logL, logNs, logNseq, tw, src, dst);
}

struct NoDst {
  template <typename C> __device__ void store(int, int, C) const {}
};

// Device view of the twiddle tables of one transform length L = L1 * L2.
template <typename T> struct FftDev {
  typedef typename CxOf<T>::type C;
  int logL, logL1, logL2;  // single-CTA plans: logL1 = logL, logL2 = 0
  const C *tw1;            // exp(+2 pi i q / L1), q < L1
  const C *tw2;            // exp(+2 pi i q / L2), q < L2
  const C *twlo;           // exp(+2 pi i q / L),  q < 2048
  const C *twhi;           // exp(+2 pi i 2048 q / L), q < L / 2048
};

// W_L^q for q < L from the two-level table.
template <typename T>
__device__ __forceinline__ typename CxOf<T>::type twiddle_L(const FftDev<T> &f, int q) {
  if (f.logL <= 11) return ldtw(&f.twlo[q]);
  return cmul(ldtw(&f.twhi[q >> 11]), ldtw(&f.twlo[q & 2047]));
}

// ---------------------------------------------------------------------------
// pass A: column FFTs of length L1 (stride L2), B = blockDim.x*E/L1 columns
// per CTA, twiddle W_L^{n2 k1}, stored in place (in == out allowed: a CTA
// reads all its columns before it writes any of them).
// grid = (L2 / B, nslab)
// ---------------------------------------------------------------------------
template <typename T> struct ColSrc {
  const typename CxOf<T>::type *p;
  int L2, c0;
  __device__ __forceinline__ typename CxOf<T>::type load(int seq, int i) const {
    return p[(int64_t)i * L2 + c0 + seq];
  }
};
template <typename T> struct ColDst {
  typename CxOf<T>::type *p;
  int L2, c0;
  FftDev<T> f;
  __device__ __forceinline__ void store(int seq, int k, typename CxOf<T>::type v) const {
    p[(int64_t)k * L2 + c0 + seq] = cmul(v, twiddle_L(f, (c0 + seq) * k));
  }
};

// Column FFTs [c0, c0 + B) of one slab; B = blockDim.x * kFftE / L1.
template <typename T>
__device__ __forceinline__ void colpass_body(const typename CxOf<T>::type *in, typename CxOf<T>::type *out,
                                             const FftDev<T> &f, int cblock) {
  typedef typename CxOf<T>::type C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *s = reinterpret_cast<C *>(smem_raw);
  const int L2 = 1 << f.logL2;
  const int logB = ilog2i((int64_t)blockDim.x * kFftE) - f.logL1;
  const int B = 1 << logB;
  const int pitch = fft_pitch(1 << f.logL1, B);
  const int c0 = cblock * B;
  ColSrc<T> src{in, L2, c0};
  ColDst<T> dst{out, L2, c0, f};
  // a CTA's reads all precede the barrier after the first stage, its writes
  // all follow it, so in == out is safe
  fft_fused<T, true, true, true>(s, pitch, f.logL1, logB, f.tw1, src, dst);
}

template <typename T>
__global__ void __launch_bounds__(sizeof(T) == 4 ? 512 : 256) k_fft_colpass(const typename CxOf<T>::type *in,
                                                                            typename CxOf<T>::type *out,
                                                                            FftDev<T> f, int64_t slab_stride) {
  colpass_body<T>(in + blockIdx.y * slab_stride, out + blockIdx.y * slab_stride, f, blockIdx.x);
}

}  // namespace
}  // namespace cuna
