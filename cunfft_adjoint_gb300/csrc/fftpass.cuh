// fftpass.cuh -- the accurate transform's four-step row pass (real unpack,
// deconvolution and centring fused in) with compile-time geometry; the
// stages and the column pass are in fftpass_core.cuh.
#pragma once
#include "accurate_kernels.cuh"
#include "fftpass_core.cuh"

namespace cuna {
namespace {

// ---------------------------------------------------------------------------
// row pass with the accurate epilogue: a CTA owns the row-pair slots
// p in [p0, p0 + B/2), transforms their rows (length L2) into shared memory,
// then unpacks, deconvolves and centres every output k = k1 + L1 k2 <= K.
// Slot p >= 1 holds rows (p, L1 - p), whose outputs need each other's
// values; rows 0 and L1/2 each pair with themselves and share slot 0, so
// there are exactly L1/2 slots and every CTA's slots are all used.
// ---------------------------------------------------------------------------
template <int LOG1> __host__ __device__ constexpr int ct_pair_row(int p, int half) {
  return half ? (p == 0 ? (1 << LOG1) / 2 : (1 << LOG1) - p) : p;
}

// Sequence seq of the CTA's buffer holds row ct_pair_row(p0 + i, half) with
// seq = half P + i (first rows k1 of the CTA's slots, then their partners), so
// that the epilogue's lanes, which take consecutive slots i, read rows one
// odd pitch apart: conflict-free 8-byte shared loads.
template <typename T, int LOG1, int LOG2, int LOGP> struct CtPairSrc {
  const typename MemOf<T>::type *p;  // slab
  int p0;
  __device__ __forceinline__ typename CxOf<T>::type load(int seq, int j, int dr) const {
    // through L2: the column pass may still have been writing when this kernel started
    return cx_load<typename CxOf<T>::type>(
        __ldcg(p + (ct_pair_row<LOG1>(p0 + (seq & ((1 << LOGP) - 1)), seq >> LOGP) << LOG2) + j + dr));
  }
};

struct CtNoDst {
  template <int R, int LOGNS, typename C> __device__ void store(int, int, C *) const {}
};

// row-pair block `pblock` of one packed grid z; outputs Fs[0 .. nf)
template <typename T, int LOGL>
__device__ __forceinline__ void ct_rowpass_body(const typename MemOf<T>::type *slab, const FftDev<T> &f,
                                                const AccParams<typename AccOf<T>::type> &e,
                                                typename MemOf<T>::type *Fs, int pblock) {
  typedef typename CxOf<T>::type C;
  typedef typename AccOf<T>::type A;
  constexpr int LOG1 = (LOGL + 1) / 2, LOG2 = LOGL / 2;
  constexpr int L2 = 1 << LOG2;
  constexpr int LOGB = ilog2c(PassCfg<T>::ELEMS) - LOG2;
  constexpr int B = 1 << LOGB, LOGP = LOGB - 1, P = B >> 1;
  constexpr int PITCH = fft_pitch(L2, B);
  constexpr int THREADS = PassCfg<T>::THREADS;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *s = reinterpret_cast<C *>(smem_raw);
  // unpack twiddles W_ng^k = W_ng^{k1} W_ng^{k2 L1} from two small tables
  // behind the FFT buffer: the CTA's 2P rows and all L2 columns
  C *twr = s + PITCH * B, *twc = twr + B;
  const int p0 = pblock * P;
  pdl_trigger();
  for (int u = threadIdx.x; u < B + L2; u += THREADS) {
    const int q = u < B ? ct_pair_row<LOG1>(p0 + (u >> 1), u & 1) : (u - B) << LOG1;
    A sn, cs;
    sincospi_t((A)q * e.twk, &sn, &cs);
    twr[u] = cmk((T)cs, (T)sn);  // twr[B + k2] is twc[k2]
  }
  pdl_wait();  // the rows come from the column pass
  CtPairSrc<T, LOG1, LOG2, LOGP> src{slab, p0};
  ct_fft<T, LOG2, LOGB, false, false, false>(s, f.tw2, src, CtNoDst());
#pragma unroll 4
  for (int idx = threadIdx.x; idx < (B << LOG2); idx += THREADS) {
    const int i = idx & (P - 1), half = (idx >> LOGP) & 1, k2 = idx >> (LOGP + 1);
    const int p = p0 + i;
    const int k1 = ct_pair_row<LOG1>(p, half);
    const int64_t k = (int64_t)k1 + ((int64_t)k2 << LOG1);
    if (k > e.K) continue;
    // Z[L - k] is in row (L1 - k1) mod L1: the slot's other row, or the
    // same row for the self-paired rows 0 and L1/2 of slot 0
    const int k2m = k1 == 0 ? ((L2 - k2) & (L2 - 1)) : (L2 - 1 - k2);
    const int seqm = p == 0 ? half * P + i : (1 - half) * P + i;
    const C Zk = s[(half * P + i) * PITCH + cpad16(k2)];
    const C Zm = cconj(s[seqm * PITCH + cpad16(k2m)]);
    acc_output_tw<T>(e, k, Zk, Zm, Fs, cmul(twr[2 * i + half], twc[k2]));
  }
}

// three CTAs per SM for the short rows of many small grids (bootstrap), where
// the pass streams from HBM and more bytes in flight pay
template <typename T, int LOGL>
__global__ void __launch_bounds__(PassCfg<T>::THREADS, (sizeof(T) == 4 && LOGL <= 15) ? 3 : 2) k_ct_rowpass_acc(const typename MemOf<T>::type *grid,
                                                                        FftDev<T> f, AccParams<typename AccOf<T>::type> e,
                                                                        typename MemOf<T>::type *F) {
  ct_rowpass_body<T, LOGL>(grid + ((int64_t)blockIdx.y << LOGL), f, e, F + (int64_t)blockIdx.y * e.nf, blockIdx.x);
}

// CTAs per packed grid of the row pass: L1/2 slots, B/2 per CTA
template <typename T, int LOGL> constexpr int ct_rowpass_ctas() {
  return ((1 << ((LOGL + 1) / 2)) / 2) / ((PassCfg<T>::ELEMS >> (LOGL / 2)) / 2);
}

template <typename T, int LOGL> constexpr size_t ct_rowpass_smem() {
  constexpr int LOG2 = LOGL / 2;
  constexpr int B = PassCfg<T>::ELEMS >> LOG2;
  return sizeof(typename CxOf<T>::type) * ((size_t)fft_pitch(1 << LOG2, B) * B + B + (1 << LOG2));
}

}  // namespace
}  // namespace cuna
