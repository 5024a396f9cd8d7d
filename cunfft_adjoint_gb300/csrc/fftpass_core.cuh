// fftpass_core.cuh -- Stockham stages and the four-step column pass with the
// whole geometry fixed at compile time (shared by the accurate and compat
// transforms; the accurate row pass is in fftpass.cuh).
//
// Same Stockham algorithm as fft.cuh (one leading radix 2/4/8/16 stage, then
// radix-16 stages; 16 values per thread; one shared buffer), but lengths,
// strides, masks and shifts are template constants, one kernel instance per
// transform length L = 2^LOGL (L1 = 2^ceil(LOGL/2), L2 = 2^floor(LOGL/2)).
// The shared-memory index of a thread's r-th value splits as
//     pad16(j + (r << s)) = pad16(j) + pad16(r << s)      (j < 2^s, or s >= 4)
// because the two addends never carry across bit 4, so the 16 accesses of a
// stage use one base address and immediate offsets.  The column pass takes
// its W_L^{c k} twiddles as (per-butterfly base) x (per-CTA table of 16 x B
// steps in shared memory) instead of two global table reads per value.
#pragma once
#include <type_traits>
#include "fft.cuh"
#include "runtime.h"
#include "tma.cuh"

namespace cuna {
namespace {

__host__ __device__ constexpr int ilog2c(int v) { return v <= 1 ? 0 : 1 + ilog2c(v >> 1); }

template <int R> struct RLog {
  static constexpr int v = R == 2 ? 1 : R == 4 ? 2 : R == 8 ? 3 : 4;
};

__host__ __device__ constexpr int cpad16(int i) { return i + (i >> 4); }

// Sources and destinations that live in the stage's own shared buffer
// (kShared = true) need a barrier between the stage's reads and its writes.
template <class X, class = void> struct in_smem : std::false_type {};
template <class X> struct in_smem<X, std::void_t<decltype(X::kShared)>> : std::bool_constant<X::kShared> {};

template <typename T> struct PassCfg {
  static constexpr int ELEMS = sizeof(T) == 4 ? kPassElemsF32 : kPassElemsF64;
  static constexpr int THREADS = ELEMS / kFftE;
};

// One Stockham stage of radix R over the 2^LOGS sequences of length 2^LOGN a
// CTA holds; 2^LOGNS points already transformed.  IN_G / OUT_G: the stage
// reads from src / writes to dst instead of shared memory.  SEQ_FAST: thread
// g takes sequence g mod 2^LOGS (else point-fastest).
template <typename T, int R, int LOGN, int LOGNS, int LOGS, bool IN_G, bool OUT_G, bool SEQ_FAST, class Src,
          class Dst>
__device__ __forceinline__ void ct_stage(typename CxOf<T>::type *s, const typename CxOf<T>::type *__restrict__ tw,
                                         const Src &src, const Dst &dst) {
  typedef typename CxOf<T>::type C;
  constexpr int LOGR = RLog<R>::v;
  constexpr int NB = kFftE / R;
  constexpr int LOGLR = LOGN - LOGR;
  constexpr int THREADS = 1 << (LOGN + LOGS - 4);
  constexpr int PITCH = fft_pitch(1 << LOGN, 1 << LOGS);
  constexpr int TWSH = LOGN - LOGNS - LOGR;
  static_assert(THREADS * kFftE == (1 << (LOGN + LOGS)), "one value set per thread");
  C v[NB][R];
#pragma unroll
  for (int u = 0; u < NB; ++u) {
    const int g = threadIdx.x + u * THREADS;
    const int seq = SEQ_FAST ? (g & ((1 << LOGS) - 1)) : (g >> LOGLR);
    const int j = SEQ_FAST ? (g >> LOGS) : (g & ((1 << LOGLR) - 1));
    if (IN_G) {
#pragma unroll
      for (int r = 0; r < R; ++r) v[u][r] = src.load(seq, j, r << LOGLR);
    } else {
      const C *b = s + seq * PITCH + cpad16(j);
#pragma unroll
      for (int r = 0; r < R; ++r) v[u][r] = b[cpad16(r << LOGLR)];
    }
    if (LOGNS > 0) {
      // tw[q] = exp(+2 pi i q / 2^LOGN): W_{R Ns}^{r k} = tw[(r k) << TWSH].
      // float: six table reads per radix-16 butterfly, w_1..w_3 and w_4, w_8,
      // w_12, with w_{a + 4b} = w_a w_{4b} (one rounding more than a table
      // value); double reads all 15 (the FP64 pipe, not the loads, bounds it).
      const int step = (j & ((1 << LOGNS) - 1)) << TWSH;
      if (sizeof(T) == 8) {
#pragma unroll
        for (int r = 1; r < R; ++r) v[u][r] = cmul(v[u][r], ldtw(tw + r * step));
      } else {
      C wa[4];
#pragma unroll
      for (int a = 1; a < (R < 4 ? R : 4); ++a) wa[a] = ldtw(tw + a * step);
#pragma unroll
      for (int b = 0; b < R; b += 4) {
        C wb = cmk((T)1, (T)0);
        if (b > 0) wb = ldtw(tw + b * step);
#pragma unroll
        for (int a = 0; a < 4 && a < R; ++a) {
          const int r = a + b;
          if (r == 0) continue;
          const C w = b == 0 ? wa[a] : (a == 0 ? wb : cmul(wa[a], wb));
          v[u][r] = cmul(v[u][r], w);
        }
      }
      }
    }
    dftR<R>(v[u]);
  }
  if ((!IN_G || in_smem<Src>::value) && (!OUT_G || in_smem<Dst>::value)) __syncthreads();
#pragma unroll
  for (int u = 0; u < NB; ++u) {
    const int g = threadIdx.x + u * THREADS;
    const int seq = SEQ_FAST ? (g & ((1 << LOGS) - 1)) : (g >> LOGLR);
    const int j = SEQ_FAST ? (g >> LOGS) : (g & ((1 << LOGLR) - 1));
    const int idxD = ((j >> LOGNS) << (LOGNS + LOGR)) + (j & ((1 << LOGNS) - 1));
    if (OUT_G) {
      dst.template store<R, LOGNS>(seq, idxD, v[u]);
    } else {
      C *b = s + seq * PITCH + cpad16(idxD);
#pragma unroll
      for (int r = 0; r < R; ++r) b[cpad16(r << LOGNS)] = v[u][r];
    }
  }
  if (!OUT_G) __syncthreads();
}

// radix-16 stages from LOGNS on; the last one writes to dst when TO_GLOBAL
template <typename T, int LOGN, int LOGS, int LOGNS, bool TO_GLOBAL, bool FSF, bool LSF, class Src, class Dst>
__device__ __forceinline__ void ct_rest(typename CxOf<T>::type *s, const typename CxOf<T>::type *__restrict__ tw,
                                        const Src &src, const Dst &dst) {
  if constexpr (LOGNS + 4 >= LOGN) {
    ct_stage<T, 16, LOGN, LOGNS, LOGS, false, TO_GLOBAL, TO_GLOBAL ? LSF : FSF>(s, tw, src, dst);
  } else {
    ct_stage<T, 16, LOGN, LOGNS, LOGS, false, false, FSF>(s, tw, src, dst);
    ct_rest<T, LOGN, LOGS, LOGNS + 4, TO_GLOBAL, FSF, LSF>(s, tw, src, dst);
  }
}

// Src -> stages -> Dst (TO_GLOBAL) or -> shared memory s[seq*PITCH + pad16(k)]
// followed by a barrier.  FSF / LSF: thread mapping of the loading stages /
// of the storing stage.
template <typename T, int LOGN, int LOGS, bool TO_GLOBAL, bool FSF, bool LSF, class Src, class Dst>
__device__ __forceinline__ void ct_fft(typename CxOf<T>::type *s, const typename CxOf<T>::type *__restrict__ tw,
                                       const Src &src, const Dst &dst) {
  constexpr int R0L = (LOGN & 3) == 0 ? 4 : (LOGN & 3);
  if constexpr (R0L == LOGN) {
    ct_stage<T, (1 << R0L), LOGN, 0, LOGS, true, TO_GLOBAL, TO_GLOBAL ? LSF : FSF>(s, tw, src, dst);
  } else {
    ct_stage<T, (1 << R0L), LOGN, 0, LOGS, true, false, FSF>(s, tw, src, dst);
    ct_rest<T, LOGN, LOGS, R0L, TO_GLOBAL, FSF, LSF>(s, tw, src, dst);
  }
}

// ---------------------------------------------------------------------------
// column pass: FFTs of length L1 down the columns [c0, c0 + B) of one slab
// (row-major L1 x L2), times W_L^{c k1}, stored in place.
// ---------------------------------------------------------------------------
template <typename T, int LOG1, int LOG2> struct CtColSrc {
  const typename MemOf<T>::type *p;  // slab + c0
  __device__ __forceinline__ typename CxOf<T>::type load(int seq, int j, int dr) const {
    // through L2: the gridding may still have been writing when this kernel started
    return cx_load<typename CxOf<T>::type>(__ldcg(p + ((j + dr) << LOG2) + seq));
  }
};

template <typename T, int LOG1, int LOG2, int LOGB> struct CtColDst {
  typename MemOf<T>::type *p;             // slab + c0
  const typename CxOf<T>::type *steps;    // shared: steps[seq * 17 + r] = W_L^{c (r << LOGNS_last)}
  FftDev<T> f;
  int c0;
  template <int R, int LOGNS>
  __device__ __forceinline__ void store(int seq, int idxD, typename CxOf<T>::type *v) const {
    typedef typename CxOf<T>::type C;
    static_assert(R == 16 || LOGNS == 0, "the storing stage is radix 16 or the only stage");
    const C w0 = twiddle_L(f, (c0 + seq) * idxD);
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const C w = r == 0 ? w0 : cmul(w0, steps[seq * 17 + r]);
      p[((idxD + (r << LOGNS)) << LOG2) + seq] = cx_to_mem(cmul(v[r], w));
    }
  }
};

// last stage's point stride 2^LOGNS for a length-2^LOGN transform
template <int LOGN> __host__ __device__ constexpr int last_logns() {
  return LOGN <= 4 ? 0 : LOGN - 4;
}

// column block `cblock` of one packed grid (L1 x L2 complex, row-major), from
// `in` to `out` (in == out allowed: every read precedes the first barrier,
// every write follows it)
template <typename T, int LOGL>
__device__ __forceinline__ void ct_colpass_body(const typename MemOf<T>::type *in, typename MemOf<T>::type *out,
                                                const FftDev<T> &f, int cblock) {
  typedef typename CxOf<T>::type C;
  constexpr int LOG1 = (LOGL + 1) / 2, LOG2 = LOGL / 2;
  constexpr int LOGB = ilog2c(PassCfg<T>::ELEMS) - LOG1;
  constexpr int B = 1 << LOGB;
  constexpr int PITCH = fft_pitch(1 << LOG1, B);
  constexpr int LNS = last_logns<LOG1>();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *s = reinterpret_cast<C *>(smem_raw);
  C *steps = s + PITCH * B;
  const int c0 = cblock * B;
  pdl_trigger();
  // stride 17 so that the columns of one row of the table fall in different banks
  for (int i = threadIdx.x; i < 16 * B; i += PassCfg<T>::THREADS)
    steps[(i >> 4) * 17 + (i & 15)] = twiddle_L(f, (c0 + (i >> 4)) * ((i & 15) << LNS));
  // the steps table is read only by the storing stage, after at least one barrier
  pdl_wait();  // the grid comes from the gridding
  CtColSrc<T, LOG1, LOG2> src{in + c0};
  CtColDst<T, LOG1, LOG2, LOGB> dst{out + c0, steps, f, c0};
  // reads all precede the first barrier, writes all follow it: in place is safe
  ct_fft<T, LOG1, LOGB, true, true, true>(s, f.tw1, src, dst);
}

template <typename T, int LOGL>
__global__ void __launch_bounds__(PassCfg<T>::THREADS) k_ct_colpass(typename MemOf<T>::type *grid, FftDev<T> f,
                                                                    int64_t slab_stride) {
  typename MemOf<T>::type *z = grid + blockIdx.y * slab_stride;
  ct_colpass_body<T, LOGL>(z, z, f, blockIdx.x);
}

template <typename T, int LOGL> constexpr size_t ct_colpass_smem() {
  constexpr int LOG1 = (LOGL + 1) / 2;
  constexpr int B = PassCfg<T>::ELEMS >> LOG1;
  return sizeof(typename CxOf<T>::type) * ((size_t)fft_pitch(1 << LOG1, B) * B + 17 * B);
}

// ---------------------------------------------------------------------------
// column pass with TMA (float, B >= 2 columns per CTA): the CTA's B columns
// (L1 rows x 8B bytes, one row every L2 complex) come in as L1/256 boxes of a
// 3D tensor map {2 L2 floats, L1 rows, slabs} into shared memory, row-major
// [row][column] ("dense"); the first stage reads them from there, the last
// stage writes the twiddled result back in the same dense order and the
// boxes go out with TMA stores.  No strided global access is left to the
// load/store units.  A copy that does not complete within the bounded wait
// is counted in `timeouts` and the CTA leaves its columns unwritten.
// ---------------------------------------------------------------------------
template <typename T, int LOGB> struct CtDenseSrc {
  static constexpr bool kShared = true;
  const typename CxOf<T>::type *s;
  __device__ __forceinline__ typename CxOf<T>::type load(int seq, int j, int dr) const {
    return s[((j + dr) << LOGB) + seq];
  }
};

template <typename T, int LOGB> struct CtDenseDst {
  static constexpr bool kShared = true;
  typename CxOf<T>::type *s;
  const typename CxOf<T>::type *steps;  // shared: steps[seq * 17 + r] = W_L^{c (r << LOGNS_last)}
  FftDev<T> f;
  int c0;
  template <int R, int LOGNS>
  __device__ __forceinline__ void store(int seq, int idxD, typename CxOf<T>::type *v) const {
    typedef typename CxOf<T>::type C;
    static_assert(R == 16 || LOGNS == 0, "the storing stage is radix 16 or the only stage");
    const C w0 = twiddle_L(f, (c0 + seq) * idxD);
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const C w = r == 0 ? w0 : cmul(w0, steps[seq * 17 + r]);
      s[((idxD + (r << LOGNS)) << LOGB) + seq] = cmul(v[r], w);
    }
  }
};

template <int LOGL> struct TmaCol {
  static constexpr int LOG1 = (LOGL + 1) / 2, LOG2 = LOGL / 2;
  static constexpr int LOGB = ilog2c(PassCfg<float>::ELEMS) - LOG1;
  static constexpr int B = 1 << LOGB;
  static constexpr int ROWS = (1 << LOG1) < 256 ? (1 << LOG1) : 256;  // rows per box
  static constexpr int NBOX = (1 << LOG1) / ROWS;
  static constexpr bool ok = B >= 2;  // box rows of >= 16 bytes
};

template <int LOGL>
__global__ void __launch_bounds__(PassCfg<float>::THREADS) k_ct_colpass_tma(const __grid_constant__ CUtensorMap map,
                                                                           FftDev<float> f, int *timeouts) {
  typedef TmaCol<LOGL> G;
  typedef typename CxOf<float>::type C;
  constexpr int LOG1 = G::LOG1, LOGB = G::LOGB, B = G::B;
  constexpr int PITCH = fft_pitch(1 << LOG1, B);
  constexpr int LNS = last_logns<LOG1>();
  static_assert(G::ok, "TMA column pass needs two columns per CTA");
  extern __shared__ __align__(128) unsigned char smem_tma[];
  C *s = reinterpret_cast<C *>(smem_tma);
  C *steps = s + PITCH * B;
  uint64_t *bar = reinterpret_cast<uint64_t *>(steps + 17 * B);
  const int c0 = blockIdx.x * B, slab = blockIdx.y;
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    mbar_arrive_expect_tx(bar, (uint32_t)(sizeof(C) << (LOG1 + LOGB)));
#pragma unroll 1
    for (int b = 0; b < G::NBOX; ++b) tma_load_3d(s + b * G::ROWS * B, &map, 2 * c0, b * G::ROWS, slab, bar);
  }
  for (int i = threadIdx.x; i < 16 * B; i += PassCfg<float>::THREADS)
    steps[(i >> 4) * 17 + (i & 15)] = twiddle_L(f, (c0 + (i >> 4)) * ((i & 15) << LNS));
  if (!__syncthreads_and(mbar_wait(bar, 0))) {
    if (threadIdx.x == 0) atomicAdd(timeouts, 1);
    return;
  }
  CtDenseSrc<float, LOGB> src{s};
  CtDenseDst<float, LOGB> dst{s, steps, f, c0};
  ct_fft<float, LOG1, LOGB, true, true, true>(s, f.tw1, src, dst);
  fence_proxy_async_smem();
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll 1
    for (int b = 0; b < G::NBOX; ++b) tma_store_3d(&map, 2 * c0, b * G::ROWS, slab, s + b * G::ROWS * B);
    bulk_commit();
    bulk_wait_all();
  }
}

template <int LOGL> constexpr size_t ct_colpass_tma_smem() { return ct_colpass_smem<float, LOGL>() + 16; }

// The tensor map of k_ct_colpass_tma for `nslab` packed grids of L = 2^LOGL
// complex at `z` (slab stride L).
template <int LOGL> bool ct_colpass_tma_map(void *map, const void *z, int nslab) {
  typedef TmaCol<LOGL> G;
  const uint64_t L2 = 1ull << G::LOG2, L1 = 1ull << G::LOG1;
  return encode_tmap_f32_3d(map, z, 2 * L2, L1, (uint64_t)nslab, 2 * L2 * sizeof(float),
                            (L1 * L2) * 2 * sizeof(float), 2 * G::B, G::ROWS);
}

}  // namespace
}  // namespace cuna
