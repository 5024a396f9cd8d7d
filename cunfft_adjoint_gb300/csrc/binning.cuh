// binning.cuh -- counting sort of samples into grid tiles (the bucket sort in
// front of the tiled gridding).
//
// A tile is a run of TL consecutive grid cells that one gridding CTA owns.
// Each sample is binned into every tile its filter taps touch (one, or two
// near a tile edge, because the tap span 2m is shorter than a tile), so the
// gridding CTA of a tile finds all its contributions in one contiguous range
// of the sorted record array and owns its cells outright: no global atomics,
// a fixed-order flush.
//
//   k_bin_count   per-CTA shared histogram of tile indices -> counts[tile]
//   k_scan_tiles  exclusive scan counts -> offsets[0..ntiles], cursor = 0
//   k_bin_scatter per-CTA shared ranks + one global reservation per
//                 (CTA, tile) -> records in tile order
//   k_bin_count_resv + k_bin_scatter_resv  for up to kScanFuseTiles tiles:
//                 the count pass also reserves each CTA's range per tile, the
//                 scatter pass scans the counts itself (see there)
//   k_bin_local   one pass, records in chunk-local tile order (see there)
//
// The tile index of a sample is an exact integer function of its input (the
// bucket indices are bit-exact); only the order of records inside a tile
// depends on scheduling.
//
// A Sampler provides `int64_t n`, a `Raw` struct of per-sample inputs and
//   __device__ Raw  load(int64_t i, bool with_value)
//   __device__ void prep(int64_t i, const Raw& r, Prep<Rec>& p)
// prep fills p.nt (0..2), p.t[0..nt) and p.rec.  The kernels issue the loads
// of all of a thread's samples before computing any of them, so that every
// warp keeps several global loads in flight.
#pragma once
#include <algorithm>
#include "common.cuh"

namespace cuna {
namespace {

constexpr int kBinSmemTiles = 6144;  // shared histogram limit (scatter: 2 x 24 KB)
constexpr int kScatterItems = 4;     // samples per thread in k_bin_scatter
constexpr int kCountItems = 8;       // samples per thread in k_bin_count

template <typename Rec> struct Prep {
  int nt;
  int t[2];
  Rec rec;
};

template <class S>
__global__ void __launch_bounds__(512) k_bin_count(S smp, int *__restrict__ counts, int ntiles) {
  extern __shared__ int lc[];
  const bool sm = ntiles <= kBinSmemTiles;
  if (sm) {
    for (int t = threadIdx.x; t < ntiles; t += blockDim.x) lc[t] = 0;
    __syncthreads();
  }
  const int64_t span = (int64_t)blockDim.x * kCountItems;
  for (int64_t c0 = (int64_t)blockIdx.x * span; c0 < smp.n; c0 += (int64_t)gridDim.x * span) {
    typename S::Raw raw[kCountItems];
#pragma unroll
    for (int it = 0; it < kCountItems; ++it) {
      const int64_t i = c0 + (int64_t)it * blockDim.x + threadIdx.x;
      if (i < smp.n) raw[it] = smp.load(i, false);
    }
#pragma unroll
    for (int it = 0; it < kCountItems; ++it) {
      const int64_t i = c0 + (int64_t)it * blockDim.x + threadIdx.x;
      if (i >= smp.n) continue;
      Prep<typename S::Rec> p;
      smp.prep(i, raw[it], p);
      for (int q = 0; q < p.nt; ++q) {
        if (sm) atomicAdd(&lc[p.t[q]], 1);
        else atomicAdd(&counts[p.t[q]], 1);
      }
    }
  }
  if (sm) {
    __syncthreads();
    for (int t = threadIdx.x; t < ntiles; t += blockDim.x)
      if (lc[t]) atomicAdd(&counts[t], lc[t]);
  }
}

// Single CTA (1024 threads): offsets[t] = sum_{u<t} counts[u], offsets[ntiles]
// = total, cursor[t] = 0.
__global__ void __launch_bounds__(1024) k_scan_tiles(const int *__restrict__ counts,
                                                     int *__restrict__ offsets,
                                                     int *__restrict__ cursor, int ntiles) {
  __shared__ int wsum[32];
  const int tid = threadIdx.x, nt = blockDim.x;
  const int per = (ntiles + nt - 1) / nt;
  const int beg = min(tid * per, ntiles), end = min(beg + per, ntiles);
  int sum = 0;
  for (int i = beg; i < end; ++i) sum += counts[i];
  const int lane = tid & 31, w = tid >> 5;
  int v = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int u = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += u;
  }
  if (lane == 31) wsum[w] = v;
  __syncthreads();
  if (w == 0) {
    int s = lane < (nt >> 5) ? wsum[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int u = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += u;
    }
    wsum[lane] = s;
  }
  __syncthreads();
  int run = v - sum + (w > 0 ? wsum[w - 1] : 0);
  for (int i = beg; i < end; ++i) {
    offsets[i] = run;
    run += counts[i];
    cursor[i] = 0;
  }
  if (tid == nt - 1) offsets[ntiles] = wsum[(nt >> 5) - 1];
}

template <class S>
__global__ void __launch_bounds__(512) k_bin_scatter(S smp, const int *__restrict__ offsets,
                                                     int *__restrict__ cursor,
                                                     typename S::Rec *__restrict__ recs,
                                                     int ntiles) {
  typedef typename S::Rec Rec;
  extern __shared__ int sh[];
  int *lc = sh, *lbase = sh + ntiles;
  const bool sm = ntiles <= kBinSmemTiles;
  if (sm) {
    for (int t = threadIdx.x; t < ntiles; t += blockDim.x) lc[t] = 0;
    __syncthreads();
  }
  const int64_t chunk0 = (int64_t)blockIdx.x * blockDim.x * kScatterItems;
  Prep<Rec> p[kScatterItems];
  int rk[kScatterItems][2];
  typename S::Raw raw[kScatterItems];
#pragma unroll
  for (int it = 0; it < kScatterItems; ++it) {
    const int64_t i = chunk0 + (int64_t)it * blockDim.x + threadIdx.x;
    if (i < smp.n) raw[it] = smp.load(i, true);
  }
#pragma unroll
  for (int it = 0; it < kScatterItems; ++it) {
    const int64_t i = chunk0 + (int64_t)it * blockDim.x + threadIdx.x;
    p[it].nt = 0;
    if (i < smp.n) smp.prep(i, raw[it], p[it]);
    for (int q = 0; q < p[it].nt; ++q) {
      const int t = p[it].t[q];
      rk[it][q] = sm ? atomicAdd(&lc[t], 1) : offsets[t] + atomicAdd(&cursor[t], 1);
    }
  }
  if (sm) {
    __syncthreads();
    for (int t = threadIdx.x; t < ntiles; t += blockDim.x)
      if (lc[t]) lbase[t] = offsets[t] + atomicAdd(&cursor[t], lc[t]);
    __syncthreads();
  }
#pragma unroll
  for (int it = 0; it < kScatterItems; ++it)
    for (int q = 0; q < p[it].nt; ++q) {
      const int pos = sm ? lbase[p[it].t[q]] + rk[it][q] : rk[it][q];
      recs[pos] = p[it].rec;
    }
}

// Exclusive scan of n ints in shared memory by the whole CTA (blockDim.x a
// multiple of 32, <= 1024): out[i] = sum_{u<i} in[u], out[n] = total.  `in`
// and `out` may not alias.  Ends with a barrier.
__device__ __forceinline__ void cta_exclusive_scan(const int *in, int *out, int n) {
  __shared__ int wsum[32];
  const int nt = blockDim.x, tid = threadIdx.x;
  const int per = (n + nt - 1) / nt;
  const int beg = min(tid * per, n), end = min(beg + per, n);
  int sum = 0;
  for (int i = beg; i < end; ++i) sum += in[i];
  const int lane = tid & 31, w = tid >> 5;
  int v = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int u = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += u;
  }
  if (lane == 31) wsum[w] = v;
  __syncthreads();
  if (w == 0) {
    int s = lane < (nt >> 5) ? wsum[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += u;
    }
    wsum[lane] = s;
  }
  __syncthreads();
  int run = v - sum + (w > 0 ? wsum[w - 1] : 0);
  for (int i = beg; i < end; ++i) {
    out[i] = run;
    run += in[i];
  }
  if (tid == nt - 1) out[n] = wsum[(nt >> 5) - 1];
  __syncthreads();
}

// Reserved binning for up to kScanFuseTiles tiles, two launches.  Both passes
// split the samples the same way: CTA b owns [b*span, min((b+1)*span, n)).
//   k_bin_count_resv    shared histogram of the CTA's tiles; per touched tile
//                       one returning global atomic on counts[t] reserves the
//                       CTA's range inside the tile: resv[b*ntiles + t] is its
//                       start relative to the tile's start.
//   k_bin_scatter_resv  scans the tile counts itself (CTA 0 publishes
//                       offsets[0..ntiles]), then ranks each sample with a
//                       shared atomic and writes its record straight to
//                       offsets[t] + resv[b*ntiles + t] + rank.
// The ranks of CTA b in the second pass cover exactly the counts it reserved
// in the first, so the positions are a permutation of [0, offsets[ntiles]).
// No global atomic is left in the scatter pass and nothing waits on one.
// Both are launched with 512 threads; span is a multiple of 512.
constexpr int kScanFuseTiles = 4096;  // 3 shared arrays of ntiles ints: 48 KB
constexpr int kResvEntries = 1 << 22; // reservation table limit (ints)

template <class S>
__global__ void __launch_bounds__(512) k_bin_count_resv(S smp, int *__restrict__ counts, int *__restrict__ resv,
                                                        int ntiles, int64_t span) {
  extern __shared__ int lc[];
  constexpr int TPT = kScanFuseTiles / 512;
  pdl_trigger();  // the scatter pass may launch and wait for this grid
#pragma unroll
  for (int k = 0; k < TPT; ++k) {
    const int t = threadIdx.x + k * 512;
    if (t < ntiles) lc[t] = 0;
  }
  __syncthreads();
  const int64_t beg = (int64_t)blockIdx.x * span, end = min(beg + span, smp.n);
  for (int64_t c0 = beg; c0 < end; c0 += 512 * kCountItems) {
    typename S::Raw raw[kCountItems];
#pragma unroll
    for (int it = 0; it < kCountItems; ++it) {
      const int64_t i = c0 + it * 512 + threadIdx.x;
      if (i < end) raw[it] = smp.load(i, false);
    }
#pragma unroll
    for (int it = 0; it < kCountItems; ++it) {
      const int64_t i = c0 + it * 512 + threadIdx.x;
      if (i >= end) continue;
      Prep<typename S::Rec> p;
      smp.prep(i, raw[it], p);
      for (int q = 0; q < p.nt; ++q) atomicAdd(&lc[p.t[q]], 1);
    }
  }
  __syncthreads();
  int res[TPT];
#pragma unroll
  for (int k = 0; k < TPT; ++k) {
    const int t = threadIdx.x + k * 512;
    const int c = t < ntiles ? lc[t] : 0;
    res[k] = c ? atomicAdd(&counts[t], c) : 0;
  }
  int *rv = resv + (int64_t)blockIdx.x * ntiles;
#pragma unroll
  for (int k = 0; k < TPT; ++k) {
    const int t = threadIdx.x + k * 512;
    if (t < ntiles && lc[t]) rv[t] = res[k];
  }
}

template <class S>
__global__ void __launch_bounds__(512) k_bin_scatter_resv(S smp, const int *counts, const int *resv, int *offsets,
                                                          typename S::Rec *recs, int ntiles, int64_t span) {
  typedef typename S::Rec Rec;
  extern __shared__ int sh[];
  int *lc = sh, *base = sh + ntiles, *off = sh + 2 * ntiles;  // off: ntiles + 1
  constexpr int TPT = kScanFuseTiles / 512;
  const int *rv = resv + (int64_t)blockIdx.x * ntiles;
  pdl_trigger();
  pdl_wait();  // counts and reservations come from the count pass
  int res[TPT];
#pragma unroll
  for (int k = 0; k < TPT; ++k) {
    const int t = threadIdx.x + k * 512;
    res[k] = 0;
    if (t < ntiles) {
      lc[t] = 0;
      base[t] = __ldcg(counts + t);  // the count pass's output, through L2
      res[k] = __ldcg(rv + t);       // entries of untouched tiles are stale and never used
    }
  }
  __syncthreads();
  cta_exclusive_scan(base, off, ntiles);
  if (blockIdx.x == 0)
    for (int t = threadIdx.x; t <= ntiles; t += blockDim.x) offsets[t] = off[t];
#pragma unroll
  for (int k = 0; k < TPT; ++k) {
    const int t = threadIdx.x + k * 512;
    if (t < ntiles) base[t] = off[t] + res[k];
  }
  __syncthreads();
  const int64_t beg = (int64_t)blockIdx.x * span, end = min(beg + span, smp.n);
  for (int64_t c0 = beg; c0 < end; c0 += 512 * kCountItems) {
    typename S::Raw raw[kCountItems];
#pragma unroll
    for (int it = 0; it < kCountItems; ++it) {
      const int64_t i = c0 + it * 512 + threadIdx.x;
      if (i < end) raw[it] = smp.load(i, true);
    }
#pragma unroll
    for (int it = 0; it < kCountItems; ++it) {
      const int64_t i = c0 + it * 512 + threadIdx.x;
      if (i >= end) continue;
      Prep<Rec> p;
      smp.prep(i, raw[it], p);
      for (int q = 0; q < p.nt; ++q) {
        const int t = p.t[q];
        recs[base[t] + atomicAdd(&lc[t], 1)] = p.rec;
      }
    }
  }
}

// Samples per CTA of the reserved binning: about two CTAs per SM (nsm SMs)
// so that the one wave is balanced, a multiple of 512, at least 512, and
// enough that the reservation table (CTAs x ntiles ints) stays within
// kResvEntries.
inline int64_t resv_span(int64_t n, int ntiles, int nsm) {
  const int64_t maxb = std::max<int64_t>(1, kResvEntries / std::max(ntiles, 1));
  int64_t span = std::max((n + maxb - 1) / maxb, (n + 2 * (int64_t)nsm - 1) / (2 * (int64_t)std::max(nsm, 1)));
  span = std::max<int64_t>(512, (span + 511) / 512 * 512);
  return span;
}

// Multi-CTA form of k_scan_tiles for long tile lists: k_scan_blocks scans
// chunks of kScanChunk counts per CTA (local exclusive offsets + chunk
// totals), k_scan_add adds each chunk's prefix of totals, writes
// offsets[ntiles] and zeroes cursor.
constexpr int kScanChunk = 4096;  // 1024 threads x 4

__global__ void __launch_bounds__(1024) k_scan_blocks(const int *__restrict__ counts, int *__restrict__ offsets,
                                                      int *__restrict__ totals, int ntiles) {
  __shared__ int in[kScanChunk], out[kScanChunk + 1];
  const int base = blockIdx.x * kScanChunk, cnt = min(kScanChunk, ntiles - base);
  for (int i = threadIdx.x; i < cnt; i += blockDim.x) in[i] = counts[base + i];
  __syncthreads();
  cta_exclusive_scan(in, out, cnt);
  for (int i = threadIdx.x; i < cnt; i += blockDim.x) offsets[base + i] = out[i];
  if (threadIdx.x == 0) totals[blockIdx.x] = out[cnt];
}

__global__ void __launch_bounds__(1024) k_scan_add(int *__restrict__ offsets, const int *__restrict__ totals,
                                                   int *__restrict__ cursor, int ntiles, int nblocks) {
  __shared__ int add;
  if (threadIdx.x == 0) {
    int a = 0;
    for (int b = 0; b < (int)blockIdx.x; ++b) a += totals[b];
    add = a;
    if (blockIdx.x == nblocks - 1) offsets[ntiles] = a + totals[blockIdx.x];
  }
  __syncthreads();
  const int base = blockIdx.x * kScanChunk, cnt = min(kScanChunk, ntiles - base);
  for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
    offsets[base + i] += add;
    cursor[base + i] = 0;
  }
}

// k_bin_local: single-pass binning into chunk-local tile order.  CTA c takes
// the samples [c CH, (c+1) CH), counts its records per tile in shared memory,
// scans the counts, and writes its records tile by tile into its own region
// recs[c 2CH ..] (a sample makes at most two records).  loc[tau nch + c] =
// start | count << 16 describes chunk c's run of tile tau, so the gridding CTA
// of tau finds its records as nch runs (SegSrc).  No global atomics and no
// separate count pass: each sample's phase is computed twice (count, write),
// the second time from an L2-resident t.  Needs 2 CH < 2^16, ntiles <=
// kScanFuseTiles.
template <class S>
__global__ void __launch_bounds__(512) k_bin_local(S smp, typename S::Rec *__restrict__ recs,
                                                   int *__restrict__ loc, int ntiles, int nch, int CH) {
  typedef typename S::Rec Rec;
  extern __shared__ int sh[];
  int *hist = sh, *cur = sh + ntiles;  // cur: ntiles + 1
  const int c = blockIdx.x;
  const int64_t i0 = (int64_t)c * CH, i1 = min(i0 + (int64_t)CH, smp.n);
  for (int t = threadIdx.x; t < ntiles; t += blockDim.x) hist[t] = 0;
  __syncthreads();
  for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
    Prep<Rec> p;
    smp.prep(i, smp.load(i, false), p);
    for (int q = 0; q < p.nt; ++q) atomicAdd(&hist[p.t[q]], 1);
  }
  __syncthreads();
  cta_exclusive_scan(hist, cur, ntiles);
  for (int t = threadIdx.x; t < ntiles; t += blockDim.x) loc[(int64_t)t * nch + c] = cur[t] | (hist[t] << 16);
  __syncthreads();
  Rec *out = recs + (int64_t)c * 2 * CH;
  for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
    Prep<Rec> p;
    smp.prep(i, smp.load(i, true), p);
    for (int q = 0; q < p.nt; ++q) out[atomicAdd(&cur[p.t[q]], 1)] = p.rec;
  }
}

}  // namespace
}  // namespace cuna
