// rng.cuh -- the reference's bootstrap draw stream: d = xorshift32(wang_hash(
// seed + i)) % n (src/gridding.cu:67-82,101), shared by compat and accurate
// bootstrap.
#pragma once

namespace cuna {
namespace {

// wang_hash, src/gridding.cu:67-74
__device__ __forceinline__ unsigned wang_hash(unsigned s) {
  s = (s ^ 61u) ^ (s >> 16);
  s *= 9u;
  s = s ^ (s >> 4);
  s *= 0x27d4eb2du;
  s = s ^ (s >> 15);
  return s;
}
// rand_XORSHIFT, src/gridding.cu:76-82
__device__ __forceinline__ unsigned xorshift32(unsigned s) {
  s ^= (s << 13);
  s ^= (s >> 17);
  s ^= (s << 5);
  return s;
}
// draw number i of the stream: the sample index d = xorshift32(wang_hash(
// seed + i)) % n (src/gridding.cu:101, unsigned arithmetic throughout)
__device__ __forceinline__ unsigned boot_draw(unsigned seed, unsigned i, unsigned n) {
  return xorshift32(wang_hash(seed + i)) % n;
}

}  // namespace
}  // namespace cuna
