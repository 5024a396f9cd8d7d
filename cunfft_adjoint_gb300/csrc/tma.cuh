// tma.cuh -- Tensor Memory Accelerator copies and mbarrier waits (inline PTX,
// sm_90+ forms as on sm_103a).
//
// A CTA stages a box of global memory into shared memory with
// cp.async.bulk.tensor (one elected thread issues the copies, an mbarrier
// counts the bytes in) and writes shared memory back with the store form
// (bulk async-group, waited on before the CTA ends).  Every wait is bounded:
// mbar_wait gives up after kWaitRounds rounds of try_wait (each suspends for
// at most kWaitHintNs), about a second, so a copy that never lands turns into
// a counted error instead of a hung CTA.
#pragma once
#include <cuda.h>
#include <stdint.h>

namespace cuna {
namespace {

constexpr int kWaitRounds = 1 << 20;
constexpr uint32_t kWaitHintNs = 1000;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// the initialised barrier is visible to the async proxy (the copy engine)
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// shared-memory writes of this thread are visible to the async proxy
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity), "r"(kWaitHintNs)
      : "memory");
  return ok != 0;
}

// true once the barrier's phase `parity` has completed; false after the limit
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
  for (int i = 0; i < kWaitRounds; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// box at element coordinates (x, y, z) of `map` -> shared memory `dst`
// (x * element size a multiple of 16 bytes); completes bytes on `bar`
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

// shared memory `src` -> box at (x, y, z) of `map`, in the current bulk group
__device__ __forceinline__ void tma_store_3d(const CUtensorMap *map, int x, int y, int z, const void *src) {
  asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3}], [%4];" ::"l"(
                   reinterpret_cast<uint64_t>(map)),
               "r"(x), "r"(y), "r"(z), "r"(smem_u32(src))
               : "memory");
}

__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }

// every committed bulk store of this thread has completed (writes performed)
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

}  // namespace
}  // namespace cuna
