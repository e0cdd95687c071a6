// async.cuh -- mbarrier and bulk-copy (cp.async.bulk) helpers for sm_103a.
//
// Every wait is bounded: after kSpinLimit failed try_wait polls the caller
// gets `false`, records an error code in a device status word and leaves
// the pipeline, so a lost arrival can never hang the GPU.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace opir {

// status codes written to the device status word
constexpr uint32_t kErrWaitFull = 1u;   // consumer gave up waiting for a copy
constexpr uint32_t kErrWaitEmpty = 2u;  // producer gave up waiting for a free stage
constexpr uint32_t kErrDrain = 4u;      // producer gave up draining its copies

constexpr uint32_t kSpinLimit = 1u << 22;
constexpr uint32_t kSuspendHintNs = 2000;  // per try_wait; the wait stays bounded by kSpinLimit tries

// A kernel's status area is kStatusWords words: [0] the error bits above,
// [1] a test hook read by the single-query scan -- nonzero: its first CTA
// withholds the copies of its first pipeline stage and its waits give up
// after that many polls, so a test can make a consumer wait run out (the
// host sets it through opir_debug_withhold_scan_stage; 0 in production).
constexpr int kStatusWords = 4;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// try_wait with a suspend-time hint: a waiting warp sleeps (up to the hint)
// instead of spinning, leaving issue slots to the warps that have work.
__device__ __forceinline__ bool mbar_try_wait_hint(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity), "r"(kSuspendHintNs)
      : "memory");
  return ok != 0;
}

// Bounded wait for the phase with the given parity to complete.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity,
                                          uint32_t limit = kSpinLimit) {
  for (uint32_t i = 0; i < limit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// Bounded wait that sleeps between polls (consumer side of a pipeline).
__device__ __forceinline__ bool mbar_wait_sleep(uint64_t *bar, uint32_t parity,
                                                uint32_t limit = kSpinLimit) {
  for (uint32_t i = 0; i < limit; ++i)
    if (mbar_try_wait_hint(bar, parity)) return true;
  return false;
}

// Bulk copy global -> shared, completion signalled on `bar` (complete_tx).
// dst, src 16-byte aligned; bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes,
                                         uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// Prefetch [src, src + bytes) into L2 (16-byte aligned, multiple of 16).
__device__ __forceinline__ void bulk_prefetch_l2(const void *src, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

__device__ __forceinline__ void report_error(uint32_t *status, uint32_t code) {
  if (status) atomicOr(status, code);
}

}  // namespace opir
