// Bulk asynchronous copies global -> shared memory (cp.async.bulk, the TMA unit's untiled
// form) completed through shared-memory mbarriers, for kernels that stream long rows.
//
// Use: one thread initialises the stage barriers (mbar_init + fence_barrier_init, then a
// block barrier); the producing thread arms a stage with mbar_expect_tx(total bytes) and
// issues bulk_g2s for each segment; consumers wait with mbar_wait_bounded(phase), and
// release the stage (mbar_arrive on its empty barrier) after their last read of it; the
// producer refills it once that barrier completes.
// Addresses and sizes of bulk_g2s must be multiples of 16 bytes.
//
// Every wait is bounded: mbar_wait_bounded gives up after kBulkWaitCycles clock cycles
// (about half a second) and returns false, so a kernel never spins forever on a copy that
// does not complete.
#pragma once

#include <cstdint>

namespace bgb {

constexpr long long kBulkWaitCycles = 1000000000LL;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// makes initialised barriers visible to the asynchronous (bulk copy) proxy
__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// orders this thread's earlier shared-memory accesses before later bulk copies into it
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// arrive on the barrier (count 1) and add bytes to the transaction count it waits for
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

// global -> shared bulk copy of bytes (multiple of 16, both addresses 16-byte aligned),
// completing its bytes on bar
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// plain arrival (count 1) on the barrier, releasing this thread's earlier accesses
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t phase) {
  uint32_t done;
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(phase)
      : "memory");
  return done != 0;
}

// wait for the completion of the barrier's phase `phase` (parity); false after
// kBulkWaitCycles without completion
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t phase) {
  if (mbar_try_wait(bar, phase)) return true;
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, phase))
    if (clock64() - t0 > kBulkWaitCycles) return false;
  return true;
}

}  // namespace bgb
