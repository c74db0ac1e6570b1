// Staging of contiguous global byte ranges in shared memory by the bulk
// asynchronous copy engine (cp.async.bulk, TMA) with mbarrier completion, for
// the streaming matvec kernels: one elected lane starts the copies of a stage
// and the warp consumes earlier stages meanwhile, so the bytes in flight per
// SM do not depend on registers or on how long the arithmetic of a stage takes.
//
// Every wait is bounded: mbar_wait gives up after kWaitNs (2 s); the
// kernels then count the event in a device counter (matvec.cu:
// g_stream_timeouts, read by the host after a solve or matvec) and drain
// their own copies, again with a bound, before they return.
// The bulk copy needs 16-byte aligned shared and global addresses and a size
// that is a multiple of 16 bytes; callers state why theirs are.
#pragma once
#include <cstdint>

namespace hodlr {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// makes barrier initialisation visible to the copy engine
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// orders this thread's earlier shared-memory accesses before later
// asynchronous-proxy (bulk copy) writes
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

// raises the phase's expected transaction bytes without arriving
__device__ __forceinline__ void mbar_expect_tx_only(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}

// One poll that suspends the thread (no issue slots used) until the phase
// completes or about kSuspendNs nanoseconds pass.
constexpr uint32_t kSuspendNs = 1000000;

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n"
      " .reg .pred p;\n"
      " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
      " selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity), "r"(kSuspendNs)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Waits for the phase with the given parity; false once kWaitNs nanoseconds
// have passed without it completing.
constexpr uint64_t kWaitNs = 2000000000ull;

__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  for (;;) {
    if (mbar_try_wait(bar, parity)) return true;
    if (global_ns() - t0 > kWaitNs) return false;
  }
}

__device__ __forceinline__ const void* align_down16(const void* p) {
  return reinterpret_cast<const void*>(reinterpret_cast<uintptr_t>(p) & ~uintptr_t(15));
}

}  // namespace hodlr
