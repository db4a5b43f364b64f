// Bulk asynchronous copies global -> shared memory (the TMA unit's 1-D
// cp.async.bulk) completing on shared-memory mbarriers, with bounded waits.
//
// A copy moves `bytes` (a multiple of 16) from a 16-byte aligned global
// address to a 16-byte aligned shared address; the issuing thread first
// registers the byte count on the barrier (arrive.expect_tx, one arrival),
// and the phase completes when all the bytes have landed.  Waiters poll the
// phase parity with try_wait for at most kWaitNs of global time (and a fixed
// number of polls); a wait that gives up returns false and the kernel records
// an error status instead of hanging.
#pragma once

#include <cstdint>

namespace bdda {
namespace acp {

constexpr unsigned long long kWaitNs = 2000000000ull;  // 2 s
constexpr int kWaitPolls = 1 << 26;

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void bar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(bar)), "r"(count) : "memory");
}
// Makes the barrier initialisation visible to the async proxy and the other threads (then a CTA barrier).
__device__ __forceinline__ void fence_bar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// Orders this thread's earlier shared-memory accesses before later async-proxy (bulk copy) writes.
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   saddr(dst)),
               "l"(src), "r"(bytes), "r"(saddr(bar))
               : "memory");
}

__device__ __forceinline__ bool try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(saddr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ unsigned long long now_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Waits for the phase of the given parity to complete; false after the time limit.
__device__ __forceinline__ bool wait(uint64_t* bar, uint32_t parity) {
  if (try_wait(bar, parity)) return true;
  const unsigned long long t0 = now_ns();
  for (int i = 0; i < kWaitPolls; ++i) {
    if (try_wait(bar, parity)) return true;
    if ((i & 63) == 63 && now_ns() - t0 > kWaitNs) return false;
  }
  return false;
}

}  // namespace acp
}  // namespace bdda
