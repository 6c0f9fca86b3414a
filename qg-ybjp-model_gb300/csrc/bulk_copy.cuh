// Bulk global -> shared copies completed on a shared-memory mbarrier
// (cp.async.bulk, the untiled TMA path), with a bounded wait.
//
// Use: one thread initialises the barrier (mbar_init) before a CTA barrier;
// per use, one thread arms it with the byte count (mbar_expect_tx) and
// issues the copies (bulk_g2s, 16-byte aligned addresses, sizes multiples of
// 16); every consumer waits on the phase parity (mbar_wait) and flips it
// after each use.  Before copies overwrite a buffer that threads have read
// through ordinary loads, the issuing thread runs fence_proxy_async() after
// the CTA barrier that ends those reads.
#pragma once
#include <cstdint>

namespace qg {

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0u;
}

// Waits for the phase with this parity to complete; gives up (false) after
// about kMbarWaitCycles SM clocks (~0.5 s), so that a copy that never lands
// ends the kernel with an error instead of a hang.
constexpr long long kMbarWaitCycles = 1LL << 30;
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity))
    if (clock64() - t0 > kMbarWaitCycles) return false;
  return true;
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

// Sets the flag a host reads after the stream drains (mapped page-locked
// word: a plain store, no system-scope atomic needed).
__device__ __forceinline__ void raise_wait_flag(int* wflag) { *reinterpret_cast<volatile int*>(wflag) = 1; }

// The failure path of the bounded waits, on demand: one CTA waits on an
// mbarrier phase that nothing completes, gives up after kMbarWaitCycles and
// raises the flag, as a row kernel does when a bulk copy never lands.
static __global__ void k_wait_expire(int* wflag) {
  __shared__ __align__(8) unsigned long long bar;
  const unsigned b = smem_u32(&bar);
  if (threadIdx.x == 0) mbar_init(b, 1);
  __syncthreads();
  const bool ok = mbar_wait(b, 0);
  if (__syncthreads_or(!ok) && threadIdx.x == 0) raise_wait_flag(wflag);
}

}  // namespace qg
