// k_mbar.cuh -- mbarrier, bulk-copy (TMA) and bounded-wait helpers shared
// by the sweep kernels (device code, sm_103a).
#pragma once
#include "dfg_common.cuh"

namespace dfg {

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.shared::cta.b64 st, [%0];\n}" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}" ::"r"(smem_u32(bar)),
               "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool mbar_test_wait(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// First failure of a launch: err[0] = code, err[1..3] = where it happened
// (wait site, slot, range or row); later failures leave the record alone.
__device__ __forceinline__ void record_fail(int* err, int code, int site, int a, int b) {
  if (atomicCAS(err, 0, code) == 0) {
    err[1] = site;
    err[2] = a;
    err[3] = b;
    __threadfence();
  }
}

// Bounded wait for a copy known to be in flight (no failure record).
__device__ __forceinline__ void mbar_drain(uint64_t* bar, unsigned parity) {
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity) && clock64() - t0 < kDrainCycles) {
  }
}

// Bounded wait: false when another waiter of the launch has already failed
// (checked every 32 polls) or after kWaitCycles, when it records a timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, int* err, int site, int slot, int range) {
  if (mbar_test_wait(bar, parity)) return true;
  const long long t0 = clock64();
  for (unsigned n = 1;; ++n) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((n & 31) == 0) {
      if (ld_relaxed_int(err) != 0) return false;
      if (clock64() - t0 > kWaitCycles) {
        record_fail(err, kErrTimeout, site, slot, range);
        return false;
      }
    }
  }
}
__device__ __forceinline__ void tma_load_1d(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void cp_async_arrive_noinc(uint64_t* bar) {
  asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void named_sync(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

}  // namespace dfg
