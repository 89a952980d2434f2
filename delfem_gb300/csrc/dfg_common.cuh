// dfg_common.cuh -- shared device helpers for libdfg (sm_103a only).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#ifndef __CUDACC__
#error "dfg_common.cuh is device code"
#endif

namespace dfg {

// Sentinels marking "not yet written" in sweep output buffers.  They are
// negative quiet NaNs with a payload that GPU arithmetic never produces
// (arithmetic NaNs are canonical), so a consumer that reads anything else
// has read the producer's final value.
constexpr uint64_t kSentinel64 = 0xFFF4BADBADBADBADull;
constexpr uint32_t kSentinel32 = 0xFFB4BADBu;

__device__ __forceinline__ bool is_sentinel(double v) {
  return (uint64_t)__double_as_longlong(v) == kSentinel64;
}
__device__ __forceinline__ bool is_sentinel(float v) {
  return __float_as_uint(v) == kSentinel32;
}
template <typename T> __device__ __forceinline__ T sentinel_value();
template <> __device__ __forceinline__ double sentinel_value<double>() {
  return __longlong_as_double((long long)kSentinel64);
}
template <> __device__ __forceinline__ float sentinel_value<float>() {
  return __uint_as_float(kSentinel32);
}

// gpu-scope relaxed accesses (morally strong: a poll sees the producer's store)
__device__ __forceinline__ double ld_relaxed(const double* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return __longlong_as_double((long long)v);
}
__device__ __forceinline__ float ld_relaxed(const float* p) {
  unsigned v;
  asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return __uint_as_float(v);
}
__device__ __forceinline__ void st_relaxed(double* p, double v) {
  asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"((unsigned long long)__double_as_longlong(v)) : "memory");
}
__device__ __forceinline__ void st_relaxed(float* p, float v) {
  asm volatile("st.relaxed.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(__float_as_uint(v)) : "memory");
}
__device__ __forceinline__ int ld_relaxed_int(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Ampere-style asynchronous global->shared copies
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
  unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
  unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Programmatic dependent launch (kernels launched with
// cudaLaunchAttributeProgrammaticStreamSerialization): wait until the
// previous kernel in the stream has finished and its writes are visible,
// then let the next kernel launch so that its start overlaps this one.  In a
// kernel launched in plain stream order both are no-ops.
__device__ __forceinline__ void pdl_enter() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// error word shared by all kernels of a context (0 = ok)
enum : int { kErrNone = 0, kErrTimeout = 1, kErrBadIndex = 2 };

// Device-side wait budget: a wait gives up after this many SM clock cycles
// (about two seconds at 2 GHz), records kErrTimeout with where it happened,
// and every other waiter of the launch leaves as soon as it sees the record.
constexpr long long kWaitCycles = 4000000000ll;
// Bound on waiting for a copy already in flight before a failing CTA leaves.
constexpr long long kDrainCycles = 2000000ll;
// wait sites recorded with a timeout (error word [1])
enum : int { kSiteEmpty = 1, kSiteRecLoad = 2, kSitePoll = 3, kSiteRecCompute = 4, kSiteFull = 5, kSiteRange = 6 };

}  // namespace dfg
