// k_level.cu -- level-scheduled triangular sweeps: one launch per dependency
// level, one warp per row of the level.
//
// CMatDiaFrac_BlkCrs::ForwardSubstitution / BackwardSubstitution
// (src/matvec/matdiafrac_blkcrs.cpp:332-669) over the factor's block CRS,
// rows of one level at a time: every row of a level depends only on rows of
// earlier levels, which earlier launches finished, so there is no waiting
// inside a launch.  This is the schedule for matrices whose levels are wide
// (3D meshes: a few hundred levels of thousands of rows), where the ranged
// sweep of k_sweep.cu spends its time on hand-offs between ranges; the
// preconditioner's set-up times both and keeps the faster.
#include "dfg_common.cuh"
#include "k_sweep.h"

namespace dfg {

// One warp per row: lane e takes the row's entries e, e+32, ..., so the
// dependency and factor loads of a row are issued together; the partial sums
// meet in a shuffle tree and lane 0 finishes the row.
template <typename T, int B, bool FWD>
__global__ void __launch_bounds__(128) k_sweep_level(LevelSweepArgs a, int first, int cnt) {
  if (a.done && *a.done) return;
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= cnt) return;
  constexpr int BS = B * B;
  const T* __restrict__ in = reinterpret_cast<const T*>(a.in);
  T* out = reinterpret_cast<T*>(a.out);
  const T* __restrict__ fo = reinterpret_cast<const T*>(a.foffd);
  const int i = a.rows[first + w];
  const int c0 = FWD ? a.rowptr[i] : a.diaind[i];
  const int c1 = FWD ? a.diaind[i] : a.rowptr[i + 1];
  T part[B];
#pragma unroll
  for (int p = 0; p < B; ++p) part[p] = 0;
  for (int c = c0 + lane; c < c1; c += 32) {
    const int j = a.colind[c];
    const T* blk = fo + (size_t)c * BS;
    T x[B];
#pragma unroll
    for (int q = 0; q < B; ++q) x[q] = out[(size_t)j * B + q];
#pragma unroll
    for (int p = 0; p < B; ++p)
#pragma unroll
      for (int q = 0; q < B; ++q) part[p] += blk[p * B + q] * x[q];
  }
#pragma unroll
  for (int p = 0; p < B; ++p)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) part[p] += __shfl_xor_sync(0xffffffffu, part[p], o);
  if (lane != 0) return;
  T acc[B];
#pragma unroll
  for (int p = 0; p < B; ++p) acc[p] = in[(size_t)i * B + p] - part[p];
  if constexpr (FWD) {
    const T* dv = reinterpret_cast<const T*>(a.fdiag) + (size_t)i * BS;
#pragma unroll
    for (int p = 0; p < B; ++p) {
      T y = dv[p * B] * acc[0];
#pragma unroll
      for (int q = 1; q < B; ++q) y += dv[p * B + q] * acc[q];
      out[(size_t)i * B + p] = y;
    }
  } else {
#pragma unroll
    for (int p = 0; p < B; ++p) out[(size_t)i * B + p] = acc[p];
  }
}

cudaError_t launch_sweep_level(bool forward, bool fp32, int b, const LevelSweepArgs& a, int first, int cnt,
                               cudaStream_t s) {
  if (cnt <= 0) return cudaSuccess;
  const unsigned grid = (unsigned)((cnt + 3) / 4);  // four rows (warps) per block
#define DFG_LVL(T, B)                                                                  \
  (forward ? (k_sweep_level<T, B, true><<<grid, 128, 0, s>>>(a, first, cnt), 0)       \
           : (k_sweep_level<T, B, false><<<grid, 128, 0, s>>>(a, first, cnt), 0))
  switch (b) {
    case 1: fp32 ? DFG_LVL(float, 1) : DFG_LVL(double, 1); break;
    case 2: fp32 ? DFG_LVL(float, 2) : DFG_LVL(double, 2); break;
    case 3: fp32 ? DFG_LVL(float, 3) : DFG_LVL(double, 3); break;
    default: return cudaErrorInvalidValue;
  }
#undef DFG_LVL
  return cudaGetLastError();
}

}  // namespace dfg
