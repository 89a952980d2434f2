// k_reduce.cuh -- deterministic reductions of the solver kernels (device
// helpers): a fixed grid, one partial per block (fixed-shape warp-shuffle
// tree), and the last block to finish sums the partials in index order, so a
// dot product gives the same bits on every run.
#pragma once
#include "dfg_common.cuh"
#include "k_solve.h"

namespace dfg {

static __device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// sum over the block (fixed order); result valid in every thread
static __device__ double block_sum(double v) {
  __shared__ double ws[32];
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) ws[w] = v;
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  double t = (threadIdx.x < nw) ? ws[threadIdx.x] : 0.0;
  if (w == 0) t = warp_sum(t);
  __syncthreads();
  if (threadIdx.x == 0) ws[0] = t;
  __syncthreads();
  return ws[0];
}

// Publishes this block's partial; returns true (in every thread) in the
// last block, which then holds the grid total in *total.
static __device__ bool grid_sum(double v, Red red, double* total) {
  __shared__ bool last;
  const double bs = block_sum(v);
  if (threadIdx.x == 0) {
    red.partials[blockIdx.x] = bs;
    __threadfence();
    const unsigned prev = atomicAdd(red.counter, 1u);
    last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double t = 0.0;
  for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) t += ld_relaxed(&red.partials[i]);
  t = block_sum(t);
  if (threadIdx.x == 0) *red.counter = 0u;
  *total = t;
  return true;
}

// Two sums in one pass (partials interleaved, 2 per block): each total is
// the same as grid_sum of that value alone would give.
static __device__ bool grid_sum2(double a, double b, Red red, double* ta, double* tb) {
  __shared__ bool last;
  const double ba = block_sum(a);
  const double bb = block_sum(b);
  if (threadIdx.x == 0) {
    red.partials[2 * blockIdx.x] = ba;
    red.partials[2 * blockIdx.x + 1] = bb;
    __threadfence();
    const unsigned prev = atomicAdd(red.counter, 1u);
    last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double sa = 0.0, sb = 0.0;
  for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) {
    sa += ld_relaxed(&red.partials[2 * i]);
    sb += ld_relaxed(&red.partials[2 * i + 1]);
  }
  sa = block_sum(sa);
  sb = block_sum(sb);
  if (threadIdx.x == 0) *red.counter = 0u;
  *ta = sa;
  *tb = sb;
  return true;
}

}  // namespace dfg
