// k_level.cu -- level-scheduled triangular sweeps: one launch per dependency
// level, a group of lanes per row of the level.
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

// G lanes per row (G a power of two, 4..32: the smallest that holds the
// widest row of the sweep), 32/G rows per warp.  Lane k of a row's group
// takes the row's entries k, k+G, ..., so the dependency and factor loads of
// a row are issued together; the partial sums meet in an xor butterfly over
// the group (every lane ends with the same totals) and lane p < B of the
// group finishes component p of the row.
//
// Levels after the first are launched as programmatic dependents of the
// level before: each launch lets the next one start at once
// (griddepcontrol.launch_dependents), and a launch loads what does not
// depend on earlier levels -- the row's descriptor {row, first entry, end
// entry}, its first entry's column and factor block -- before it waits for
// the previous level's grid to finish and its writes to be visible
// (griddepcontrol.wait).  Only the dependency values, the right-hand side
// and the arithmetic are left on the level's critical path, and the launch
// latency overlaps the previous level.  The solve's `done` flag is read before
// the wait: it is written by a kernel that precedes the sweep's first level,
// which is launched in plain stream order.
template <typename T, int B, bool FWD>
__global__ void __launch_bounds__(128) k_sweep_level(LevelSweepArgs a, int first, int cnt) {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  if (a.done && *a.done) return;
  const int G = a.G;
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  const int r = gid / G, sub = gid & (G - 1);
  const bool active = r < cnt;
  constexpr int BS = B * B;
  const T* __restrict__ in = reinterpret_cast<const T*>(a.in);
  T* out = reinterpret_cast<T*>(a.out);
  const T* __restrict__ fo = reinterpret_cast<const T*>(a.foffd);
  int4 inf = make_int4(0, 0, 0, 0);
  if (active) inf = a.info[first + r];
  const int i = inf.x, c0 = inf.y, c1 = inf.z;
  // this lane's first entry (the only one for rows of <= G entries)
  int c = c0 + sub;
  const bool have = c < c1;
  int j0 = 0;
  T blk0[BS];
  if (have) {
    j0 = a.colind[c];
#pragma unroll
    for (int e = 0; e < BS; ++e) blk0[e] = fo[(size_t)c * BS + e];
  }
  asm volatile("griddepcontrol.wait;" ::: "memory");
  T part[B];
#pragma unroll
  for (int p = 0; p < B; ++p) part[p] = 0;
  if (have) {
    T x[B];
#pragma unroll
    for (int q = 0; q < B; ++q) x[q] = out[(size_t)j0 * B + q];
#pragma unroll
    for (int p = 0; p < B; ++p)
#pragma unroll
      for (int q = 0; q < B; ++q) part[p] += blk0[p * B + q] * x[q];
  }
  for (c += G; c < c1; c += G) {
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
  for (int o = G >> 1; o > 0; o >>= 1)
#pragma unroll
    for (int p = 0; p < B; ++p) part[p] += __shfl_xor_sync(0xffffffffu, part[p], o);
  if (!active || sub >= B) return;
  T acc[B];
#pragma unroll
  for (int p = 0; p < B; ++p) acc[p] = in[(size_t)i * B + p] - part[p];
  T y = acc[0];
  if constexpr (FWD) {
    const T* dv = reinterpret_cast<const T*>(a.fdiag) + (size_t)i * BS + sub * B;
    y = dv[0] * acc[0];
#pragma unroll
    for (int q = 1; q < B; ++q) y += dv[q] * acc[q];
  } else {
#pragma unroll
    for (int p = 1; p < B; ++p)
      if (sub == p) y = acc[p];
  }
  out[(size_t)i * B + sub] = y;
}

template <typename T, int B, bool FWD>
static cudaError_t launch_one(const LevelSweepArgs& a, int first, int cnt, unsigned grid, bool dependent,
                              cudaStream_t s) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(128);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = dependent ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, k_sweep_level<T, B, FWD>, a, first, cnt);
}

cudaError_t launch_sweep_level(bool forward, bool fp32, int b, const LevelSweepArgs& a, int first, int cnt,
                               bool dependent, cudaStream_t s) {
  if (cnt <= 0) return cudaSuccess;
  const long long lanes = (long long)cnt * a.G;
  const unsigned grid = (unsigned)((lanes + 127) / 128);  // 128 threads per block
  cudaError_t e = cudaErrorInvalidValue;
#define DFG_LVL(T, B)                                                          \
  e = forward ? launch_one<T, B, true>(a, first, cnt, grid, dependent, s)      \
              : launch_one<T, B, false>(a, first, cnt, grid, dependent, s)
  switch (b) {
    case 1: if (fp32) { DFG_LVL(float, 1); } else { DFG_LVL(double, 1); } break;
    case 2: if (fp32) { DFG_LVL(float, 2); } else { DFG_LVL(double, 2); } break;
    case 3: if (fp32) { DFG_LVL(float, 3); } else { DFG_LVL(double, 3); } break;
    default: return cudaErrorInvalidValue;
  }
#undef DFG_LVL
  return e;
}

}  // namespace dfg
