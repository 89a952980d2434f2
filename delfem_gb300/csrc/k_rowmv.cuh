// k_rowmv.cuh -- one block row of the block-CRS product (device helper).
#pragma once

namespace dfg {

// y_i = sum_j A_ij x_j for one block row; off-diagonal blocks in CRS order,
// then the diagonal block (the order of CMatDia_BlkCrs::MatVec).
template <typename T, typename A, int B>
__device__ __forceinline__ void row_mv(int i, const int* __restrict__ rowptr, const int* __restrict__ colind,
                                       const T* __restrict__ diag, const T* __restrict__ offd,
                                       const T* __restrict__ x, A y[B]) {
  constexpr int BS = B * B;
#pragma unroll
  for (int p = 0; p < B; ++p) y[p] = 0;
  const int c0 = rowptr[i], c1 = rowptr[i + 1];
  for (int c = c0; c < c1; ++c) {
    const int j = colind[c];
    const T* a = offd + (size_t)c * BS;
    T xv[B];
#pragma unroll
    for (int q = 0; q < B; ++q) xv[q] = x[(size_t)j * B + q];
#pragma unroll
    for (int p = 0; p < B; ++p)
#pragma unroll
      for (int q = 0; q < B; ++q) y[p] += (A)a[p * B + q] * (A)xv[q];
  }
  const T* a = diag + (size_t)i * BS;
#pragma unroll
  for (int p = 0; p < B; ++p)
#pragma unroll
    for (int q = 0; q < B; ++q) y[p] += (A)a[p * B + q] * (A)x[(size_t)i * B + q];
}

}  // namespace dfg

namespace dfg {

// ---------------------------------------------------------------------------
// Warp-cooperative block-row product.  A row is handled by a group of L lanes
// that stride over its values -- the off-diagonal blocks (contiguous in CRS
// order) followed by the diagonal block -- so a warp's loads of one row are
// coalesced.  Lane `sub` of the group always meets the same block entry
// (p, q) (L is a multiple of b*b), multiplies it by x[col*b + q], and the
// group reduces the lanes of equal p.
//   b = 1: L = 8  (4 rows per warp)
//   b = 2: L = 16 (2 rows per warp)
//   b = 3: L = 27 (1 row per warp, lanes 27..31 idle)
template <int B> struct RowLanes;
template <> struct RowLanes<1> { static constexpr int L = 8, RPW = 4; };
template <> struct RowLanes<2> { static constexpr int L = 16, RPW = 2; };
template <> struct RowLanes<3> { static constexpr int L = 27, RPW = 1; };

// Which row group of the warp this lane belongs to and its place in it;
// g >= RPW marks an idle lane.
template <int B>
__device__ __forceinline__ void row_lane(int lane, int& g, int& sub) {
  constexpr int L = RowLanes<B>::L;
  g = lane / L;
  sub = lane % L;
}

// Output component p of this lane and whether it stores it after the
// reduction (one lane per component).
template <int B>
__device__ __forceinline__ int row_comp(int sub, bool& writer) {
  constexpr int BS = B * B;
  const int e = sub % BS;
  writer = (sub < BS) && (e % B == 0);
  return e / B;
}

// (A x)_i, component row_comp(sub): valid in the group's writer lanes.  All 32
// lanes of the warp must call it together; pass i < 0 for an idle group.
template <typename T, int B>
__device__ __forceinline__ T row_mv_warp(int i, int sub, const int* __restrict__ rowptr,
                                         const int* __restrict__ colind, const T* __restrict__ diag,
                                         const T* __restrict__ offd, const T* __restrict__ x) {
  constexpr int L = RowLanes<B>::L, BS = B * B;
  T acc = 0;
  if (i >= 0 && sub < L) {
    const int q = (sub % BS) % B;
    const int c0 = rowptr[i], c1 = rowptr[i + 1];
    const int nv = (c1 - c0) * BS;
    const T* base = offd + (size_t)c0 * BS;
#pragma unroll 2
    for (int v = sub; v < nv; v += L) acc += base[v] * x[(size_t)colind[c0 + v / BS] * B + q];
    // diagonal block: entry sub % BS, by the lanes whose turn it is
    const int vd = nv + ((sub - nv) % L + L) % L;  // first v >= nv this lane meets
    if (vd < nv + BS) acc += diag[(size_t)i * BS + (vd - nv)] * x[(size_t)i * B + q];
  }
  if constexpr (B == 1) {
    acc += __shfl_xor_sync(0xffffffffu, acc, 4);
    acc += __shfl_xor_sync(0xffffffffu, acc, 2);
    acc += __shfl_xor_sync(0xffffffffu, acc, 1);
  } else if constexpr (B == 2) {
    acc += __shfl_xor_sync(0xffffffffu, acc, 1);   // q
    acc += __shfl_xor_sync(0xffffffffu, acc, 4);   // blocks of the pass
    acc += __shfl_xor_sync(0xffffffffu, acc, 8);
  } else {
    const int lane = threadIdx.x & 31;
    const T a1 = __shfl_sync(0xffffffffu, acc, min(lane + 1, 31));
    const T a2 = __shfl_sync(0xffffffffu, acc, min(lane + 2, 31));
    acc += a1 + a2;                                 // q (lanes with q == 0)
    const T b1 = __shfl_sync(0xffffffffu, acc, min(lane + 9, 31));
    const T b2 = __shfl_sync(0xffffffffu, acc, min(lane + 18, 31));
    acc += b1 + b2;                                 // the three blocks of a pass (lanes < 9)
  }
  return acc;
}

}  // namespace dfg
