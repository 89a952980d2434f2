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
// Sliced-ELL block-row product (layout: SellMap in dfg_internal.h).  Thread
// i owns row i; a warp owns one slice of 32 rows, so every load of a value
// (block w, entry e) is one coalesced 32-word access, and the width W_s is
// uniform across the warp.  The row's blocks come in CRS order, then the
// diagonal block, then zero padding: the same accumulation sequence as
// row_mv.  x may be stored narrower than the values (X = float with T =
// double: a vector from FP32 sweeps); it is widened on load.
template <typename T, int B, typename X = T>
__device__ __forceinline__ void sell_row_mv(int i, const long long* __restrict__ ptr, const int* __restrict__ width,
                                            const int* __restrict__ col, const T* __restrict__ val,
                                            const X* __restrict__ x, T y[B]) {
  constexpr int BS = B * B;
  const int s = i >> 5, lane = i & 31;
  const long long k0 = ptr[s];
  const int W = width[s];
  const int* __restrict__ c = col + k0 + lane;
  const T* __restrict__ v = val + k0 * BS + lane;
#pragma unroll
  for (int p = 0; p < B; ++p) y[p] = 0;
#pragma unroll 4
  for (int w = 0; w < W; ++w) {
    const int j = c[w * 32];
    T xv[B];
#pragma unroll
    for (int q = 0; q < B; ++q) xv[q] = (T)x[(size_t)j * B + q];
#pragma unroll
    for (int p = 0; p < B; ++p)
#pragma unroll
      for (int q = 0; q < B; ++q) y[p] += v[(w * BS + p * B + q) * 32] * xv[q];
  }
}

}  // namespace dfg
