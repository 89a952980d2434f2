// k_pattern.cu -- the block pattern and the assembly gather map built on the
// device from the element connectivity.
//
// Same results as the host builders in sched.cpp (pattern_from_elements:
// CElemAry::MakePattern_FEM, src/femfield/elem_ary.cpp:225-245, followed by
// CMatDia_BlkCrs::AddPattern; build_gather_map: the element order of
// CMatDia_BlkCrs::Mearge, src/matvec/matdia_blkcrs.cpp:165-258), bit for bit:
//   1. incidences (element e, local node i) per node, counted, placed and
//      then sorted by t = e*k + i within each node, so every list is in
//      element order whatever order the atomic placement took;
//   2. one thread per node collects the other nodes of its elements into a
//      sorted list without repeats: the row's columns;
//   3. one thread per node walks its incidences in element order and appends
//      each element block (e, i, j) to the slot of its own row that holds it
//      (blocks outside the pattern are skipped, as Mearge skips them): the
//      slot lists come out in element order without atomics.
// Lists are bounded per thread (kPatCap entries); a node beyond that sets a
// flag and the caller builds on the host instead.
#include <algorithm>
#include <cstdint>

#include "dfg_common.cuh"
#include "k_pattern.h"

namespace dfg {

namespace {

constexpr int kScanTpb = 1024, kScanPer = 4, kScanChunk = kScanTpb * kScanPer;

__global__ void k_inc_count(const int* __restrict__ conn, long long nk, int n, int* cnt, int* err) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nk; t += (long long)gridDim.x * blockDim.x) {
    const int a = conn[t];
    if (a < 0 || a >= n) {
      atomicExch(err, kPatErrRange);
      continue;
    }
    atomicAdd(&cnt[a], 1);
  }
}

__global__ void k_inc_fill(const int* __restrict__ conn, long long nk, int n, const long long* __restrict__ ptr,
                           int* cursor, int* inc) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nk; t += (long long)gridDim.x * blockDim.x) {
    const int a = conn[t];
    if (a < 0 || a >= n) continue;
    inc[ptr[a] + atomicAdd(&cursor[a], 1)] = (int)t;
  }
}

// insertion sort of each node's incidences (short lists)
__global__ void k_inc_sort(int n, const long long* __restrict__ ptr, int* inc) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= n) return;
  const long long p0 = ptr[a], p1 = ptr[a + 1];
  for (long long p = p0 + 1; p < p1; ++p) {
    const int v = inc[p];
    long long q = p;
    while (q > p0 && inc[q - 1] > v) {
      inc[q] = inc[q - 1];
      --q;
    }
    inc[q] = v;
  }
}

// the other nodes of node a's elements, ascending, without repeats; -1 on overflow
__device__ int collect_row(int a, int k, const int* __restrict__ conn, const long long* __restrict__ ptr,
                           const int* __restrict__ inc, int* buf) {
  int m = 0;
  for (long long p = ptr[a]; p < ptr[a + 1]; ++p) {
    const int t = inc[p];
    const long long base = (long long)(t / k) * k;
    const int i = t - (int)base;
    for (int j = 0; j < k; ++j) {
      if (j == i) continue;
      const int b = conn[base + j];
      if (b == a) continue;
      int q = m;
      while (q > 0 && buf[q - 1] > b) --q;
      if (q > 0 && buf[q - 1] == b) continue;
      if (m == kPatCap) return -1;
      for (int r = m; r > q; --r) buf[r] = buf[r - 1];
      buf[q] = b;
      ++m;
    }
  }
  return m;
}

__global__ void k_row_count(int n, int k, const int* __restrict__ conn, const long long* __restrict__ ptr,
                            const int* __restrict__ inc, int* rowcnt, int* err) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= n) return;
  int buf[kPatCap];
  const int m = collect_row(a, k, conn, ptr, inc, buf);
  if (m < 0) {
    atomicExch(err, kPatErrOverflow);
    rowcnt[a] = 0;
    return;
  }
  rowcnt[a] = m;
}

__global__ void k_row_fill(int n, int k, const int* __restrict__ conn, const long long* __restrict__ ptr,
                           const int* __restrict__ inc, const int* __restrict__ rowptr, int* colind) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= n) return;
  int buf[kPatCap];
  const int m = collect_row(a, k, conn, ptr, inc, buf);
  if (m != rowptr[a + 1] - rowptr[a]) return;  // overflow: the count pass flagged it
  for (int q = 0; q < m; ++q) colind[rowptr[a] + q] = buf[q];
}

// CRS slot of column b in row a, or -1
__device__ __forceinline__ int find_col(const int* __restrict__ colind, int c0, int c1, int b) {
  int lo = c0, hi = c1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (colind[mid] < b) lo = mid + 1;
    else hi = mid;
  }
  return (lo < c1 && colind[lo] == b) ? lo : -1;
}

// slot counts: diagonal slot a = incidences of a; CRS slot c of row a =
// elements holding both ends (each thread owns its row's slots)
__global__ void k_slot_count(int n, int k, const int* __restrict__ conn, const long long* __restrict__ ptr,
                             const int* __restrict__ inc, const int* __restrict__ rowptr,
                             const int* __restrict__ colind, int* slotcnt, int* err) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= n) return;
  const int c0 = rowptr[a], c1 = rowptr[a + 1];
  if (c1 - c0 > kPatCap) {
    atomicExch(err, kPatErrOverflow);
    return;
  }
  slotcnt[a] = (int)(ptr[a + 1] - ptr[a]);
  for (long long p = ptr[a]; p < ptr[a + 1]; ++p) {
    const int t = inc[p];
    const long long base = (long long)(t / k) * k;
    const int i = t - (int)base;
    for (int j = 0; j < k; ++j) {
      if (j == i) continue;
      const int c = find_col(colind, c0, c1, conn[base + j]);
      if (c >= 0) slotcnt[n + c] += 1;
    }
  }
}

// slot lists in element order: block index (e*k + i)*k + j = t*k + j
__global__ void k_slot_fill(int n, int k, const int* __restrict__ conn, const long long* __restrict__ ptr,
                            const int* __restrict__ inc, const int* __restrict__ rowptr,
                            const int* __restrict__ colind, const long long* __restrict__ slot_ptr, int* slot_src) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= n) return;
  const int c0 = rowptr[a], c1 = rowptr[a + 1];
  if (c1 - c0 > kPatCap) return;
  int cur[kPatCap];
  for (int q = 0; q < c1 - c0; ++q) cur[q] = 0;
  long long dpos = slot_ptr[a];
  for (long long p = ptr[a]; p < ptr[a + 1]; ++p) {
    const int t = inc[p];
    const long long base = (long long)(t / k) * k;
    const int i = t - (int)base;
    for (int j = 0; j < k; ++j) {
      if (j == i) {
        slot_src[dpos++] = t * k + j;
        continue;
      }
      const int c = find_col(colind, c0, c1, conn[base + j]);
      if (c < 0) continue;
      slot_src[slot_ptr[n + c] + cur[c - c0]++] = t * k + j;
    }
  }
}

// ---- exclusive scan of int counts into T offsets, out[m] = total ----------

template <typename T>
__global__ void __launch_bounds__(kScanTpb) k_scan_local(const int* __restrict__ in, long long m, T* out, T* bsum) {
  __shared__ T s[kScanTpb];
  const long long base = blockIdx.x * (long long)kScanChunk + (long long)threadIdx.x * kScanPer;
  T v[kScanPer];
  T own = 0;
#pragma unroll
  for (int q = 0; q < kScanPer; ++q) {
    v[q] = (base + q < m) ? (T)in[base + q] : (T)0;
    own += v[q];
  }
  s[threadIdx.x] = own;
  __syncthreads();
  for (int off = 1; off < kScanTpb; off <<= 1) {
    const T x = threadIdx.x >= (unsigned)off ? s[threadIdx.x - off] : (T)0;
    __syncthreads();
    s[threadIdx.x] += x;
    __syncthreads();
  }
  T run = s[threadIdx.x] - own;
#pragma unroll
  for (int q = 0; q < kScanPer; ++q) {
    if (base + q < m) out[base + q] = run;
    run += v[q];
  }
  if (threadIdx.x == kScanTpb - 1) bsum[blockIdx.x] = s[kScanTpb - 1];
}

// one block: exclusive scan of the block sums, total into *total
template <typename T>
__global__ void __launch_bounds__(kScanTpb) k_scan_sums(T* bsum, long long nb, T* total) {
  __shared__ T s[kScanTpb];
  T carry = 0;
  for (long long c0 = 0; c0 < nb; c0 += kScanTpb) {
    const long long idx = c0 + threadIdx.x;
    const T v = idx < nb ? bsum[idx] : (T)0;
    s[threadIdx.x] = v;
    __syncthreads();
    for (int off = 1; off < kScanTpb; off <<= 1) {
      const T x = threadIdx.x >= (unsigned)off ? s[threadIdx.x - off] : (T)0;
      __syncthreads();
      s[threadIdx.x] += x;
      __syncthreads();
    }
    if (idx < nb) bsum[idx] = carry + s[threadIdx.x] - v;
    const T chunk = s[kScanTpb - 1];
    __syncthreads();
    carry += chunk;
  }
  if (threadIdx.x == 0) *total = carry;
}

template <typename T>
__global__ void k_scan_add(T* out, long long m, const T* __restrict__ bsum) {
  const long long base = blockIdx.x * (long long)kScanChunk;
  const T add = bsum[blockIdx.x];
  for (long long i = threadIdx.x; i < kScanChunk && base + i < m; i += blockDim.x) out[base + i] += add;
}

// grid-stride launches are capped; one-thread-per-node launches are not
int grid_for(long long m, int tpb) { return (int)std::min<long long>((m + tpb - 1) / tpb, 1 << 20); }
unsigned grid_nodes(int n, int tpb) { return (unsigned)(((long long)n + tpb - 1) / tpb); }

}  // namespace

long long scan_blocks(long long m) { return (m + kScanChunk - 1) / kScanChunk; }

template <typename T>
cudaError_t exclusive_scan(const int* in, long long m, T* out, T* bsum, cudaStream_t s) {
  const long long nb = scan_blocks(m);
  if (nb == 0) return cudaMemsetAsync(out, 0, sizeof(T), s);
  k_scan_local<T><<<(unsigned)nb, kScanTpb, 0, s>>>(in, m, out, bsum);
  k_scan_sums<T><<<1, kScanTpb, 0, s>>>(bsum, nb, out + m);
  k_scan_add<T><<<(unsigned)nb, 256, 0, s>>>(out, m, bsum);
  return cudaGetLastError();
}
template cudaError_t exclusive_scan<int>(const int*, long long, int*, int*, cudaStream_t);
template cudaError_t exclusive_scan<long long>(const int*, long long, long long*, long long*, cudaStream_t);

cudaError_t incidence_count(const int* conn, long long nk, int n, int* cnt, int* err, cudaStream_t s) {
  if (nk > 0) k_inc_count<<<grid_for(nk, 256), 256, 0, s>>>(conn, nk, n, cnt, err);
  return cudaGetLastError();
}
cudaError_t incidence_fill(const int* conn, long long nk, int n, const long long* ptr, int* cursor, int* inc,
                           cudaStream_t s) {
  if (nk > 0) k_inc_fill<<<grid_for(nk, 256), 256, 0, s>>>(conn, nk, n, ptr, cursor, inc);
  if (n > 0) k_inc_sort<<<grid_nodes(n, 128), 128, 0, s>>>(n, ptr, inc);
  return cudaGetLastError();
}
cudaError_t pattern_count(int n, int k, const int* conn, const long long* ptr, const int* inc, int* rowcnt, int* err,
                          cudaStream_t s) {
  if (n > 0) k_row_count<<<grid_nodes(n, 128), 128, 0, s>>>(n, k, conn, ptr, inc, rowcnt, err);
  return cudaGetLastError();
}
cudaError_t pattern_fill(int n, int k, const int* conn, const long long* ptr, const int* inc, const int* rowptr,
                         int* colind, cudaStream_t s) {
  if (n > 0) k_row_fill<<<grid_nodes(n, 128), 128, 0, s>>>(n, k, conn, ptr, inc, rowptr, colind);
  return cudaGetLastError();
}
cudaError_t slots_count(int n, int k, const int* conn, const long long* ptr, const int* inc, const int* rowptr,
                        const int* colind, int* slotcnt, int* err, cudaStream_t s) {
  if (n > 0) k_slot_count<<<grid_nodes(n, 128), 128, 0, s>>>(n, k, conn, ptr, inc, rowptr, colind, slotcnt, err);
  return cudaGetLastError();
}
cudaError_t slots_fill(int n, int k, const int* conn, const long long* ptr, const int* inc, const int* rowptr,
                       const int* colind, const long long* slot_ptr, int* slot_src, cudaStream_t s) {
  if (n > 0) k_slot_fill<<<grid_nodes(n, 128), 128, 0, s>>>(n, k, conn, ptr, inc, rowptr, colind, slot_ptr, slot_src);
  return cudaGetLastError();
}

}  // namespace dfg
