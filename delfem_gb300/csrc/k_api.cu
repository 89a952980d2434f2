// k_api.cu -- elementwise kernels behind the strict drop-in solver interface
// (CLinearSystem::MATVEC / AXPY / SCAL / DOT, src/ls/linearsystem.cpp:250-415,
// over CMatDia_BlkCrs::MatVec and CVector_Blk, src/matvec/matdia_blkcrs.cpp:
// 921-1094, src/matvec/vector_blk.cpp:37-112).  Compiled with -fmad=false and
// written with the reference's operand order, so MATVEC / AXPY / SCAL / COPY
// give bit-identical vectors; DOT is a deterministic tree sum and differs
// from the reference's sequential sum only in rounding.
#include "dfg_common.cuh"
#include "k_solve.h"

namespace dfg {

__device__ double block_sum_api(double v) {
  __shared__ double ws[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) ws[w] = v;
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  double t = (threadIdx.x < nw) ? ws[threadIdx.x] : 0.0;
  if (w == 0) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  }
  __syncthreads();
  if (threadIdx.x == 0) ws[0] = t;
  __syncthreads();
  return ws[0];
}

// y := beta*y; y += alpha*(A_ij x_j) per off-diagonal block in CRS order;
// y += alpha*(D_i x_i)  (b = 1 keeps the reference's alpha*a*x grouping)
template <int B>
__global__ void k_api_matvec(MatView Am, double alpha, const double* __restrict__ x, double beta, double* y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= Am.n) return;
  constexpr int BS = B * B;
  const double* diag = reinterpret_cast<const double*>(Am.diag);
  const double* offd = reinterpret_cast<const double*>(Am.offd);
  double yi[B];
#pragma unroll
  for (int p = 0; p < B; ++p) yi[p] = y[(size_t)i * B + p] * beta;
  for (int c = Am.rowptr[i]; c < Am.rowptr[i + 1]; ++c) {
    const double* a = offd + (size_t)c * BS;
    const double* xj = x + (size_t)Am.colind[c] * B;
    if constexpr (B == 1) {
      yi[0] += alpha * a[0] * xj[0];
    } else {
#pragma unroll
      for (int p = 0; p < B; ++p) {
        double s = a[p * B] * xj[0];
#pragma unroll
        for (int q = 1; q < B; ++q) s += a[p * B + q] * xj[q];
        yi[p] += alpha * s;
      }
    }
  }
  const double* a = diag + (size_t)i * BS;
  const double* xi = x + (size_t)i * B;
  if constexpr (B == 1) {
    yi[0] += alpha * a[0] * xi[0];
  } else {
#pragma unroll
    for (int p = 0; p < B; ++p) {
      double s = a[p * B] * xi[0];
#pragma unroll
      for (int q = 1; q < B; ++q) s += a[p * B + q] * xi[q];
      yi[p] += alpha * s;
    }
  }
#pragma unroll
  for (int p = 0; p < B; ++p) y[(size_t)i * B + p] = yi[p];
}

__global__ void k_api_axpy(long long m, double alpha, const double* x, double* y) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < m; k += (long long)gridDim.x * blockDim.x)
    y[k] += alpha * x[k];
}
__global__ void k_api_scal(long long m, double alpha, double* x) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < m; k += (long long)gridDim.x * blockDim.x)
    x[k] *= alpha;
}
__global__ void k_api_dot(long long m, const double* x, const double* y, Red red) {
  double part = 0.0;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < m; k += (long long)gridDim.x * blockDim.x)
    part += x[k] * y[k];
  __shared__ bool last;
  const double bs = block_sum_api(part);
  if (threadIdx.x == 0) {
    red.partials[blockIdx.x] = bs;
    __threadfence();
    last = (atomicAdd(red.counter, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double t = 0.0;
  for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) t += ld_relaxed(&red.partials[i]);
  t = block_sum_api(t);
  if (threadIdx.x == 0) {
    *red.counter = 0u;
    *red.result = 0.0 + t;
  }
}

cudaError_t api_matvec(const MatView& A, double alpha, const double* x, double beta, double* y, cudaStream_t s) {
  if (A.n == 0) return cudaSuccess;
  const int tpb = 128, g = (A.n + tpb - 1) / tpb;
  switch (A.b) {
    case 1: k_api_matvec<1><<<g, tpb, 0, s>>>(A, alpha, x, beta, y); break;
    case 2: k_api_matvec<2><<<g, tpb, 0, s>>>(A, alpha, x, beta, y); break;
    case 3: k_api_matvec<3><<<g, tpb, 0, s>>>(A, alpha, x, beta, y); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}
cudaError_t api_axpy(long long m, double alpha, const double* x, double* y, cudaStream_t s) {
  if (m > 0) k_api_axpy<<<kRedGrid, kRedTpb, 0, s>>>(m, alpha, x, y);
  return cudaGetLastError();
}
cudaError_t api_scal(long long m, double alpha, double* x, cudaStream_t s) {
  if (m > 0) k_api_scal<<<kRedGrid, kRedTpb, 0, s>>>(m, alpha, x);
  return cudaGetLastError();
}
cudaError_t api_dot(long long m, const double* x, const double* y, Red red, cudaStream_t s) {
  k_api_dot<<<kRedGrid, kRedTpb, 0, s>>>(m, x, y, red);
  return cudaGetLastError();
}

}  // namespace dfg
