// k_ilu.cu -- numeric block ILU factorisation, level-scheduled.
//
// Restates CMatDiaFrac_BlkCrs::DoILUDecomp (src/matvec/matdiafrac_blkcrs.cpp:
// 774-1107) for 1x1, 2x2 and 3x3 blocks, on the factor's own pattern (A's
// for ILU(0), with fill-in for ILU(k)).  Row i only reads rows k < i that
// are finished (they sit in earlier levels of the forward dependency DAG)
// and only writes its own row, so all rows of one level run in parallel, one
// thread each.  This file is compiled with -fmad=false and every expression
// keeps the reference's operand order, so the factor is bit-identical to the
// reference's (the division 1.0/det is IEEE-rounded on both sides).
#include "dfg_common.cuh"
#include "k_ilu.h"

namespace dfg {

// position of column j inside row i (CRS slot) or -1; the reference uses a
// scatter array row2crs_f for the same lookup
__device__ __forceinline__ int find_slot(const int* colind, int c0, int c1, int j) {
  int lo = c0, hi = c1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (colind[mid] < j) lo = mid + 1; else hi = mid;
  }
  return (lo < c1 && colind[lo] == j) ? lo : -1;
}

template <int B>
__global__ void k_ilu_level(const int* __restrict__ rows, int cnt, const int* __restrict__ rowptr,
                            const int* __restrict__ colind, const int* __restrict__ diaind,
                            double* fdiag, double* foffd, int* nsing) {
  constexpr int BS = B * B;
  pdl_enter();  // the previous level (a programmatic dependency) is complete
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= cnt) return;
  const int i = rows[t];
  const int r0 = rowptr[i], r1 = rowptr[i + 1], di = diaind[i];
  double* pii = fdiag + (size_t)i * BS;
  for (int ik = r0; ik < di; ++ik) {
    const int k = colind[ik];
    const double* pik = foffd + (size_t)ik * BS;
    double lik[BS];
#pragma unroll
    for (int m = 0; m < BS; ++m) lik[m] = pik[m];  // A_ik already holds the updates of all k' < k
    for (int kj = diaind[k]; kj < rowptr[k + 1]; ++kj) {
      const int j = colind[kj];
      const double* pkj = foffd + (size_t)kj * BS;
      double* pij;
      if (j != i) {
        const int ij = find_slot(colind, r0, r1, j);
        if (ij < 0) continue;
        pij = foffd + (size_t)ij * BS;
      } else {
        pij = pii;
      }
      if constexpr (B == 1) {
        pij[0] -= lik[0] * pkj[0];
      } else if constexpr (B == 2) {
        pij[0] -= lik[0] * pkj[0] + lik[1] * pkj[2];
        pij[1] -= lik[0] * pkj[1] + lik[1] * pkj[3];
        pij[2] -= lik[2] * pkj[0] + lik[3] * pkj[2];
        pij[3] -= lik[2] * pkj[1] + lik[3] * pkj[3];
      } else {
#pragma unroll
        for (int r = 0; r < 3; ++r) {
          pij[r * 3 + 0] -= lik[r * 3 + 0] * pkj[0] + lik[r * 3 + 1] * pkj[3] + lik[r * 3 + 2] * pkj[6];
          pij[r * 3 + 1] -= lik[r * 3 + 0] * pkj[1] + lik[r * 3 + 1] * pkj[4] + lik[r * 3 + 2] * pkj[7];
          pij[r * 3 + 2] -= lik[r * 3 + 0] * pkj[2] + lik[r * 3 + 1] * pkj[5] + lik[r * 3 + 2] * pkj[8];
        }
      }
    }
  }
  // pivot inverse (matdiafrac_blkcrs.cpp:885-895 / 933-951 / 998-1013)
  bool sing = false;
  if constexpr (B == 1) {
    const double v = pii[0];
    if (fabs(v) > 1.0e-30) pii[0] = 1.0 / v; else sing = true;
  } else if constexpr (B == 2) {
    const double det = pii[0] * pii[3] - pii[1] * pii[2];
    if (fabs(det) > 1.0e-30) {
      const double inv_det = 1.0 / det;
      const double t0 = pii[0];
      pii[0] = inv_det * pii[3];
      pii[1] = -inv_det * pii[1];
      pii[2] = -inv_det * pii[2];
      pii[3] = inv_det * t0;
    } else {
      sing = true;
    }
  } else {
    const double* a = pii;
    const double det = a[0] * a[4] * a[8] + a[3] * a[7] * a[2] + a[6] * a[1] * a[5]
                     - a[0] * a[7] * a[5] - a[6] * a[4] * a[2] - a[3] * a[1] * a[8];
    if (fabs(det) > 1.0e-30) {
      const double inv_det = 1.0 / det;
      double t[9];
#pragma unroll
      for (int m = 0; m < 9; ++m) t[m] = pii[m];
      pii[0] = inv_det * (t[4] * t[8] - t[5] * t[7]);
      pii[1] = inv_det * (t[2] * t[7] - t[1] * t[8]);
      pii[2] = inv_det * (t[1] * t[5] - t[2] * t[4]);
      pii[3] = inv_det * (t[5] * t[6] - t[3] * t[8]);
      pii[4] = inv_det * (t[0] * t[8] - t[2] * t[6]);
      pii[5] = inv_det * (t[2] * t[3] - t[0] * t[5]);
      pii[6] = inv_det * (t[3] * t[7] - t[4] * t[6]);
      pii[7] = inv_det * (t[1] * t[6] - t[0] * t[7]);
      pii[8] = inv_det * (t[0] * t[4] - t[1] * t[3]);
    } else {
      sing = true;
    }
  }
  if (sing) atomicAdd(nsing, 1);
  // U'_ij = D_i^-1 A_ij, j > i
  double d[BS];
#pragma unroll
  for (int m = 0; m < BS; ++m) d[m] = pii[m];
  for (int ij = di; ij < r1; ++ij) {
    double* p = foffd + (size_t)ij * BS;
    if constexpr (B == 1) {
      p[0] = p[0] * d[0];
    } else if constexpr (B == 2) {
      const double t0 = p[0], t1 = p[1], t2 = p[2], t3 = p[3];
      p[0] = d[0] * t0 + d[1] * t2;
      p[1] = d[0] * t1 + d[1] * t3;
      p[2] = d[2] * t0 + d[3] * t2;
      p[3] = d[2] * t1 + d[3] * t3;
    } else {
      double t[9];
#pragma unroll
      for (int m = 0; m < 9; ++m) t[m] = p[m];
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        p[r * 3 + 0] = d[r * 3 + 0] * t[0] + d[r * 3 + 1] * t[3] + d[r * 3 + 2] * t[6];
        p[r * 3 + 1] = d[r * 3 + 0] * t[1] + d[r * 3 + 1] * t[4] + d[r * 3 + 2] * t[7];
        p[r * 3 + 2] = d[r * 3 + 0] * t[2] + d[r * 3 + 1] * t[5] + d[r * 3 + 2] * t[8];
      }
    }
  }
}

// SetValue_Initialize for a factor with fill-in (matvec/matdiafrac_blkcrs.h:
// 90-96): the factor storage was zeroed; every block of A goes to the slot of
// the same column in the factor pattern.  One thread per value.
__global__ void k_factor_init(long long nval, int bs, const int* __restrict__ a2f, const double* __restrict__ offd,
                              double* __restrict__ foffd) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nval) return;
  const long long c = t / bs;
  foffd[(size_t)a2f[c] * bs + (t - c * bs)] = offd[t];
}

cudaError_t launch_factor_init(int B, long long nnz_a, const int* a2f, const double* offd, double* foffd,
                               cudaStream_t st) {
  const long long nval = nnz_a * B * B;
  if (nval <= 0) return cudaSuccess;
  const int tpb = 256;
  k_factor_init<<<(unsigned)((nval + tpb - 1) / tpb), tpb, 0, st>>>(nval, B * B, a2f, offd, foffd);
  return cudaGetLastError();
}

cudaError_t launch_ilu_level(int B, const int* rows, int cnt, const int* rowptr, const int* colind,
                             const int* diaind, double* fdiag, double* foffd, int* nsing, cudaStream_t st,
                             bool dependent) {
  if (cnt <= 0) return cudaSuccess;
  const int tpb = 64;
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3((cnt + tpb - 1) / tpb);
  cfg.blockDim = dim3(tpb);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = dependent ? 1 : 0;
  switch (B) {
    case 1: return cudaLaunchKernelEx(&cfg, k_ilu_level<1>, rows, cnt, rowptr, colind, diaind, fdiag, foffd, nsing);
    case 2: return cudaLaunchKernelEx(&cfg, k_ilu_level<2>, rows, cnt, rowptr, colind, diaind, fdiag, foffd, nsing);
    case 3: return cudaLaunchKernelEx(&cfg, k_ilu_level<3>, rows, cnt, rowptr, colind, diaind, fdiag, foffd, nsing);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace dfg
