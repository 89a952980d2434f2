// k_assemble.cu -- element assembly and Dirichlet finalize.
//
// Assembly is two data-parallel passes with no atomics:
//  1. element pass (one thread per element): shape-function gradients and the
//     element matrix / residual with the reference's expressions
//     (TriArea/TriDlDx, src/femeqn/ker_emat_tri.cpp:13-69; TetVolume/TetDlDx,
//     include/delfem/femeqn/ker_emat_tet.h:32-77; element equations of
//     eqn_poisson.cpp:49-125,249-323, eqn_diffusion.cpp:240-347,
//     eqn_linear_solid2d.cpp:505-598, eqn_linear_solid3d.cpp:241-334),
//     written to an element-block buffer;
//  2. slot gather (one thread per matrix entry / residual entry): each CRS
//     slot adds the blocks that land on it in increasing element order,
//     which is the order CMatDia_BlkCrs::Mearge (src/matvec/matdia_blkcrs.cpp:
//     165-258) and CVector_Blk::AddValue apply them.
// This file is compiled with -fmad=false: with the same operand order and no
// contraction the assembled matrix and residual are bit-identical to the
// reference's.
#include "dfg_common.cuh"
#include "k_assemble.h"

namespace dfg {

__device__ __forceinline__ double tri_area(const double* p0, const double* p1, const double* p2) {
  return 0.5 * ((p1[0] - p0[0]) * (p2[1] - p0[1]) - (p2[0] - p0[0]) * (p1[1] - p0[1]));
}
__device__ __forceinline__ void tri_dldx(double d[3][2], const double* p0, const double* p1, const double* p2) {
  const double area = tri_area(p0, p1, p2);
  const double tmp1 = 0.5 / area;
  d[0][0] = tmp1 * (p1[1] - p2[1]);
  d[1][0] = tmp1 * (p2[1] - p0[1]);
  d[2][0] = tmp1 * (p0[1] - p1[1]);
  d[0][1] = tmp1 * (p2[0] - p1[0]);
  d[1][1] = tmp1 * (p0[0] - p2[0]);
  d[2][1] = tmp1 * (p1[0] - p0[0]);
}
__device__ __forceinline__ double tet_volume(const double* p0, const double* p1, const double* p2, const double* p3) {
  double vol = (p1[0] - p0[0]) * ((p2[1] - p0[1]) * (p3[2] - p0[2]) - (p3[1] - p0[1]) * (p2[2] - p0[2]))
             - (p1[1] - p0[1]) * ((p2[0] - p0[0]) * (p3[2] - p0[2]) - (p3[0] - p0[0]) * (p2[2] - p0[2]))
             + (p1[2] - p0[2]) * ((p2[0] - p0[0]) * (p3[1] - p0[1]) - (p3[0] - p0[0]) * (p2[1] - p0[1]));
  vol *= 0.1666666666666;
  return vol;
}
__device__ __forceinline__ void tet_dldx(double d[4][3], const double* p0, const double* p1, const double* p2, const double* p3) {
  const double vol = tet_volume(p0, p1, p2, p3);
  const double t = 1.0 / (vol * 6.0);
  d[0][0] = -t * ((p2[1] - p1[1]) * (p3[2] - p1[2]) - (p3[1] - p1[1]) * (p2[2] - p1[2]));
  d[0][1] = +t * ((p2[0] - p1[0]) * (p3[2] - p1[2]) - (p3[0] - p1[0]) * (p2[2] - p1[2]));
  d[0][2] = -t * ((p2[0] - p1[0]) * (p3[1] - p1[1]) - (p3[0] - p1[0]) * (p2[1] - p1[1]));
  d[1][0] = +t * ((p3[1] - p2[1]) * (p0[2] - p2[2]) - (p0[1] - p2[1]) * (p3[2] - p2[2]));
  d[1][1] = -t * ((p3[0] - p2[0]) * (p0[2] - p2[2]) - (p0[0] - p2[0]) * (p3[2] - p2[2]));
  d[1][2] = +t * ((p3[0] - p2[0]) * (p0[1] - p2[1]) - (p0[0] - p2[0]) * (p3[1] - p2[1]));
  d[2][0] = -t * ((p0[1] - p3[1]) * (p1[2] - p3[2]) - (p1[1] - p3[1]) * (p0[2] - p3[2]));
  d[2][1] = +t * ((p0[0] - p3[0]) * (p1[2] - p3[2]) - (p1[0] - p3[0]) * (p0[2] - p3[2]));
  d[2][2] = -t * ((p0[0] - p3[0]) * (p1[1] - p3[1]) - (p1[0] - p3[0]) * (p0[1] - p3[1]));
  d[3][0] = +t * ((p1[1] - p0[1]) * (p2[2] - p0[2]) - (p2[1] - p0[1]) * (p1[2] - p0[2]));
  d[3][1] = -t * ((p1[0] - p0[0]) * (p2[2] - p0[2]) - (p2[0] - p0[0]) * (p1[2] - p0[2]));
  d[3][2] = +t * ((p1[0] - p0[0]) * (p2[1] - p0[1]) - (p2[0] - p0[0]) * (p1[1] - p0[1]));
}

// element-block buffer layout: em[((e*k + i)*k + j)*bs + m], er[(e*k + i)*b + d]

__global__ void k_elem_poisson2d(ElemArgs a) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= a.nelem) return;
  const int* no = a.conn + e * 3;
  const double alpha = a.coef ? a.p[0] * a.coef[e] : a.p[0];
  const double source = a.p[1];
  double c[3][2], val[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    c[k][0] = a.coords[no[k] * 2 + 0]; c[k][1] = a.coords[no[k] * 2 + 1];
    val[k] = a.u ? a.u[no[k]] : 0.0;
  }
  const double area = tri_area(c[0], c[1], c[2]);
  double d[3][2];
  tri_dldx(d, c[0], c[1], c[2]);
  double* em = a.em + e * 9;
  double eres[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) eres[i] = source * area * 0.33333333333333333;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const double v = alpha * area * (d[i][0] * d[j][0] + d[i][1] * d[j][1]);
      em[i * 3 + j] = v;
      eres[i] -= v * val[j];
    }
#pragma unroll
  for (int i = 0; i < 3; ++i) a.er[e * 3 + i] = eres[i];
}

__global__ void k_elem_poisson3d(ElemArgs a) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= a.nelem) return;
  const int* no = a.conn + e * 4;
  const double alpha = a.coef ? a.p[0] * a.coef[e] : a.p[0];
  const double source = a.p[1];
  double c[4][3], val[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
#pragma unroll
    for (int q = 0; q < 3; ++q) c[k][q] = a.coords[no[k] * 3 + q];
    val[k] = a.u ? a.u[no[k]] : 0.0;
  }
  const double vol = tet_volume(c[0], c[1], c[2], c[3]);
  double d[4][3];
  tet_dldx(d, c[0], c[1], c[2], c[3]);
  double* em = a.em + e * 16;
  double eres[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) eres[i] = source * vol * 0.25;
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const double v = alpha * vol * (d[i][0] * d[j][0] + d[i][1] * d[j][1] + d[i][2] * d[j][2]);
      em[i * 4 + j] = v;
      eres[i] -= v * val[j];
    }
#pragma unroll
  for (int i = 0; i < 4; ++i) a.er[e * 4 + i] = eres[i];
}

// p = {rho, alpha, source, gamma, dt}
__global__ void k_elem_diffusion2d(ElemArgs a) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= a.nelem) return;
  const int* no = a.conn + e * 3;
  const double rho = a.p[0], source = a.p[2], gamma = a.p[3], dt = a.p[4];
  const double alpha = a.coef ? a.p[1] * a.coef[e] : a.p[1];
  double c[3][2], val[3], vval[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    c[k][0] = a.coords[no[k] * 2 + 0]; c[k][1] = a.coords[no[k] * 2 + 1];
    val[k] = a.u ? a.u[no[k]] : 0.0;
    vval[k] = a.v ? a.v[no[k]] : 0.0;
  }
  const double area = tri_area(c[0], c[1], c[2]);
  double d[3][2];
  tri_dldx(d, c[0], c[1], c[2]);
  double eC[3][3], eM[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) eC[i][j] = alpha * area * (d[i][0] * d[j][0] + d[i][1] * d[j][1]);
  {
    const double t = rho * area * 0.08333333333333333;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
#pragma unroll
      for (int j = 0; j < 3; ++j) eM[i][j] = t;
      eM[i][i] += t;
    }
  }
  double eres[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) eres[i] = source * area * 0.333333333333333333;
  double* em = a.em + e * 9;
  const double gdt = gamma * dt;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) em[i * 3 + j] = eM[i][j] + gdt * eC[i][j];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) eres[i] -= eC[i][j] * (val[j] + dt * vval[j]) + eM[i][j] * vval[j];
#pragma unroll
  for (int i = 0; i < 3; ++i) a.er[e * 3 + i] = eres[i];
}

// p = {lambda, myu, rho, g_x, g_y}
__global__ void k_elem_solid2d(ElemArgs a) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= a.nelem) return;
  const int* no = a.conn + e * 3;
  const double lambda = a.coef ? a.p[0] * a.coef[e] : a.p[0];
  const double myu = a.coef ? a.p[1] * a.coef[e] : a.p[1];
  const double rho = a.p[2], g_x = a.p[3], g_y = a.p[4];
  double c[3][2], disp[3][2];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    c[k][0] = a.coords[no[k] * 2 + 0]; c[k][1] = a.coords[no[k] * 2 + 1];
    disp[k][0] = a.u ? a.u[no[k] * 2 + 0] : 0.0;
    disp[k][1] = a.u ? a.u[no[k] * 2 + 1] : 0.0;
  }
  const double area = tri_area(c[0], c[1], c[2]);
  double d[3][2];
  tri_dldx(d, c[0], c[1], c[2]);
  double eres[3][2];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    eres[i][0] = area * rho * g_x * 0.33333333333333333;
    eres[i][1] = area * rho * g_y * 0.33333333333333333;
  }
  double* em = a.em + e * 36;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      double m00 = area * (lambda + myu) * d[i][0] * d[j][0];
      const double m01 = area * (lambda * d[i][0] * d[j][1] + myu * d[j][0] * d[i][1]);
      const double m10 = area * (lambda * d[i][1] * d[j][0] + myu * d[j][1] * d[i][0]);
      double m11 = area * (lambda + myu) * d[i][1] * d[j][1];
      const double t = (d[i][1] * d[j][1] + d[i][0] * d[j][0]) * area * myu;
      m00 += t;
      m11 += t;
      double* blk = em + (i * 3 + j) * 4;
      blk[0] = m00; blk[1] = m01; blk[2] = m10; blk[3] = m11;
      eres[i][0] -= m00 * disp[j][0] + m01 * disp[j][1];
      eres[i][1] -= m10 * disp[j][0] + m11 * disp[j][1];
    }
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    a.er[(e * 3 + i) * 2 + 0] = eres[i][0];
    a.er[(e * 3 + i) * 2 + 1] = eres[i][1];
  }
}

// p = {lambda, myu, rho, g_x, g_y, g_z}
__global__ void k_elem_solid3d(ElemArgs a) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= a.nelem) return;
  const int* no = a.conn + e * 4;
  const double lambda = a.coef ? a.p[0] * a.coef[e] : a.p[0];
  const double myu = a.coef ? a.p[1] * a.coef[e] : a.p[1];
  const double rho = a.p[2], g_x = a.p[3], g_y = a.p[4], g_z = a.p[5];
  double c[4][3], disp[4][3];
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      c[k][q] = a.coords[no[k] * 3 + q];
      disp[k][q] = a.u ? a.u[no[k] * 3 + q] : 0.0;
    }
  const double vol = tet_volume(c[0], c[1], c[2], c[3]);
  double d[4][3];
  tet_dldx(d, c[0], c[1], c[2], c[3]);
  double* em = a.em + e * 144;
  double* er = a.er + e * 12;
#pragma unroll 1
  for (int i = 0; i < 4; ++i) {
    double r0 = vol * rho * g_x * 0.25;
    double r1 = vol * rho * g_y * 0.25;
    double r2 = vol * rho * g_z * 0.25;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      double m[3][3];
#pragma unroll
      for (int p = 0; p < 3; ++p)
#pragma unroll
        for (int q = 0; q < 3; ++q) m[p][q] = vol * (lambda * d[i][p] * d[j][q] + myu * d[j][p] * d[i][q]);
      const double t = d[i][0] * d[j][0] + d[i][1] * d[j][1] + d[i][2] * d[j][2];
      m[0][0] += vol * myu * t;
      m[1][1] += vol * myu * t;
      m[2][2] += vol * myu * t;
      double* blk = em + (i * 4 + j) * 9;
#pragma unroll
      for (int p = 0; p < 3; ++p)
#pragma unroll
        for (int q = 0; q < 3; ++q) blk[p * 3 + q] = m[p][q];
      r0 -= m[0][0] * disp[j][0] + m[0][1] * disp[j][1] + m[0][2] * disp[j][2];
      r1 -= m[1][0] * disp[j][0] + m[1][1] * disp[j][1] + m[1][2] * disp[j][2];
      r2 -= m[2][0] * disp[j][0] + m[2][1] * disp[j][1] + m[2][2] * disp[j][2];
    }
    er[i * 3 + 0] = r0; er[i * 3 + 1] = r1; er[i * 3 + 2] = r2;
  }
}

// slot gather: matrix entry (slot s, element m); slots < n are diagonal blocks
__global__ void k_gather_matrix(GatherArgs a) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long total = (a.n + a.nnz) * (long long)a.bs;
  if (t >= total) return;
  const long long s = t / a.bs;
  const int m = (int)(t - s * a.bs);
  double* dst = s < a.n ? a.diag + s * a.bs + m : a.offd + (s - a.n) * a.bs + m;
  double acc = *dst;
  for (long long p = a.slot_ptr[s]; p < a.slot_ptr[s + 1]; ++p) acc += a.em[(long long)a.slot_src[p] * a.bs + m];
  *dst = acc;
}

// residual entry (node i, dof d)
__global__ void k_gather_residual(GatherArgs a) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)a.n * a.b) return;
  const long long i = t / a.b;
  const int d = (int)(t - i * a.b);
  double acc = a.res[t];
  for (long long p = a.res_ptr[i]; p < a.res_ptr[i + 1]; ++p) acc += a.er[(long long)a.res_src[p] * a.b + d];
  a.res[t] = acc;
}

__global__ void k_add_vec(long long m, const double* f, double* r) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t < m) r[t] = r[t] + f[t];
}

// Dirichlet finalize (CMatDia_BlkCrs::SetBoundaryCondition, src/matvec/matdia_blkcrs.cpp:
// 314-343): entry (r,q) of diagonal block i becomes 1 if r==q and DOF (i,r) is
// fixed, 0 if (i,r) or (i,q) is fixed; entry (r,q) of off-diagonal block
// (i,j) becomes 0 if (i,r) or (j,q) is fixed.
__global__ void k_bc_matrix(BcArgs a) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int b = a.b, bs = b * b;
  const long long total = (a.n + a.nnz) * (long long)bs;
  if (t >= total) return;
  const long long s = t / bs;
  const int m = (int)(t - s * bs), r = m / b, q = m - (m / b) * b;
  if (s < a.n) {
    const int fr = a.flag[s * b + r], fq = a.flag[s * b + q];
    if (r == q && fr) a.diag[t] = 1.0;
    else if (fr || fq) a.diag[t] = 0.0;
  } else {
    const long long c = s - a.n;
    // row of slot c: last i with rowptr[i] <= c
    int lo = 0, hi = a.n;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (a.rowptr[mid] <= c) lo = mid; else hi = mid;
    }
    const int i = lo, j = a.colind[c];
    if (a.flag[(long long)i * b + r] || a.flag[(long long)j * b + q]) a.offd[c * bs + m] = 0.0;
  }
}

__global__ void k_bc_residual(long long m, const int* flag, double* res) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t < m && flag[t] == 1) res[t] = 0;
}

static inline int nblk(long long n, int tpb) { return (int)((n + tpb - 1) / tpb); }

cudaError_t launch_elem(int kind, const ElemArgs& a, cudaStream_t st) {
  if (a.nelem == 0) return cudaSuccess;
  const int tpb = 128;
  switch (kind) {
    case 1: k_elem_poisson2d<<<nblk(a.nelem, tpb), tpb, 0, st>>>(a); break;
    case 2: k_elem_poisson3d<<<nblk(a.nelem, tpb), tpb, 0, st>>>(a); break;
    case 3: k_elem_diffusion2d<<<nblk(a.nelem, tpb), tpb, 0, st>>>(a); break;
    case 4: k_elem_solid2d<<<nblk(a.nelem, tpb), tpb, 0, st>>>(a); break;
    case 5: k_elem_solid3d<<<nblk(a.nelem, 64), 64, 0, st>>>(a); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_gather(const GatherArgs& a, cudaStream_t st) {
  const int tpb = 256;
  const long long tm = (a.n + a.nnz) * (long long)a.bs;
  if (tm > 0) k_gather_matrix<<<nblk(tm, tpb), tpb, 0, st>>>(a);
  const long long tr = (long long)a.n * a.b;
  if (tr > 0) k_gather_residual<<<nblk(tr, tpb), tpb, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_add_vec(long long m, const double* f, double* r, cudaStream_t st) {
  if (m > 0) k_add_vec<<<nblk(m, 256), 256, 0, st>>>(m, f, r);
  return cudaGetLastError();
}

cudaError_t launch_bc(const BcArgs& a, cudaStream_t st) {
  const long long tm = (a.n + a.nnz) * (long long)a.b * a.b;
  if (tm > 0) k_bc_matrix<<<nblk(tm, 256), 256, 0, st>>>(a);
  const long long tr = (long long)a.n * a.b;
  if (tr > 0) k_bc_residual<<<nblk(tr, 256), 256, 0, st>>>(tr, a.flag, a.res);
  return cudaGetLastError();
}

}  // namespace dfg
