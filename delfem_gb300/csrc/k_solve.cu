// k_solve.cu -- SpMV, reductions and the device-resident PCG iteration.
//
// The PCG loop of LsSol::Solve_PCG (src/ls/solver_ls_iter.cpp:100-172) is
// cut into a few kernels whose scalars (alpha, beta, rho) live in a device
// state, so a whole iteration -- and a chunk of iterations captured in a CUDA
// graph -- runs without any host round trip.  Convergence is checked on the
// device; once `done` is set every later kernel of the chunk returns at once.
//
// Dot products are deterministic: a fixed grid, one partial per block
// (fixed-shape warp-shuffle tree), and the last block to finish sums the
// partials in index order.
#include <cmath>

#include <utility>

#include "dfg_common.cuh"
#include "k_reduce.cuh"
#include "k_rowmv.cuh"
#include "k_solve.h"

namespace dfg {

// ------------------------------------------------------------------- SpMV

// q = A p and pAp = p.q; the last block sets alpha = rz / pAp.  Thread per
// block row over the sliced-ELL copy (coalesced value loads).
template <typename T, int B>
__global__ void __launch_bounds__(kSpmvTpb, 2) k_spmv_pap(MatView Am, const T* __restrict__ p, T* __restrict__ q,
                                                         PcgState* st, Red red) {
  pdl_enter();
  if (st->done) return;
  const T* sval = reinterpret_cast<const T*>(Am.sval);
  double part = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < Am.n; i += gridDim.x * blockDim.x) {
    T y[B];
    sell_row_mv<T, B>(i, Am.sptr, Am.swidth, Am.scol, sval, p, y);
#pragma unroll
    for (int d = 0; d < B; ++d) {
      q[(size_t)i * B + d] = y[d];
      part += (double)p[(size_t)i * B + d] * (double)y[d];
    }
  }
  double tot;
  if (grid_sum(part, red, &tot) && threadIdx.x == 0) {
    st->pap = tot;
    st->alpha = st->rz / tot;
  }
}

// one block per slice: value (w, e) of lane l from the block named by src
template <typename T, int B>
__global__ void k_sell_pack(const long long* __restrict__ ptr, const int* __restrict__ src,
                            const double* __restrict__ diag, const double* __restrict__ offd, T* __restrict__ out) {
  constexpr int BS = B * B;
  const int s = blockIdx.x;
  const long long k0 = ptr[s];
  const int nval = (int)(ptr[s + 1] - k0) * BS;
  for (int o = threadIdx.x; o < nval; o += blockDim.x) {
    const int lane = o & 31, e = (o >> 5) % BS, w = (o >> 5) / BS;
    const int v = src[k0 + w * 32 + lane];
    const double a = v >= 0 ? offd[(size_t)v * BS + e] : v == -1 ? 0.0 : diag[(size_t)(-v - 2) * BS + e];
    out[k0 * BS + o] = (T)a;
  }
}

cudaError_t sell_pack(int nslices, int b, const long long* ptr, const int* src, const double* diag,
                      const double* offd, void* out, bool fp32, cudaStream_t s) {
  if (nslices == 0) return cudaSuccess;
#define DFG_SELL(B)                                                                                        \
  if (fp32) k_sell_pack<float, B><<<nslices, 256, 0, s>>>(ptr, src, diag, offd, static_cast<float*>(out)); \
  else k_sell_pack<double, B><<<nslices, 256, 0, s>>>(ptr, src, diag, offd, static_cast<double*>(out));
  switch (b) {
    case 1: DFG_SELL(1) break;
    case 2: DFG_SELL(2) break;
    case 3: DFG_SELL(3) break;
    default: return cudaErrorInvalidValue;
  }
#undef DFG_SELL
  return cudaGetLastError();
}

// ------------------------------------------------------------- FP64 PCG

template <typename Z>
__device__ __forceinline__ double zval(const void* z, long long k) {
  return (double)reinterpret_cast<const Z*>(z)[k];
}

// x := 0 * x (SCAL(0,x)); rr0 = r.r; early exit below 1e-30; sentinels
template <typename Z>
__global__ void k_pcg_init(PcgVecs v, PcgState* st, Red red, double tol, int maxit, int* tickets) {
  double part = 0.0;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < v.m; k += (long long)gridDim.x * blockDim.x) {
    v.x[k] = v.x[k] * 0.0;
    const double r = v.r[k];
    part += r * r;
    reinterpret_cast<Z*>(v.y)[k] = sentinel_value<Z>();
    reinterpret_cast<Z*>(v.z)[k] = sentinel_value<Z>();
    if constexpr (sizeof(Z) == 4) v.r32[k] = (float)r;
  }
  double tot;
  if (grid_sum(part, red, &tot) && threadIdx.x == 0) {
    st->rr0 = tot;
    st->it = 0;
    st->maxit = maxit;
    st->iter_out = 0;
    st->tol2 = tol * tol;
    if (tot < 1.0e-30) {
      st->done = 1;
      st->conv = 0.0;
    } else {
      st->done = (maxit <= 0) ? 2 : 0;
      st->inv_rr0 = 1.0 / tot;
      st->conv = 1.0;
    }
    tickets[0] = 0;
    tickets[1] = 0;
  }
}

// p := z; rz = r.z
template <typename Z>
__global__ void k_pcg_after_precond0(PcgVecs v, PcgState* st, Red red) {
  if (st->done) return;
  double part = 0.0;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < v.m; k += (long long)gridDim.x * blockDim.x) {
    const double z = zval<Z>(v.z, k);
    v.p[k] = z;
    part += v.r[k] * z;
  }
  double tot;
  if (grid_sum(part, red, &tot) && threadIdx.x == 0) st->rz = tot;
}

// r := r - alpha q; x := x + alpha p (AXPY, no-op for alpha == 0); rr = r.r;
// convergence check; sentinel refill for the sweeps; sweep tickets reset
template <typename Z>
__global__ void k_pcg_update_rx(PcgVecs v, PcgState* st, Red red, int* tickets) {
  pdl_enter();
  if (st->done) return;
  const double alpha = st->alpha;
  double part = 0.0;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < v.m; k += (long long)gridDim.x * blockDim.x) {
    double r = v.r[k];
    if (alpha != 0.0) {
      r = __dadd_rn(r, __dmul_rn(-alpha, v.q[k]));
      v.r[k] = r;
      v.x[k] = __dadd_rn(v.x[k], __dmul_rn(alpha, v.p[k]));
    }
    part += r * r;
    reinterpret_cast<Z*>(v.y)[k] = sentinel_value<Z>();
    reinterpret_cast<Z*>(v.z)[k] = sentinel_value<Z>();
    if constexpr (sizeof(Z) == 4) v.r32[k] = (float)r;
  }
  double tot;
  if (grid_sum(part, red, &tot) && threadIdx.x == 0) {
    st->rr = tot;
    const double ratio = tot * st->inv_rr0;
    if (ratio < st->tol2) {
      st->done = 1;
      st->conv = sqrt(ratio);
      st->iter_out = st->it;
    } else if (st->it + 1 >= st->maxit) {
      st->done = 2;
      st->conv = sqrt(ratio);
      st->iter_out = st->maxit;
    } else if (!(ratio == ratio)) {
      st->done = 3;  // NaN
      st->conv = ratio;
      st->iter_out = st->it;
    }
    tickets[0] = 0;
    tickets[1] = 0;
  }
}

// rz_new = r.z; beta = rz_new / rz
template <typename Z>
__global__ void k_pcg_rz_beta(PcgVecs v, PcgState* st, Red red) {
  pdl_enter();
  if (st->done) return;
  double part = 0.0;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < v.m; k += (long long)gridDim.x * blockDim.x)
    part += v.r[k] * zval<Z>(v.z, k);
  double tot;
  if (grid_sum(part, red, &tot) && threadIdx.x == 0) {
    st->beta = tot / st->rz;
    st->rz = tot;
  }
}

// p := beta p; p := p + 1.0 z (SCAL + AXPY); iteration counter
template <typename Z>
__global__ void k_pcg_update_p(PcgVecs v, PcgState* st) {
  pdl_enter();
  if (st->done) return;
  const double beta = st->beta;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < v.m; k += (long long)gridDim.x * blockDim.x)
    v.p[k] = __dadd_rn(__dmul_rn(v.p[k], beta), zval<Z>(v.z, k));
  if (blockIdx.x == 0 && threadIdx.x == 0) st->it += 1;
}

// rd = b - A x; st->rr = rd.rd
template <int B>
__global__ void k_pcg_true_residual(MatView Am, PcgVecs v, PcgState* st, Red red) {
  const double* diag = reinterpret_cast<const double*>(Am.diag);
  const double* offd = reinterpret_cast<const double*>(Am.offd);
  double part = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < Am.n; i += gridDim.x * blockDim.x) {
    double y[B];
    row_mv<double, double, B>(i, Am.rowptr, Am.colind, diag, offd, v.x, y);
#pragma unroll
    for (int d = 0; d < B; ++d) {
      const double r = v.b[(size_t)i * B + d] - y[d];
      v.rd[(size_t)i * B + d] = r;
      part += r * r;
    }
  }
  double tot;
  if (grid_sum(part, red, &tot) && threadIdx.x == 0) st->rr = tot;
}

// residual replacement: continue the recursion from the true residual
template <typename Z>
__global__ void k_pcg_replace(PcgVecs v, PcgState* st, int* tickets) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < v.m; k += (long long)gridDim.x * blockDim.x) {
    const double r = v.rd[k];
    v.r[k] = r;
    if constexpr (sizeof(Z) == 4) v.r32[k] = (float)r;
    reinterpret_cast<Z*>(v.y)[k] = sentinel_value<Z>();
    reinterpret_cast<Z*>(v.z)[k] = sentinel_value<Z>();
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    st->done = 0;
    tickets[0] = 0;
    tickets[1] = 0;
  }
}

// ----------------------------------------------------------- mixed precision

// rd = b - A x (FP64); rr = rd.rd
template <int B>
__global__ void k_mix_true_residual(MatView Am, MixVecs v, PcgState* st, Red red) {
  const double* diag = reinterpret_cast<const double*>(Am.diag);
  const double* offd = reinterpret_cast<const double*>(Am.offd);
  double part = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < Am.n; i += gridDim.x * blockDim.x) {
    double y[B];
    row_mv<double, double, B>(i, Am.rowptr, Am.colind, diag, offd, v.x, y);
#pragma unroll
    for (int d = 0; d < B; ++d) {
      const double r = v.b[(size_t)i * B + d] - y[d];
      v.rd[(size_t)i * B + d] = r;
      part += r * r;
    }
  }
  double tot;
  if (grid_sum(part, red, &tot) && threadIdx.x == 0) st->rr = tot;
}

__global__ void k_mix_start(PcgState* st, double tol, double bb, double delta, int maxit) {
  st->it = 0;
  st->maxit = maxit;
  st->iter_out = 0;
  st->done = 0;
  st->tolb2 = tol * tol * bb;
  st->delta2 = delta * delta;
  st->rr0 = bb;
  st->inv_rr0 = bb > 0 ? 1.0 / bb : 0.0;
  st->conv = 1.0;
}

// residual replacement: the FP32 recursive residual restarts from the FP64
// true residual; the correction is folded into the FP64 solution
__global__ void k_mix_replace(MixVecs v, PcgState* st, int* tickets) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < v.m; k += (long long)gridDim.x * blockDim.x) {
    v.r[k] = (float)v.rd[k];
    v.y[k] = sentinel_value<float>();
    v.z[k] = sentinel_value<float>();
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    st->rr_ref = st->rr;
    st->done = 0;
    tickets[0] = 0;
    tickets[1] = 0;
  }
}

__global__ void k_mix_after_precond0(MixVecs v, PcgState* st, Red red) {
  if (st->done) return;
  double part = 0.0;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < v.m; k += (long long)gridDim.x * blockDim.x) {
    const float z = v.z[k];
    v.p[k] = z;
    part += (double)v.r[k] * (double)z;
  }
  double tot;
  if (grid_sum(part, red, &tot) && threadIdx.x == 0) st->rz = tot;
}

__global__ void k_mix_update_rx(MixVecs v, PcgState* st, Red red, int* tickets) {
  if (st->done) return;
  const double alpha = st->alpha;
  const float alpha32 = (float)alpha;
  double part = 0.0;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < v.m; k += (long long)gridDim.x * blockDim.x) {
    float r = v.r[k];
    if (alpha != 0.0) {
      r = r - alpha32 * v.q[k];
      v.r[k] = r;
      v.d[k] = v.d[k] + alpha * (double)v.p[k];
    }
    part += (double)r * (double)r;
    v.y[k] = sentinel_value<float>();
    v.z[k] = sentinel_value<float>();
  }
  double tot;
  if (grid_sum(part, red, &tot) && threadIdx.x == 0) {
    st->rr = tot;
    if (!(tot == tot)) {
      st->done = 3;
    } else if (tot < st->tolb2) {
      st->done = 5;
    } else if (tot < st->delta2 * st->rr_ref) {
      st->done = 4;
    } else if (st->it + 1 >= st->maxit) {
      st->done = 2;
    }
    st->iter_out = st->it + 1;
    tickets[0] = 0;
    tickets[1] = 0;
  }
}

__global__ void k_mix_rz_beta(MixVecs v, PcgState* st, Red red) {
  if (st->done) return;
  double part = 0.0;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < v.m; k += (long long)gridDim.x * blockDim.x)
    part += (double)v.r[k] * (double)v.z[k];
  double tot;
  if (grid_sum(part, red, &tot) && threadIdx.x == 0) {
    st->beta = tot / st->rz;
    st->rz = tot;
  }
}

__global__ void k_mix_update_p(MixVecs v, PcgState* st) {
  if (st->done) return;
  const float beta = (float)st->beta;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < v.m; k += (long long)gridDim.x * blockDim.x)
    v.p[k] = v.z[k] + beta * v.p[k];
  if (blockIdx.x == 0 && threadIdx.x == 0) st->it += 1;
}

__global__ void k_mix_accumulate(MixVecs v) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < v.m; k += (long long)gridDim.x * blockDim.x) {
    v.x[k] = v.x[k] + v.d[k];
    v.d[k] = 0.0;
  }
}

__global__ void k_mix_clear_done(PcgState* st) { st->done = 0; }

__global__ void k_to_fp32(long long m, const double* a, float* b) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < m; k += (long long)gridDim.x * blockDim.x)
    b[k] = (float)a[k];
}

__global__ void k_fill_sentinel64(long long m, double* p) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < m; k += (long long)gridDim.x * blockDim.x)
    p[k] = sentinel_value<double>();
}
__global__ void k_fill_sentinel32(long long m, float* p) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < m; k += (long long)gridDim.x * blockDim.x)
    p[k] = sentinel_value<float>();
}

// ------------------------------------------------------------- launchers

// reductions always use the fixed grid (deterministic regardless of timing)
#define RED_LAUNCH <<<kRedGrid, kRedTpb, 0, s>>>

// dep: launch as a programmatic dependent of the previous kernel in the
// stream (the kernel waits for it at entry, see pdl_enter)
template <typename... KArgs, typename... Args>
static cudaError_t launch_dep(void (*k)(KArgs...), int grid, int block, cudaStream_t s, bool dep, Args&&... args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = dep ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, k, std::forward<Args>(args)...);
}

#define ZDISPATCH(kern, ...)                               \
  do {                                                     \
    if (fp32z) kern<float> RED_LAUNCH(__VA_ARGS__);        \
    else kern<double> RED_LAUNCH(__VA_ARGS__);             \
  } while (0)

cudaError_t pcg_init(const PcgVecs& v, PcgState* st, Red red, double tol, int maxit, int* tickets, bool fp32z, cudaStream_t s) {
  ZDISPATCH(k_pcg_init, v, st, red, tol, maxit, tickets);
  return cudaGetLastError();
}
cudaError_t pcg_after_precond0(const PcgVecs& v, PcgState* st, Red red, bool fp32z, cudaStream_t s) {
  ZDISPATCH(k_pcg_after_precond0, v, st, red);
  return cudaGetLastError();
}
cudaError_t pcg_spmv_pap(const MatView& A, const PcgVecs& v, PcgState* st, Red red, cudaStream_t s, bool dep) {
  const double* p = v.p;
  double* q = v.q;
  switch (A.b) {
    case 1: return launch_dep(k_spmv_pap<double, 1>, kRedGrid, kSpmvTpb, s, dep, A, p, q, st, red);
    case 2: return launch_dep(k_spmv_pap<double, 2>, kRedGrid, kSpmvTpb, s, dep, A, p, q, st, red);
    case 3: return launch_dep(k_spmv_pap<double, 3>, kRedGrid, kSpmvTpb, s, dep, A, p, q, st, red);
    default: return cudaErrorInvalidValue;
  }
}
cudaError_t pcg_update_rx(const PcgVecs& v, PcgState* st, Red red, int* tickets, bool fp32z, cudaStream_t s, bool dep) {
  if (fp32z) return launch_dep(k_pcg_update_rx<float>, kRedGrid, kRedTpb, s, dep, v, st, red, tickets);
  return launch_dep(k_pcg_update_rx<double>, kRedGrid, kRedTpb, s, dep, v, st, red, tickets);
}
cudaError_t pcg_rz_beta(const PcgVecs& v, PcgState* st, Red red, bool fp32z, cudaStream_t s, bool dep) {
  if (fp32z) return launch_dep(k_pcg_rz_beta<float>, kRedGrid, kRedTpb, s, dep, v, st, red);
  return launch_dep(k_pcg_rz_beta<double>, kRedGrid, kRedTpb, s, dep, v, st, red);
}
cudaError_t pcg_update_p(const PcgVecs& v, PcgState* st, bool fp32z, cudaStream_t s, bool dep) {
  if (fp32z) return launch_dep(k_pcg_update_p<float>, kRedGrid, kRedTpb, s, dep, v, st);
  return launch_dep(k_pcg_update_p<double>, kRedGrid, kRedTpb, s, dep, v, st);
}
cudaError_t pcg_true_residual(const MatView& A, const PcgVecs& v, PcgState* st, Red red, cudaStream_t s) {
  switch (A.b) {
    case 1: k_pcg_true_residual<1> RED_LAUNCH(A, v, st, red); break;
    case 2: k_pcg_true_residual<2> RED_LAUNCH(A, v, st, red); break;
    case 3: k_pcg_true_residual<3> RED_LAUNCH(A, v, st, red); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}
cudaError_t pcg_replace(const PcgVecs& v, PcgState* st, int* tickets, bool fp32z, cudaStream_t s) {
  ZDISPATCH(k_pcg_replace, v, st, tickets);
  return cudaGetLastError();
}

cudaError_t mix_true_residual(const MatView& A64, const MixVecs& v, PcgState* st, Red red, cudaStream_t s) {
  switch (A64.b) {
    case 1: k_mix_true_residual<1> RED_LAUNCH(A64, v, st, red); break;
    case 2: k_mix_true_residual<2> RED_LAUNCH(A64, v, st, red); break;
    case 3: k_mix_true_residual<3> RED_LAUNCH(A64, v, st, red); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}
cudaError_t mix_replace(const MixVecs& v, PcgState* st, int* tickets, cudaStream_t s) {
  k_mix_replace RED_LAUNCH(v, st, tickets);
  return cudaGetLastError();
}
cudaError_t mix_start(PcgState* st, double tol, double bb, double delta, int maxit, cudaStream_t s) {
  k_mix_start<<<1, 1, 0, s>>>(st, tol, bb, delta, maxit);
  return cudaGetLastError();
}
cudaError_t mix_clear_done(PcgState* st, cudaStream_t s) {
  k_mix_clear_done<<<1, 1, 0, s>>>(st);
  return cudaGetLastError();
}
cudaError_t mix_after_precond0(const MixVecs& v, PcgState* st, Red red, cudaStream_t s) {
  k_mix_after_precond0 RED_LAUNCH(v, st, red);
  return cudaGetLastError();
}
cudaError_t mix_spmv_pap(const MatView& A32, const MixVecs& v, PcgState* st, Red red, cudaStream_t s) {
  switch (A32.b) {
    case 1: k_spmv_pap<float, 1><<<kRedGrid, kSpmvTpb, 0, s>>>(A32, v.p, v.q, st, red); break;
    case 2: k_spmv_pap<float, 2><<<kRedGrid, kSpmvTpb, 0, s>>>(A32, v.p, v.q, st, red); break;
    case 3: k_spmv_pap<float, 3><<<kRedGrid, kSpmvTpb, 0, s>>>(A32, v.p, v.q, st, red); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}
cudaError_t mix_update_rx(const MixVecs& v, PcgState* st, Red red, int* tickets, cudaStream_t s) {
  k_mix_update_rx RED_LAUNCH(v, st, red, tickets);
  return cudaGetLastError();
}
cudaError_t mix_rz_beta(const MixVecs& v, PcgState* st, Red red, cudaStream_t s) {
  k_mix_rz_beta RED_LAUNCH(v, st, red);
  return cudaGetLastError();
}
cudaError_t mix_update_p(const MixVecs& v, PcgState* st, cudaStream_t s) {
  k_mix_update_p RED_LAUNCH(v, st);
  return cudaGetLastError();
}
cudaError_t mix_accumulate(const MixVecs& v, cudaStream_t s) {
  k_mix_accumulate RED_LAUNCH(v);
  return cudaGetLastError();
}
cudaError_t to_fp32(long long m, const double* a, float* b, cudaStream_t s) {
  if (m > 0) k_to_fp32 RED_LAUNCH(m, a, b);
  return cudaGetLastError();
}
cudaError_t fill_sentinel(long long m, void* p, bool fp32, cudaStream_t s) {
  if (m <= 0) return cudaSuccess;
  if (fp32) k_fill_sentinel32 RED_LAUNCH(m, static_cast<float*>(p));
  else k_fill_sentinel64 RED_LAUNCH(m, static_cast<double*>(p));
  return cudaGetLastError();
}

}  // namespace dfg
