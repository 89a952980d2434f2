// k_bicg.cu -- device-resident preconditioned BiCGSTAB.
//
// LsSol::Solve_PBiCGSTAB (src/ls/solver_ls_iter.cpp:291-408) cut into
// kernels whose scalars (rho, alpha, omega, beta) live in a device state, so
// a chunk of iterations captured in a CUDA graph runs without host round
// trips.  One iteration:
//   sweeps(p -> Mp); AMp = A Mp, (AMp, r2) -> alpha;          [k_bicg_amp]
//   s = r - alpha AMp;                                          [k_bicg_s]
//   sweeps(s -> Ms); AMs = A Ms, (s, AMs), (AMs, AMs) -> omega; [k_bicg_ams]
//   x += alpha Mp; x += omega Ms; r = s - omega AMs;
//   (r, r), (r, r2) -> convergence, beta;                       [k_bicg_update]
//   p = beta p + r - beta omega AMp                             [k_bicg_p]
// The reference's (r, r2) at the top of an iteration is the same product as
// the beta numerator of the iteration before (r does not change in between),
// so it is carried over in the state instead of being recomputed.  Vector
// updates round like the reference's AXPY / SCAL (separate multiply and add,
// AXPY skipped for a zero coefficient).  Everything is FP64: BiCGSTAB's
// shadow-residual recurrences do not survive a preconditioner applied in
// FP32 (fresh rounding at every application makes it a different operator
// each time; on a 200x100 cantilever that doubles the iterations, and with
// the factor rounded too the iteration diverges), unlike CG's.
#include <cmath>

#include "dfg_common.cuh"
#include "k_reduce.cuh"
#include "k_rowmv.cuh"
#include "k_solve.h"

namespace dfg {

// y := y + a x, rounded as CVector_Blk's AXPY (no contraction)
__device__ __forceinline__ double axpy1(double y, double a, double x) { return __dadd_rn(y, __dmul_rn(a, x)); }

// rr0 = (r, r); a residual below 1e-60 ends the solve before anything is
// touched (the reference returns with ratio sqrt(rr0) and x as it is)
__global__ void k_bicg_init0(BicgVecs v, BicgState* st, Red red, double tol, int maxit) {
  double part = 0.0;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < v.m; k += (long long)gridDim.x * blockDim.x) {
    const double r = v.r[k];
    part += r * r;
  }
  double tot;
  if (grid_sum(part, red, &tot) && threadIdx.x == 0) {
    st->rr0 = tot;
    st->rr = tot;
    st->tol2 = tol * tol;
    st->maxit = maxit;
    st->it = 1;
    st->iter_out = 0;
    st->conv = tol;
    if (tot < 1.0e-60) {
      st->done = 4;
      st->conv = sqrt(tot);
    } else {
      st->inv_rr0 = 1.0 / tot;
      st->rho = tot;  // (r, r2) with r2 = r
      st->done = (maxit <= 1) ? 2 : 0;
      if (maxit <= 1) st->iter_out = maxit;
    }
  }
}

// x := 0 x; r2 = r; p = r; sweep outputs to the sentinel; tickets reset
__global__ void k_bicg_init1(BicgVecs v, BicgState* st, int* tickets) {
  if (st->done == 4) return;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < v.m; k += (long long)gridDim.x * blockDim.x) {
    v.x[k] = v.x[k] * 0.0;
    const double r = v.r[k];
    v.r2[k] = r;
    v.p[k] = r;
    v.y[k] = sentinel_value<double>();
    v.mp[k] = sentinel_value<double>();
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    tickets[0] = 0;
    tickets[1] = 0;
  }
}

// AMp = A Mp; alpha = rho / (AMp, r2)
template <int B>
__global__ void __launch_bounds__(kSpmvTpb, 2) k_bicg_amp(MatView Am, BicgVecs v, BicgState* st, Red red) {
  if (st->done) return;
  const double* sval = reinterpret_cast<const double*>(Am.sval);
  double part = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < Am.n; i += gridDim.x * blockDim.x) {
    double y[B];
    sell_row_mv<double, B>(i, Am.sptr, Am.swidth, Am.scol, sval, v.mp, y);
#pragma unroll
    for (int d = 0; d < B; ++d) {
      v.amp[(size_t)i * B + d] = y[d];
      part += y[d] * v.r2[(size_t)i * B + d];
    }
  }
  double tot;
  if (grid_sum(part, red, &tot) && threadIdx.x == 0) st->alpha = st->rho / tot;
}

// s = r; s += -alpha AMp; sweep outputs to the sentinel; tickets reset
__global__ void k_bicg_s(BicgVecs v, BicgState* st, int* tickets) {
  if (st->done) return;
  const double na = -st->alpha;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < v.m; k += (long long)gridDim.x * blockDim.x) {
    double s = v.r[k];
    if (na != 0.0) s = axpy1(s, na, v.amp[k]);
    v.s[k] = s;
    v.y[k] = sentinel_value<double>();
    v.ms[k] = sentinel_value<double>();
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    tickets[0] = 0;
    tickets[1] = 0;
  }
}

// AMs = A Ms; omega = (s, AMs) / (AMs, AMs)
template <int B>
__global__ void __launch_bounds__(kSpmvTpb, 2) k_bicg_ams(MatView Am, BicgVecs v, BicgState* st, Red red) {
  if (st->done) return;
  const double* sval = reinterpret_cast<const double*>(Am.sval);
  double tt = 0.0, ts = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < Am.n; i += gridDim.x * blockDim.x) {
    double y[B];
    sell_row_mv<double, B>(i, Am.sptr, Am.swidth, Am.scol, sval, v.ms, y);
#pragma unroll
    for (int d = 0; d < B; ++d) {
      v.ams[(size_t)i * B + d] = y[d];
      tt += y[d] * y[d];
      ts += v.s[(size_t)i * B + d] * y[d];
    }
  }
  double den, num;
  if (grid_sum2(tt, ts, red, &den, &num) && threadIdx.x == 0) st->omega = num / den;
}

// x += alpha Mp; x += omega Ms; r = s; r += -omega AMs; (r, r) -> stop test;
// (r, r2) -> beta and the next rho
__global__ void k_bicg_update(BicgVecs v, BicgState* st, Red red) {
  if (st->done) return;
  const double alpha = st->alpha, omega = st->omega, no = -omega;
  double rr = 0.0, rr2 = 0.0;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < v.m; k += (long long)gridDim.x * blockDim.x) {
    double x = v.x[k];
    if (alpha != 0.0) x = axpy1(x, alpha, v.mp[k]);
    if (omega != 0.0) x = axpy1(x, omega, v.ms[k]);
    v.x[k] = x;
    double r = v.s[k];
    if (no != 0.0) r = axpy1(r, no, v.ams[k]);
    v.r[k] = r;
    rr += r * r;
    rr2 += r * v.r2[k];
  }
  double trr, trr2;
  if (grid_sum2(rr, rr2, red, &trr, &trr2) && threadIdx.x == 0) {
    st->rr = trr;
    const double sq = trr * st->inv_rr0;
    if (sq < st->tol2) {
      st->done = 1;
      st->conv = sqrt(sq);
      st->iter_out = st->it;
    } else if (!(sq == sq)) {
      st->done = 3;
      st->iter_out = st->it;
    } else {
      st->beta = trr2 * alpha / (st->rho * omega);
      st->rho = trr2;
      if (st->it + 1 >= st->maxit) {
        st->done = 2;  // the reference's loop ends; ratio left as given
        st->iter_out = st->maxit;
      }
    }
  }
}

// p := beta p; p += 1.0 r; p += -beta omega AMp; next iteration
__global__ void k_bicg_p(BicgVecs v, BicgState* st, int* tickets) {
  if (st->done) return;
  const double beta = st->beta, c = -beta * st->omega;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < v.m; k += (long long)gridDim.x * blockDim.x) {
    double p = __dmul_rn(v.p[k], beta);
    p = __dadd_rn(p, v.r[k]);
    if (c != 0.0) p = axpy1(p, c, v.amp[k]);
    v.p[k] = p;
    v.y[k] = sentinel_value<double>();
    v.mp[k] = sentinel_value<double>();
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    tickets[0] = 0;
    tickets[1] = 0;
    st->it += 1;
  }
}

#define DFG_BDISPATCH(kern, ...)                                                    \
  do {                                                                              \
    switch (A.b) {                                                                  \
      case 1: kern<1><<<kRedGrid, kSpmvTpb, 0, s>>>(__VA_ARGS__); break;            \
      case 2: kern<2><<<kRedGrid, kSpmvTpb, 0, s>>>(__VA_ARGS__); break;            \
      case 3: kern<3><<<kRedGrid, kSpmvTpb, 0, s>>>(__VA_ARGS__); break;            \
      default: return cudaErrorInvalidValue;                                        \
    }                                                                               \
  } while (0)

cudaError_t bicg_init(const BicgVecs& v, BicgState* st, Red red, double tol, int maxit, int* tickets,
                      cudaStream_t s) {
  k_bicg_init0<<<kRedGrid, kRedTpb, 0, s>>>(v, st, red, tol, maxit);
  k_bicg_init1<<<kRedGrid, kRedTpb, 0, s>>>(v, st, tickets);
  return cudaGetLastError();
}
cudaError_t bicg_amp(const MatView& A, const BicgVecs& v, BicgState* st, Red red, cudaStream_t s) {
  DFG_BDISPATCH(k_bicg_amp, A, v, st, red);
  return cudaGetLastError();
}
cudaError_t bicg_s(const BicgVecs& v, BicgState* st, int* tickets, cudaStream_t s) {
  k_bicg_s<<<kRedGrid, kRedTpb, 0, s>>>(v, st, tickets);
  return cudaGetLastError();
}
cudaError_t bicg_ams(const MatView& A, const BicgVecs& v, BicgState* st, Red red2, cudaStream_t s) {
  DFG_BDISPATCH(k_bicg_ams, A, v, st, red2);
  return cudaGetLastError();
}
cudaError_t bicg_update(const BicgVecs& v, BicgState* st, Red red2, cudaStream_t s) {
  k_bicg_update<<<kRedGrid, kRedTpb, 0, s>>>(v, st, red2);
  return cudaGetLastError();
}
cudaError_t bicg_p(const BicgVecs& v, BicgState* st, int* tickets, cudaStream_t s) {
  k_bicg_p<<<kRedGrid, kRedTpb, 0, s>>>(v, st, tickets);
  return cudaGetLastError();
}

#undef DFG_BDISPATCH

}  // namespace dfg
