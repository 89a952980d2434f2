// k_serve.cu -- the PCG iteration of many independent solves in one set of
// launches (the serving path).
//
// Each launch walks a global chunk space: chunk c belongs to the slot s with
// chunk_start[s] <= c < chunk_start[s+1] and covers kSrvRows block rows of
// it (vector kernels: a thread per element; products: a thread per block
// row over the slot's sliced-ELL matrix).  Blocks loop over chunks (fixed grid), so a launch's shape does not
// depend on the slots in flight and one captured graph serves every mix.
// A slot whose state says `done` is skipped.
//
// Per-slot reductions are deterministic and independent of the mix: each
// chunk publishes one partial (fixed block tree), and the last chunk of the
// slot to arrive sums the slot's partials in chunk order.
//
// The iteration follows LsSol::Solve_PCG (src/ls/solver_ls_iter.cpp:100-172)
// with the first iteration folded into the common body (beta = 0, p = z).
#include <algorithm>
#include <cmath>

#include "dfg_common.cuh"
#include "k_rowmv.cuh"
#include "k_serve.h"

static_assert(dfg::kSrvTpb <= 1024 && dfg::kSrvTpb % 32 == 0, "batched kernels: block size");

namespace dfg {

namespace {

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ double block_sum(double v) {
  __shared__ double ws[kSrvTpb / 32];
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) ws[w] = v;
  __syncthreads();
  double t = (threadIdx.x < kSrvTpb / 32) ? ws[threadIdx.x] : 0.0;
  if (w == 0) t = warp_sum(t);
  __syncthreads();
  if (threadIdx.x == 0) ws[0] = t;
  __syncthreads();
  return ws[0];
}

__device__ __forceinline__ int find_slot(const SrvTable* T, int c) {
  int lo = 0, hi = T->nslots - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (T->chunk_start[mid] <= c) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Publishes this chunk's partial; true (block-uniform) in the slot's last
// arriving block, which then holds the slot total in *tot.
__device__ bool slot_sum(double v, int c, const SrvSlot& S, double* partials, double* tot) {
  __shared__ bool last;
  const double bs = block_sum(v);
  if (threadIdx.x == 0) {
    partials[c] = bs;
    __threadfence();
    last = (atomicAdd(S.cnt, 1u) == (unsigned)S.nchunks - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double t = 0.0;
  for (int i = threadIdx.x; i < S.nchunks; i += kSrvTpb) t += ld_relaxed(&partials[S.chunk0 + i]);
  t = block_sum(t);
  if (threadIdx.x == 0) *S.cnt = 0u;
  *tot = t;
  return true;
}

template <typename Z>
__device__ __forceinline__ double zval(const void* z, long long k) {
  return (double)reinterpret_cast<const Z*>(z)[k];
}

// element range [e0, e1) of chunk c of slot S
__device__ __forceinline__ void chunk_elems(const SrvSlot& S, int c, long long& e0, long long& e1) {
  const long long row0 = (long long)(c - S.chunk0) * kSrvRows;
  const long long row1 = min(row0 + kSrvRows, (long long)S.n);
  e0 = row0 * S.b;
  e1 = row1 * S.b;
}

// q = A p over rows [row0, row1) of one chunk (thread per row, sliced ELL);
// returns this thread's share of p.q
template <int B>
__device__ __forceinline__ double chunk_q_pap(const SrvSlot& S, int row0, int row1) {
  double part = 0.0;
  for (int i = row0 + threadIdx.x; i < row1; i += kSrvTpb) {
    double y[B];
    sell_row_mv<double, B>(i, S.sptr, S.swidth, S.scol, S.sval, S.p, y);
#pragma unroll
    for (int d = 0; d < B; ++d) {
      S.q[(size_t)i * B + d] = y[d];
      part += S.p[(size_t)i * B + d] * y[d];
    }
  }
  return part;
}

// rd = b - A x over one chunk; returns this thread's share of rd.rd
template <int B>
__device__ __forceinline__ double chunk_true_res(const SrvSlot& S, int row0, int row1) {
  double part = 0.0;
  for (int i = row0 + threadIdx.x; i < row1; i += kSrvTpb) {
    double y[B];
    sell_row_mv<double, B>(i, S.sptr, S.swidth, S.scol, S.sval, S.x, y);
#pragma unroll
    for (int d = 0; d < B; ++d) {
      const double rv = S.rhs[(size_t)i * B + d] - y[d];
      S.rd[(size_t)i * B + d] = rv;
      part += rv * rv;
    }
  }
  return part;
}

__device__ __forceinline__ void chunk_rows(const SrvSlot& S, int c, int& row0, int& row1) {
  row0 = (c - S.chunk0) * kSrvRows;
  row1 = min(row0 + kSrvRows, S.n);
}

// rz_new = r.z; beta = rz_new / rz (0 in the first iteration)
template <typename Z>
__global__ void __launch_bounds__(kSrvTpb) k_srv_rz_beta(const SrvTable* T, double* partials, int* tickets,
                                                         int ntickets) {
  if (blockIdx.x == 0 && threadIdx.x < ntickets) tickets[threadIdx.x] = 0;
  const int nch = T->total_chunks;
  for (int c = blockIdx.x; c < nch; c += gridDim.x) {
    const SrvSlot S = T->slot[find_slot(T, c)];
    if (ld_relaxed_int(&S.st->done) != 0) continue;
    long long e0, e1;
    chunk_elems(S, c, e0, e1);
    double part = 0.0;
    for (long long k = e0 + threadIdx.x; k < e1; k += kSrvTpb) part += S.r[k] * zval<Z>(S.z, k);
    double tot;
    if (slot_sum(part, c, S, partials, &tot) && threadIdx.x == 0) {
      PcgState* st = S.st;
      st->beta = (st->it == 0) ? 0.0 : tot / st->rz;
      st->rz = tot;
    }
  }
}

// p := z in the first iteration, else p := beta p + z (SCAL + AXPY)
template <typename Z>
__global__ void __launch_bounds__(kSrvTpb) k_srv_update_p(const SrvTable* T) {
  const int nch = T->total_chunks;
  for (int c = blockIdx.x; c < nch; c += gridDim.x) {
    const SrvSlot S = T->slot[find_slot(T, c)];
    if (ld_relaxed_int(&S.st->done) != 0) continue;
    long long e0, e1;
    chunk_elems(S, c, e0, e1);
    const bool first = S.st->it == 0;
    const double beta = S.st->beta;
    for (long long k = e0 + threadIdx.x; k < e1; k += kSrvTpb)
      S.p[k] = first ? zval<Z>(S.z, k) : __dadd_rn(__dmul_rn(S.p[k], beta), zval<Z>(S.z, k));
  }
}

// q = A p; pAp; alpha = rz / pAp
__global__ void __launch_bounds__(kSrvTpb) k_srv_spmv_pap(const SrvTable* T, double* partials) {
  const int nch = T->total_chunks;
  for (int c = blockIdx.x; c < nch; c += gridDim.x) {
    const SrvSlot S = T->slot[find_slot(T, c)];
    if (ld_relaxed_int(&S.st->done) != 0) continue;
    int row0, row1;
    chunk_rows(S, c, row0, row1);
    const double part = S.b == 1 ? chunk_q_pap<1>(S, row0, row1)
                        : S.b == 2 ? chunk_q_pap<2>(S, row0, row1) : chunk_q_pap<3>(S, row0, row1);
    double tot;
    if (slot_sum(part, c, S, partials, &tot) && threadIdx.x == 0) {
      S.st->pap = tot;
      S.st->alpha = S.st->rz / tot;
    }
  }
}

// r := r - alpha q; x := x + alpha p; rr = r.r; stop test; sweep outputs back
// to the sentinel; FP32 copy of r for FP32 sweeps
template <typename Z>
__global__ void __launch_bounds__(kSrvTpb) k_srv_update_rx(const SrvTable* T, double* partials) {
  const int nch = T->total_chunks;
  for (int c = blockIdx.x; c < nch; c += gridDim.x) {
    const SrvSlot S = T->slot[find_slot(T, c)];
    if (ld_relaxed_int(&S.st->done) != 0) continue;
    long long e0, e1;
    chunk_elems(S, c, e0, e1);
    const double alpha = S.st->alpha;
    double part = 0.0;
    for (long long k = e0 + threadIdx.x; k < e1; k += kSrvTpb) {
      double r = S.r[k];
      if (alpha != 0.0) {
        r = __dadd_rn(r, __dmul_rn(-alpha, S.q[k]));
        S.r[k] = r;
        S.x[k] = __dadd_rn(S.x[k], __dmul_rn(alpha, S.p[k]));
      }
      part += r * r;
      reinterpret_cast<Z*>(S.y)[k] = sentinel_value<Z>();
      reinterpret_cast<Z*>(S.z)[k] = sentinel_value<Z>();
      if constexpr (sizeof(Z) == 4) S.r32[k] = (float)r;
    }
    double tot;
    if (slot_sum(part, c, S, partials, &tot) && threadIdx.x == 0) {
      PcgState* st = S.st;
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
        st->done = 3;
        st->conv = ratio;
        st->iter_out = st->it;
      }
      st->it += 1;
    }
  }
}

constexpr int kMaxReplace = 8;

// done == 1 and not yet verified: rd = b - A x, rr_true; verified when
// ||rd||^2 <= tol^2 ||b||^2, else marked for residual replacement (done = 6),
// or given up (done = 7) after kMaxReplace replacements
__global__ void __launch_bounds__(kSrvTpb) k_srv_check_true(const SrvTable* T, double* partials) {
  const int nch = T->total_chunks;
  for (int c = blockIdx.x; c < nch; c += gridDim.x) {
    const SrvSlot S = T->slot[find_slot(T, c)];
    if (ld_relaxed_int(&S.st->done) != 1 || ld_relaxed_int(&S.st->verified) != 0) continue;
    int row0, row1;
    chunk_rows(S, c, row0, row1);
    const double part = S.b == 1 ? chunk_true_res<1>(S, row0, row1)
                        : S.b == 2 ? chunk_true_res<2>(S, row0, row1) : chunk_true_res<3>(S, row0, row1);
    double tot;
    if (slot_sum(part, c, S, partials, &tot) && threadIdx.x == 0) {
      PcgState* st = S.st;
      st->rr_true = tot;
      if (tot * st->inv_rr0 <= st->tol2) st->verified = 1;
      else st->done = (st->nreplace >= kMaxReplace) ? 7 : 6;
    }
  }
}

// done == 6: r := rd and the recursion continues (residual replacement)
template <typename Z>
__global__ void __launch_bounds__(kSrvTpb) k_srv_replace(const SrvTable* T, double* partials) {
  const int nch = T->total_chunks;
  for (int c = blockIdx.x; c < nch; c += gridDim.x) {
    const SrvSlot S = T->slot[find_slot(T, c)];
    if (ld_relaxed_int(&S.st->done) != 6) continue;
    long long e0, e1;
    chunk_elems(S, c, e0, e1);
    for (long long k = e0 + threadIdx.x; k < e1; k += kSrvTpb) {
      const double r = S.rd[k];
      S.r[k] = r;
      if constexpr (sizeof(Z) == 4) S.r32[k] = (float)r;
      reinterpret_cast<Z*>(S.y)[k] = sentinel_value<Z>();
      reinterpret_cast<Z*>(S.z)[k] = sentinel_value<Z>();
    }
    double tot;
    if (slot_sum(0.0, c, S, partials, &tot) && threadIdx.x == 0) {
      S.st->nreplace += 1;
      S.st->done = 0;
    }
  }
}

__global__ void k_srv_collect(const SrvTable* T, SrvStatus* out) {
  for (int s = threadIdx.x; s < T->nslots; s += blockDim.x) {
    const PcgState* st = T->slot[s].st;
    SrvStatus o;
    o.done = st->done;
    o.iter_out = st->iter_out;
    o.verified = st->verified;
    o.nreplace = st->nreplace;
    o.conv = st->conv;
    o.rel_true = st->verified ? sqrt(st->rr_true * st->inv_rr0) : -1.0;
    out[s] = o;
  }
}

template <typename Z>
__global__ void k_srv_init_vectors(long long m, const double* rhs, double* r, double* x, double* p, Z* y, Z* z,
                                   float* r32) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < m; k += (long long)gridDim.x * blockDim.x) {
    const double v = rhs[k];
    r[k] = v;
    x[k] = 0.0;
    p[k] = 0.0;
    y[k] = sentinel_value<Z>();
    z[k] = sentinel_value<Z>();
    if constexpr (sizeof(Z) == 4) r32[k] = (float)v;
  }
}

__global__ void k_srv_init_state(PcgState* st, const double* rr0p, double tol, int maxit) {
  const double rr0 = *rr0p;
  PcgState s{};
  s.rr0 = rr0;
  s.tol2 = tol * tol;
  s.maxit = maxit;
  if (rr0 < 1.0e-30) {  // Solve_PCG returns at once; x = 0
    s.done = 1;
    s.verified = 1;
    s.conv = 0.0;
    s.inv_rr0 = 0.0;
  } else {
    s.done = (maxit <= 0) ? 2 : 0;
    s.inv_rr0 = 1.0 / rr0;
    s.conv = 1.0;
  }
  *st = s;
}

}  // namespace

// ------------------------------------------------------------------ launchers

cudaError_t srv_rz_beta(const SrvTable* T, double* partials, int* tickets, int ntickets, bool fp32z, int grid,
                        cudaStream_t s) {
  if (fp32z) k_srv_rz_beta<float><<<grid, kSrvTpb, 0, s>>>(T, partials, tickets, ntickets);
  else k_srv_rz_beta<double><<<grid, kSrvTpb, 0, s>>>(T, partials, tickets, ntickets);
  return cudaGetLastError();
}
cudaError_t srv_update_p(const SrvTable* T, bool fp32z, int grid, cudaStream_t s) {
  if (fp32z) k_srv_update_p<float><<<grid, kSrvTpb, 0, s>>>(T);
  else k_srv_update_p<double><<<grid, kSrvTpb, 0, s>>>(T);
  return cudaGetLastError();
}
cudaError_t srv_spmv_pap(const SrvTable* T, double* partials, int grid, cudaStream_t s) {
  k_srv_spmv_pap<<<grid, kSrvTpb, 0, s>>>(T, partials);
  return cudaGetLastError();
}
cudaError_t srv_update_rx(const SrvTable* T, double* partials, bool fp32z, int grid, cudaStream_t s) {
  if (fp32z) k_srv_update_rx<float><<<grid, kSrvTpb, 0, s>>>(T, partials);
  else k_srv_update_rx<double><<<grid, kSrvTpb, 0, s>>>(T, partials);
  return cudaGetLastError();
}
cudaError_t srv_check_true(const SrvTable* T, double* partials, int grid, cudaStream_t s) {
  k_srv_check_true<<<grid, kSrvTpb, 0, s>>>(T, partials);
  return cudaGetLastError();
}
cudaError_t srv_replace(const SrvTable* T, double* partials, bool fp32z, int grid, cudaStream_t s) {
  if (fp32z) k_srv_replace<float><<<grid, kSrvTpb, 0, s>>>(T, partials);
  else k_srv_replace<double><<<grid, kSrvTpb, 0, s>>>(T, partials);
  return cudaGetLastError();
}
cudaError_t srv_collect(const SrvTable* T, SrvStatus* out, cudaStream_t s) {
  k_srv_collect<<<1, 256, 0, s>>>(T, out);
  return cudaGetLastError();
}
cudaError_t srv_init_vectors(long long m, const double* rhs, double* r, double* x, double* p, void* y, void* z,
                             float* r32, bool fp32z, cudaStream_t s) {
  const int grid = (int)std::min<long long>((m + 255) / 256, 1216);
  if (m == 0) return cudaSuccess;
  if (fp32z) k_srv_init_vectors<float><<<grid, 256, 0, s>>>(m, rhs, r, x, p, (float*)y, (float*)z, r32);
  else k_srv_init_vectors<double><<<grid, 256, 0, s>>>(m, rhs, r, x, p, (double*)y, (double*)z, r32);
  return cudaGetLastError();
}
cudaError_t srv_init_state(PcgState* st, const double* rr0, double tol, int maxit, cudaStream_t s) {
  k_srv_init_state<<<1, 1, 0, s>>>(st, rr0, tol, maxit);
  return cudaGetLastError();
}

}  // namespace dfg
