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
// chunk publishes one partial (fixed block tree), and the slot's partials are
// summed in chunk order -- for the three reductions of every PCG iteration by
// a finishing launch (one block per slot), so that no fence or atomic stands
// between a block's chunks; for the rest by the slot's last arriving block.
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

// the batched kernels of every iteration are held to the registers of six
// blocks per SM and launched six blocks per SM, all resident in one wave:
// more rows in flight per SM (the SpMV and vector kernels are latency-bound
// at four blocks; 78.4 against 74.7 solves/s on the saturated 2D stream)
constexpr int kSrvVecBlocks = 6;

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

// This block's chunks (blockIdx.x, + gridDim.x, ...) with their slot index,
// the next chunk's index loaded one chunk ahead so that only the slot's
// fields and state stand between a chunk and its data.
struct ChunkWalk {
  const unsigned char* map;
  int nch, c, si_next;
  __device__ explicit ChunkWalk(const SrvTable* T) : map(T->chunk_slot), nch(T->total_chunks), c(blockIdx.x) {
    si_next = c < nch ? __ldg(map + c) : 0;
  }
  __device__ bool next(int& cc, int& si) {
    if (c >= nch) return false;
    cc = c;
    si = si_next;
    c += gridDim.x;
    si_next = c < nch ? __ldg(map + c) : 0;
    return true;
  }
};

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

// Publishes this chunk's partial (a fixed block tree) for the slot's total,
// which a separate launch takes (slot_total): no fence or atomic stands
// between a block's chunks.
__device__ __forceinline__ void publish(double v, int c, double* partials) {
  const double bs = block_sum(v);
  if (threadIdx.x == 0) partials[c] = bs;
}

// The slot's partials summed in chunk order, as the slot's last arriving
// block sums them in slot_sum: one block per slot.
__device__ __forceinline__ double slot_total(const SrvSlot& S, const double* partials) {
  double t = 0.0;
  for (int i = threadIdx.x; i < S.nchunks; i += kSrvTpb) t += partials[S.chunk0 + i];
  return block_sum(t);
}

// the slots a finishing launch works on: block s takes slot s while its
// solve runs (its state is read once, by every thread)
__device__ __forceinline__ bool live_slot(const SrvTable* T, int s) {
  return s < T->nslots && ld_relaxed_int(&T->slot[s].st->done) == 0;
}

template <typename Z>
__device__ __forceinline__ double zval(const void* z, long long k) {
  return (double)reinterpret_cast<const Z*>(z)[k];
}

// A new forward-sweep input value r of element k: in the sweep's step order
// for one-CTA-per-solve sweeps, else as the FP32 copy ranged FP32 sweeps read
// (FP64 ranged sweeps read r itself).
template <typename Z>
__device__ __forceinline__ void put_sweep_input(const SrvSlot& S, long long k, double r) {
  if (S.posf) {
    const long long row = k / S.b;
    reinterpret_cast<Z*>(S.rperm)[(long long)S.posf[row] * S.b + (k - row * S.b)] = (Z)r;
  } else if constexpr (sizeof(Z) == 4) {
    S.r32[k] = (float)r;
  }
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
__global__ void __launch_bounds__(kSrvTpb, kSrvVecBlocks) k_srv_rz_beta(const SrvTable* T, double* partials, int* tickets,
                                                         int ntickets) {
  if (blockIdx.x == 0 && threadIdx.x < ntickets) tickets[threadIdx.x] = 0;
  ChunkWalk w(T);
  for (int c, si; w.next(c, si);) {
    const SrvSlot S = T->slot[si];
    if (ld_relaxed_int(&S.st->done) != 0) continue;
    long long e0, e1;
    chunk_elems(S, c, e0, e1);
    double part = 0.0;
    #pragma unroll 4
    for (long long k = e0 + threadIdx.x; k < e1; k += kSrvTpb) part += S.r[k] * zval<Z>(S.z, k);
    publish(part, c, partials);
  }
}

__global__ void __launch_bounds__(kSrvTpb) k_srv_fin_rz_beta(const SrvTable* T, const double* partials) {
  if (!live_slot(T, blockIdx.x)) return;
  const SrvSlot& S = T->slot[blockIdx.x];
  const double tot = slot_total(S, partials);
  if (threadIdx.x == 0) {
    PcgState* st = S.st;
    st->beta = (st->it == 0) ? 0.0 : tot / st->rz;
    st->rz = tot;
  }
}

// p := z in the first iteration, else p := beta p + z (SCAL + AXPY)
template <typename Z>
__global__ void __launch_bounds__(kSrvTpb, kSrvVecBlocks) k_srv_update_p(const SrvTable* T) {
  ChunkWalk w(T);
  for (int c, si; w.next(c, si);) {
    const SrvSlot S = T->slot[si];
    if (ld_relaxed_int(&S.st->done) != 0) continue;
    long long e0, e1;
    chunk_elems(S, c, e0, e1);
    const bool first = S.st->it == 0;
    const double beta = S.st->beta;
    #pragma unroll 4
    for (long long k = e0 + threadIdx.x; k < e1; k += kSrvTpb)
      S.p[k] = first ? zval<Z>(S.z, k) : __dadd_rn(__dmul_rn(S.p[k], beta), zval<Z>(S.z, k));
  }
}

// q = A p; pAp; alpha = rz / pAp
__global__ void __launch_bounds__(kSrvTpb, kSrvVecBlocks) k_srv_spmv_pap(const SrvTable* T, double* partials) {
  ChunkWalk w(T);
  for (int c, si; w.next(c, si);) {
    const SrvSlot S = T->slot[si];
    if (ld_relaxed_int(&S.st->done) != 0) continue;
    int row0, row1;
    chunk_rows(S, c, row0, row1);
    const double part = S.b == 1 ? chunk_q_pap<1>(S, row0, row1)
                        : S.b == 2 ? chunk_q_pap<2>(S, row0, row1) : chunk_q_pap<3>(S, row0, row1);
    publish(part, c, partials);
  }
}

__global__ void __launch_bounds__(kSrvTpb) k_srv_fin_pap(const SrvTable* T, const double* partials) {
  if (!live_slot(T, blockIdx.x)) return;
  const SrvSlot& S = T->slot[blockIdx.x];
  const double tot = slot_total(S, partials);
  if (threadIdx.x == 0) {
    S.st->pap = tot;
    S.st->alpha = S.st->rz / tot;
  }
}

// r := r - alpha q; x := x + alpha p; rr = r.r; stop test; sweep outputs back
// to the sentinel; FP32 copy of r for FP32 sweeps
template <typename Z>
__global__ void __launch_bounds__(kSrvTpb, kSrvVecBlocks) k_srv_update_rx(const SrvTable* T, double* partials) {
  ChunkWalk w(T);
  for (int c, si; w.next(c, si);) {
    const SrvSlot S = T->slot[si];
    if (ld_relaxed_int(&S.st->done) != 0) continue;
    long long e0, e1;
    chunk_elems(S, c, e0, e1);
    const double alpha = S.st->alpha;
    double part = 0.0;
    #pragma unroll 4
    for (long long k = e0 + threadIdx.x; k < e1; k += kSrvTpb) {
      double r = S.r[k];
      if (alpha != 0.0) {
        r = __dadd_rn(r, __dmul_rn(-alpha, S.q[k]));
        S.r[k] = r;
        S.x[k] = __dadd_rn(S.x[k], __dmul_rn(alpha, S.p[k]));
      }
      part += r * r;
      if (!S.posf) {  // ranged sweeps hand values over through these sentinels
        reinterpret_cast<Z*>(S.y)[k] = sentinel_value<Z>();
        reinterpret_cast<Z*>(S.z)[k] = sentinel_value<Z>();
      }
      put_sweep_input<Z>(S, k, r);
    }
    publish(part, c, partials);
  }
}

__global__ void __launch_bounds__(kSrvTpb) k_srv_fin_rx(const SrvTable* T, const double* partials) {
  if (!live_slot(T, blockIdx.x)) return;
  const SrvSlot& S = T->slot[blockIdx.x];
  const double tot = slot_total(S, partials);
  if (threadIdx.x == 0) {
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

constexpr int kMaxReplace = 8;

// done == 1 and not yet verified: rd = b - A x, rr_true; verified when
// ||rd||^2 <= tol^2 ||b||^2, else marked for residual replacement (done = 6),
// or given up (done = 7) after kMaxReplace replacements
__global__ void __launch_bounds__(kSrvTpb) k_srv_check_true(const SrvTable* T, double* partials) {
  ChunkWalk w(T);
  for (int c, si; w.next(c, si);) {
    const SrvSlot S = T->slot[si];
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
__global__ void __launch_bounds__(kSrvTpb, kSrvVecBlocks) k_srv_replace(const SrvTable* T, double* partials) {
  ChunkWalk w(T);
  for (int c, si; w.next(c, si);) {
    const SrvSlot S = T->slot[si];
    if (ld_relaxed_int(&S.st->done) != 6) continue;
    long long e0, e1;
    chunk_elems(S, c, e0, e1);
    #pragma unroll 4
    for (long long k = e0 + threadIdx.x; k < e1; k += kSrvTpb) {
      const double r = S.rd[k];
      S.r[k] = r;
      put_sweep_input<Z>(S, k, r);
      if (!S.posf) {
        reinterpret_cast<Z*>(S.y)[k] = sentinel_value<Z>();
        reinterpret_cast<Z*>(S.z)[k] = sentinel_value<Z>();
      }
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

// ------------------------------------------------------------ mixed form
//
// The loop of the single-solve mixed form (dfg_solve_pcg_mixed) on every
// slot at once: FP32 recursion, FP64 reductions and correction, and reliable
// updates (the FP64 true residual replaces the FP32 recursive one, the
// search direction is kept) once the recursive residual has dropped by the
// factor delta since the last update, or below the tolerance.  Updates fall
// due inside a replay and are carried out at its end (srvm_fold,
// srvm_refine); the stop is decided on the FP64 true residual only.

__device__ __forceinline__ bool mixed_live(const PcgState* st) { return ld_relaxed_int(&st->done) == 0; }

// rz_new = r.z (FP64 accumulation of FP32 products); beta = rz_new / rz
__global__ void __launch_bounds__(kSrvTpb, kSrvVecBlocks) k_srvm_rz_beta(const SrvTable* T, double* partials, int* tickets,
                                                          int ntickets) {
  if (blockIdx.x == 0 && threadIdx.x < ntickets) tickets[threadIdx.x] = 0;
  ChunkWalk w(T);
  for (int c, si; w.next(c, si);) {
    const SrvSlot S = T->slot[si];
    if (!mixed_live(S.st)) continue;
    long long e0, e1;
    chunk_elems(S, c, e0, e1);
    const float* z = reinterpret_cast<const float*>(S.z);
    double part = 0.0;
    #pragma unroll 4
    for (long long k = e0 + threadIdx.x; k < e1; k += kSrvTpb) part += (double)S.r32[k] * (double)z[k];
    double tot;
    if (slot_sum(part, c, S, partials, &tot) && threadIdx.x == 0) {
      PcgState* st = S.st;
      st->beta = (st->it == 0) ? 0.0 : tot / st->rz;
      st->rz = tot;
    }
  }
}

// p := z in the first iteration, else p := z + beta p (FP32)
__global__ void __launch_bounds__(kSrvTpb, kSrvVecBlocks) k_srvm_update_p(const SrvTable* T) {
  ChunkWalk w(T);
  for (int c, si; w.next(c, si);) {
    const SrvSlot S = T->slot[si];
    if (!mixed_live(S.st)) continue;
    long long e0, e1;
    chunk_elems(S, c, e0, e1);
    const bool first = S.st->it == 0;
    const float beta = (float)S.st->beta;
    const float* z = reinterpret_cast<const float*>(S.z);
    #pragma unroll 4
    for (long long k = e0 + threadIdx.x; k < e1; k += kSrvTpb) S.p32[k] = first ? z[k] : z[k] + beta * S.p32[k];
  }
}

// q = A p on the FP32 values with FP32 accumulation; pAp in FP64; alpha
template <int B>
__device__ __forceinline__ double chunk_q_pap32(const SrvSlot& S, int row0, int row1) {
  double part = 0.0;
  for (int i = row0 + threadIdx.x; i < row1; i += kSrvTpb) {
    float y[B];
    sell_row_mv<float, B>(i, S.sptr, S.swidth, S.scol, S.sval32, S.p32, y);
#pragma unroll
    for (int d = 0; d < B; ++d) {
      S.q32[(size_t)i * B + d] = y[d];
      part += (double)S.p32[(size_t)i * B + d] * (double)y[d];
    }
  }
  return part;
}

__global__ void __launch_bounds__(kSrvTpb) k_srvm_spmv_pap(const SrvTable* T, double* partials) {
  ChunkWalk w(T);
  for (int c, si; w.next(c, si);) {
    const SrvSlot S = T->slot[si];
    if (!mixed_live(S.st)) continue;
    int row0, row1;
    chunk_rows(S, c, row0, row1);
    const double part = S.b == 1 ? chunk_q_pap32<1>(S, row0, row1)
                        : S.b == 2 ? chunk_q_pap32<2>(S, row0, row1) : chunk_q_pap32<3>(S, row0, row1);
    double tot;
    if (slot_sum(part, c, S, partials, &tot) && threadIdx.x == 0) {
      S.st->pap = tot;
      S.st->alpha = S.st->rz / tot;
    }
  }
}

// r := r - alpha q (FP32); d := d + alpha p (FP64); rr = r.r (FP64); the
// recursive stop (done 5: the true residual decides at the end of the replay),
// the reliable-update trigger, the iteration limit; sweep outputs back to the
// sentinel
__global__ void __launch_bounds__(kSrvTpb, kSrvVecBlocks) k_srvm_update_rx(const SrvTable* T, double* partials) {
  ChunkWalk w(T);
  for (int c, si; w.next(c, si);) {
    const SrvSlot S = T->slot[si];
    if (!mixed_live(S.st)) continue;
    long long e0, e1;
    chunk_elems(S, c, e0, e1);
    const double alpha = S.st->alpha;
    const float alpha32 = (float)alpha;
    float* y = reinterpret_cast<float*>(S.y);
    float* z = reinterpret_cast<float*>(S.z);
    double part = 0.0;
    #pragma unroll 4
    for (long long k = e0 + threadIdx.x; k < e1; k += kSrvTpb) {
      float r = S.r32[k];
      if (alpha != 0.0) {
        r = r - alpha32 * S.q32[k];
        S.r32[k] = r;
        S.d[k] = S.d[k] + alpha * (double)S.p32[k];
        if (S.posf) put_sweep_input<float>(S, k, r);
      }
      part += (double)r * (double)r;
      if (!S.posf) {
        y[k] = sentinel_value<float>();
        z[k] = sentinel_value<float>();
      }
    }
    double tot;
    if (slot_sum(part, c, S, partials, &tot) && threadIdx.x == 0) {
      PcgState* st = S.st;
      st->rr = tot;
      st->iter_out = st->it;
      if (!(tot == tot)) {
        st->done = 3;
      } else if (tot * st->inv_rr0 < st->tol2) {
        st->done = 5;
      } else {
        if (tot < st->delta2 * st->rr_ref) st->refine = 1;
        if (st->it + 1 >= st->maxit) {
          st->done = 2;
          st->iter_out = st->maxit;
        }
      }
      st->conv = sqrt(tot * st->inv_rr0);
      st->it += 1;
    }
  }
}

__device__ __forceinline__ bool mixed_due(const PcgState* st) {
  const int dn = ld_relaxed_int(&st->done);
  return dn == 5 || (dn == 0 && ld_relaxed_int(&st->refine) != 0);
}

// x := x + d, d := 0 for slots due for a reliable update, stopped, or at
// the end (limit, NaN)
__global__ void __launch_bounds__(kSrvTpb, kSrvVecBlocks) k_srvm_fold(const SrvTable* T) {
  ChunkWalk w(T);
  for (int c, si; w.next(c, si);) {
    const SrvSlot S = T->slot[si];
    const int dn = ld_relaxed_int(&S.st->done);
    if (!(mixed_due(S.st) || dn == 2 || dn == 3)) continue;
    long long e0, e1;
    chunk_elems(S, c, e0, e1);
    #pragma unroll 4
    for (long long k = e0 + threadIdx.x; k < e1; k += kSrvTpb) {
      S.x[k] = S.x[k] + S.d[k];
      S.d[k] = 0.0;
    }
  }
}

// rd = b - A x with the FP64 values; r := rd (FP32); true-residual stop:
// converged and verified, or the recursion continues from rd
template <int B>
__device__ __forceinline__ double chunk_refine(const SrvSlot& S, int row0, int row1) {
  double part = 0.0;
  for (int i = row0 + threadIdx.x; i < row1; i += kSrvTpb) {
    double y[B];
    sell_row_mv<double, B>(i, S.sptr, S.swidth, S.scol, S.sval, S.x, y);
#pragma unroll
    for (int d = 0; d < B; ++d) {
      const double rv = S.rhs[(size_t)i * B + d] - y[d];
      S.r32[(size_t)i * B + d] = (float)rv;
      if (S.posf) reinterpret_cast<float*>(S.rperm)[(size_t)S.posf[i] * B + d] = (float)rv;
      part += rv * rv;
    }
  }
  return part;
}

__global__ void __launch_bounds__(kSrvTpb) k_srvm_refine(const SrvTable* T, double* partials) {
  ChunkWalk w(T);
  for (int c, si; w.next(c, si);) {
    const SrvSlot S = T->slot[si];
    if (!mixed_due(S.st)) continue;
    int row0, row1;
    chunk_rows(S, c, row0, row1);
    const double part = S.b == 1 ? chunk_refine<1>(S, row0, row1)
                        : S.b == 2 ? chunk_refine<2>(S, row0, row1) : chunk_refine<3>(S, row0, row1);
    double tot;
    if (slot_sum(part, c, S, partials, &tot) && threadIdx.x == 0) {
      PcgState* st = S.st;
      st->rr_true = tot;
      st->refine = 0;
      st->nreplace += 1;
      if (tot * st->inv_rr0 <= st->tol2) {
        st->done = 1;
        st->verified = 1;
      } else if (!(tot == tot)) {
        st->done = 3;
      } else if (st->it >= st->maxit) {
        st->done = 2;
        st->iter_out = st->maxit;
      } else {
        st->rr_ref = tot;
        st->done = 0;
      }
    }
  }
}

__global__ void k_srvm_init_vectors(long long m, const double* rhs, double* x, double* d, float* r32, float* p32,
                                    float* y, float* z) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < m; k += (long long)gridDim.x * blockDim.x) {
    x[k] = 0.0;
    d[k] = 0.0;
    r32[k] = (float)rhs[k];
    p32[k] = 0.0f;
    y[k] = sentinel_value<float>();
    z[k] = sentinel_value<float>();
  }
}

__global__ void k_srv_init_state(PcgState* st, const double* rr0p, double tol, int maxit, double delta2) {
  const double rr0 = *rr0p;
  PcgState s{};
  s.rr0 = rr0;
  s.rr_ref = rr0;
  s.delta2 = delta2;
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
  k_srv_fin_rz_beta<<<kSrvMaxSlots, kSrvTpb, 0, s>>>(T, partials);
  return cudaGetLastError();
}
cudaError_t srv_update_p(const SrvTable* T, bool fp32z, int grid, cudaStream_t s) {
  if (fp32z) k_srv_update_p<float><<<grid, kSrvTpb, 0, s>>>(T);
  else k_srv_update_p<double><<<grid, kSrvTpb, 0, s>>>(T);
  return cudaGetLastError();
}
cudaError_t srv_spmv_pap(const SrvTable* T, double* partials, int grid, cudaStream_t s) {
  k_srv_spmv_pap<<<grid, kSrvTpb, 0, s>>>(T, partials);
  k_srv_fin_pap<<<kSrvMaxSlots, kSrvTpb, 0, s>>>(T, partials);
  return cudaGetLastError();
}
cudaError_t srv_update_rx(const SrvTable* T, double* partials, bool fp32z, int grid, cudaStream_t s) {
  if (fp32z) k_srv_update_rx<float><<<grid, kSrvTpb, 0, s>>>(T, partials);
  else k_srv_update_rx<double><<<grid, kSrvTpb, 0, s>>>(T, partials);
  k_srv_fin_rx<<<kSrvMaxSlots, kSrvTpb, 0, s>>>(T, partials);
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
cudaError_t srv_init_state(PcgState* st, const double* rr0, double tol, int maxit, double delta2, cudaStream_t s) {
  k_srv_init_state<<<1, 1, 0, s>>>(st, rr0, tol, maxit, delta2);
  return cudaGetLastError();
}
cudaError_t srvm_rz_beta(const SrvTable* T, double* partials, int* tickets, int ntickets, int grid, cudaStream_t s) {
  k_srvm_rz_beta<<<grid, kSrvTpb, 0, s>>>(T, partials, tickets, ntickets);
  return cudaGetLastError();
}
cudaError_t srvm_update_p(const SrvTable* T, int grid, cudaStream_t s) {
  k_srvm_update_p<<<grid, kSrvTpb, 0, s>>>(T);
  return cudaGetLastError();
}
cudaError_t srvm_spmv_pap(const SrvTable* T, double* partials, int grid, cudaStream_t s) {
  k_srvm_spmv_pap<<<grid, kSrvTpb, 0, s>>>(T, partials);
  return cudaGetLastError();
}
cudaError_t srvm_update_rx(const SrvTable* T, double* partials, int grid, cudaStream_t s) {
  k_srvm_update_rx<<<grid, kSrvTpb, 0, s>>>(T, partials);
  return cudaGetLastError();
}
cudaError_t srvm_fold(const SrvTable* T, int grid, cudaStream_t s) {
  k_srvm_fold<<<grid, kSrvTpb, 0, s>>>(T);
  return cudaGetLastError();
}
cudaError_t srvm_refine(const SrvTable* T, double* partials, int grid, cudaStream_t s) {
  k_srvm_refine<<<grid, kSrvTpb, 0, s>>>(T, partials);
  return cudaGetLastError();
}
template <typename Z>
__global__ void k_srv_permute_rhs(long long m, int b, const double* rhs, const int* posf, Z* rperm) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < m; k += (long long)gridDim.x * blockDim.x) {
    const long long row = k / b;
    rperm[(long long)posf[row] * b + (k - row * b)] = (Z)rhs[k];
  }
}

cudaError_t srv_permute_rhs(const SrvSlot& s, bool fp32, cudaStream_t st) {
  const long long m = (long long)s.n * s.b;
  if (m == 0 || !s.posf) return cudaSuccess;
  const int grid = (int)std::min<long long>((m + 255) / 256, 1216);
  if (fp32) k_srv_permute_rhs<float><<<grid, 256, 0, st>>>(m, s.b, s.rhs, s.posf, static_cast<float*>(s.rperm));
  else k_srv_permute_rhs<double><<<grid, 256, 0, st>>>(m, s.b, s.rhs, s.posf, static_cast<double*>(s.rperm));
  return cudaGetLastError();
}

cudaError_t srvm_init_vectors(long long m, const double* rhs, double* x, double* d, float* r32, float* p32,
                              float* y, float* z, cudaStream_t s) {
  if (m == 0) return cudaSuccess;
  const int grid = (int)std::min<long long>((m + 255) / 256, 1216);
  k_srvm_init_vectors<<<grid, 256, 0, s>>>(m, rhs, x, d, r32, p32, y, z);
  return cudaGetLastError();
}

}  // namespace dfg
