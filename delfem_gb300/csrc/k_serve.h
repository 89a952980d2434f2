// k_serve.h -- batched PCG kernels of the serving path: one launch works on
// every in-flight solve listed in a device-side slot table.
#pragma once
#include <cuda_runtime.h>

#include "k_solve.h"

namespace dfg {

constexpr int kSrvRows = 2048;      // block rows per chunk
constexpr int kSrvMaxSlots = 256;   // in-flight solves per server
constexpr int kSrvTpb = 256;        // threads per block of the batched kernels

// One in-flight solve.  Its rows are cut into chunks of kSrvRows; chunk k of
// the slot is chunk chunk0 + k of the launch's chunk space.  Reductions sum a
// slot's per-chunk partials in chunk order, so a slot's result does not
// depend on which other solves share the launch.
struct SrvSlot {
  int n, b;
  int chunk0, nchunks;
  const long long* sptr;  // FP64 matrix, sliced-ELL copy (SellMap layout)
  const int* swidth;
  const int* scol;
  const double* sval;
  const double* rhs;    // finalized right-hand side
  double* r;            // recursive residual
  double* x;            // solution
  double* p;
  double* q;            // A p
  double* rd;           // true residual b - A x
  void* y;              // forward-sweep output (sweep precision)
  void* z;              // backward-sweep output
  float* r32;           // FP32 sweep input (FP32 factor), else nullptr; the
                        // recursive residual itself in the mixed form
  PcgState* st;
  unsigned* cnt;        // reduction arrival counter (0 between launches)
  // mixed form (DFG_PREC_MIXED) only, else nullptr: FP32 sliced-ELL values,
  // FP32 direction and product, FP64 correction accumulated since the last
  // reliable update
  const float* sval32;
  float* p32;
  float* q32;
  double* d;
  // one-CTA-per-solve sweeps (k_solo.cu), else nullptr: the forward sweep's
  // input stored in its step order, rperm[posf[row]*b + c] = r[row*b + c]
  // (the sweep's element type: FP32 in the FP32 modes)
  const int* posf;
  void* rperm;
};

struct SrvTable {
  int nslots;
  int total_chunks;
  const unsigned char* chunk_slot;  // per chunk of the launch: its slot
  int chunk_start[kSrvMaxSlots + 1];
  SrvSlot slot[kSrvMaxSlots];
};
static_assert(kSrvMaxSlots <= 256, "chunk_slot holds a slot index in one byte");

// What the host reads after each replay, one entry per table slot.
struct SrvStatus {
  int done, iter_out, verified, nreplace;
  double conv;      // recursive sqrt(rr / rr0) at the stop
  double rel_true;  // ||b - A x|| / ||b|| at the last check (-1 if none)
};

// fp32z: sweep outputs y, z are float (FP32 factor); tickets: the batched
// sweep launches' counters, reset once the sweeps of an iteration are over.
// srv_rz_beta, srv_spmv_pap and srv_update_rx are two launches each: the
// batched kernel, then one block per slot for the slot's reduction.
cudaError_t srv_rz_beta(const SrvTable* T, double* partials, int* tickets, int ntickets, bool fp32z, int grid,
                        cudaStream_t s);
cudaError_t srv_update_p(const SrvTable* T, bool fp32z, int grid, cudaStream_t s);
cudaError_t srv_spmv_pap(const SrvTable* T, double* partials, int grid, cudaStream_t s);
cudaError_t srv_update_rx(const SrvTable* T, double* partials, bool fp32z, int grid, cudaStream_t s);
// for slots with a converged recursion not yet verified: rd = b - A x and the
// true residual check; failures are marked for replacement
cudaError_t srv_check_true(const SrvTable* T, double* partials, int grid, cudaStream_t s);
// slots marked for replacement continue from r = rd
cudaError_t srv_replace(const SrvTable* T, double* partials, bool fp32z, int grid, cudaStream_t s);
cudaError_t srv_collect(const SrvTable* T, SrvStatus* out, cudaStream_t s);

// admission: r = rhs, x = p = 0, sweep outputs = sentinel, r32 = r; then the
// state from rr0 = r.r (computed by the caller into *rr0)
cudaError_t srv_init_vectors(long long m, const double* rhs, double* r, double* x, double* p, void* y, void* z,
                             float* r32, bool fp32z, cudaStream_t s);
// delta2 > 0 (mixed form): a reliable update falls due once the recursive
// residual norm^2 drops below delta2 times its value at the last update
cudaError_t srv_init_state(PcgState* st, const double* rr0, double tol, int maxit, double delta2, cudaStream_t s);

// ---- the mixed form (DFG_PREC_MIXED): FP32 SpMV on FP32-stored values with
// FP32 accumulation, FP32 Krylov vectors r, p, q and preconditioned vectors;
// FP64 for the dot reductions (alpha, beta, r.r), the solution x += d and the
// reliable-update residual b - A x.  Each iteration: sweeps, srvm_rz_beta,
// srvm_update_p, srvm_spmv_pap, srvm_update_rx; each replay ends with
// srvm_fold and srvm_refine.
cudaError_t srvm_rz_beta(const SrvTable* T, double* partials, int* tickets, int ntickets, int grid, cudaStream_t s);
cudaError_t srvm_update_p(const SrvTable* T, int grid, cudaStream_t s);
cudaError_t srvm_spmv_pap(const SrvTable* T, double* partials, int grid, cudaStream_t s);
// r -= alpha q, d += alpha p, rr; the recursive stop (done = 5) and the
// reliable-update trigger (refine = 1)
cudaError_t srvm_update_rx(const SrvTable* T, double* partials, int grid, cudaStream_t s);
// slots due for a reliable update or stopped: x += d, d = 0
cudaError_t srvm_fold(const SrvTable* T, int grid, cudaStream_t s);
// slots due for a reliable update or stopped on the recursion: r = b - A x in
// FP64 (rounded to FP32 for the recursion) and the true-residual stop
cudaError_t srvm_refine(const SrvTable* T, double* partials, int grid, cudaStream_t s);
// admission of a solve with one-CTA-per-solve sweeps: its first forward
// input, rperm[posf[row]*b + c] = rhs[row*b + c] (fp32: as float)
cudaError_t srv_permute_rhs(const SrvSlot& s, bool fp32, cudaStream_t st);
// admission: x = d = p = 0, r = rhs (FP32), sweep outputs = sentinel
cudaError_t srvm_init_vectors(long long m, const double* rhs, double* x, double* d, float* r32, float* p32,
                              float* y, float* z, cudaStream_t s);

}  // namespace dfg
