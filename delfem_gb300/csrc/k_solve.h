// k_solve.h -- launch interface of the SpMV / BLAS-1 / PCG kernels.
#pragma once
#include <cuda_runtime.h>

namespace dfg {

// device-resident Krylov state (one per solve)
struct PcgState {
  double rz, alpha, beta, rr, inv_rr0, tol2, conv, rr0;
  double pap;
  double rr_ref;   // mixed: recursive residual norm^2 at the last reliable update
  double delta2;   // mixed: reliable update once rr < delta2 * rr_ref
  double tolb2;    // mixed: tol^2 * ||b||^2
  double rr_true;  // serving: ||b - A x||^2 at the last check
  int it, maxit, done, iter_out;
  int verified;    // serving: the true residual met the tolerance
  int nreplace;    // serving: residual replacements so far
  int refine;      // serving, mixed: a reliable update is due at the end of the replay
  int pad;
};
// done codes: 0 running, 1 converged, 2 iteration limit, 3 NaN,
//             4 reliable update due (mixed), 5 recursive residual below tol (mixed)

// deterministic reductions: fixed grid, per-block partials, the last block
// to finish sums the partials in index order
struct Red {
  double* partials;     // >= kRedGrid
  unsigned* counter;    // one counter per concurrent reduction channel
  double* result;       // where the finished sum goes (may be nullptr)
};
constexpr int kRedGrid = 304;   // 2 x 152 SMs
constexpr int kRedTpb = 256;
constexpr int kSpmvTpb = 512;   // SpMV blocks: 16 warps, two blocks per SM at the reduction grid

struct MatView {
  int n, b;
  const int* rowptr;
  const int* colind;
  const void* diag;   // double or float
  const void* offd;
  // sliced-ELL copy of the same matrix (SellMap layout), used by the PCG
  // products; values of the same type as diag/offd
  const long long* sptr;
  const int* swidth;
  const int* scol;
  const void* sval;
};

// Packs a block matrix (reference layout) into its sliced-ELL value array,
// converting to FP32 when fp32 is set.
cudaError_t sell_pack(int nslices, int b, const long long* ptr, const int* src, const double* diag,
                      const double* offd, void* out, bool fp32, cudaStream_t s);

// ---- FP64 PCG (plain path) -------------------------------------------------
struct PcgVecs {
  double* r;   // residual slot
  double* x;   // update slot
  double* p;
  double* q;   // A p
  void* y;     // forward-sweep output (double, or float with an FP32 factor)
  void* z;     // backward-sweep output (preconditioned residual)
  long long m; // n*b
  float* r32;  // FP32 copy of r fed to FP32 sweeps (nullptr with an FP64 factor)
  double* rd;  // true-residual scratch (b - A x)
  const double* b;  // finalized right-hand side (true-residual checks)
};
// fp32z: the preconditioned vectors y, z are float (FP32 factor and sweeps)
cudaError_t pcg_init(const PcgVecs& v, PcgState* st, Red red, double tol, int maxit, int* tickets, bool fp32z, cudaStream_t s);
cudaError_t pcg_after_precond0(const PcgVecs& v, PcgState* st, Red red, bool fp32z, cudaStream_t s);
// dep (the four iteration kernels): launch as a programmatic dependent of the
// previous kernel in the stream, which must be a kernel (a graph's chain)
cudaError_t pcg_spmv_pap(const MatView& A, const PcgVecs& v, PcgState* st, Red red, cudaStream_t s, bool dep = false);
cudaError_t pcg_update_rx(const PcgVecs& v, PcgState* st, Red red, int* tickets, bool fp32z, cudaStream_t s,
                          bool dep = false);
cudaError_t pcg_rz_beta(const PcgVecs& v, PcgState* st, Red red, bool fp32z, cudaStream_t s, bool dep = false);
cudaError_t pcg_update_p(const PcgVecs& v, PcgState* st, bool fp32z, cudaStream_t s, bool dep = false);
// rd = b - A x, rr = rd.rd (into st->rr; state otherwise untouched)
cudaError_t pcg_true_residual(const MatView& A, const PcgVecs& v, PcgState* st, Red red, cudaStream_t s);
// r = rd (and r32), sentinels, tickets reset, done = 0: continue from the true residual
cudaError_t pcg_replace(const PcgVecs& v, PcgState* st, int* tickets, bool fp32z, cudaStream_t s);

// ---- mixed precision ----------------------------------------------------
struct MixVecs {
  double* b;       // right-hand side (FP64)
  double* x;       // solution (FP64)
  double* rd;      // FP64 true residual b - A x at the last reliable update
  double* d;       // FP64 correction accumulated since the last reliable update
  float* r;        // inner residual
  float* p;
  float* q;
  float* y;
  float* z;
  long long m;
};
// rd = b - A64 x; rr = rd.rd (FP64)
cudaError_t mix_true_residual(const MatView& A64, const MixVecs& v, PcgState* st, Red red, cudaStream_t s);
// r32 = rd; rr_ref = rr; done = 0; sweep outputs refilled; tickets reset
cudaError_t mix_replace(const MixVecs& v, PcgState* st, int* tickets, cudaStream_t s);
// first call: state reset for a solve (tolerance, limits)
cudaError_t mix_start(PcgState* st, double tol, double bb, double delta, int maxit, cudaStream_t s);
cudaError_t mix_after_precond0(const MixVecs& v, PcgState* st, Red red, cudaStream_t s);
cudaError_t mix_spmv_pap(const MatView& A32, const MixVecs& v, PcgState* st, Red red, cudaStream_t s);
cudaError_t mix_update_rx(const MixVecs& v, PcgState* st, Red red, int* tickets, cudaStream_t s);
cudaError_t mix_rz_beta(const MixVecs& v, PcgState* st, Red red, cudaStream_t s);
cudaError_t mix_update_p(const MixVecs& v, PcgState* st, cudaStream_t s);
// x += d; d = 0
cudaError_t mix_accumulate(const MixVecs& v, cudaStream_t s);
cudaError_t mix_clear_done(PcgState* st, cudaStream_t s);
cudaError_t to_fp32(long long m, const double* a, float* b, cudaStream_t s);

// ---- preconditioned BiCGSTAB (k_bicg.cu) ----------------------------------
struct BicgState {
  double rho;            // (r, r2) of the current iteration
  double alpha, omega, beta;
  double rr, rr0, inv_rr0, tol2, conv;
  int it;                // current iteration, 1-based as the reference counts
  int maxit, done, iter_out;
};
// done codes: 0 running, 1 converged, 2 iteration limit, 3 NaN,
//             4 residual below 1e-60 at the start (nothing touched)
struct BicgVecs {
  double* r;   // residual slot
  double* x;   // update slot
  double* r2;  // shadow residual (the initial r)
  double* p;
  double* amp; // A M^-1 p
  double* s;
  double* ams; // A M^-1 s
  double* mp;  // M^-1 p
  double* ms;  // M^-1 s
  double* y;   // forward-sweep output
  long long m;
};
// red2: partials for 2 x kRedGrid values and its own counter
cudaError_t bicg_init(const BicgVecs& v, BicgState* st, Red red, double tol, int maxit, int* tickets, cudaStream_t s);
cudaError_t bicg_amp(const MatView& A, const BicgVecs& v, BicgState* st, Red red, cudaStream_t s);
cudaError_t bicg_s(const BicgVecs& v, BicgState* st, int* tickets, cudaStream_t s);
cudaError_t bicg_ams(const MatView& A, const BicgVecs& v, BicgState* st, Red red2, cudaStream_t s);
cudaError_t bicg_update(const BicgVecs& v, BicgState* st, Red red2, cudaStream_t s);
cudaError_t bicg_p(const BicgVecs& v, BicgState* st, int* tickets, cudaStream_t s);

// ---- strict drop-in BLAS (k_api.cu, bit-exact elementwise ops) ------------
cudaError_t api_matvec(const MatView& A, double alpha, const double* x, double beta, double* y, cudaStream_t s);
cudaError_t api_axpy(long long m, double alpha, const double* x, double* y, cudaStream_t s);
cudaError_t api_scal(long long m, double alpha, double* x, cudaStream_t s);
cudaError_t api_dot(long long m, const double* x, const double* y, Red red, cudaStream_t s);
cudaError_t fill_sentinel(long long m, void* p, bool fp32, cudaStream_t s);

}  // namespace dfg
