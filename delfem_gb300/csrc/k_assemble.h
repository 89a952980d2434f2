// k_assemble.h -- launch interface of the assembly / finalize kernels.
#pragma once
#include <cuda_runtime.h>

namespace dfg {

struct ElemArgs {
  long long nelem;
  const int* conn;
  const double* coords;
  const double* coef;   // per-element multiplier or nullptr
  const double* u;      // field value per DOF or nullptr
  const double* v;      // field velocity per DOF or nullptr
  double p[8];          // equation parameters (order per kind, see dfg.h)
  double* em;           // element blocks
  double* er;           // element residuals
};

struct GatherArgs {
  long long n, nnz;
  int b, bs;
  const long long* slot_ptr;
  const int* slot_src;
  const long long* res_ptr;
  const int* res_src;
  const double* em;
  const double* er;
  double* diag;
  double* offd;
  double* res;
};

struct BcArgs {
  int n;
  long long nnz;
  int b;
  const int* rowptr;
  const int* colind;
  const int* flag;
  double* diag;
  double* offd;
  double* res;
};

// kind: 1 poisson2d, 2 poisson3d, 3 diffusion2d, 4 solid2d, 5 solid3d
cudaError_t launch_elem(int kind, const ElemArgs& a, cudaStream_t st);
cudaError_t launch_gather(const GatherArgs& a, cudaStream_t st);
cudaError_t launch_add_vec(long long m, const double* f, double* r, cudaStream_t st);
cudaError_t launch_bc(const BcArgs& a, cudaStream_t st);

}  // namespace dfg
