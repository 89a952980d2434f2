// k_ilu.h -- launch interface of the numeric block ILU factorisation.
#pragma once
#include <cuda_runtime.h>

namespace dfg {
// factorises the rows of one level (rows[0..cnt)) in place; dependent:
// launched as a programmatic dependent of the previous kernel in the stream
// (the previous level), which it waits for before touching memory
cudaError_t launch_ilu_level(int B, const int* rows, int cnt, const int* rowptr, const int* colind,
                             const int* diaind, double* fdiag, double* foffd, int* nsing, cudaStream_t st,
                             bool dependent = false);
// scatters A's off-diagonal blocks into a zeroed factor with fill-in
cudaError_t launch_factor_init(int B, long long nnz_a, const int* a2f, const double* offd, double* foffd,
                               cudaStream_t st);
}  // namespace dfg
