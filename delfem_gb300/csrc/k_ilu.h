// k_ilu.h -- launch interface of the ILU(0) numeric factorisation.
#pragma once
#include <cuda_runtime.h>

namespace dfg {
// factorises the rows of one level (rows[0..cnt)) in place
cudaError_t launch_ilu_level(int B, const int* rows, int cnt, const int* rowptr, const int* colind,
                             const int* diaind, double* fdiag, double* foffd, int* nsing, cudaStream_t st);
}  // namespace dfg
