// k_pattern.h -- launch interface of the device pattern / gather-map build.
#pragma once
#include <cuda_runtime.h>

namespace dfg {

constexpr int kPatCap = 256;          // per-node list bound (neighbours, row width)
constexpr int kPatErrRange = 1;       // a connectivity entry outside [0, n)
constexpr int kPatErrOverflow = 2;    // a node's list exceeds kPatCap: build on the host

// number of block sums exclusive_scan needs scratch for
long long scan_blocks(long long m);
// out[0..m] = exclusive prefix sums of in[0..m), out[m] = total; bsum: scan_blocks(m) entries
template <typename T>
cudaError_t exclusive_scan(const int* in, long long m, T* out, T* bsum, cudaStream_t s);

// incidences t = e*k + i per node: counts (cnt zeroed), then the lists
// (cursor zeroed, ptr = exclusive scan of the counts) sorted by t
cudaError_t incidence_count(const int* conn, long long nk, int n, int* cnt, int* err, cudaStream_t s);
cudaError_t incidence_fill(const int* conn, long long nk, int n, const long long* ptr, int* cursor, int* inc,
                           cudaStream_t s);
// row lengths, then columns (rowptr = exclusive scan of the lengths)
cudaError_t pattern_count(int n, int k, const int* conn, const long long* ptr, const int* inc, int* rowcnt, int* err,
                          cudaStream_t s);
cudaError_t pattern_fill(int n, int k, const int* conn, const long long* ptr, const int* inc, const int* rowptr,
                         int* colind, cudaStream_t s);
// gather-map slot counts (n diagonal + nnz CRS slots, zeroed), then lists
cudaError_t slots_count(int n, int k, const int* conn, const long long* ptr, const int* inc, const int* rowptr,
                        const int* colind, int* slotcnt, int* err, cudaStream_t s);
cudaError_t slots_fill(int n, int k, const int* conn, const long long* ptr, const int* inc, const int* rowptr,
                       const int* colind, const long long* slot_ptr, int* slot_src, cudaStream_t s);

}  // namespace dfg
