// noalloc.cu -- dfg_dot_noalloc: the deterministic dot product of dfg_dot
// (k_api.cu) with its reduction scratch in a fixed, file-scope device array
// instead of a context's allocation, for callers that may not allocate
// device memory.  Nothing here calls cudaMalloc, cudaFree or any allocating
// library routine.
#include <cuda.h>  // CUcontext / CUresult types only

#include <mutex>
#include <string>

#include "dfg_common.cuh"
#include "dfg_internal.h"

namespace dfg {
void set_noctx_error(const std::string& m);  // capi.cu: the text dfg_last_error(NULL) returns
}

using namespace dfg;

namespace {

constexpr int kTpb = 256;
constexpr int kPerThread = 16;
constexpr long long kChunk = (long long)kTpb * kPerThread;  // elements per block
constexpr int kMaxPartials = 8192;                          // blocks per launch, at most
static_assert(kChunk * kMaxPartials == DFG_DOT_NOALLOC_MAX_LEN, "maximum length and scratch size disagree");

// [0, kMaxPartials)   per-block partial sums
// [kMaxPartials]      the finished sum
// [kMaxPartials + 1]  arrival counter (an unsigned in a double's slot)
// 8194 doubles = 65,552 bytes per device, rounded up to 256-byte alignment.
constexpr int kResult = kMaxPartials;
constexpr int kCounter = kMaxPartials + 1;
static __device__ __align__(256) double g_dot_scratch[kMaxPartials + 2];

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// fixed-shape sum over the block; the result is valid in every thread
__device__ double block_sum(double v) {
  __shared__ double ws[kTpb / 32];
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) ws[w] = v;
  __syncthreads();
  double t = (threadIdx.x < kTpb / 32) ? ws[threadIdx.x] : 0.0;
  if (w == 0) t = warp_sum(t);
  __syncthreads();
  if (threadIdx.x == 0) ws[0] = t;
  __syncthreads();
  return ws[0];
}

// Block k sums elements [k*kChunk, (k+1)*kChunk) in a fixed order and
// publishes the partial; the last block to arrive sums the partials in index
// order.  The grid is ceil(m / kChunk) <= kMaxPartials blocks.
__global__ void __launch_bounds__(kTpb) k_dot_noalloc(long long m, const double* __restrict__ x,
                                                      const double* __restrict__ y, double* scratch) {
  const long long base = (long long)blockIdx.x * kChunk;
  double t = 0.0;
#pragma unroll
  for (int j = 0; j < kPerThread; ++j) {
    const long long k = base + (long long)j * kTpb + threadIdx.x;
    if (k < m) t += x[k] * y[k];
  }
  const double bs = block_sum(t);
  __shared__ bool last;
  unsigned* counter = reinterpret_cast<unsigned*>(scratch + kCounter);
  if (threadIdx.x == 0) {
    scratch[blockIdx.x] = bs;
    __threadfence();
    last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double s = 0.0;
  for (int i = threadIdx.x; i < (int)gridDim.x; i += kTpb) s += ld_relaxed(&scratch[i]);
  s = block_sum(s);
  if (threadIdx.x == 0) {
    scratch[kResult] = s;
    *counter = 0u;
  }
}

// Device address of g_dot_scratch, looked up once per CUDA context with that
// context current.  A device's array lives in the module the context loaded,
// so the address belongs to the context, not to the device ordinal: a device
// reset (a new primary context) or a caller's own driver-API context gets a
// lookup of its own.  Contexts are told apart by their unique ID
// (cuCtxGetId, reached through the runtime's driver entry points: the
// library does not link the driver API).
typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);

struct AddrEntry {
  unsigned long long ctx_id;
  double* addr;
};
constexpr int kMaxEntries = 64;
std::mutex g_mu;
AddrEntry g_addr[kMaxEntries] = {};
int g_nentries = 0, g_next = 0;
CtxGetCurrentFn g_get_current = nullptr;
CtxGetIdFn g_get_id = nullptr;

// ID of the calling thread's current context, 0 when none is current.
cudaError_t current_context_id(unsigned long long* id) {
  *id = 0;
  if (!g_get_current || !g_get_id) {
    cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = cudaDriverEntryPointSymbolNotFound;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", (void**)&g_get_current, 12000,
                                                     cudaEnableDefault, &q1);
    if (e == cudaSuccess)
      e = cudaGetDriverEntryPointByVersion("cuCtxGetId", (void**)&g_get_id, 12000, cudaEnableDefault, &q2);
    if (e != cudaSuccess) return e;
    if (q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !g_get_current || !g_get_id) {
      g_get_current = nullptr;
      g_get_id = nullptr;
      return cudaErrorNotSupported;
    }
  }
  CUcontext c = nullptr;
  if (g_get_current(&c) != CUDA_SUCCESS) return cudaErrorDeviceUninitialized;
  if (c && g_get_id(c, id) != CUDA_SUCCESS) return cudaErrorDeviceUninitialized;
  return cudaSuccess;
}

cudaError_t scratch_address(double** out) {
  std::lock_guard<std::mutex> lock(g_mu);
  unsigned long long id = 0;
  cudaError_t e = current_context_id(&id);
  if (e != cudaSuccess) return e;
  for (int k = 0; id != 0 && k < g_nentries; ++k)
    if (g_addr[k].ctx_id == id) {
      *out = g_addr[k].addr;
      return cudaSuccess;
    }
  // first call in this context (the lookup also makes the device's primary
  // context current on a thread that had none)
  double* p = nullptr;
  if ((e = cudaGetSymbolAddress((void**)&p, g_dot_scratch)) != cudaSuccess) return e;
  if ((e = current_context_id(&id)) != cudaSuccess) return e;
  if (id != 0) {
    AddrEntry& slot = g_addr[g_nentries < kMaxEntries ? g_nentries++ : g_next];
    if (g_nentries == kMaxEntries) g_next = (g_next + 1) % kMaxEntries;
    slot.ctx_id = id;
    slot.addr = p;
  }
  *out = p;
  return cudaSuccess;
}

int cuda_fail(const char* what, cudaError_t e) {
  cudaGetLastError();
  set_noctx_error(std::string("dfg_dot_noalloc: ") + what + ": " + cudaGetErrorString(e));
  return DFG_CUDA_ERROR;
}

}  // namespace

extern "C" int dfg_dot_noalloc(const double* x, const double* y, long long m, double* out, void* stream) {
  if (!out || m < 0 || (m > 0 && (!x || !y))) {
    set_noctx_error("dfg_dot_noalloc: out must be non-NULL, m >= 0, and x, y non-NULL when m > 0");
    return DFG_INVALID_ARGUMENT;
  }
  if (m > DFG_DOT_NOALLOC_MAX_LEN) {
    set_noctx_error("dfg_dot_noalloc: length " + std::to_string(m) + " exceeds the maximum of " +
                    std::to_string(DFG_DOT_NOALLOC_MAX_LEN) + " elements (" + std::to_string(kMaxPartials) +
                    " partial sums of " + std::to_string(kChunk) + " elements in the static scratch)");
    return DFG_INVALID_ARGUMENT;
  }
  if (m == 0) {
    *out = 0.0;
    return DFG_OK;
  }
  double* scratch = nullptr;
  cudaError_t e = scratch_address(&scratch);
  if (e != cudaSuccess) return cuda_fail("looking up the scratch array's address", e);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // the arrival counter must start at zero
  if ((e = cudaMemsetAsync(scratch + kCounter, 0, sizeof(unsigned), st)) != cudaSuccess)
    return cuda_fail("clearing the arrival counter", e);
  const int grid = (int)((m + kChunk - 1) / kChunk);
  k_dot_noalloc<<<grid, kTpb, 0, st>>>(m, x, y, scratch);
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail("kernel launch", e);
  if ((e = cudaMemcpyAsync(out, scratch + kResult, sizeof(double), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
    return cuda_fail("reading the result", e);
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cuda_fail("cudaStreamSynchronize", e);
  return DFG_OK;
}
