// capi.cu -- the extern "C" entry points of libdfg (declared in include/dfg.h).
//
// Host-side orchestration only: argument checks, device memory, symbolic
// set-up (sched.cpp) and kernel launches on the context's stream.  The PCG
// loop runs device-resident: a chunk of iterations is captured once into a
// CUDA graph and replayed until the device-side state reports convergence.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "dfg_internal.h"
#include "k_assemble.h"
#include "k_ilu.h"
#include "k_pattern.h"
#include "k_solve.h"
#include "k_sweep.h"

using namespace dfg;

#define DFG_VERSION "dfg 0.1.0 (sm_103a)"

namespace dfg {

void DBuf::release() {
  if (p) cudaFree(p);
  p = nullptr;
  bytes = 0;
}

}  // namespace dfg

namespace {

struct Fail {
  int status;
};

inline void set_err(dfg_ctx c, const std::string& m) {
  if (c) c->last_error = m;
}

#define CK(call)                                                                            \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess) {                                                                \
      set_err(ctx_, std::string("CUDA error: ") + cudaGetErrorString(e_) + " at " #call);  \
      throw Fail{e_ == cudaErrorMemoryAllocation ? DFG_OOM_REJECTED : DFG_CUDA_ERROR};    \
    }                                                                                       \
  } while (0)

#define REQUIRE(cond, status, msg)   \
  do {                               \
    if (!(cond)) {                   \
      set_err(ctx_, msg);            \
      throw Fail{status};            \
    }                                \
  } while (0)

template <class F>
int guarded(dfg_ctx ctx, F&& f) {
  try {
    if (ctx) {
      cudaError_t e = cudaSetDevice(ctx->device);
      if (e != cudaSuccess) {
        ctx->last_error = std::string("cudaSetDevice: ") + cudaGetErrorString(e);
        return DFG_CUDA_ERROR;
      }
    }
    return f();
  } catch (const Fail& x) {
    return x.status;
  } catch (const std::bad_alloc&) {
    set_err(ctx, "host allocation failed");
    return DFG_OOM_REJECTED;
  } catch (...) {
    set_err(ctx, "unexpected host exception");
    return DFG_CUDA_ERROR;
  }
}

void dalloc(dfg_ctx ctx_, DBuf& b, size_t bytes) {
  if (b.p && b.bytes >= bytes) return;
  b.release();
  if (bytes == 0) bytes = 16;
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_err(ctx_, "device allocation of " + std::to_string(bytes) + " bytes refused: " + cudaGetErrorString(e));
    throw Fail{DFG_OOM_REJECTED};
  }
  b.p = p;
  b.bytes = bytes;
}

template <class T>
void upload(dfg_ctx ctx_, DBuf& b, const T* h, size_t count, size_t slack = 0) {
  dalloc(ctx_, b, count * sizeof(T) + slack);
  if (count) CK(cudaMemcpyAsync(b.p, h, count * sizeof(T), cudaMemcpyHostToDevice, ctx_->stream));
}

void launched(dfg_ctx c, long long n = 1) { c->launches += n; }

// scratch layout in ctx->scratch: [partials kRedGrid doubles][counters 16][results 16 doubles][tickets 16 ints]
struct Scratch {
  double* partials;
  unsigned* counters;
  double* results;
  int* tickets;
};
Scratch scratch_of(dfg_ctx c) {
  char* base = c->scratch.as<char>();
  Scratch s;
  s.partials = reinterpret_cast<double*>(base);
  s.counters = reinterpret_cast<unsigned*>(base + kRedGrid * 8);
  s.results = reinterpret_cast<double*>(base + kRedGrid * 8 + 16 * 4);
  s.tickets = reinterpret_cast<int*>(base + kRedGrid * 8 + 16 * 4 + 16 * 8);
  return s;
}
Red red_of(dfg_ctx c, int channel = 0) {
  Scratch s = scratch_of(c);
  return Red{s.partials, s.counters + channel, s.results + channel};
}

double* vec_ptr(dfg_ctx ctx_, dfg_system s, int iv) {
  if (iv == -1) return s->res.as<double>();
  if (iv == -2) return s->upd.as<double>();
  REQUIRE(iv >= 0 && iv < (int)s->tmp.size(), DFG_INVALID_ARGUMENT, "vector slot " + std::to_string(iv) + " out of range");
  return s->tmp[iv].as<double>();
}

MatView view64(dfg_system s) {
  return MatView{s->n, s->b, s->rowptr.as<int>(), s->colind.as<int>(), s->diag.p, s->offd.p,
                 s->s_ptr.as<long long>(), s->s_width.as<int>(), s->s_col.as<int>(), s->s_val64.p};
}
MatView view32(dfg_system s) {
  return MatView{s->n, s->b, s->rowptr.as<int>(), s->colind.as<int>(), s->diag32.p, s->offd32.p,
                 s->s_ptr.as<long long>(), s->s_width.as<int>(), s->s_col.as<int>(), s->s_val32.p};
}

// Packs the sliced-ELL values of the current matrix (FP64 or FP32) if the
// matrix changed since the last pack.
void ensure_sell(dfg_ctx ctx_, dfg_system s, bool fp32) {
  long long& ver = fp32 ? s->sell32_version : s->sell64_version;
  if (ver == s->mat_version) return;
  DBuf& out = fp32 ? s->s_val32 : s->s_val64;
  dalloc(ctx_, out, (size_t)std::max<long long>(s->sell_blocks, 1) * s->b * s->b * (fp32 ? 4 : 8) + 64);
  CK(sell_pack(s->sell_nslices, s->b, s->s_ptr.as<long long>(), s->s_src.as<int>(), s->diag.as<double>(),
               s->offd.as<double>(), out.p, fp32, ctx_->stream));
  ctx_->launches += 1;
  ver = s->mat_version;
}

size_t vec_bytes(dfg_system s, size_t elem) { return (size_t)s->n * s->b * elem + 64; }

void system_alloc(dfg_ctx ctx_, dfg_system s) {
  const size_t bs = (size_t)s->b * s->b;
  dalloc(ctx_, s->diag, (size_t)s->n * bs * 8);
  dalloc(ctx_, s->offd, (size_t)std::max<long long>(s->nnz, 1) * bs * 8);
  dalloc(ctx_, s->res, vec_bytes(s, 8));
  dalloc(ctx_, s->upd, vec_bytes(s, 8));
  CK(cudaMemsetAsync(s->diag.p, 0, s->diag.bytes, ctx_->stream));
  CK(cudaMemsetAsync(s->offd.p, 0, s->offd.bytes, ctx_->stream));
  CK(cudaMemsetAsync(s->res.p, 0, s->res.bytes, ctx_->stream));
  CK(cudaMemsetAsync(s->upd.p, 0, s->upd.bytes, ctx_->stream));
  s->h_diaind.resize(s->n);
  for (int i = 0; i < s->n; ++i) {
    int d = s->h_rowptr[i + 1];
    for (int c = s->h_rowptr[i]; c < s->h_rowptr[i + 1]; ++c)
      if (s->h_colind[c] > i) { d = c; break; }
    s->h_diaind[i] = d;
  }
  upload(ctx_, s->rowptr, s->h_rowptr.data(), s->h_rowptr.size());
  upload(ctx_, s->colind, s->h_colind.data(), s->h_colind.size());
  upload(ctx_, s->diaind, s->h_diaind.data(), s->h_diaind.size());
  const SellMap M = build_sell(s->n, s->h_rowptr.data(), s->h_colind.data());
  s->sell_nslices = M.nslices;
  s->sell_blocks = M.ptr.back();
  upload(ctx_, s->s_ptr, M.ptr.data(), M.ptr.size());
  upload(ctx_, s->s_width, M.width.data(), std::max<size_t>(M.width.size(), 1));
  upload(ctx_, s->s_col, M.col.data(), std::max<size_t>(M.col.size(), 1));
  upload(ctx_, s->s_src, M.src.data(), std::max<size_t>(M.src.size(), 1));
  CK(cudaStreamSynchronize(ctx_->stream));  // the host map is about to go away
}

void check_pattern(dfg_ctx ctx_, int n, const int* rowptr, const int* colind) {
  REQUIRE(rowptr[0] == 0, DFG_INVALID_ARGUMENT, "rowptr[0] must be 0");
  for (int i = 0; i < n; ++i) {
    REQUIRE(rowptr[i + 1] >= rowptr[i], DFG_INVALID_ARGUMENT, "rowptr must be non-decreasing");
    for (int c = rowptr[i]; c < rowptr[i + 1]; ++c) {
      REQUIRE(colind[c] >= 0 && colind[c] < n, DFG_INVALID_ARGUMENT, "column index out of range");
      REQUIRE(colind[c] != i, DFG_INVALID_ARGUMENT, "pattern must not hold the diagonal block (CMatDia_BlkCrs::AddPattern)");
      REQUIRE(c == rowptr[i] || colind[c] > colind[c - 1], DFG_INVALID_ARGUMENT, "columns must be strictly ascending within a row");
    }
  }
}

int read_state(dfg_ctx ctx_, PcgState* d_state, PcgState& h) {
  CK(cudaMemcpyAsync(&h, d_state, sizeof(PcgState), cudaMemcpyDeviceToHost, ctx_->stream));
  CK(cudaStreamSynchronize(ctx_->stream));
  return 0;
}

int read_err(dfg_ctx ctx_) {
  int e = 0;
  CK(cudaMemcpyAsync(&e, ctx_->err_word.p, sizeof(int), cudaMemcpyDeviceToHost, ctx_->stream));
  CK(cudaStreamSynchronize(ctx_->stream));
  return e;
}

}  // namespace

// ===================================================================== context

extern "C" const char* dfg_version(void) { return DFG_VERSION; }

// error text of the last failed dfg_ctx_create (there is no context to hold it)
static thread_local std::string g_create_error = "no error";

namespace dfg {
// errors of entry points that take no context (dfg_dot_noalloc)
void set_noctx_error(const std::string& m) { g_create_error = m; }
}  // namespace dfg

extern "C" int dfg_ctx_create(int device, dfg_ctx* out) {
  if (!out) return DFG_INVALID_ARGUMENT;
  *out = nullptr;
  int ndev = 0;
  const cudaError_t ce = cudaGetDeviceCount(&ndev);
  if (ce != cudaSuccess || device < 0 || device >= ndev) {
    g_create_error = ce != cudaSuccess ? std::string("cudaGetDeviceCount: ") + cudaGetErrorString(ce)
                                       : "device index out of range";
    cudaGetLastError();
    return DFG_CUDA_ERROR;
  }
  dfg_ctx c = new (std::nothrow) dfg_ctx_s;
  if (!c) return DFG_OOM_REJECTED;
  c->device = device;
  int rc = guarded(c, [&]() -> int {
    dfg_ctx ctx_ = c;
    CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    CK(cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, device));
    int optin = 0;
    CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
    // dynamic shared memory a kernel may request: the opt-in limit less a
    // margin for the kernels' own static shared memory
    c->smem_optin = (size_t)optin - 1024;
    dalloc(c, c->err_word, 64);
    dalloc(c, c->scratch, kRedGrid * 8 + 16 * 4 + 16 * 8 + 16 * 4 + 256);
    CK(cudaMemsetAsync(c->err_word.p, 0, 64, c->stream));
    CK(cudaMemsetAsync(c->scratch.p, 0, c->scratch.bytes, c->stream));
    CK(sweep_set_smem_limits(c->smem_optin));
    CK(cudaStreamSynchronize(c->stream));
    return DFG_OK;
  });
  if (rc != DFG_OK) {
    g_create_error = c->last_error;
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return rc;
  }
  *out = c;
  return DFG_OK;
}

extern "C" int dfg_ctx_destroy(dfg_ctx ctx) {
  if (!ctx) return DFG_INVALID_ARGUMENT;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  ctx->err_word.release();
  ctx->scratch.release();
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  return DFG_OK;
}

extern "C" const char* dfg_last_error(dfg_ctx ctx) { return ctx ? ctx->last_error.c_str() : g_create_error.c_str(); }

extern "C" int dfg_ctx_synchronize(dfg_ctx ctx) {
  if (!ctx) return DFG_INVALID_ARGUMENT;
  return guarded(ctx, [&]() -> int {
    dfg_ctx ctx_ = ctx;
    CK(cudaStreamSynchronize(ctx->stream));
    return DFG_OK;
  });
}

extern "C" long long dfg_ctx_kernel_launches(dfg_ctx ctx) { return ctx ? ctx->launches : -1; }

extern "C" int dfg_ctx_get_stream(dfg_ctx ctx, void** stream) {
  if (!ctx || !stream) return DFG_INVALID_ARGUMENT;
  *stream = (void*)ctx->stream;
  return DFG_OK;
}

// ===================================================================== system

extern "C" int dfg_system_create(dfg_ctx ctx, int nblk, int blklen, const int* rowptr, const int* colind,
                                 dfg_system* out) {
  if (!ctx || !out) return DFG_INVALID_ARGUMENT;
  *out = nullptr;
  return guarded(ctx, [&]() -> int {
    dfg_ctx ctx_ = ctx;
    REQUIRE(nblk >= 0 && rowptr, DFG_INVALID_ARGUMENT, "bad nblk / rowptr");
    REQUIRE(blklen >= 1 && blklen <= 3, DFG_INVALID_ARGUMENT, "block length must be 1, 2 or 3");
    check_pattern(ctx, nblk, rowptr, colind);
    dfg_system s = new dfg_system_s;
    s->ctx = ctx;
    s->n = nblk;
    s->b = blklen;
    s->nnz = rowptr[nblk];
    s->h_rowptr.assign(rowptr, rowptr + nblk + 1);
    s->h_colind.assign(colind, colind + s->nnz);
    try {
      system_alloc(ctx, s);
      CK(cudaStreamSynchronize(ctx->stream));
    } catch (...) {
      delete s;
      throw;
    }
    *out = s;
    return DFG_OK;
  });
}

namespace {

int read_flag(dfg_ctx ctx_, const int* d) {
  int h = 0;
  CK(cudaMemcpyAsync(&h, d, sizeof(int), cudaMemcpyDeviceToHost, ctx_->stream));
  CK(cudaStreamSynchronize(ctx_->stream));
  return h;
}

// Element incidences per node on the device (ptr: n+1 offsets, inc: e*k+i
// sorted per node); returns the error flag (0, or kPatErrRange).
int build_incidence(dfg_ctx ctx_, int n, long long nk, const int* d_conn, DBuf& ptr, DBuf& inc, DBuf& flag) {
  DBuf cnt, bsum;
  dalloc(ctx_, cnt, (size_t)std::max(n, 1) * 4);
  dalloc(ctx_, flag, 16);
  dalloc(ctx_, ptr, (size_t)(n + 1) * 8);
  dalloc(ctx_, bsum, (size_t)std::max<long long>(scan_blocks(n), 1) * 8);
  dalloc(ctx_, inc, (size_t)std::max<long long>(nk, 1) * 4);
  CK(cudaMemsetAsync(cnt.p, 0, cnt.bytes, ctx_->stream));
  CK(cudaMemsetAsync(flag.p, 0, flag.bytes, ctx_->stream));
  CK(incidence_count(d_conn, nk, n, cnt.as<int>(), flag.as<int>(), ctx_->stream));
  CK(exclusive_scan<long long>(cnt.as<int>(), n, ptr.as<long long>(), bsum.as<long long>(), ctx_->stream));
  CK(cudaMemsetAsync(cnt.p, 0, cnt.bytes, ctx_->stream));  // now the placement cursors
  CK(incidence_fill(d_conn, nk, n, ptr.as<long long>(), cnt.as<int>(), inc.as<int>(), ctx_->stream));
  launched(ctx_, 6);
  return read_flag(ctx_, flag.as<int>());
}

// The element pattern (MakePattern_FEM + AddPattern) built on the device and
// copied to the host; false when a node's neighbour list overflows the
// per-thread bound, and the caller builds on the host.
bool device_pattern(dfg_ctx ctx_, int n, int nelem, int k, const int* conn, std::vector<int>& rp,
                    std::vector<int>& ci) {
  const long long nk = (long long)nelem * k;
  if ((long long)n * kPatCap > INT32_MAX || nk > INT32_MAX) return false;  // int offsets and incidence ids
  DBuf dconn, ptr, inc, flag, rowcnt, rowptr, colind, bsum;
  upload(ctx_, dconn, conn, (size_t)nk, 16);
  REQUIRE(build_incidence(ctx_, n, nk, dconn.as<int>(), ptr, inc, flag) == 0, DFG_INVALID_ARGUMENT,
          "connectivity index out of range");
  dalloc(ctx_, rowcnt, (size_t)std::max(n, 1) * 4);
  CK(pattern_count(n, k, dconn.as<int>(), ptr.as<long long>(), inc.as<int>(), rowcnt.as<int>(), flag.as<int>(),
                   ctx_->stream));
  launched(ctx_);
  if (read_flag(ctx_, flag.as<int>()) != 0) return false;
  dalloc(ctx_, rowptr, (size_t)(n + 1) * 4);
  dalloc(ctx_, bsum, (size_t)std::max<long long>(scan_blocks(n), 1) * 4);
  CK(exclusive_scan<int>(rowcnt.as<int>(), n, rowptr.as<int>(), bsum.as<int>(), ctx_->stream));
  launched(ctx_, 3);
  rp.assign(n + 1, 0);
  CK(cudaMemcpyAsync(rp.data(), rowptr.p, (size_t)(n + 1) * 4, cudaMemcpyDeviceToHost, ctx_->stream));
  CK(cudaStreamSynchronize(ctx_->stream));
  const int nnz = rp[n];
  dalloc(ctx_, colind, (size_t)std::max(nnz, 1) * 4);
  CK(pattern_fill(n, k, dconn.as<int>(), ptr.as<long long>(), inc.as<int>(), rowptr.as<int>(), colind.as<int>(),
                  ctx_->stream));
  launched(ctx_);
  ci.assign(nnz, 0);
  if (nnz) CK(cudaMemcpyAsync(ci.data(), colind.p, (size_t)nnz * 4, cudaMemcpyDeviceToHost, ctx_->stream));
  CK(cudaStreamSynchronize(ctx_->stream));
  return true;
}

struct DeviceGather {
  DBuf slot_ptr, slot_src, res_ptr, res_src;
};

// The assembly gather map (the element order of Mearge) built on the device
// from the connectivity d_conn against the system's pattern; false when a
// row is wider than the per-thread bound (build on the host).
bool device_gather_map(dfg_ctx ctx_, dfg_system sys, int nelem, int k, const int* d_conn, DeviceGather& G) {
  const int n = sys->n;
  const long long nnz = sys->nnz, nk = (long long)nelem * k;
  REQUIRE(nk * k <= INT32_MAX, DFG_INVALID_ARGUMENT, "mesh too large for 32-bit element-block indices");
  DBuf ptr, inc, flag, slotcnt, bsum;
  REQUIRE(build_incidence(ctx_, n, nk, d_conn, ptr, inc, flag) == 0, DFG_INVALID_ARGUMENT,
          "connectivity index out of range");
  const long long ns = n + nnz;
  dalloc(ctx_, slotcnt, (size_t)std::max<long long>(ns, 1) * 4);
  CK(cudaMemsetAsync(slotcnt.p, 0, slotcnt.bytes, ctx_->stream));
  CK(slots_count(n, k, d_conn, ptr.as<long long>(), inc.as<int>(), sys->rowptr.as<int>(), sys->colind.as<int>(),
                 slotcnt.as<int>(), flag.as<int>(), ctx_->stream));
  launched(ctx_);
  if (read_flag(ctx_, flag.as<int>()) != 0) return false;
  dalloc(ctx_, G.slot_ptr, (size_t)(ns + 1) * 8);
  dalloc(ctx_, bsum, (size_t)std::max<long long>(scan_blocks(ns), 1) * 8);
  CK(exclusive_scan<long long>(slotcnt.as<int>(), ns, G.slot_ptr.as<long long>(), bsum.as<long long>(),
                               ctx_->stream));
  launched(ctx_, 3);
  long long total = 0;
  CK(cudaMemcpyAsync(&total, G.slot_ptr.as<long long>() + ns, 8, cudaMemcpyDeviceToHost, ctx_->stream));
  CK(cudaStreamSynchronize(ctx_->stream));
  REQUIRE(total <= INT32_MAX, DFG_INVALID_ARGUMENT, "mesh too large for 32-bit element-block indices");
  dalloc(ctx_, G.slot_src, (size_t)std::max<long long>(total, 1) * 4);
  CK(slots_fill(n, k, d_conn, ptr.as<long long>(), inc.as<int>(), sys->rowptr.as<int>(), sys->colind.as<int>(),
                G.slot_ptr.as<long long>(), G.slot_src.as<int>(), ctx_->stream));
  launched(ctx_);
  G.res_ptr = std::move(ptr);
  G.res_src = std::move(inc);
  CK(cudaStreamSynchronize(ctx_->stream));
  return true;
}

}  // namespace

extern "C" int dfg_system_create_from_elements(dfg_ctx ctx, int nblk, int blklen, int nelem, int nnoel,
                                               const int* conn, dfg_system* out) {
  if (!ctx || !out) return DFG_INVALID_ARGUMENT;
  *out = nullptr;
  std::vector<int> rp, ci;
  int rc = guarded(ctx, [&]() -> int {
    dfg_ctx ctx_ = ctx;
    REQUIRE(nblk >= 0 && nelem >= 0 && nnoel >= 1 && (conn || nelem == 0), DFG_INVALID_ARGUMENT, "bad element arguments");
    for (long long k = 0; k < (long long)nelem * nnoel; ++k)
      REQUIRE(conn[k] >= 0 && conn[k] < nblk, DFG_INVALID_ARGUMENT, "connectivity index out of range");
    // on the device; the host builder when a node has more neighbours than a thread's list holds
    if (!device_pattern(ctx, nblk, nelem, nnoel, conn, rp, ci)) pattern_from_elements(nblk, nelem, nnoel, conn, rp, ci);
    return DFG_OK;
  });
  if (rc != DFG_OK) return rc;
  return dfg_system_create(ctx, nblk, blklen, rp.data(), ci.data(), out);
}

extern "C" int dfg_system_destroy(dfg_system sys) {
  if (!sys) return DFG_INVALID_ARGUMENT;
  cudaSetDevice(sys->ctx->device);
  cudaStreamSynchronize(sys->ctx->stream);
  delete sys;
  return DFG_OK;
}

extern "C" int dfg_system_info(dfg_system sys, int* nblk, int* blklen, long long* nnz) {
  if (!sys) return DFG_INVALID_ARGUMENT;
  if (nblk) *nblk = sys->n;
  if (blklen) *blklen = sys->b;
  if (nnz) *nnz = sys->nnz;
  return DFG_OK;
}

extern "C" int dfg_system_get_pattern(dfg_system sys, int* rowptr, int* colind) {
  if (!sys) return DFG_INVALID_ARGUMENT;
  if (rowptr) std::memcpy(rowptr, sys->h_rowptr.data(), sys->h_rowptr.size() * sizeof(int));
  if (colind) std::memcpy(colind, sys->h_colind.data(), sys->h_colind.size() * sizeof(int));
  return DFG_OK;
}

extern "C" int dfg_system_set_mesh(dfg_system sys, int ndim, const double* coords, int nelem, int nnoel,
                                   const int* conn) {
  if (!sys) return DFG_INVALID_ARGUMENT;
  dfg_ctx ctx = sys->ctx;
  return guarded(ctx, [&]() -> int {
    dfg_ctx ctx_ = ctx;
    REQUIRE(ndim == 2 || ndim == 3, DFG_INVALID_ARGUMENT, "ndim must be 2 or 3");
    REQUIRE((ndim == 2 && nnoel == 3) || (ndim == 3 && nnoel == 4), DFG_INVALID_ARGUMENT,
            "elements must be P1 triangles (2D) or P1 tetrahedra (3D)");
    REQUIRE(nelem >= 0 && coords && (conn || nelem == 0), DFG_INVALID_ARGUMENT, "bad mesh arguments");
    // everything is built aside and replaces the system's mesh only once complete
    DBuf dconn, dcoords;
    DeviceGather D;
    upload(ctx, dconn, conn, (size_t)nelem * nnoel, 16);
    upload(ctx, dcoords, coords, (size_t)sys->n * ndim);
    // gather map on the device; the host builder when a row is wider than a thread's list holds
    if (!device_gather_map(ctx, sys, nelem, nnoel, dconn.as<int>(), D)) {
      GatherMap G;
      std::string err;
      REQUIRE(build_gather_map(sys->n, sys->h_rowptr.data(), sys->h_colind.data(), nelem, nnoel, conn, G, err),
              DFG_INVALID_ARGUMENT, err);
      upload(ctx, D.slot_ptr, G.slot_ptr.data(), G.slot_ptr.size());
      upload(ctx, D.slot_src, G.slot_src.data(), G.slot_src.size(), 16);
      upload(ctx, D.res_ptr, G.res_ptr.data(), G.res_ptr.size());
      upload(ctx, D.res_src, G.res_src.data(), G.res_src.size(), 16);
    }
    CK(cudaStreamSynchronize(ctx->stream));
    sys->conn = std::move(dconn);
    sys->coords = std::move(dcoords);
    sys->slot_ptr = std::move(D.slot_ptr);
    sys->slot_src = std::move(D.slot_src);
    sys->res_ptr = std::move(D.res_ptr);
    sys->res_src = std::move(D.res_src);
    sys->ndim = ndim;
    sys->nelem = nelem;
    sys->nnoel = nnoel;
    return DFG_OK;
  });
}

extern "C" int dfg_system_set_coef(dfg_system sys, const double* coef) {
  if (!sys) return DFG_INVALID_ARGUMENT;
  dfg_ctx ctx = sys->ctx;
  return guarded(ctx, [&]() -> int {
    dfg_ctx ctx_ = ctx;
    REQUIRE(sys->conn.p || sys->nelem == 0, DFG_NOT_READY, "set the mesh before the coefficients");
    if (!coef) { sys->has_coef = false; return DFG_OK; }
    upload(ctx, sys->coef, coef, (size_t)sys->nelem);
    CK(cudaStreamSynchronize(ctx->stream));
    sys->has_coef = true;
    return DFG_OK;
  });
}

extern "C" int dfg_system_set_field(dfg_system sys, const double* u, const double* v) {
  if (!sys) return DFG_INVALID_ARGUMENT;
  dfg_ctx ctx = sys->ctx;
  return guarded(ctx, [&]() -> int {
    dfg_ctx ctx_ = ctx;
    const size_t m = (size_t)sys->n * sys->b;
    sys->has_u = u != nullptr;
    sys->has_v = v != nullptr;
    if (u) upload(ctx, sys->fu, u, m);
    if (v) upload(ctx, sys->fv, v, m);
    CK(cudaStreamSynchronize(ctx->stream));
    return DFG_OK;
  });
}

extern "C" int dfg_system_update_field(dfg_system sys, int fdt) {
  if (!sys) return DFG_INVALID_ARGUMENT;
  dfg_ctx ctx = sys->ctx;
  return guarded(ctx, [&]() -> int {
    dfg_ctx ctx_ = ctx;
    REQUIRE(fdt == 0 || fdt == 1, DFG_INVALID_ARGUMENT, "fdt must be 0 (VALUE) or 1 (VELOCITY)");
    const long long m = (long long)sys->n * sys->b;
    DBuf& f = fdt == 0 ? sys->fu : sys->fv;
    bool& has = fdt == 0 ? sys->has_u : sys->has_v;
    if (!has) {
      dalloc(ctx, f, (size_t)m * 8);
      CK(cudaMemsetAsync(f.p, 0, (size_t)m * 8, ctx->stream));
      has = true;
    }
    CK(api_axpy(m, 1.0, sys->upd.as<double>(), f.as<double>(), ctx->stream));  // AddValueToNodeSegment(.., 1.0)
    launched(ctx);
    CK(cudaStreamSynchronize(ctx->stream));
    return DFG_OK;
  });
}

extern "C" int dfg_system_get_field(dfg_system sys, double* u, double* v) {
  if (!sys) return DFG_INVALID_ARGUMENT;
  dfg_ctx ctx = sys->ctx;
  return guarded(ctx, [&]() -> int {
    dfg_ctx ctx_ = ctx;
    const size_t bytes = (size_t)sys->n * sys->b * 8;
    if (u) {
      if (sys->has_u) CK(cudaMemcpyAsync(u, sys->fu.p, bytes, cudaMemcpyDeviceToHost, ctx->stream));
      else std::memset(u, 0, bytes);
    }
    if (v) {
      if (sys->has_v) CK(cudaMemcpyAsync(v, sys->fv.p, bytes, cudaMemcpyDeviceToHost, ctx->stream));
      else std::memset(v, 0, bytes);
    }
    CK(cudaStreamSynchronize(ctx->stream));
    return DFG_OK;
  });
}

extern "C" int dfg_set_bcflags(dfg_system sys, const int* flags) {
  if (!sys) return DFG_INVALID_ARGUMENT;
  dfg_ctx ctx = sys->ctx;
  return guarded(ctx, [&]() -> int {
    dfg_ctx ctx_ = ctx;
    const size_t m = (size_t)sys->n * sys->b;
    if (!flags) {
      dalloc(ctx, sys->bcflag, m * 4 + 16);
      CK(cudaMemsetAsync(sys->bcflag.p, 0, sys->bcflag.bytes, ctx->stream));
    } else {
      upload(ctx, sys->bcflag, flags, m);
    }
    CK(cudaStreamSynchronize(ctx->stream));
    sys->has_bc = true;
    return DFG_OK;
  });
}

// ===================================================================== assembly

extern "C" int dfg_initialize_marge(dfg_system sys) {
  if (!sys) return DFG_INVALID_ARGUMENT;
  dfg_ctx ctx = sys->ctx;
  return guarded(ctx, [&]() -> int {
    dfg_ctx ctx_ = ctx;
    CK(cudaMemsetAsync(sys->diag.p, 0, sys->diag.bytes, ctx->stream));
    CK(cudaMemsetAsync(sys->offd.p, 0, sys->offd.bytes, ctx->stream));
    CK(cudaMemsetAsync(sys->res.p, 0, sys->res.bytes, ctx->stream));
    CK(cudaMemsetAsync(sys->upd.p, 0, sys->upd.bytes, ctx->stream));
    sys->mat32_valid = false;
    ++sys->mat_version;
    sys->rhs0_valid = false;
    return DFG_OK;
  });
}

static int assemble(dfg_system sys, int kind, int need_b, int need_ndim, const double* p, int np) {
  if (!sys) return DFG_INVALID_ARGUMENT;
  dfg_ctx ctx = sys->ctx;
  return guarded(ctx, [&]() -> int {
    dfg_ctx ctx_ = ctx;
    REQUIRE(sys->conn.p && sys->nelem >= 0, DFG_NOT_READY, "dfg_system_set_mesh must come before assembly");
    REQUIRE(sys->b == need_b, DFG_INVALID_ARGUMENT, "block length does not match the equation");
    REQUIRE(need_ndim == 0 || sys->ndim == need_ndim, DFG_INVALID_ARGUMENT, "mesh dimension does not match the equation");
    const int k = sys->nnoel, bs = sys->b * sys->b;
    dalloc(ctx, sys->em, (size_t)sys->nelem * k * k * bs * 8);
    dalloc(ctx, sys->er, (size_t)sys->nelem * k * sys->b * 8);
    ElemArgs a{};
    a.nelem = sys->nelem;
    a.conn = sys->conn.as<int>();
    a.coords = sys->coords.as<double>();
    a.coef = sys->has_coef ? sys->coef.as<double>() : nullptr;
    a.u = sys->has_u ? sys->fu.as<double>() : nullptr;
    a.v = sys->has_v ? sys->fv.as<double>() : nullptr;
    for (int i = 0; i < 8; ++i) a.p[i] = i < np ? p[i] : 0.0;
    a.em = sys->em.as<double>();
    a.er = sys->er.as<double>();
    CK(launch_elem(kind, a, ctx->stream));
    GatherArgs g{};
    g.n = sys->n;
    g.nnz = sys->nnz;
    g.b = sys->b;
    g.bs = bs;
    g.slot_ptr = sys->slot_ptr.as<long long>();
    g.slot_src = sys->slot_src.as<int>();
    g.res_ptr = sys->res_ptr.as<long long>();
    g.res_src = sys->res_src.as<int>();
    g.em = a.em;
    g.er = a.er;
    g.diag = sys->diag.as<double>();
    g.offd = sys->offd.as<double>();
    g.res = sys->res.as<double>();
    CK(launch_gather(g, ctx->stream));
    launched(ctx, 3);
    sys->mat32_valid = false;
    ++sys->mat_version;
    return DFG_OK;
  });
}

extern "C" int dfg_assemble_poisson(dfg_system sys, double alpha, double source) {
  if (!sys) return DFG_INVALID_ARGUMENT;
  const double p[2] = {alpha, source};
  return assemble(sys, sys->ndim == 3 ? 2 : 1, 1, 0, p, 2);
}
extern "C" int dfg_assemble_diffusion(dfg_system sys, double dt, double gamma, double rho, double alpha,
                                      double source) {
  const double p[5] = {rho, alpha, source, gamma, dt};
  return assemble(sys, 3, 1, 2, p, 5);
}
extern "C" int dfg_assemble_solid2d(dfg_system sys, double lambda, double myu, double rho, double g_x,
                                    double g_y) {
  const double p[5] = {lambda, myu, rho, g_x, g_y};
  return assemble(sys, 4, 2, 2, p, 5);
}
extern "C" int dfg_assemble_solid3d(dfg_system sys, double lambda, double myu, double rho, double g_x,
                                    double g_y, double g_z) {
  const double p[6] = {lambda, myu, rho, g_x, g_y, g_z};
  return assemble(sys, 5, 3, 3, p, 6);
}

extern "C" int dfg_add_residual(dfg_system sys, const double* f) {
  if (!sys) return DFG_INVALID_ARGUMENT;
  dfg_ctx ctx = sys->ctx;
  return guarded(ctx, [&]() -> int {
    dfg_ctx ctx_ = ctx;
    REQUIRE(f, DFG_INVALID_ARGUMENT, "null load vector");
    const size_t m = (size_t)sys->n * sys->b;
    DBuf tmp;
    upload(ctx, tmp, f, m);
    CK(launch_add_vec((long long)m, tmp.as<double>(), sys->res.as<double>(), ctx->stream));
    launched(ctx);
    CK(cudaStreamSynchronize(ctx->stream));
    return DFG_OK;
  });
}

extern "C" int dfg_system_set_load(dfg_system sys, const double* f) {
  if (!sys) return DFG_INVALID_ARGUMENT;
  dfg_ctx ctx = sys->ctx;
  return guarded(ctx, [&]() -> int {
    dfg_ctx ctx_ = ctx;
    if (!f) { sys->has_load = false; return DFG_OK; }
    upload(ctx, sys->load, f, (size_t)sys->n * sys->b);
    CK(cudaStreamSynchronize(ctx->stream));
    sys->has_load = true;
    return DFG_OK;
  });
}

extern "C" int dfg_finalize_marge(dfg_system sys, double* norm_res) {
  if (!sys) return DFG_INVALID_ARGUMENT;
  dfg_ctx ctx = sys->ctx;
  return guarded(ctx, [&]() -> int {
    dfg_ctx ctx_ = ctx;
    if (sys->has_load) {
      CK(launch_add_vec((long long)sys->n * sys->b, sys->load.as<double>(), sys->res.as<double>(), ctx->stream));
      launched(ctx);
    }
    if (sys->has_bc) {
      BcArgs a{};
      a.n = sys->n;
      a.nnz = sys->nnz;
      a.b = sys->b;
      a.rowptr = sys->rowptr.as<int>();
      a.colind = sys->colind.as<int>();
      a.flag = sys->bcflag.as<int>();
      a.diag = sys->diag.as<double>();
      a.offd = sys->offd.as<double>();
      a.res = sys->res.as<double>();
      CK(launch_bc(a, ctx->stream));
      launched(ctx, 2);
    }
    const size_t m = (size_t)sys->n * sys->b;
    dalloc(ctx, sys->rhs0, vec_bytes(sys, 8));
    CK(cudaMemcpyAsync(sys->rhs0.p, sys->res.p, m * 8, cudaMemcpyDeviceToDevice, ctx->stream));
    sys->rhs0_valid = true;
    sys->mat32_valid = false;
    ++sys->mat_version;
    Red r = red_of(ctx, 0);
    CK(api_dot((long long)m, sys->res.as<double>(), sys->res.as<double>(), r, ctx->stream));
    launched(ctx);
    double s = 0.0;
    CK(cudaMemcpyAsync(&s, r.result, 8, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (norm_res) *norm_res = std::sqrt(s);
    return DFG_OK;
  });
}

extern "C" int dfg_get_matrix(dfg_system sys, double* diag, double* offd) {
  if (!sys) return DFG_INVALID_ARGUMENT;
  dfg_ctx ctx = sys->ctx;
  return guarded(ctx, [&]() -> int {
    dfg_ctx ctx_ = ctx;
    const size_t bs = (size_t)sys->b * sys->b;
    if (diag) CK(cudaMemcpyAsync(diag, sys->diag.p, (size_t)sys->n * bs * 8, cudaMemcpyDeviceToHost, ctx->stream));
    if (offd && sys->nnz) CK(cudaMemcpyAsync(offd, sys->offd.p, (size_t)sys->nnz * bs * 8, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return DFG_OK;
  });
}

extern "C" int dfg_set_matrix(dfg_system sys, const double* diag, const double* offd) {
  if (!sys) return DFG_INVALID_ARGUMENT;
  dfg_ctx ctx = sys->ctx;
  return guarded(ctx, [&]() -> int {
    dfg_ctx ctx_ = ctx;
    const size_t bs = (size_t)sys->b * sys->b;
    if (diag) CK(cudaMemcpyAsync(sys->diag.p, diag, (size_t)sys->n * bs * 8, cudaMemcpyHostToDevice, ctx->stream));
    if (offd && sys->nnz) CK(cudaMemcpyAsync(sys->offd.p, offd, (size_t)sys->nnz * bs * 8, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    sys->mat32_valid = false;
    ++sys->mat_version;
    return DFG_OK;
  });
}

extern "C" int dfg_get_vector(dfg_system sys, int iv, double* out) {
  if (!sys || !out) return DFG_INVALID_ARGUMENT;
  dfg_ctx ctx = sys->ctx;
  return guarded(ctx, [&]() -> int {
    dfg_ctx ctx_ = ctx;
    double* p = vec_ptr(ctx, sys, iv);
    CK(cudaMemcpyAsync(out, p, (size_t)sys->n * sys->b * 8, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return DFG_OK;
  });
}

extern "C" int dfg_set_vector(dfg_system sys, int iv, const double* in) {
  if (!sys || !in) return DFG_INVALID_ARGUMENT;
  dfg_ctx ctx = sys->ctx;
  return guarded(ctx, [&]() -> int {
    dfg_ctx ctx_ = ctx;
    double* p = vec_ptr(ctx, sys, iv);
    CK(cudaMemcpyAsync(p, in, (size_t)sys->n * sys->b * 8, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return DFG_OK;
  });
}

// ============================================================ solver interface

extern "C" int dfg_get_tmp_vector_size(dfg_system sys, unsigned* size) {
  if (!sys || !size) return DFG_INVALID_ARGUMENT;
  *size = (unsigned)sys->tmp.size();
  return DFG_OK;
}

extern "C" int dfg_resize_tmp_vec(dfg_system sys, unsigned size) {
  if (!sys) return DFG_INVALID_ARGUMENT;
  dfg_ctx ctx = sys->ctx;
  return guarded(ctx, [&]() -> int {
    dfg_ctx ctx_ = ctx;
    while (sys->tmp.size() > size) sys->tmp.pop_back();
    while (sys->tmp.size() < size) {
      sys->tmp.emplace_back();
      dalloc(ctx, sys->tmp.back(), vec_bytes(sys, 8));
      CK(cudaMemsetAsync(sys->tmp.back().p, 0, sys->tmp.back().bytes, ctx->stream));
    }
    return DFG_OK;
  });
}

extern "C" int dfg_dot(dfg_system sys, int iv1, int iv2, double* out) {
  if (!sys || !out) return DFG_INVALID_ARGUMENT;
  dfg_ctx ctx = sys->ctx;
  return guarded(ctx, [&]() -> int {
    dfg_ctx ctx_ = ctx;
    const double* a = vec_ptr(ctx, sys, iv1);
    const double* b = vec_ptr(ctx, sys, iv2);
    Red r = red_of(ctx, 0);
    CK(api_dot((long long)sys->n * sys->b, a, b, r, ctx->stream));
    launched(ctx);
    CK(cudaMemcpyAsync(out, r.result, 8, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return DFG_OK;
  });
}

extern "C" int dfg_copy(dfg_system sys, int iv1, int iv2) {
  if (!sys) return DFG_INVALID_ARGUMENT;
  if (iv1 == iv2) return DFG_OK;
  dfg_ctx ctx = sys->ctx;
  return guarded(ctx, [&]() -> int {
    dfg_ctx ctx_ = ctx;
    const double* a = vec_ptr(ctx, sys, iv1);
    double* b = vec_ptr(ctx, sys, iv2);
    CK(cudaMemcpyAsync(b, a, (size_t)sys->n * sys->b * 8, cudaMemcpyDeviceToDevice, ctx->stream));
    return DFG_OK;
  });
}

extern "C" int dfg_scal(dfg_system sys, double alpha, int iv1) {
  if (!sys) return DFG_INVALID_ARGUMENT;
  dfg_ctx ctx = sys->ctx;
  return guarded(ctx, [&]() -> int {
    dfg_ctx ctx_ = ctx;
    CK(api_scal((long long)sys->n * sys->b, alpha, vec_ptr(ctx, sys, iv1), ctx->stream));
    launched(ctx);
    return DFG_OK;
  });
}

extern "C" int dfg_axpy(dfg_system sys, double alpha, int iv1, int iv2) {
  if (!sys) return DFG_INVALID_ARGUMENT;
  dfg_ctx ctx = sys->ctx;
  return guarded(ctx, [&]() -> int {
    dfg_ctx ctx_ = ctx;
    if (alpha == 0) return DFG_OK;  // CLinearSystem::AXPY returns early
    REQUIRE(iv1 != iv2, DFG_INVALID_ARGUMENT, "AXPY on one slot (the reference asserts)");
    CK(api_axpy((long long)sys->n * sys->b, alpha, vec_ptr(ctx, sys, iv1), vec_ptr(ctx, sys, iv2), ctx->stream));
    launched(ctx);
    return DFG_OK;
  });
}

extern "C" int dfg_matvec(dfg_system sys, double alpha, int iv1, double beta, int iv2) {
  if (!sys) return DFG_INVALID_ARGUMENT;
  dfg_ctx ctx = sys->ctx;
  return guarded(ctx, [&]() -> int {
    dfg_ctx ctx_ = ctx;
    double* y = vec_ptr(ctx, sys, iv2);
    if (alpha == 0.0) {  // CLinearSystem::MATVEC -> SCAL(beta, iv2)
      CK(api_scal((long long)sys->n * sys->b, beta, y, ctx->stream));
      launched(ctx);
      return DFG_OK;
    }
    REQUIRE(iv1 != iv2, DFG_INVALID_ARGUMENT, "MATVEC on one slot (the reference asserts)");
    CK(api_matvec(view64(sys), alpha, vec_ptr(ctx, sys, iv1), beta, y, ctx->stream));
    launched(ctx);
    return DFG_OK;
  });
}

// =============================================================== preconditioner

namespace {

void build_records(dfg_ctx ctx_, SweepDev& S, int elem, DBuf& rec, DBuf& rec_off, long long& total, long long& max_rec) {
  std::vector<long long> off;
  const std::vector<unsigned char> h = pack_record_headers(S.plan, elem, off, max_rec);
  total = off.back();
  upload(ctx_, rec, h.data(), h.size(), 64);
  upload(ctx_, rec_off, off.data(), off.size());
}

void setup_sweep_plan(dfg_ctx ctx_, SweepDev& S) {
  const SweepPlan& P = S.plan;
  build_records(ctx_, S, 8, S.rec64, S.rec_off64, S.rec_total64, S.max_rec64);
  build_records(ctx_, S, 4, S.rec32, S.rec_off32, S.rec_total32, S.max_rec32);
  upload(ctx_, S.range_steps, P.range_steps.data(), P.range_steps.size());
  upload(ctx_, S.ent_off, P.ent_off.data(), P.ent_off.size());
  upload(ctx_, S.ent_slot, P.ent_slot.data(), std::max<size_t>(P.ent_slot.size(), 1));
  upload(ctx_, S.step_rows, P.step_rows.data(), std::max<size_t>(P.step_rows.size(), 1));
}

void pack_sweep(dfg_ctx ctx_, dfg_precond pr, SweepDev& S, bool fp32) {
  if (S.levels) return;  // the level-scheduled sweep reads the factor itself
  if (S.solo) {
    SweepDev::SoloDev& D = S.sd[fp32 ? 1 : 0];
    PackArgs a{};
    a.nsteps = D.plan.P.nsteps;
    a.rec = D.rec.as<unsigned char>();
    a.rec_off = D.rec_off.as<long long>();
    a.ent_off = D.ent_off.as<long long>();
    a.ent_slot = D.ent_slot.as<int>();
    a.step_rows = D.step_rows.as<int>();
    a.fdiag = pr->fdiag.as<double>();
    a.foffd = pr->foffd.as<double>();
    a.code_bytes = 128;
    CK(launch_pack(S.forward, fp32, pr->b, a, ctx_->stream));
    launched(ctx_);
    return;
  }
  PackArgs a{};
  a.nsteps = S.plan.nsteps;
  a.rec = fp32 ? S.rec32.as<unsigned char>() : S.rec64.as<unsigned char>();
  a.rec_off = fp32 ? S.rec_off32.as<long long>() : S.rec_off64.as<long long>();
  a.ent_off = S.ent_off.as<long long>();
  a.ent_slot = S.ent_slot.as<int>();
  a.step_rows = S.step_rows.as<int>();
  a.fdiag = pr->fdiag.as<double>();
  a.foffd = pr->foffd.as<double>();
  CK(launch_pack(S.plan.forward, fp32, pr->b, a, ctx_->stream));
  launched(ctx_);
}

struct SweepLaunch {
  bool forward = true, fp32 = false;
  int b = 1;
  // ranged
  SweepArgs args;
  int grid = 0;
  size_t smem = 0;
  // level-scheduled
  bool levels = false;
  const Levels* lev = nullptr;
  LevelSweepArgs la{};
  // one CTA: permute `src` (row order) into the plan's step order, then the sweep
  bool solo = false;
  SoloArgs sa{};
  size_t ssmem = 0;
  long long sn = 0;
  const int* spos = nullptr;
  const void* ssrc = nullptr;
  void* sdst = nullptr;
};

// The factor's block pattern: the system's for ILU(0), the preconditioner's
// own when fill-in changed it.
struct FactorPattern {
  const int *rowptr, *colind, *diaind;        // host
  const int *d_rowptr, *d_colind, *d_diaind;  // device
};
FactorPattern factor_pattern(dfg_precond pr) {
  if (pr->own_pattern)
    return {pr->h_rowptr.data(), pr->h_colind.data(), pr->h_diaind.data(),
            pr->rowptr.as<int>(), pr->colind.as<int>(), pr->diaind.as<int>()};
  const dfg_system s = pr->sys;
  return {s->h_rowptr.data(), s->h_colind.data(), s->h_diaind.data(),
          s->rowptr.as<int>(), s->colind.as<int>(), s->diaind.as<int>()};
}

constexpr int kSoloBatchRing = 8;  // single-slot batches kept per sweep (a BiCGSTAB solve uses two)

// A single-slot batch for the one-CTA sweep of S writing `out`, in the next
// entry of S's batch ring (uploaded in stream order), and its launch args.
SoloArgs solo_launch_args(dfg_ctx ctx_, SweepDev& S, bool fp32, void* out, int* ticket, const int* done) {
  const SweepDev::SoloDev& D = S.sd[fp32 ? 1 : 0];
  if (!S.solo_batch.p) dalloc(ctx_, S.solo_batch, sizeof(SoloBatch) * kSoloBatchRing);
  SoloBatch* dev = S.solo_batch.as<SoloBatch>() + (S.solo_next++ % kSoloBatchRing);
  SoloBatch h{};
  h.nslots = 1;
  SoloSlot& w = h.slot[0];
  w.rec = D.rec.as<unsigned char>();
  w.chunks = D.chunks.as<SoloChunk>();
  w.lev_chunks = D.lev_chunks.as<int>();
  w.nlevels = D.plan.P.nranges;
  w.nchunks = (int)D.plan.chunks.size();
  w.in = S.solo_in.p;
  w.out = out;
  w.done = done;
  const size_t head = offsetof(SoloBatch, slot) + sizeof(SoloSlot);
  CK(cudaMemcpyAsync(dev, &h, head, cudaMemcpyHostToDevice, ctx_->stream));
  CK(cudaStreamSynchronize(ctx_->stream));  // h is on this frame
  SoloArgs a{};
  a.batch = dev;
  a.ticket = ticket;
  a.err = ctx_->err_word.as<int>();
  a.rec_stage = D.shape.rec_stage;
  a.ch_max = D.shape.ch_max;
  a.NS = D.shape.ns;
  a.R = D.shape.R;
  a.max_nent = D.plan.P.max_nent;
  return a;
}

// Builds the one-CTA sweep of one direction for both precisions into S (plans,
// record headers, chunk tables, packing indices, the row -> position map);
// false when its stages do not fit in shared memory.
bool setup_solo(dfg_ctx ctx_, dfg_precond pr, SweepDev& S, const FactorPattern& F, bool forward) {
  const int n = pr->n, b = pr->b;
  if (n == 0) return false;
  int maxe = 0;
  for (int i = 0; i < n; ++i)
    maxe = std::max(maxe, forward ? F.diaind[i] - F.rowptr[i] : F.rowptr[i + 1] - F.diaind[i]);
  int per_sm = 0;
  cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, ctx_->device);
  const size_t budget = std::min<size_t>(ctx_->smem_optin, (size_t)per_sm) - 4096;
  std::vector<int> ident(n);
  for (int i = 0; i < n; ++i) ident[i] = i;
  for (int k = 0; k < 2; ++k) {
    const int elem = k ? 4 : 8;
    SweepDev::SoloDev& D = S.sd[k];
    D.shape = solo_shape(b, maxe, elem, forward, budget);
    if (D.shape.ns < 2 || D.shape.smem > ctx_->smem_optin) return false;
    D.plan = solo_sweep_plan(n, b, F.rowptr, F.colind, F.diaind, forward, D.shape.R, elem, D.shape.rec_stage,
                             D.shape.ch_max);
    std::vector<long long> off;
    const std::vector<unsigned char> h = pack_solo_headers(D.plan, elem, ident.data(), ident.data(), off);
    const SweepPlan& P = D.plan.P;
    upload(ctx_, D.rec, h.data(), std::max<size_t>(h.size(), 1), 64);
    upload(ctx_, D.rec_off, off.data(), off.size());
    upload(ctx_, D.chunks, D.plan.chunks.data(), std::max<size_t>(D.plan.chunks.size(), 1));
    upload(ctx_, D.lev_chunks, D.plan.lev_chunks.data(), D.plan.lev_chunks.size());
    upload(ctx_, D.ent_off, P.ent_off.data(), P.ent_off.size());
    upload(ctx_, D.ent_slot, P.ent_slot.data(), std::max<size_t>(P.ent_slot.size(), 1));
    upload(ctx_, D.step_rows, P.step_rows.data(), std::max<size_t>(P.step_rows.size(), 1));
  }
  upload(ctx_, S.solo_pos, S.sd[0].plan.pos.data(), std::max<size_t>(S.sd[0].plan.pos.size(), 1));
  dalloc(ctx_, S.solo_in, (size_t)std::max(S.sd[0].plan.P.nsteps, 1) * 32 * b * 8 + 64);
  CK(cudaMemsetAsync(S.solo_in.p, 0, S.solo_in.bytes, ctx_->stream));
  S.solo_maxe = maxe;
  CK(solo_set_smem_limits(ctx_->smem_optin));
  return true;
}

SweepLaunch sweep_launch(dfg_ctx ctx_, dfg_precond pr, SweepDev& S, bool fp32, const void* in, void* out,
                         int* ticket, const int* done) {
  const int elem = fp32 ? 4 : 8;
  SweepLaunch L{};
  L.forward = S.forward;
  L.fp32 = fp32;
  L.b = pr->b;
  if (S.levels) {
    const FactorPattern F = factor_pattern(pr);
    L.levels = true;
    L.lev = &S.lev;
    L.la = LevelSweepArgs{S.lev_info.as<int4>(), F.d_colind, fp32 ? pr->fdiag32.p : pr->fdiag.p,
                          fp32 ? pr->foffd32.p : pr->foffd.p, in, out, done, S.lev_G};
    return L;
  }
  if (S.solo) {
    L.solo = true;
    L.sa = solo_launch_args(ctx_, S, fp32, out, ticket, done);
    L.ssmem = S.sd[fp32 ? 1 : 0].shape.smem;
    L.sn = pr->n;
    L.spos = S.solo_pos.as<int>();
    L.ssrc = in;
    L.sdst = S.solo_in.p;
    return L;
  }
  SweepArgs& a = L.args;
  a.rec = fp32 ? S.rec32.as<unsigned char>() : S.rec64.as<unsigned char>();
  a.rec_off = fp32 ? S.rec_off32.as<long long>() : S.rec_off64.as<long long>();
  a.range_steps = S.range_steps.as<int>();
  a.nranges = S.plan.nranges;
  a.in = in;
  a.out = out;
  a.ticket = ticket;
  a.err = ctx_->err_word.as<int>();
  a.done = done;
  a.rec_stage = (int)((fp32 ? S.max_rec32 : S.max_rec64) + 15) / 16 * 16;
  a.val_stage = sweep_val_stage(S.plan.max_nent, pr->b, elem);
  a.R = S.plan.R;
  a.max_nent = S.plan.max_nent;
  // pipeline depth: as deep as 16 stages while the CTA fits in ~200 KB
  const size_t budget = std::min<size_t>(ctx_->smem_optin, 200 * 1024);
  int NS = 16;
  while (NS > 2 && sweep_smem_bytes(NS, a.rec_stage, a.val_stage, a.R, pr->b, elem) > budget) --NS;
  a.NS = NS;
  L.smem = sweep_smem_bytes(NS, a.rec_stage, a.val_stage, a.R, pr->b, elem);
  REQUIRE(L.smem <= ctx_->smem_optin, DFG_INVALID_ARGUMENT, "sweep records exceed shared memory");
  int per_sm_bytes = 0;
  cudaDeviceGetAttribute(&per_sm_bytes, cudaDevAttrMaxSharedMemoryPerMultiprocessor, ctx_->device);
  int per_sm = std::max(1, std::min(16, (int)(per_sm_bytes / (L.smem + 1024))));
  L.grid = std::max(1, std::min(S.plan.nranges, ctx_->nsm * per_sm));
  return L;
}

// Launches one sweep on stream st (no error check and no launch count, so
// that it can be captured into a graph); the ranged kernel or one launch per
// level.  dep: the ranged kernel as a programmatic dependent of the previous
// kernel in the stream (a level sweep's first launch always waits in stream
// order: it reads the solve's stop flag before waiting).
cudaError_t enqueue_sweep(const SweepLaunch& L, cudaStream_t st, bool dep = false) {
  if (L.solo) {
    const cudaError_t e = launch_solo_permute(L.fp32, L.sn, L.b, L.spos, L.ssrc, L.sdst, st);
    if (e != cudaSuccess) return e;
    return launch_solo(L.forward, L.fp32, L.b, L.sa, 1, L.ssmem, st);
  }
  if (!L.levels) return launch_sweep(L.forward, L.fp32, L.b, L.args, L.grid, L.smem, st, dep);
  const Levels& V = *L.lev;
  for (size_t l = 0; l + 1 < V.ptr.size(); ++l) {
    const cudaError_t e = launch_sweep_level(L.forward, L.fp32, L.b, L.la, V.ptr[l], V.ptr[l + 1] - V.ptr[l], l > 0, st);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}
long long launches_of(const SweepLaunch& L) {
  return L.solo ? 2 : L.levels ? (long long)L.lev->ptr.size() - 1 : 1;
}

void run_sweep(dfg_ctx ctx_, const SweepLaunch& L) {
  CK(enqueue_sweep(L, ctx_->stream));
  launched(ctx_, launches_of(L));
}

struct GraphHolder {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  ~GraphHolder() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
  }
};

// Schedule choice.  Ranged: the cost model keeps a few candidate range sizes
// and the fullest-step plan joins them.  Level-scheduled: one launch per
// dependency level.  Each candidate is timed on the device as one FP32 sweep
// of the real structure (values do not change the timing; the level launches
// as a graph, as the solvers replay them) and the fastest wins.  The
// preconditioner's sweep mode can restrict the choice to one kind.
void setup_sweep(dfg_ctx ctx_, dfg_precond pr, SweepDev& S, const dfg_system sys, bool forward) {
  const FactorPattern F = factor_pattern(pr);
  const int mode = pr->sweep_mode;
  const long long m = (long long)sys->n * sys->b;
  S.forward = forward;
  S.levels = false;
  S.t_ranged = S.t_levels = -1.f;
  DBuf vin, vout;
  dalloc(ctx_, vin, (size_t)m * 4 + 64);
  dalloc(ctx_, vout, (size_t)m * 4 + 64);
  CK(cudaMemsetAsync(vin.p, 0, vin.bytes, ctx_->stream));
  Scratch sc = scratch_of(ctx_);
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  struct EventPair {
    cudaEvent_t a, b;
    ~EventPair() { cudaEventDestroy(a); cudaEventDestroy(b); }
  } ev{e0, e1};
  auto elapsed = [&](auto&& run) {
    float best = 1e30f;
    for (int rep = 0; rep < 2; ++rep) {
      CK(cudaEventRecord(e0, ctx_->stream));
      run();
      CK(cudaEventRecord(e1, ctx_->stream));
      CK(cudaEventSynchronize(e1));
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, e0, e1));
      best = std::min(best, ms);
    }
    return best;
  };
  // ranged candidates
  std::vector<SweepPlan> cands;
  size_t best = 0;
  float best_ms = 1e30f;
  if (mode != 2) {
    cands = candidate_sweep_plans(sys->n, sys->b, F.rowptr, F.colind, F.diaind, forward, 32, 4);
    // and the fullest-step plan (ranges of up to 32 grid lines), if it differs
    SweepPlan full = fullest_sweep_plan(sys->n, sys->b, F.rowptr, F.colind, F.diaind, forward, 32);
    bool seen = false;
    for (const SweepPlan& c : cands) seen |= (c.nranges == full.nranges && c.nsteps == full.nsteps);
    if (!seen) cands.push_back(std::move(full));
    if (cands.size() > 1 || mode == 0) {
      for (size_t c = 0; c < cands.size(); ++c) {
        SweepDev T;
        T.forward = forward;
        T.plan = std::move(cands[c]);
        // the uploaded records carry the real headers and dependency codes; their
        // value regions are zero (no factor packed), which does not change the timing
        build_records(ctx_, T, 4, T.rec32, T.rec_off32, T.rec_total32, T.max_rec32);
        upload(ctx_, T.range_steps, T.plan.range_steps.data(), T.plan.range_steps.size());
        SweepLaunch L = sweep_launch(ctx_, pr, T, true, vin.p, vout.p, sc.tickets + 2, nullptr);
        const float ms = elapsed([&] {
          CK(fill_sentinel(m, vout.p, true, ctx_->stream));
          CK(cudaMemsetAsync(sc.tickets + 2, 0, sizeof(int), ctx_->stream));
          CK(enqueue_sweep(L, ctx_->stream));
        });
        launched(ctx_, 4);
        if (ms < best_ms) { best_ms = ms; best = c; }
        cands[c] = std::move(T.plan);
      }
      if (read_err(ctx_) != 0) {
        CK(cudaMemsetAsync(ctx_->err_word.p, 0, sizeof(int), ctx_->stream));
        set_err(ctx_, "a triangular-sweep wait timed out while choosing the schedule");
        throw Fail{DFG_TIMEOUT};
      }
      S.t_ranged = best_ms;
    }
  }
  // one-CTA candidate (k_solo.cu), timed in FP32 with its input permutation
  S.solo = false;
  S.t_solo = -1.f;
  if (mode == 0 || mode == 3) {
    const bool fits = setup_solo(ctx_, pr, S, F, forward);
    REQUIRE(fits || mode != 3, DFG_INVALID_ARGUMENT, "the one-CTA sweep's records do not fit in shared memory");
    if (fits) {
      S.solo = true;
      SweepLaunch L = sweep_launch(ctx_, pr, S, true, vin.p, vout.p, sc.tickets + 2, nullptr);
      const float ms = elapsed([&] {
        CK(cudaMemsetAsync(sc.tickets + 2, 0, sizeof(int), ctx_->stream));
        CK(enqueue_sweep(L, ctx_->stream));
      });
      launched(ctx_, 4);
      if (read_err(ctx_) != 0) {
        CK(cudaMemsetAsync(ctx_->err_word.p, 0, sizeof(int), ctx_->stream));
        set_err(ctx_, "a triangular-sweep wait timed out while choosing the schedule");
        throw Fail{DFG_TIMEOUT};
      }
      S.t_solo = ms;
      if (mode == 3 || ms < best_ms) {
        best_ms = ms;
      } else {
        S.solo = false;
        for (SweepDev::SoloDev& D : S.sd) D = SweepDev::SoloDev{};
        S.solo_pos.release();
        S.solo_in.release();
      }
    }
  }
  // level-scheduled candidate
  if (mode != 1 && mode != 3) {
    Levels V = build_levels(sys->n, F.rowptr, F.colind, F.diaind, forward);
    // per position: the row and its entry range in this direction
    std::vector<int4> info(std::max<size_t>(V.rows.size(), 1), make_int4(0, 0, 0, 0));
    int widest = 0;
    for (size_t k = 0; k < V.rows.size(); ++k) {
      const int row = V.rows[k];
      const int c0 = forward ? F.rowptr[row] : F.diaind[row];
      const int c1 = forward ? F.diaind[row] : F.rowptr[row + 1];
      info[k] = make_int4(row, c0, c1, 0);
      widest = std::max(widest, c1 - c0);
    }
    const int G = level_group_lanes(widest);
    DBuf rows;
    upload(ctx_, rows, info.data(), info.size());
    bool take = mode == 2 || V.ptr.size() <= 1;  // no rows: nothing to launch or time
    if (!take) {
      const size_t bs = (size_t)sys->b * sys->b;
      DBuf zd, zo;
      dalloc(ctx_, zd, (size_t)sys->n * bs * 4 + 64);
      dalloc(ctx_, zo, (size_t)std::max<long long>(pr->nnz, 1) * bs * 4 + 64);
      CK(cudaMemsetAsync(zd.p, 0, zd.bytes, ctx_->stream));
      CK(cudaMemsetAsync(zo.p, 0, zo.bytes, ctx_->stream));
      SweepLaunch L{};
      L.forward = forward;
      L.fp32 = true;
      L.b = sys->b;
      L.levels = true;
      L.lev = &V;
      L.la = LevelSweepArgs{rows.as<int4>(), F.d_colind, zd.p, zo.p, vin.p, vout.p, nullptr, G};
      GraphHolder g;
      CK(cudaStreamBeginCapture(ctx_->stream, cudaStreamCaptureModeThreadLocal));
      const cudaError_t ce = enqueue_sweep(L, ctx_->stream);
      CK(cudaStreamEndCapture(ctx_->stream, &g.graph));
      CK(ce);
      CK(cudaGraphInstantiate(&g.exec, g.graph, 0));
      CK(cudaGraphLaunch(g.exec, ctx_->stream));  // first replay uploads the graph
      const float ms = elapsed([&] { CK(cudaGraphLaunch(g.exec, ctx_->stream)); });
      launched(ctx_, 3 * launches_of(L));
      S.t_levels = ms;
      take = ms < best_ms;
    }
    if (take) {
      S.levels = true;
      S.solo = false;
      for (SweepDev::SoloDev& D : S.sd) D = SweepDev::SoloDev{};
      S.solo_pos.release();
      S.solo_in.release();
      S.lev = std::move(V);
      S.lev_info = std::move(rows);
      S.lev_G = G;
      S.plan = SweepPlan{};
      return;
    }
  }
  if (S.solo) {
    S.plan = SweepPlan{};
    return;
  }
  S.plan = std::move(cands[best]);
  setup_sweep_plan(ctx_, S);
}

}  // namespace

extern "C" int dfg_precond_create(dfg_ctx ctx, dfg_precond* out) {
  if (!ctx || !out) return DFG_INVALID_ARGUMENT;
  dfg_precond p = new (std::nothrow) dfg_precond_s;
  if (!p) return DFG_OOM_REJECTED;
  p->ctx = ctx;
  *out = p;
  return DFG_OK;
}

extern "C" int dfg_precond_destroy(dfg_precond prec) {
  if (!prec) return DFG_INVALID_ARGUMENT;
  cudaSetDevice(prec->ctx->device);
  cudaStreamSynchronize(prec->ctx->stream);
  delete prec;
  return DFG_OK;
}

extern "C" int dfg_precond_set_fill_level(dfg_precond prec, int lev) {
  if (!prec) return DFG_INVALID_ARGUMENT;
  if (lev < -1) {
    prec->ctx->last_error = "fill-in level must be >= -1 (-1: no limit)";
    return DFG_INVALID_ARGUMENT;
  }
  prec->lev = lev;
  return DFG_OK;
}

extern "C" int dfg_precond_set_sweep_mode(dfg_precond prec, int mode) {
  if (!prec) return DFG_INVALID_ARGUMENT;
  if (mode < 0 || mode > 3) {
    prec->ctx->last_error =
        "sweep mode must be 0 (timed choice), 1 (ranged), 2 (level-scheduled) or 3 (one CTA)";
    return DFG_INVALID_ARGUMENT;
  }
  prec->sweep_mode = mode;
  return DFG_OK;
}

extern "C" int dfg_precond_get_sweep_mode(dfg_precond prec, int* fwd, int* bwd) {
  if (!prec) return DFG_INVALID_ARGUMENT;
  if (!prec->symbolic) {
    prec->ctx->last_error = "dfg_precond_set_linear_system must come first";
    return DFG_NOT_READY;
  }
  if (fwd) *fwd = prec->fwd.solo ? 3 : prec->fwd.levels ? 2 : 1;
  if (bwd) *bwd = prec->bwd.solo ? 3 : prec->bwd.levels ? 2 : 1;
  return DFG_OK;
}

extern "C" int dfg_precond_get_sweep_timing(dfg_precond prec, float* ms) {
  if (!prec || !ms) return DFG_INVALID_ARGUMENT;
  if (!prec->symbolic) {
    prec->ctx->last_error = "dfg_precond_set_linear_system must come first";
    return DFG_NOT_READY;
  }
  ms[0] = prec->fwd.t_ranged;
  ms[1] = prec->fwd.t_levels;
  ms[2] = prec->bwd.t_ranged;
  ms[3] = prec->bwd.t_levels;
  return DFG_OK;
}

extern "C" int dfg_precond_get_solo_timing(dfg_precond prec, float* ms) {
  if (!prec || !ms) return DFG_INVALID_ARGUMENT;
  if (!prec->symbolic) {
    prec->ctx->last_error = "dfg_precond_set_linear_system must come first";
    return DFG_NOT_READY;
  }
  ms[0] = prec->fwd.t_solo;
  ms[1] = prec->bwd.t_solo;
  return DFG_OK;
}

extern "C" int dfg_precond_set_linear_system(dfg_precond prec, dfg_system sys) {
  if (!prec || !sys) return DFG_INVALID_ARGUMENT;
  dfg_ctx ctx = prec->ctx;
  return guarded(ctx, [&]() -> int {
    dfg_ctx ctx_ = ctx;
    REQUIRE(sys->ctx == ctx, DFG_INVALID_ARGUMENT, "system and preconditioner belong to different contexts");
    prec->sys = sys;
    prec->n = sys->n;
    prec->b = sys->b;
    prec->symbolic = prec->numeric = prec->numeric32 = false;
    // fill-in (CPreconditioner_ILU::SetLinearSystem -> AddFracPtn)
    prec->own_pattern = false;
    prec->h_rowptr.clear(); prec->h_colind.clear(); prec->h_diaind.clear();
    prec->rowptr.release(); prec->colind.release(); prec->diaind.release(); prec->a2f.release();
    if (prec->lev != 0) {
      std::vector<int> rp, ci;
      REQUIRE(ilu_fill_pattern(sys->n, sys->h_rowptr.data(), sys->h_colind.data(), prec->lev, rp, ci, INT32_MAX - 1),
              DFG_INVALID_ARGUMENT, "the ILU fill-in pattern exceeds 2^31 blocks");
      if ((long long)ci.size() != sys->nnz) {
        std::vector<int> a2f;
        REQUIRE(factor_slot_map(sys->n, sys->h_rowptr.data(), sys->h_colind.data(), rp.data(), ci.data(), a2f),
                DFG_INVALID_ARGUMENT, "the fill-in pattern does not contain the matrix pattern");
        prec->h_diaind.resize(sys->n);
        for (int i = 0; i < sys->n; ++i) {
          int d = rp[i + 1];
          for (int c = rp[i]; c < rp[i + 1]; ++c)
            if (ci[c] > i) { d = c; break; }
          prec->h_diaind[i] = d;
        }
        prec->h_rowptr = std::move(rp);
        prec->h_colind = std::move(ci);
        upload(ctx, prec->rowptr, prec->h_rowptr.data(), prec->h_rowptr.size());
        upload(ctx, prec->colind, prec->h_colind.data(), std::max<size_t>(prec->h_colind.size(), 1));
        upload(ctx, prec->diaind, prec->h_diaind.data(), prec->h_diaind.size());
        upload(ctx, prec->a2f, a2f.data(), std::max<size_t>(a2f.size(), 1));
        prec->own_pattern = true;
      }
    }
    const FactorPattern F = factor_pattern(prec);
    prec->nnz = F.rowptr[sys->n];
    const size_t bs = (size_t)sys->b * sys->b;
    dalloc(ctx, prec->fdiag, (size_t)sys->n * bs * 8);
    dalloc(ctx, prec->foffd, (size_t)std::max<long long>(prec->nnz, 1) * bs * 8);
    prec->lev_fwd = build_levels(sys->n, F.rowptr, F.colind, F.diaind, true);
    upload(ctx, prec->lev_rows, prec->lev_fwd.rows.data(), std::max<size_t>(prec->lev_fwd.rows.size(), 1));
    setup_sweep(ctx, prec, prec->fwd, sys, true);
    setup_sweep(ctx, prec, prec->bwd, sys, false);
    dalloc(ctx, prec->ybuf64, vec_bytes(sys, 8));
    dalloc(ctx, prec->ybuf32, vec_bytes(sys, 4));
    CK(cudaStreamSynchronize(ctx->stream));
    prec->symbolic = true;
    prec->numeric = prec->numeric32 = false;
    return DFG_OK;
  });
}

extern "C" int dfg_precond_set_value(dfg_precond prec, dfg_system sys) {
  if (!prec || !sys) return DFG_INVALID_ARGUMENT;
  dfg_ctx ctx = prec->ctx;
  return guarded(ctx, [&]() -> int {
    dfg_ctx ctx_ = ctx;
    REQUIRE(prec->symbolic && prec->sys == sys, DFG_NOT_READY, "dfg_precond_set_linear_system must come first");
    const size_t bs = (size_t)sys->b * sys->b;
    // SetValue_Initialize: copy A into the factor storage (zero at fill-in)
    CK(cudaMemcpyAsync(prec->fdiag.p, sys->diag.p, (size_t)sys->n * bs * 8, cudaMemcpyDeviceToDevice, ctx->stream));
    if (prec->own_pattern) {
      CK(cudaMemsetAsync(prec->foffd.p, 0, (size_t)prec->nnz * bs * 8, ctx->stream));
      CK(launch_factor_init(sys->b, sys->nnz, prec->a2f.as<int>(), sys->offd.as<double>(), prec->foffd.as<double>(),
                            ctx->stream));
      launched(ctx);
    } else if (sys->nnz) {
      CK(cudaMemcpyAsync(prec->foffd.p, sys->offd.p, (size_t)sys->nnz * bs * 8, cudaMemcpyDeviceToDevice, ctx->stream));
    }
    const FactorPattern F = factor_pattern(prec);
    Scratch sc = scratch_of(ctx);
    int* nsing = sc.tickets + 8;
    CK(cudaMemsetAsync(nsing, 0, sizeof(int), ctx->stream));
    const Levels& L = prec->lev_fwd;
    const int nl = (int)L.ptr.size() - 1;
    for (int l = 0; l < nl; ++l)
      CK(launch_ilu_level(sys->b, prec->lev_rows.as<int>() + L.ptr[l], L.ptr[l + 1] - L.ptr[l], F.d_rowptr,
                          F.d_colind, F.d_diaind, prec->fdiag.as<double>(), prec->foffd.as<double>(), nsing,
                          ctx->stream, l > 0));
    launched(ctx, nl);
    int h_nsing = 0;
    CK(cudaMemcpyAsync(&h_nsing, nsing, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    pack_sweep(ctx, prec, prec->fwd, false);
    pack_sweep(ctx, prec, prec->bwd, false);
    CK(cudaStreamSynchronize(ctx->stream));
    prec->numeric = true;
    prec->numeric32 = false;
    if (h_nsing > 10) {
      set_err(ctx, "ILU: " + std::to_string(h_nsing) + " singular pivots (more than 10)");
      return DFG_SINGULAR_PIVOT;
    }
    return DFG_OK;
  });
}

namespace {
void ensure_numeric32(dfg_ctx ctx_, dfg_precond prec) {
  if (prec->numeric32) return;
  pack_sweep(ctx_, prec, prec->fwd, true);
  pack_sweep(ctx_, prec, prec->bwd, true);
  if (prec->fwd.levels || prec->bwd.levels) {  // the level-scheduled sweeps read the factor in CRS
    const long long bs = (long long)prec->b * prec->b;
    dalloc(ctx_, prec->fdiag32, (size_t)prec->n * bs * 4 + 64);
    dalloc(ctx_, prec->foffd32, (size_t)std::max<long long>(prec->nnz, 1) * bs * 4 + 64);
    CK(to_fp32((long long)prec->n * bs, prec->fdiag.as<double>(), prec->fdiag32.as<float>(), ctx_->stream));
    CK(to_fp32(prec->nnz * bs, prec->foffd.as<double>(), prec->foffd32.as<float>(), ctx_->stream));
    launched(ctx_, 2);
  }
  prec->numeric32 = true;
}
}  // namespace

extern "C" int dfg_precond_solve(dfg_precond prec, dfg_system sys, int iv) {
  if (!prec || !sys) return DFG_INVALID_ARGUMENT;
  dfg_ctx ctx = prec->ctx;
  return guarded(ctx, [&]() -> int {
    dfg_ctx ctx_ = ctx;
    REQUIRE(prec->numeric && prec->sys == sys, DFG_NOT_READY, "dfg_precond_set_value must come first");
    double* v = vec_ptr(ctx, sys, iv);
    const long long m = (long long)sys->n * sys->b;
    Scratch sc = scratch_of(ctx);
    CK(cudaMemsetAsync(sc.tickets, 0, 2 * sizeof(int), ctx->stream));
    CK(fill_sentinel(m, prec->ybuf64.p, false, ctx->stream));
    SweepLaunch F = sweep_launch(ctx, prec, prec->fwd, false, v, prec->ybuf64.p, sc.tickets, nullptr);
    run_sweep(ctx, F);
    CK(fill_sentinel(m, v, false, ctx->stream));
    SweepLaunch B = sweep_launch(ctx, prec, prec->bwd, false, prec->ybuf64.p, v, sc.tickets + 1, nullptr);
    run_sweep(ctx, B);
    launched(ctx, 2);  // the two sentinel fills
    if (read_err(ctx) != 0) {
      CK(cudaMemsetAsync(ctx->err_word.p, 0, sizeof(int), ctx->stream));
      set_err(ctx, "a triangular-sweep wait timed out");
      return DFG_TIMEOUT;
    }
    return DFG_OK;
  });
}

extern "C" int dfg_precond_get_pattern(dfg_precond prec, long long* nnz, int* rowptr, int* colind) {
  if (!prec) return DFG_INVALID_ARGUMENT;
  if (!prec->symbolic) {
    prec->ctx->last_error = "dfg_precond_set_linear_system must come first";
    return DFG_NOT_READY;
  }
  const FactorPattern F = factor_pattern(prec);
  if (nnz) *nnz = prec->nnz;
  if (rowptr) std::memcpy(rowptr, F.rowptr, sizeof(int) * (size_t)(prec->n + 1));
  if (colind) std::memcpy(colind, F.colind, sizeof(int) * (size_t)prec->nnz);
  return DFG_OK;
}

extern "C" int dfg_precond_get_factor(dfg_precond prec, double* fdiag, double* foffd) {
  if (!prec) return DFG_INVALID_ARGUMENT;
  dfg_ctx ctx = prec->ctx;
  return guarded(ctx, [&]() -> int {
    dfg_ctx ctx_ = ctx;
    REQUIRE(prec->numeric, DFG_NOT_READY, "no numeric factor yet");
    const size_t bs = (size_t)prec->b * prec->b;
    if (fdiag) CK(cudaMemcpyAsync(fdiag, prec->fdiag.p, (size_t)prec->n * bs * 8, cudaMemcpyDeviceToHost, ctx->stream));
    if (foffd && prec->nnz) CK(cudaMemcpyAsync(foffd, prec->foffd.p, (size_t)prec->nnz * bs * 8, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return DFG_OK;
  });
}

// ===================================================================== solvers

namespace {

struct Chunk {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  ~Chunk() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
  }
};

// Reads and clears the error word (code, wait site, slot, range or row) and
// reports the timeout; the context stays usable.
int timeout_status(dfg_ctx ctx_) {
  int w[4] = {0, 0, 0, 0};
  CK(cudaMemcpyAsync(w, ctx_->err_word.p, sizeof(w), cudaMemcpyDeviceToHost, ctx_->stream));
  CK(cudaMemsetAsync(ctx_->err_word.p, 0, sizeof(w), ctx_->stream));
  CK(cudaStreamSynchronize(ctx_->stream));
  set_err(ctx_, "a triangular-sweep wait timed out (site " + std::to_string(w[1]) + ", slot " +
                    std::to_string(w[2]) + ", range/row " + std::to_string(w[3]) + ")");
  ctx_->last_timeout_site = w[1];
  return DFG_TIMEOUT;
}

}  // namespace

extern "C" int dfg_selftest_wait_timeout(dfg_ctx ctx, int* site) {
  if (!ctx) return DFG_INVALID_ARGUMENT;
  return guarded(ctx, [&]() -> int {
    dfg_ctx ctx_ = ctx;
    DBuf never;
    dalloc(ctx, never, 64);
    CK(fill_sentinel(1, never.p, false, ctx->stream));
    CK(launch_wait_selftest(never.as<double>(), ctx->err_word.as<int>(), ctx->stream));
    launched(ctx);
    if (read_err(ctx) == 0) {
      set_err(ctx, "the wait self-test did not time out");
      return DFG_CUDA_ERROR;
    }
    const int st = timeout_status(ctx);
    if (site) *site = ctx->last_timeout_site;
    return st;
  });
}

// FP64-vector PCG with an FP64 or FP32 factor (dfg_solve_pcg / _ex).
static int solve_pcg_f64vec(dfg_system sys, dfg_precond prec, bool fp32z, bool target_true, double* conv_ratio,
                            unsigned* iteration, unsigned* refinements) {
  dfg_ctx ctx = sys->ctx;
  return guarded(ctx, [&]() -> int {
    dfg_ctx ctx_ = ctx;
    REQUIRE(prec->numeric && prec->sys == sys, DFG_NOT_READY, "preconditioner value not set for this system");
    REQUIRE(!target_true || sys->rhs0_valid, DFG_NOT_READY, "dfg_finalize_marge must come before a true-residual solve");
    const long long m = (long long)sys->n * sys->b;
    if (fp32z) ensure_numeric32(ctx, prec);
    dalloc(ctx, sys->w_p, vec_bytes(sys, 8));
    dalloc(ctx, sys->w_q, vec_bytes(sys, 8));
    dalloc(ctx, sys->w_z, vec_bytes(sys, 8));
    dalloc(ctx, sys->w_rd, vec_bytes(sys, 8));
    dalloc(ctx, sys->w_state, sizeof(PcgState));
    if (fp32z) {
      dalloc(ctx, sys->w_r32, vec_bytes(sys, 4));
      dalloc(ctx, sys->w_z32, vec_bytes(sys, 4));
    }
    PcgState* st = sys->w_state.as<PcgState>();
    Scratch sc = scratch_of(ctx);
    Red red = red_of(ctx, 1);
    PcgVecs v{};
    v.r = sys->res.as<double>();
    v.x = sys->upd.as<double>();
    v.p = sys->w_p.as<double>();
    v.q = sys->w_q.as<double>();
    v.y = fp32z ? prec->ybuf32.p : prec->ybuf64.p;
    v.z = fp32z ? sys->w_z32.p : sys->w_z.p;
    v.m = m;
    v.r32 = fp32z ? sys->w_r32.as<float>() : nullptr;
    v.rd = sys->w_rd.as<double>();
    v.b = sys->rhs0_valid ? sys->rhs0.as<double>() : nullptr;
    const int* done = reinterpret_cast<const int*>(reinterpret_cast<const char*>(st) + offsetof(PcgState, done));
    const void* sweep_in = fp32z ? (const void*)v.r32 : (const void*)v.r;
    SweepLaunch F = sweep_launch(ctx, prec, prec->fwd, fp32z, sweep_in, v.y, sc.tickets, done);
    SweepLaunch B = sweep_launch(ctx, prec, prec->bwd, fp32z, v.y, v.z, sc.tickets + 1, done);
    const int maxit = (int)std::min<unsigned>(*iteration, 0x7fffffffu);
    const double tol = *conv_ratio;
    // prologue (solver_ls_iter.cpp:106-128)
    CK(pcg_init(v, st, red, tol, maxit, sc.tickets, fp32z, ctx->stream));
    run_sweep(ctx, F);
    run_sweep(ctx, B);
    CK(pcg_after_precond0(v, st, red, fp32z, ctx->stream));
    launched(ctx, 2);
    PcgState h{};
    read_state(ctx, st, h);
    // iterations: a graph of `chunk` iterations, replayed until done
    const long long per_it = 4 + launches_of(F) + launches_of(B);
    // level-scheduled sweeps put one graph node per level: fewer iterations per graph
    const int chunk = std::max(2, std::min(m < 200000 ? 8 : 32, (int)(4096 / per_it)));
    ensure_sell(ctx, sys, false);
    const MatView A = view64(sys);
    Chunk g;
    CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    for (int c = 0; c < chunk; ++c) {
      // each kernel after the chunk's first starts as a programmatic
      // dependent of the one before: its launch overlaps that kernel, and it
      // waits for it at entry
      pcg_spmv_pap(A, v, st, red, ctx->stream, c > 0);
      pcg_update_rx(v, st, red, sc.tickets, fp32z, ctx->stream, true);
      enqueue_sweep(F, ctx->stream, true);
      enqueue_sweep(B, ctx->stream, true);
      pcg_rz_beta(v, st, red, fp32z, ctx->stream, true);
      pcg_update_p(v, st, fp32z, ctx->stream, true);
    }
    CK(cudaStreamEndCapture(ctx->stream, &g.graph));
    CK(cudaGraphInstantiate(&g.exec, g.graph, 0));
    unsigned refin = 0;
    long long guard = 0;
    double bb = 0.0;
    for (;;) {
      while (!h.done) {
        CK(cudaGraphLaunch(g.exec, ctx->stream));
        launched(ctx, per_it * chunk);
        read_state(ctx, st, h);
        if (read_err(ctx) != 0) return timeout_status(ctx);
        if (++guard > (long long)maxit / chunk + 64) break;
      }
      if (h.done != 1 || !target_true) break;
      // recursive residual converged: check the true one
      if (bb == 0.0) {
        CK(api_dot(m, v.b, v.b, red_of(ctx, 0), ctx->stream));
        launched(ctx);
        CK(cudaMemcpyAsync(&bb, red_of(ctx, 0).result, 8, cudaMemcpyDeviceToHost, ctx->stream));
      }
      CK(pcg_true_residual(A, v, st, red, ctx->stream));
      launched(ctx);
      ++refin;
      PcgState t{};
      read_state(ctx, st, t);
      const double rel = bb > 0 ? std::sqrt(t.rr / bb) : 0.0;
      h.conv = rel;
      if (rel <= tol || h.it + 1 >= maxit) {
        if (rel > tol) h.done = 2;
        break;
      }
      // continue from the true residual: finish this iteration and resume
      CK(pcg_replace(v, st, sc.tickets, fp32z, ctx->stream));
      run_sweep(ctx, F);
      run_sweep(ctx, B);
      CK(pcg_rz_beta(v, st, red, fp32z, ctx->stream));
      CK(pcg_update_p(v, st, fp32z, ctx->stream));
      launched(ctx, 3);
      read_state(ctx, st, h);
    }
    *conv_ratio = h.conv;
    if (refinements) *refinements = refin;
    if (h.done == 1) {
      *iteration = (unsigned)h.iter_out;
      return DFG_OK;
    }
    if (h.done == 3) {
      set_err(ctx, "NaN in the residual");
      return DFG_NAN_DETECTED;
    }
    set_err(ctx, "PCG did not converge within the iteration limit");
    return DFG_NOT_CONVERGED;
  });
}

extern "C" int dfg_solve_pcg(dfg_system sys, dfg_precond prec, double* conv_ratio, unsigned* iteration) {
  if (!sys || !prec || !conv_ratio || !iteration) return DFG_INVALID_ARGUMENT;
  return solve_pcg_f64vec(sys, prec, false, false, conv_ratio, iteration, nullptr);
}

// Mixed precision: PCG whose SpMV, factor, sweeps and vectors are FP32, with
// the reductions and alpha/beta in FP64 and the solution accumulated in FP64.
// Whenever the FP32 recursive residual has dropped by 10x since the last
// refinement point -- or below the tolerance -- the solution absorbs the
// FP64 correction, the FP64 true residual b - A x is recomputed, and the
// recursion continues from it with the current search direction (iterative
// refinement by residual replacement, without restarting the Krylov space).
extern "C" int dfg_solve_pcg_mixed(dfg_system sys, dfg_precond prec, double* conv_ratio, unsigned* iteration,
                                   unsigned* outer) {
  if (!sys || !prec || !conv_ratio || !iteration) return DFG_INVALID_ARGUMENT;
  dfg_ctx ctx = sys->ctx;
  return guarded(ctx, [&]() -> int {
    dfg_ctx ctx_ = ctx;
    REQUIRE(prec->numeric && prec->sys == sys, DFG_NOT_READY, "preconditioner value not set for this system");
    REQUIRE(sys->rhs0_valid, DFG_NOT_READY, "dfg_finalize_marge must come before the mixed solve");
    const long long m = (long long)sys->n * sys->b;
    const size_t bs = (size_t)sys->b * sys->b;
    if (!sys->mat32_valid) {
      dalloc(ctx, sys->diag32, (size_t)sys->n * bs * 4 + 64);
      dalloc(ctx, sys->offd32, (size_t)std::max<long long>(sys->nnz, 1) * bs * 4 + 64);
      CK(to_fp32((long long)sys->n * bs, sys->diag.as<double>(), sys->diag32.as<float>(), ctx->stream));
      CK(to_fp32(sys->nnz * (long long)bs, sys->offd.as<double>(), sys->offd32.as<float>(), ctx->stream));
      launched(ctx, 2);
      sys->mat32_valid = true;
    }
    ensure_numeric32(ctx, prec);
    dalloc(ctx, sys->w_rd, vec_bytes(sys, 8));
    dalloc(ctx, sys->w_d, vec_bytes(sys, 8));
    dalloc(ctx, sys->w_r32, vec_bytes(sys, 4));
    dalloc(ctx, sys->w_p32, vec_bytes(sys, 4));
    dalloc(ctx, sys->w_q32, vec_bytes(sys, 4));
    dalloc(ctx, sys->w_z32, vec_bytes(sys, 4));
    dalloc(ctx, sys->w_state, sizeof(PcgState));
    PcgState* st = sys->w_state.as<PcgState>();
    Scratch sc = scratch_of(ctx);
    Red red = red_of(ctx, 2);
    MixVecs v{sys->rhs0.as<double>(), sys->upd.as<double>(), sys->w_rd.as<double>(), sys->w_d.as<double>(),
              sys->w_r32.as<float>(), sys->w_p32.as<float>(), sys->w_q32.as<float>(), prec->ybuf32.as<float>(),
              sys->w_z32.as<float>(), m};
    ensure_sell(ctx, sys, true);
    const MatView A64 = view64(sys);
    const MatView A32 = view32(sys);
    const int* done = reinterpret_cast<const int*>(reinterpret_cast<const char*>(st) + offsetof(PcgState, done));
    SweepLaunch F = sweep_launch(ctx, prec, prec->fwd, true, v.r, v.y, sc.tickets, done);
    SweepLaunch B = sweep_launch(ctx, prec, prec->bwd, true, v.y, v.z, sc.tickets + 1, done);
    CK(cudaMemsetAsync(v.x, 0, (size_t)m * 8, ctx->stream));
    CK(cudaMemsetAsync(v.d, 0, (size_t)m * 8, ctx->stream));
    CK(api_dot(m, v.b, v.b, red, ctx->stream));
    launched(ctx);
    double bb = 0.0;
    CK(cudaMemcpyAsync(&bb, red.result, 8, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    const double tol = *conv_ratio;
    const int maxit = (int)std::min<unsigned>(*iteration, 0x7fffffffu);
    if (bb < 1.0e-30) {
      *conv_ratio = 0.0;
      *iteration = 0;
      if (outer) *outer = 0;
      return DFG_OK;
    }
    CK(mix_start(st, tol, bb, 0.1, maxit, ctx->stream));
    // true residual of x = 0 is b; start the recursion from it
    CK(mix_true_residual(A64, v, st, red, ctx->stream));
    CK(mix_replace(v, st, sc.tickets, ctx->stream));
    run_sweep(ctx, F);
    run_sweep(ctx, B);
    CK(mix_after_precond0(v, st, red, ctx->stream));
    launched(ctx, 4);
    const long long per_it = 4 + launches_of(F) + launches_of(B);
    const int chunk = std::max(2, std::min(m < 200000 ? 8 : 32, (int)(4096 / per_it)));
    Chunk g;
    CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    for (int c = 0; c < chunk; ++c) {
      mix_spmv_pap(A32, v, st, red, ctx->stream);
      mix_update_rx(v, st, red, sc.tickets, ctx->stream);
      enqueue_sweep(F, ctx->stream);
      enqueue_sweep(B, ctx->stream);
      mix_rz_beta(v, st, red, ctx->stream);
      mix_update_p(v, st, ctx->stream);
    }
    CK(cudaStreamEndCapture(ctx->stream, &g.graph));
    CK(cudaGraphInstantiate(&g.exec, g.graph, 0));
    PcgState h{};
    unsigned refinements = 0;
    double rel = 1.0;
    int status = DFG_NOT_CONVERGED;
    long long guard = 0;
    for (;;) {
      CK(cudaGraphLaunch(g.exec, ctx->stream));
      launched(ctx, per_it * chunk);
      read_state(ctx, st, h);
      if (read_err(ctx) != 0) return timeout_status(ctx);
      if (h.done == 0) {
        if (++guard > (long long)maxit / chunk + 64) break;
        continue;
      }
      if (h.done == 3) { status = DFG_NAN_DETECTED; set_err(ctx, "NaN in the residual"); break; }
      // refinement point: fold the correction in, recompute the true residual
      CK(mix_accumulate(v, ctx->stream));
      CK(mix_true_residual(A64, v, st, red, ctx->stream));
      launched(ctx, 2);
      ++refinements;
      PcgState t{};
      read_state(ctx, st, t);
      rel = std::sqrt(t.rr / bb);
      if (!(rel == rel)) { status = DFG_NAN_DETECTED; set_err(ctx, "NaN in the residual"); break; }
      if (rel <= tol) { status = DFG_OK; break; }
      if (h.done == 2) { set_err(ctx, "mixed PCG did not converge within the iteration limit"); break; }
      // continue the recursion from the true residual: finish this iteration
      // (preconditioner, beta, direction) and resume the graph
      CK(mix_replace(v, st, sc.tickets, ctx->stream));
      run_sweep(ctx, F);
      run_sweep(ctx, B);
      CK(mix_rz_beta(v, st, red, ctx->stream));
      CK(mix_update_p(v, st, ctx->stream));
      launched(ctx, 3);
    }
    *conv_ratio = rel;
    *iteration = (unsigned)h.iter_out;
    if (outer) *outer = refinements;
    return status;
  });
}

// Preconditioned BiCGSTAB (LsSol::Solve_PBiCGSTAB) on the device, all FP64;
// chunks of iterations captured in a graph and replayed until the device
// state says done.
extern "C" int dfg_solve_pbicgstab(dfg_system sys, dfg_precond prec, int mode, double* conv_ratio,
                                   unsigned* iteration) {
  if (!sys || !prec || !conv_ratio || !iteration) return DFG_INVALID_ARGUMENT;
  dfg_ctx ctx = sys->ctx;
  return guarded(ctx, [&]() -> int {
    dfg_ctx ctx_ = ctx;
    REQUIRE(mode == DFG_PREC_FP64, DFG_INVALID_ARGUMENT,
            "BiCGSTAB runs in DFG_PREC_FP64 only: with a preconditioner applied in FP32 its recurrences diverge "
            "on ill-conditioned systems");
    REQUIRE(prec->numeric && prec->sys == sys, DFG_NOT_READY, "preconditioner value not set for this system");
    const long long m = (long long)sys->n * sys->b;
    // workspace: r2, p, AMp, s, AMs, Mp, Ms; state; paired-sum partials
    const size_t v8 = ((size_t)m * 8 + 255) / 256 * 256;
    const size_t off_st = 7 * v8, off_red = off_st + 256, total = off_red + 2 * kRedGrid * 8 + 256;
    dalloc(ctx, sys->w_bicg, total);
    char* w = sys->w_bicg.as<char>();
    double* vec[7];
    for (int k = 0; k < 7; ++k) vec[k] = reinterpret_cast<double*>(w + k * v8);
    BicgVecs v{sys->res.as<double>(), sys->upd.as<double>(), vec[0], vec[1], vec[2], vec[3], vec[4], vec[5], vec[6],
               prec->ybuf64.as<double>(), m};
    BicgState* st = reinterpret_cast<BicgState*>(w + off_st);
    Red red2{reinterpret_cast<double*>(w + off_red), reinterpret_cast<unsigned*>(w + off_red + 2 * kRedGrid * 8),
             nullptr};
    CK(cudaMemsetAsync(red2.counter, 0, sizeof(unsigned), ctx->stream));
    Scratch sc = scratch_of(ctx);
    Red red = red_of(ctx, 1);
    const int* done = reinterpret_cast<const int*>(reinterpret_cast<const char*>(st) + offsetof(BicgState, done));
    SweepLaunch F1 = sweep_launch(ctx, prec, prec->fwd, false, v.p, v.y, sc.tickets, done);
    SweepLaunch B1 = sweep_launch(ctx, prec, prec->bwd, false, v.y, v.mp, sc.tickets + 1, done);
    SweepLaunch F2 = sweep_launch(ctx, prec, prec->fwd, false, v.s, v.y, sc.tickets, done);
    SweepLaunch B2 = sweep_launch(ctx, prec, prec->bwd, false, v.y, v.ms, sc.tickets + 1, done);
    const int maxit = (int)std::min<unsigned>(*iteration, 0x7fffffffu);
    const double tol = *conv_ratio;
    CK(bicg_init(v, st, red, tol, maxit, sc.tickets, ctx->stream));
    launched(ctx, 2);
    BicgState h{};
    CK(cudaMemcpyAsync(&h, st, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (h.done == 0) {
      ensure_sell(ctx, sys, false);
      const MatView A = view64(sys);
      const long long per_it = 5 + launches_of(F1) + launches_of(B1) + launches_of(F2) + launches_of(B2);
      const int chunk = std::max(2, std::min(m < 200000 ? 4 : 16, (int)(4096 / per_it)));
      Chunk g;
      CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
      for (int c = 0; c < chunk; ++c) {
        enqueue_sweep(F1, ctx->stream);
        enqueue_sweep(B1, ctx->stream);
        bicg_amp(A, v, st, red, ctx->stream);
        bicg_s(v, st, sc.tickets, ctx->stream);
        enqueue_sweep(F2, ctx->stream);
        enqueue_sweep(B2, ctx->stream);
        bicg_ams(A, v, st, red2, ctx->stream);
        bicg_update(v, st, red2, ctx->stream);
        bicg_p(v, st, sc.tickets, ctx->stream);
      }
      CK(cudaStreamEndCapture(ctx->stream, &g.graph));
      CK(cudaGraphInstantiate(&g.exec, g.graph, 0));
      long long guard = 0;
      while (!h.done) {
        CK(cudaGraphLaunch(g.exec, ctx->stream));
        launched(ctx, per_it * chunk);
        CK(cudaMemcpyAsync(&h, st, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        if (read_err(ctx) != 0) return timeout_status(ctx);
        if (++guard > (long long)maxit / chunk + 64) break;
      }
    }
    switch (h.done) {
      case 1:
      case 4:
        *conv_ratio = h.conv;
        *iteration = (unsigned)h.iter_out;
        return DFG_OK;
      case 3:
        *iteration = (unsigned)h.iter_out;
        set_err(ctx, "NaN in the residual");
        return DFG_NAN_DETECTED;
      default:  // the reference leaves the ratio as given and reports max_iter
        *iteration = (unsigned)maxit;
        set_err(ctx, "BiCGSTAB did not converge within the iteration limit");
        return DFG_NOT_CONVERGED;
    }
  });
}

extern "C" int dfg_solve_pcg_ex(dfg_system sys, dfg_precond prec, int mode, int target_true, double* conv_ratio,
                                unsigned* iteration, unsigned* refinements) {
  if (!sys || !prec || !conv_ratio || !iteration) return DFG_INVALID_ARGUMENT;
  switch (mode) {
    case DFG_PREC_FP64: return solve_pcg_f64vec(sys, prec, false, target_true != 0, conv_ratio, iteration, refinements);
    case DFG_PREC_FP32_FACTOR: return solve_pcg_f64vec(sys, prec, true, target_true != 0, conv_ratio, iteration, refinements);
    case DFG_PREC_MIXED: return dfg_solve_pcg_mixed(sys, prec, conv_ratio, iteration, refinements);
    default:
      sys->ctx->last_error = "unknown precision mode";
      return DFG_INVALID_ARGUMENT;
  }
}

extern "C" int dfg_true_residual(dfg_system sys, const double* b, double* rel) {
  if (!sys || !rel) return DFG_INVALID_ARGUMENT;
  dfg_ctx ctx = sys->ctx;
  return guarded(ctx, [&]() -> int {
    dfg_ctx ctx_ = ctx;
    const long long m = (long long)sys->n * sys->b;
    DBuf bb, rr;
    const double* bp;
    if (b) {
      upload(ctx, bb, b, (size_t)m);
      bp = bb.as<double>();
    } else {
      REQUIRE(sys->rhs0_valid, DFG_NOT_READY, "no finalized right-hand side");
      bp = sys->rhs0.as<double>();
    }
    dalloc(ctx, rr, (size_t)m * 8 + 64);
    CK(cudaMemcpyAsync(rr.p, bp, (size_t)m * 8, cudaMemcpyDeviceToDevice, ctx->stream));
    CK(api_matvec(view64(sys), -1.0, sys->upd.as<double>(), 1.0, rr.as<double>(), ctx->stream));
    Red red = red_of(ctx, 0);
    CK(api_dot(m, rr.as<double>(), rr.as<double>(), red, ctx->stream));
    double r2 = 0.0, b2 = 0.0;
    CK(cudaMemcpyAsync(&r2, red.result, 8, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    CK(api_dot(m, bp, bp, red, ctx->stream));
    CK(cudaMemcpyAsync(&b2, red.result, 8, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    launched(ctx, 3);
    *rel = b2 > 0 ? std::sqrt(r2 / b2) : std::sqrt(r2);
    return DFG_OK;
  });
}

extern "C" int dfg_profile_kernels(dfg_system sys, dfg_precond prec, int mode, int reps, double* ms, double* bytes) {
  if (!sys || !prec || !ms || reps < 1) return DFG_INVALID_ARGUMENT;
  dfg_ctx ctx = sys->ctx;
  return guarded(ctx, [&]() -> int {
    dfg_ctx ctx_ = ctx;
    const bool mixed = mode == DFG_PREC_MIXED;
    const bool fp32z = mode != DFG_PREC_FP64;  // sweeps in FP32
    REQUIRE(mode >= 0 && mode <= 2, DFG_INVALID_ARGUMENT, "unknown precision mode");
    REQUIRE(prec->numeric && prec->sys == sys, DFG_NOT_READY, "preconditioner value not set for this system");
    REQUIRE(mixed ? (sys->w_p32.p && sys->mat32_valid && prec->numeric32)
                  : (sys->w_p.p && (!fp32z || (sys->w_r32.p && sys->w_z32.p && prec->numeric32))),
            DFG_NOT_READY, "run a solve of this mode before profiling it");
    const long long m = (long long)sys->n * sys->b;
    Scratch sc = scratch_of(ctx);
    Red red = red_of(ctx, 3);
    dalloc(ctx, sys->w_state, sizeof(PcgState));
    PcgState* st = sys->w_state.as<PcgState>();
    // a state that never reports done, with benign scalars
    PcgState h{};
    h.rz = 1.0; h.alpha = 1e-30; h.beta = 1e-30; h.inv_rr0 = 1.0; h.tol2 = 0.0; h.maxit = 1 << 30;
    h.rr_ref = 1e300; h.delta2 = 0.0; h.tolb2 = 0.0;
    CK(cudaMemcpyAsync(st, &h, sizeof(PcgState), cudaMemcpyHostToDevice, ctx->stream));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    double acc[6] = {0, 0, 0, 0, 0, 0};
    ensure_sell(ctx, sys, mixed);
    const MatView A64 = view64(sys);
    const MatView A32 = view32(sys);
    // the update kernels run on copies, so the caller's residual, solution and
    // direction stay as the last solve left them
    DBuf tr, tx, tp, td, tr32;
    const size_t esz = mixed ? 4 : 8;
    dalloc(ctx, tr, vec_bytes(sys, esz));
    dalloc(ctx, tx, vec_bytes(sys, 8));
    dalloc(ctx, tp, vec_bytes(sys, esz));
    dalloc(ctx, td, vec_bytes(sys, 8));
    dalloc(ctx, tr32, vec_bytes(sys, 4));
    CK(cudaMemcpyAsync(tr.p, mixed ? sys->w_r32.p : sys->res.p, (size_t)m * esz, cudaMemcpyDeviceToDevice, ctx->stream));
    CK(cudaMemcpyAsync(tx.p, sys->upd.p, (size_t)m * 8, cudaMemcpyDeviceToDevice, ctx->stream));
    CK(cudaMemcpyAsync(tp.p, mixed ? sys->w_p32.p : sys->w_p.p, (size_t)m * esz, cudaMemcpyDeviceToDevice, ctx->stream));
    CK(cudaMemsetAsync(td.p, 0, (size_t)m * 8, ctx->stream));
    if (fp32z && !mixed) CK(cudaMemcpyAsync(tr32.p, sys->w_r32.p, (size_t)m * 4, cudaMemcpyDeviceToDevice, ctx->stream));
    PcgVecs v{};
    v.r = tr.as<double>(); v.x = tx.as<double>(); v.p = tp.as<double>(); v.q = sys->w_q.as<double>();
    v.y = fp32z ? prec->ybuf32.p : prec->ybuf64.p;
    v.z = fp32z ? sys->w_z32.p : sys->w_z.p;
    v.m = m; v.r32 = tr32.as<float>(); v.rd = td.as<double>(); v.b = sys->rhs0.as<double>();
    MixVecs w{sys->rhs0.as<double>(), tx.as<double>(), sys->w_rd.as<double>(), td.as<double>(),
              tr.as<float>(), tp.as<float>(), sys->w_q32.as<float>(), prec->ybuf32.as<float>(),
              sys->w_z32.as<float>(), m};
    const void* rin = mixed ? (const void*)w.r : (fp32z ? (const void*)v.r32 : (const void*)v.r);
    void* ybuf = fp32z ? prec->ybuf32.p : prec->ybuf64.p;
    void* zbuf = fp32z ? sys->w_z32.p : sys->w_z.p;
    SweepLaunch F = sweep_launch(ctx, prec, prec->fwd, fp32z, rin, ybuf, sc.tickets, nullptr);
    SweepLaunch B = sweep_launch(ctx, prec, prec->bwd, fp32z, ybuf, zbuf, sc.tickets + 1, nullptr);
    auto timed = [&](int slot, auto&& pre, auto&& body) {
      for (int r = 0; r < reps + 1; ++r) {
        pre();
        CK(cudaEventRecord(e0, ctx->stream));
        body();
        CK(cudaEventRecord(e1, ctx->stream));
        CK(cudaEventSynchronize(e1));
        float t = 0.f;
        CK(cudaEventElapsedTime(&t, e0, e1));
        if (r > 0) acc[slot] += t;  // first launch is a warm-up
      }
    };
    auto nop = [] {};
    if (mixed) timed(0, nop, [&] { CK(mix_spmv_pap(A32, w, st, red, ctx->stream)); });
    else timed(0, nop, [&] { CK(pcg_spmv_pap(A64, v, st, red, ctx->stream)); });
    timed(1, [&] {
        CK(fill_sentinel(m, ybuf, fp32z, ctx->stream));
        CK(cudaMemsetAsync(sc.tickets, 0, 2 * sizeof(int), ctx->stream));
      }, [&] { run_sweep(ctx, F); });
    timed(2, [&] {
        CK(fill_sentinel(m, zbuf, fp32z, ctx->stream));
        CK(cudaMemsetAsync(sc.tickets, 0, 2 * sizeof(int), ctx->stream));
      }, [&] { run_sweep(ctx, B); });
    if (mixed) {
      timed(3, nop, [&] { CK(mix_update_rx(w, st, red, sc.tickets, ctx->stream)); });
      timed(4, nop, [&] { CK(mix_rz_beta(w, st, red, ctx->stream)); });
      timed(5, nop, [&] { CK(mix_update_p(w, st, ctx->stream)); });
    } else {
      timed(3, nop, [&] { CK(pcg_update_rx(v, st, red, sc.tickets, fp32z, ctx->stream)); });
      timed(4, nop, [&] { CK(pcg_rz_beta(v, st, red, fp32z, ctx->stream)); });
      timed(5, nop, [&] { CK(pcg_update_p(v, st, fp32z, ctx->stream)); });
    }
    launched(ctx, 8LL * (reps + 1));
    CK(cudaStreamSynchronize(ctx->stream));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    for (int k = 0; k < 6; ++k) ms[k] = acc[k] / reps;
    if (bytes) {
      const double spmv_sz = mixed ? 4.0 : 8.0, sw_sz = fp32z ? 4.0 : 8.0;
      const double bs = (double)sys->b * sys->b, N = sys->n, Z = (double)sys->nnz;
      const FactorPattern FP = factor_pattern(prec);  // the sweeps read the factor's blocks
      long long zl = 0;
      for (int i = 0; i < sys->n; ++i) zl += FP.diaind[i] - FP.rowptr[i];
      const double Zl = (double)zl, Zu = (double)prec->nnz - Zl;
      bytes[0] = (Z + N) * bs * spmv_sz + 4.0 * (Z + N + 1) + 2.0 * N * sys->b * spmv_sz;   // values, indices, x, y
      bytes[1] = (Zl + N) * bs * sw_sz + 4.0 * (Zl + N + 1) + 2.0 * N * sys->b * sw_sz;       // L, D^-1, indices, in, out
      bytes[2] = Zu * bs * sw_sz + 4.0 * (Zu + N + 1) + 2.0 * N * sys->b * sw_sz;             // U', indices, in, out
    }
    return DFG_OK;
  });
}
