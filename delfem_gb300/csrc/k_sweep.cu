// k_sweep.cu -- forward / backward substitution of the block ILU(0) factor
// (CMatDiaFrac_BlkCrs::ForwardSubstitution / BackwardSubstitution,
// src/matvec/matdiafrac_blkcrs.cpp:332-669) in the reference's natural order.
//
// Schedule (host, sched.cpp): rows are cut into contiguous ranges; inside a
// range rows are grouped by local dependency level into steps of <= 32 rows
// (one row per lane); rows of one step are independent.
//
// Execution: a persistent CTA of two warps claims ranges in row order
// through a ticket counter and walks their steps through an NS-deep
// shared-memory pipeline:
//   * loader warp  -- per step, one TMA bulk copy of the packed step record
//     (cp.async.bulk, completion on an mbarrier with a byte count), then, once
//     the record has landed, per-lane cp.async gathers of the rows' right-hand
//     sides and of the 16-byte-aligned windows holding dependencies produced
//     by other ranges; each lane's gathers arrive on the stage's `full`
//     mbarrier when they complete (cp.async.mbarrier.arrive.noinc);
//   * compute warp -- waits for `full` (which also covers the record: each
//     loader lane arrives on it with release semantics after acquiring the
//     record's barrier), evaluates the rows (dependency values
//     come from a ring of its own recent results or from the gathered
//     windows, selected without branching), writes results to the ring and to
//     global memory, and releases the stage on its `empty` mbarrier.
// In a batched launch (SweepArgs::batch) a ticket names a range of one of
// several independent solves; the pipeline simply continues across them.
// Cross-range hand-off needs no flags or fences: outputs are pre-filled with
// a NaN sentinel and written once, so a non-sentinel value is final; a window
// copied before its producer wrote it still holds the sentinel and the
// compute warp re-polls that value from global memory (bounded).  Ranges are
// claimed in order, so a range only ever waits on ranges already running.
// Every wait is bounded (kSpinLimit); a wait that gives up records
// kErrTimeout and the launch drains and returns.
//
// Record layout (bytes; see build_records in capi.cu):
//   [hdr int4: nent][row: 32 int][code: nent x 32 int][grow: nent x 32 int]
//   [blocks: nent x B*B x 32 of T][D^-1: B*B x 32 of T, forward only]
// code: bit 31 clear -> byte offset into the ring region (0 = a zero pad);
//       bit 31 set   -> byte offset into the stage's value slot.
// grow: global row of an out-of-range dependency (else -1).
// Value slot: [rhs: 32 lanes x B of T, 16-byte padded][windows: nent x 32 x 32 B].
#include <climits>

#include "dfg_common.cuh"
#include "k_mbar.cuh"
#include "k_sweep.h"

namespace dfg {

// Rare path: a gathered window still held the sentinel (its producer wrote
// after the copy); poll those values from global memory, bounded.
template <typename T>
__device__ __noinline__ T poll_value(const T* p, int* err, int* abort, int slot, int row) {
  T x = ld_relaxed(p);
  const long long t0 = clock64();
  for (unsigned n = 1; is_sentinel(x); ++n) {
    x = ld_relaxed(p);
    if ((n & 255) == 0) {
      if (ld_relaxed_int(err) != 0) {
        *abort = 1;
        break;
      }
      if (clock64() - t0 > kWaitCycles) {
        record_fail(err, kErrTimeout, kSitePoll, slot, row);
        *abort = 1;
        break;
      }
    }
  }
  return x;
}

template <typename T, int B, bool FWD, int MAXE>
__global__ void __launch_bounds__(64) k_sweep(SweepArgs a) {
  constexpr int BS = B * B;
  constexpr int SZ = (int)sizeof(T);
  extern __shared__ __align__(128) unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int NS = a.NS;
  // layout: [bars: 3*NS u64][rstage: NS x rec_stage][vstage: NS x val_stage][zero 32 B][ring]
  uint64_t* rec_full = reinterpret_cast<uint64_t*>(smem);
  uint64_t* full = rec_full + NS;
  uint64_t* empty = full + NS;
  unsigned char* rstage = smem + (((size_t)3 * NS * 8 + 127) / 128) * 128;
  unsigned char* vstage = rstage + (size_t)NS * a.rec_stage;
  unsigned char* ringreg = vstage + (size_t)NS * a.val_stage;  // 32 zero bytes, then the ring
  __shared__ int s_range, s_slot, s_stop;

  pdl_enter();
  if (a.done && *a.done) return;
  if (threadIdx.x == 0) {
    for (int s = 0; s < NS; ++s) {
      mbar_init(&rec_full[s], 1);
      mbar_init(&full[s], 64);  // 32 copy-completion arrivals + 32 loader arrivals
      mbar_init(&empty[s], 1);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (threadIdx.x < 8) reinterpret_cast<unsigned*>(ringreg)[threadIdx.x] = 0u;
  __syncthreads();

  long long g = 0;  // steps this CTA has pushed through the pipeline (both warps count alike)
  int g_st = 0, g_ph = 0;  // stage and phase parity of pipeline position g
  bool abort = false;
  for (;;) {
    if (threadIdx.x == 0) {
      const int t = atomicAdd(a.ticket, 1);
      int r = -1, j = 0;
      if (a.batch) {
        const SweepBatch* bt = a.batch;
        const int ns = bt->nslots;
        if (t < bt->range_start[ns]) {
          int lo = 0, hi = ns - 1;  // last j with range_start[j] <= t
          while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (bt->range_start[mid] <= t) lo = mid; else hi = mid - 1;
          }
          j = lo;
          r = ld_relaxed_int(bt->slot[j].done) ? -2 : t - bt->range_start[j];
        }
      } else if (t < a.nranges) {
        r = t;
      }
      s_range = r;
      s_slot = j;
    }
    named_sync(1, 64);
    const int r = s_range, jslot = s_slot;
    named_sync(1, 64);
    if (r == -1) break;
    if (r == -2) continue;  // a finished solve: its ranges are skipped
    const unsigned char* __restrict__ recs = a.batch ? a.batch->slot[jslot].rec : a.rec;
    const long long* __restrict__ rec_off = a.batch ? a.batch->slot[jslot].rec_off : a.rec_off;
    const int* __restrict__ range_steps = a.batch ? a.batch->slot[jslot].range_steps : a.range_steps;
    const T* __restrict__ in = reinterpret_cast<const T*>(a.batch ? a.batch->slot[jslot].in : a.in);
    T* out = reinterpret_cast<T*>(a.batch ? a.batch->slot[jslot].out : a.out);
    const long long s0 = range_steps[r], s1 = range_steps[r + 1];
    const long long nsteps = s1 - s0;
    const int nst = (int)nsteps;
    if (warp == 1) {
      // ------------------------------------------------------------ loader
      // stage / phase of pipeline position g+i, advanced incrementally
      int rs_st = g_st, rs_ph = g_ph;     // next record to issue
      int n_issued = 0, n_waited = 0;     // record copies of this range issued / waited for
      int vl_st = g_st, vl_ph = g_ph;     // next step to gather for
      auto issue_rec = [&](int i) {       // step s0+i into stage rs_st
        if (g + i >= NS && !abort) {
          if (!mbar_wait(&empty[rs_st], (unsigned)(rs_ph ^ 1), a.err, kSiteEmpty, jslot, r)) abort = true;
        }
        if (abort) {  // no new copies once the launch is failing
          if (++rs_st == NS) { rs_st = 0; rs_ph ^= 1; }
          return;
        }
        ++n_issued;
        if (lane == 0) {
          const long long o0 = rec_off[s0 + i], o1 = rec_off[s0 + i + 1];
          mbar_expect_tx(&rec_full[rs_st], (unsigned)(o1 - o0));
          tma_load_1d(rstage + (size_t)rs_st * a.rec_stage, recs + o0, (unsigned)(o1 - o0), &rec_full[rs_st]);
        }
        if (++rs_st == NS) { rs_st = 0; rs_ph ^= 1; }
      };
      const int LA = NS > 3 ? NS / 2 : 1;  // record copies run LA steps ahead of the gathers
      for (int i = 0; i < LA && i < nst; ++i) issue_rec(i);
      for (int i = 0; i < nst; ++i) {
        if (i + LA < nst) issue_rec(i + LA);
        const int st = vl_st;
        if (!abort) {
          if (mbar_wait(&rec_full[st], (unsigned)vl_ph, a.err, kSiteRecLoad, jslot, r)) ++n_waited;
          else abort = true;
        }
        if (++vl_st == NS) { vl_st = 0; vl_ph ^= 1; }
        const unsigned char* rec = rstage + (size_t)st * a.rec_stage;
        unsigned char* val = vstage + (size_t)st * a.val_stage;
        const int nent = reinterpret_cast<const int*>(rec)[0];
        const int row = reinterpret_cast<const int*>(rec + 16)[lane];
        if (row >= 0 && !abort) {
          T* rhs = reinterpret_cast<T*>(val) + lane * B;
#pragma unroll
          for (int d = 0; d < B; ++d) {
            if constexpr (SZ == 8) cp_async8(rhs + d, &in[(size_t)row * B + d]);
            else cp_async4(rhs + d, &in[(size_t)row * B + d]);
          }
          const int* code = reinterpret_cast<const int*>(rec + 144);
          const int* grow = code + nent * 32;
          for (int e = 0; e < nent; ++e) {
            const int k = grow[e * 32 + lane];
            if (k < 0) continue;
            const unsigned c = (unsigned)code[e * 32 + lane] & 0x7fffffffu;
            const uintptr_t addr = reinterpret_cast<uintptr_t>(&out[(size_t)k * B]);
            const unsigned char* w = reinterpret_cast<const unsigned char*>(addr & ~(uintptr_t)15);
            unsigned char* dst = val + (c & ~15u);
            cp_async16(dst, w);
            if ((addr & 15) + B * SZ > 16) cp_async16(dst + 16, w + 16);
          }
        }
        cp_async_arrive_noinc(&full[st]);
        // release: the record this lane waited for is visible to whoever
        // acquires `full`, so the compute warp waits on one barrier per step.
        // A failing lane does not arrive: the compute warp then gives up on
        // the error word instead of reading a record that may not have landed.
        if (!abort) mbar_arrive(&full[st]);
      }
      // after a failure, record copies already issued land before the CTA
      // moves on (bounded): lane 0 issued them
      if (abort && lane == 0) {
        for (int k = n_waited; k < n_issued; ++k) {
          const long long pos = g + k;
          mbar_drain(&rec_full[pos % NS], (unsigned)((pos / NS) & 1));
        }
      }
    } else {
      // ----------------------------------------------------------- compute
      int st = g_st, ph = g_ph, rs = 0;
      for (int i = 0; i < nst; ++i) {
        if (!abort && !mbar_wait(&full[st], (unsigned)ph, a.err, kSiteFull, jslot, r)) abort = true;
        const unsigned char* rec = rstage + (size_t)st * a.rec_stage;
        const unsigned char* val = vstage + (size_t)st * a.val_stage;
        const int nent = reinterpret_cast<const int*>(rec)[0];
        const int row = reinterpret_cast<const int*>(rec + 16)[lane];
        const int* code = reinterpret_cast<const int*>(rec + 144);
        const int* grow = code + nent * 32;
        const T* blk = reinterpret_cast<const T*>(rec + 144 + nent * 256);
        if (row >= 0 && !abort) {
          T t[B];
#pragma unroll
          for (int d = 0; d < B; ++d) t[d] = reinterpret_cast<const T*>(val)[lane * B + d];
          if constexpr (MAXE > 0) {
            // all dependency values first (independent shared-memory loads),
            // one staleness test, then the FMAs
            T v[MAXE][B];
            bool stale = false;
#pragma unroll
            for (int e = 0; e < MAXE; ++e) {
              if (e < nent) {
                const int c = code[e * 32 + lane];
                const unsigned char* base = (c < 0) ? val : ringreg;
                const T* vp = reinterpret_cast<const T*>(base + (c & 0x7fffffff));
#pragma unroll
                for (int d = 0; d < B; ++d) {
                  v[e][d] = vp[d];
                  stale |= is_sentinel(v[e][d]);
                }
              }
            }
            if (stale) {
              int ab = 0;
#pragma unroll
              for (int e = 0; e < MAXE; ++e)
#pragma unroll
                for (int d = 0; d < B; ++d)
                  if (e < nent && is_sentinel(v[e][d]))
                    v[e][d] = poll_value<T>(&out[(size_t)grow[e * 32 + lane] * B + d], a.err, &ab, jslot,
                                            grow[e * 32 + lane]);
              abort |= ab != 0;
            }
#pragma unroll
            for (int e = 0; e < MAXE; ++e) {
              if (e < nent) {
#pragma unroll
                for (int p = 0; p < B; ++p) {
                  T acc = t[p];
#pragma unroll
                  for (int q = 0; q < B; ++q) acc -= blk[(e * BS + p * B + q) * 32 + lane] * v[e][q];
                  t[p] = acc;
                }
              }
            }
          } else {
            for (int e = 0; e < nent; ++e) {
              const int c = code[e * 32 + lane];
              const unsigned char* base = (c < 0) ? val : ringreg;
              const T* vp = reinterpret_cast<const T*>(base + (c & 0x7fffffff));
              T v[B];
              bool stale = false;
#pragma unroll
              for (int d = 0; d < B; ++d) {
                v[d] = vp[d];
                stale |= is_sentinel(v[d]);
              }
              if (stale) {
                int ab = 0;
#pragma unroll
                for (int d = 0; d < B; ++d)
                  if (is_sentinel(v[d]))
                    v[d] = poll_value<T>(&out[(size_t)grow[e * 32 + lane] * B + d], a.err, &ab, jslot,
                                         grow[e * 32 + lane]);
                abort |= ab != 0;
              }
#pragma unroll
              for (int p = 0; p < B; ++p) {
                T acc = t[p];
#pragma unroll
                for (int q = 0; q < B; ++q) acc -= blk[(e * BS + p * B + q) * 32 + lane] * v[q];
                t[p] = acc;
              }
            }
          }
          T y[B];
          if constexpr (FWD) {
            const T* dinv = blk + nent * BS * 32;
#pragma unroll
            for (int p = 0; p < B; ++p) {
              T acc = dinv[(p * B) * 32 + lane] * t[0];
#pragma unroll
              for (int q = 1; q < B; ++q) acc += dinv[(p * B + q) * 32 + lane] * t[q];
              y[p] = acc;
            }
          } else {
#pragma unroll
            for (int p = 0; p < B; ++p) y[p] = t[p];
          }
          T* rg = reinterpret_cast<T*>(ringreg + 32) + (rs * 32 + lane) * B;
#pragma unroll
          for (int d = 0; d < B; ++d) {
            rg[d] = y[d];
            st_relaxed(&out[(size_t)row * B + d], y[d]);
          }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[st]);
        if (++st == NS) { st = 0; ph ^= 1; }
        if (++rs == a.R) rs = 0;
      }
    }
    g += nsteps;
    g_st = (int)(g % NS);  // once per range
    g_ph = (int)((g / NS) & 1);
    if (__any_sync(0xffffffffu, abort)) {
      if (lane == 0) record_fail(a.err, kErrTimeout, kSiteRange, jslot, r);
    }
    // one read of the error word decides for both warps: a warp that left on
    // its own read while the other went on would strand it at the next bar.sync
    named_sync(1, 64);
    if (threadIdx.x == 0) s_stop = ld_relaxed_int(a.err) != 0;
    named_sync(1, 64);
    if (s_stop) break;
  }
  cp_async_wait_all();
}

// ------------------------------------------------------------------ packing

// Copies the factor blocks (reference layout) into the value regions of the
// step records, converting to T.  One CTA per step.
template <typename T, int B, bool FWD>
__global__ void k_pack(PackArgs a) {
  constexpr int BS = B * B;
  const int s = blockIdx.x;
  if (s >= a.nsteps) return;
  unsigned char* rec = a.rec + a.rec_off[s];
  const int nent = (int)(a.ent_off[s + 1] - a.ent_off[s]);
  T* blk = reinterpret_cast<T*>(rec + 144 + nent * (a.code_bytes ? a.code_bytes : 256));
  const int* slots = a.ent_slot + a.ent_off[s] * 32;
  for (int idx = threadIdx.x; idx < nent * BS * 32; idx += blockDim.x) {
    const int lane = idx & 31, m = (idx >> 5) % BS, e = (idx >> 5) / BS;
    const int slot = slots[e * 32 + lane];
    blk[idx] = slot >= 0 ? (T)a.foffd[(size_t)slot * BS + m] : (T)0;
  }
  if constexpr (FWD) {
    T* dinv = blk + nent * BS * 32;
    for (int idx = threadIdx.x; idx < BS * 32; idx += blockDim.x) {
      const int lane = idx & 31, m = idx >> 5;
      const int row = a.step_rows[(size_t)s * 32 + lane];
      dinv[idx] = row >= 0 ? (T)a.fdiag[(size_t)row * BS + m] : (T)0;
    }
  }
}

// ------------------------------------------------------------------ launchers

template <typename T, int B, bool FWD, int MAXE>
static cudaError_t launch_k(const SweepArgs& a, int grid, size_t smem, cudaStream_t st, bool dep) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(64);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = dep ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, k_sweep<T, B, FWD, MAXE>, a);
}

template <typename T, int B, bool FWD>
static cudaError_t launch_e(const SweepArgs& a, int grid, size_t smem, cudaStream_t st, bool dep) {
  if (a.max_nent <= 4) return launch_k<T, B, FWD, 4>(a, grid, smem, st, dep);
  if (a.max_nent <= 8) return launch_k<T, B, FWD, 8>(a, grid, smem, st, dep);
  return launch_k<T, B, FWD, 0>(a, grid, smem, st, dep);
}

template <typename T, bool FWD>
static cudaError_t launch_b(int B, const SweepArgs& a, int grid, size_t smem, cudaStream_t st, bool dep) {
  switch (B) {
    case 1: return launch_e<T, 1, FWD>(a, grid, smem, st, dep);
    case 2: return launch_e<T, 2, FWD>(a, grid, smem, st, dep);
    case 3: return launch_e<T, 3, FWD>(a, grid, smem, st, dep);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_sweep(bool forward, bool fp32, int B, const SweepArgs& a, int grid, size_t smem,
                         cudaStream_t st, bool dep) {
  if (fp32)
    return forward ? launch_b<float, true>(B, a, grid, smem, st, dep) : launch_b<float, false>(B, a, grid, smem, st, dep);
  return forward ? launch_b<double, true>(B, a, grid, smem, st, dep) : launch_b<double, false>(B, a, grid, smem, st, dep);
}

template <typename T, int B, bool FWD>
static cudaError_t set_attr(size_t max_smem) {
  cudaError_t e = cudaFuncSetAttribute(k_sweep<T, B, FWD, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_sweep<T, B, FWD, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_sweep<T, B, FWD, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);
  return e;
}

// Self-test of the bounded waits: one poll, with the sweep's own poll, of a
// value nothing writes (it holds the sentinel).  It gives up after the wait
// budget, records the failure in the error word and returns.
__global__ void k_wait_selftest(const double* never, int* err) {
  if (threadIdx.x != 0) return;
  int abort = 0;
  (void)poll_value<double>(never, err, &abort, -1, 0);
}

cudaError_t launch_wait_selftest(const double* never, int* err, cudaStream_t st) {
  k_wait_selftest<<<1, 32, 0, st>>>(never, err);
  return cudaGetLastError();
}

cudaError_t sweep_set_smem_limits(size_t max_smem) {
  cudaError_t e = cudaSuccess;
#define DFG_ATTR(T, B)                                        \
  if (e == cudaSuccess) e = set_attr<T, B, true>(max_smem);   \
  if (e == cudaSuccess) e = set_attr<T, B, false>(max_smem);
  DFG_ATTR(double, 1) DFG_ATTR(double, 2) DFG_ATTR(double, 3)
  DFG_ATTR(float, 1) DFG_ATTR(float, 2) DFG_ATTR(float, 3)
#undef DFG_ATTR
  return e;
}

template <typename T, bool FWD>
static cudaError_t pack_b(int B, const PackArgs& a, cudaStream_t st) {
  if (a.nsteps == 0) return cudaSuccess;
  switch (B) {
    case 1: k_pack<T, 1, FWD><<<a.nsteps, 128, 0, st>>>(a); break;
    case 2: k_pack<T, 2, FWD><<<a.nsteps, 128, 0, st>>>(a); break;
    case 3: k_pack<T, 3, FWD><<<a.nsteps, 128, 0, st>>>(a); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_pack(bool forward, bool fp32, int B, const PackArgs& a, cudaStream_t st) {
  if (fp32) return forward ? pack_b<float, true>(B, a, st) : pack_b<float, false>(B, a, st);
  return forward ? pack_b<double, true>(B, a, st) : pack_b<double, false>(B, a, st);
}

}  // namespace dfg
