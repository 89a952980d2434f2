// k_sweep.cu -- forward / backward substitution of the block ILU(0) factor
// (CMatDiaFrac_BlkCrs::ForwardSubstitution / BackwardSubstitution,
// src/matvec/matdiafrac_blkcrs.cpp:332-669) in the reference's natural order.
//
// Schedule (built on the host, sched.cpp): the rows are cut into contiguous
// ranges, one warp each; inside a range the rows are grouped by their local
// dependency level into steps of <= 32 rows (one row per lane).  A warp
// walks its steps in order; rows of one step are independent.
//
//  * a dependency produced by the same warp fewer than R steps ago is read
//    from a shared-memory ring;
//  * any other dependency is read from the output vector in global memory.
//    The output is pre-filled with a NaN sentinel and every value is written
//    exactly once, so a consumer that sees a non-sentinel value has the final
//    value: no flags, no fences.  Ranges are claimed through a ticket counter
//    in row order, so every range a warp waits on is already being worked on.
//
// Data movement per step (two-level cp.async pipeline, K steps deep):
//  record(t)  -- packed step record (row ids, dependency codes, blocks of the
//                factor, D^-1): issued at step t-2K;
//  values(t)  -- the rows' right-hand sides and the 16-byte-aligned windows
//                holding the global dependency values, whose addresses come
//                from record(t): issued at step t-K (L1-bypassing .cg copies,
//                so a window copied before its producer wrote it never
//                leaves a stale line behind; a sentinel seen in a window is
//                re-polled from global memory).
// Every wait is bounded (kSpinLimit polls); a wait that gives up records
// kErrTimeout in the error word and every warp of the launch then leaves.
//
// Record layout (bytes): [hdr int4: nent][rows: 32 int][src: nent x 32 int]
//   [blocks: nent x B*B x 32 of T][D^-1: B*B x 32 of T, forward only]
// (lane-minor, so shared-memory reads are conflict-free).
#include <climits>

#include "dfg_common.cuh"
#include "k_sweep.h"

namespace dfg {

template <typename T, int B, bool FWD, int K>
__global__ void __launch_bounds__(32) k_sweep(SweepArgs a) {
  constexpr int BS = B * B;
  constexpr int NREC = 2 * K, NVAL = K + 1;
  constexpr int RHS_BYTES = ((B * 32 * (int)sizeof(T)) + 15) / 16 * 16;
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x;
  unsigned char* rstage = smem;
  unsigned char* vstage = smem + (size_t)NREC * a.rec_stage;
  T* ring = reinterpret_cast<T*>(vstage + (size_t)NVAL * a.val_stage);
  const T* __restrict__ in = reinterpret_cast<const T*>(a.in);
  T* out = reinterpret_cast<T*>(a.out);

  if (a.done && *a.done) return;

  auto rec_ptr = [&](int slot) { return rstage + (size_t)slot * a.rec_stage; };
  auto val_ptr = [&](int slot) { return vstage + (size_t)slot * a.val_stage; };

  auto issue_record = [&](long long t, int slot) {
    const long long o0 = a.rec_off[t], o1 = a.rec_off[t + 1];
    const unsigned char* g = a.rec + o0;
    unsigned char* s = rec_ptr(slot);
    for (long long o = lane * 16; o < o1 - o0; o += 32 * 16) cp_async16(s + o, g + o);
  };
  auto issue_values = [&](int rslot, int vslot) {
    const unsigned char* r = rec_ptr(rslot);
    const int nent = reinterpret_cast<const int*>(r)[0];
    const int row = reinterpret_cast<const int*>(r + 16)[lane];
    unsigned char* v = val_ptr(vslot);
    if (row < 0) return;
    T* rhs = reinterpret_cast<T*>(v);
#pragma unroll
    for (int d = 0; d < B; ++d) {
      if constexpr (sizeof(T) == 8) cp_async8(&rhs[d * 32 + lane], &in[(size_t)row * B + d]);
      else cp_async4(&rhs[d * 32 + lane], &in[(size_t)row * B + d]);
    }
    const int* src = reinterpret_cast<const int*>(r + 144);
    for (int e = 0; e < nent; ++e) {
      const int c = src[e * 32 + lane];
      if (c >= 0 || c == INT_MIN) continue;
      const uintptr_t addr = reinterpret_cast<uintptr_t>(&out[(size_t)(-c - 1) * B]);
      const unsigned char* w = reinterpret_cast<const unsigned char*>(addr & ~(uintptr_t)15);
      unsigned char* dst = v + RHS_BYTES + (size_t)(e * 32 + lane) * 32;
      cp_async16(dst, w);
      if ((addr & 15) + B * sizeof(T) > 16) cp_async16(dst + 16, w + 16);
    }
  };

  bool abort = false;
  for (;;) {
    int r = 0;
    if (lane == 0) r = atomicAdd(a.ticket, 1);
    r = __shfl_sync(0xffffffffu, r, 0);
    if (r >= a.nranges) break;
    const long long s0 = a.range_steps[r], s1 = a.range_steps[r + 1];
    for (int i = 0; i < K; ++i)
      if (s0 + i < s1) issue_record(s0 + i, i % NREC);
    cp_async_commit();
    cp_async_wait_all();
    __syncwarp();
    for (int i = 0; i < K; ++i) {
      if (s0 + i < s1) issue_values(i % NREC, i % NVAL);
      if (s0 + K + i < s1) issue_record(s0 + K + i, (K + i) % NREC);
      cp_async_commit();
    }
    for (long long s = s0; s < s1; ++s) {
      const int loc = (int)(s - s0);
      cp_async_wait<K - 1>();  // the group carrying values(s) and record(s+K) has landed
      __syncwarp();
      if (s + K < s1) issue_values((loc + K) % NREC, (loc + K) % NVAL);
      const unsigned char* rec = rec_ptr(loc % NREC);
      const int nent = reinterpret_cast<const int*>(rec)[0];
      const int row = reinterpret_cast<const int*>(rec + 16)[lane];
      const int* src = reinterpret_cast<const int*>(rec + 144);
      const T* blk = reinterpret_cast<const T*>(rec + 144 + nent * 128);
      const unsigned char* val = val_ptr(loc % NVAL);
      if (row >= 0 && !abort) {
        T t[B];
#pragma unroll
        for (int d = 0; d < B; ++d) t[d] = reinterpret_cast<const T*>(val)[d * 32 + lane];
        for (int e = 0; e < nent; ++e) {
          const int c = src[e * 32 + lane];
          if (c == INT_MIN) continue;
          T v[B];
          if (c >= 0) {
            const int ss = c >> 5, ln = c & 31;
#pragma unroll
            for (int d = 0; d < B; ++d) v[d] = ring[(ss * B + d) * 32 + ln];
          } else {
            const size_t k = (size_t)(-c - 1);
            const uintptr_t addr = reinterpret_cast<uintptr_t>(&out[k * B]);
            const unsigned char* w = val + RHS_BYTES + (size_t)(e * 32 + lane) * 32 + (addr & 15);
#pragma unroll
            for (int d = 0; d < B; ++d) {
              T x = *reinterpret_cast<const T*>(w + d * sizeof(T));
              if (is_sentinel(x)) {
                long long spins = 0;
                for (;;) {
                  x = ld_relaxed(&out[k * B + d]);
                  if (!is_sentinel(x)) break;
                  if ((++spins & 1023) == 0) {
                    if (ld_relaxed_int(a.err) != 0) { abort = true; break; }
                    if (spins > kSpinLimit) { atomicExch(a.err, kErrTimeout); abort = true; break; }
                  }
                }
              }
              v[d] = x;
            }
          }
#pragma unroll
          for (int p = 0; p < B; ++p) {
            T acc = t[p];
#pragma unroll
            for (int q = 0; q < B; ++q) acc -= blk[(e * BS + p * B + q) * 32 + lane] * v[q];
            t[p] = acc;
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
        const int rs = loc % a.R;
#pragma unroll
        for (int d = 0; d < B; ++d) {
          ring[(rs * B + d) * 32 + lane] = y[d];
          st_relaxed(&out[(size_t)row * B + d], y[d]);
        }
      }
      abort = __any_sync(0xffffffffu, abort);
      __syncwarp();
      if (s + 2 * K < s1) issue_record(s + 2 * K, loc % NREC);
      cp_async_commit();
    }
    cp_async_wait_all();
    __syncwarp();
    if (abort) break;
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
  T* blk = reinterpret_cast<T*>(rec + 144 + nent * 128);
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

template <typename T, int B, bool FWD>
static cudaError_t launch_k(int K, const SweepArgs& a, int grid, size_t smem, cudaStream_t st) {
  switch (K) {
    case 2: k_sweep<T, B, FWD, 2><<<grid, 32, smem, st>>>(a); break;
    case 4: k_sweep<T, B, FWD, 4><<<grid, 32, smem, st>>>(a); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

template <typename T, bool FWD>
static cudaError_t launch_b(int B, int K, const SweepArgs& a, int grid, size_t smem, cudaStream_t st) {
  switch (B) {
    case 1: return launch_k<T, 1, FWD>(K, a, grid, smem, st);
    case 2: return launch_k<T, 2, FWD>(K, a, grid, smem, st);
    case 3: return launch_k<T, 3, FWD>(K, a, grid, smem, st);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_sweep(bool forward, bool fp32, int B, int K, const SweepArgs& a, int grid,
                         size_t smem, cudaStream_t st) {
  if (fp32) return forward ? launch_b<float, true>(B, K, a, grid, smem, st) : launch_b<float, false>(B, K, a, grid, smem, st);
  return forward ? launch_b<double, true>(B, K, a, grid, smem, st) : launch_b<double, false>(B, K, a, grid, smem, st);
}

template <typename T, int B, bool FWD, int K>
static cudaError_t set_attr(size_t max_smem) {
  return cudaFuncSetAttribute(k_sweep<T, B, FWD, K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);
}

cudaError_t sweep_set_smem_limits(size_t max_smem) {
  cudaError_t e = cudaSuccess;
#define DFG_ATTR(T, B)                                                                  \
  if (e == cudaSuccess) e = set_attr<T, B, true, 2>(max_smem);                          \
  if (e == cudaSuccess) e = set_attr<T, B, true, 4>(max_smem);                          \
  if (e == cudaSuccess) e = set_attr<T, B, false, 2>(max_smem);                         \
  if (e == cudaSuccess) e = set_attr<T, B, false, 4>(max_smem);
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
