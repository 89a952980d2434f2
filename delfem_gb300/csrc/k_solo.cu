// k_solo.cu -- batched forward / backward substitution of the block ILU(0)
// factor (CMatDiaFrac_BlkCrs::ForwardSubstitution / BackwardSubstitution,
// src/matvec/matdiafrac_blkcrs.cpp:332-669) with one CTA per solve.
//
// Serving keeps up to a few hundred independent solves in flight, so the
// device is filled by solves, not by splitting one solve over SMs: a CTA
// claims a whole solve and runs its sweep level after level (the dependency
// levels of the reference's natural order, build_levels), so every
// dependency was produced by the same CTA and no value crosses SMs.
//
// CTA: kSoloWarps compute warps + one producer warp.
//   * producer (one warp; lane 0 issues) -- walks the solve's chunks (runs of
//     <= ch_max steps of one level) in order, their table read 32 entries at a
//     time by the whole warp: per chunk two TMA bulk copies onto the stage's
//     `full` mbarrier (one arrival with the byte count): the chunk's packed
//     records, and its right-hand sides, which the producing kernel stored in
//     this sweep's step order so that they are contiguous; it runs up to NS
//     chunks ahead of the compute warps.
//   * compute warps -- level by level, chunk by chunk: warp w takes the steps
//     w, w + kSoloWarps, ... of the level (every record of a chunk has the
//     same size, so a step's offset is arithmetic), evaluates the step's 32 rows, writes
//     the results to the shared-memory ring (slot step mod R) and to the
//     output vector at the records' output positions, and arrives on the
//     stage's `empty` mbarrier (kSoloWarps arrivals free the stage); a named
//     barrier over the compute warps closes each level.
// A dependency is read from the ring when its step lies among the R steps
// before the end of the consuming level (never overwritten before it is
// read), else from the output vector in global memory (written at least one
// level barrier earlier).  No sentinels, flags or fences between CTAs: nothing
// is shared between CTAs but the ticket counter.  Every wait is bounded; a
// wait that gives up records kErrTimeout and the launch drains and returns.
//
// Record layout (bytes; pack_solo_headers in sched.cpp, values by k_pack):
//   [hdr int4: nent, steps in the chunk (+ 1 << 16 if the chunk closes its
//    level), step, the chunk's offset in its level]
//   [out: 32 int][code: nent x 32 int]
//   [blocks: nent x B*B x 32 of T][D^-1: B*B x 32 of T, forward only]
// out: the element offset / B where a lane's result goes (-1: empty lane);
// code >= 0: byte offset into the ring region (0 = 32 zero bytes, padding);
// code < 0: -(position + 1) of a dependency in the output vector.
#include "dfg_common.cuh"
#include "k_mbar.cuh"
#include "k_sweep.h"

namespace dfg {

template <typename T, int B, bool FWD, int MAXE>
__global__ void __launch_bounds__((kSoloWarps + 1) * 32) k_solo(SoloArgs a) {
  constexpr int BS = B * B;
  constexpr int SZ = (int)sizeof(T);
  constexpr int NW = kSoloWarps;
  constexpr int STEP_RHS = 32 * B * SZ;  // right-hand-side bytes of one step
  extern __shared__ __align__(128) unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int NS = a.NS;
  const int RM = a.R - 1;
  const int VS = a.ch_max * STEP_RHS;
  // layout: [bars: 2*NS u64][rstage: NS x rec_stage][vstage: NS x VS][zero 32 B][ring: R x 32 x B of T]
  uint64_t* full = reinterpret_cast<uint64_t*>(smem);
  uint64_t* empty = full + NS;
  unsigned char* rstage = smem + (((size_t)2 * NS * 8 + 127) / 128) * 128;
  unsigned char* vstage = rstage + (size_t)NS * a.rec_stage;
  unsigned char* ringreg = vstage + (size_t)NS * VS;
  __shared__ int s_slot, s_stop;

  if (threadIdx.x == 0) {
    for (int s = 0; s < NS; ++s) {
      mbar_init(&full[s], 1);      // the producer's arrival with the byte count
      mbar_init(&empty[s], NW);    // one arrival per compute warp
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (threadIdx.x < 8) reinterpret_cast<unsigned*>(ringreg)[threadIdx.x] = 0u;
  __syncthreads();

  int g = 0;  // chunks this CTA has pushed through the pipeline (both sides count alike)
  for (;;) {
    if (threadIdx.x == 0) {
      const int t = atomicAdd(a.ticket, 1);
      int j = -1;
      if (t < a.batch->nslots) {
        const int* dn = a.batch->slot[t].done;
        j = (dn && ld_relaxed_int(dn)) ? -2 : t;
      }
      s_slot = j;
    }
    __syncthreads();
    const int jslot = s_slot;
    __syncthreads();
    if (jslot == -1) break;
    if (jslot == -2) continue;  // a finished solve
    const SoloSlot& S = a.batch->slot[jslot];
    const int nch = S.nchunks;
    bool abort = false;
    // pipeline position g: its stage and that stage's use parity; both sides
    // then advance them chunk by chunk (every warp visits every chunk)
    const int st0 = g % NS, ph0 = (g / NS) & 1;
    if (warp == NW) {
      // ------------------------------------------------------------ producer
      // The warp reads the chunk table 32 entries at a time (one coalesced
      // load per 32 chunks, the next batch in flight while this one is
      // issued); lane 0 issues the copies with each entry taken from its
      // lane, so no global-load latency lies between two chunks' copies.
      const unsigned char* __restrict__ recs = S.rec;
      const unsigned char* __restrict__ in = reinterpret_cast<const unsigned char*>(S.in);
      const SoloChunk* __restrict__ chunks = S.chunks;
      int n_issued = 0;
      SoloChunk cur = lane < nch ? chunks[lane] : SoloChunk{};
      SoloChunk nxt = 32 + lane < nch ? chunks[32 + lane] : SoloChunk{};
      int st = st0, ph = ph0;
      for (int base = 0; base < nch && !abort; base += 32) {
        const int cnt = min(32, nch - base);
        for (int i = 0; i < cnt; ++i) {
          const long long rec_off = __shfl_sync(0xffffffffu, cur.rec_off, i);
          const int rec_bytes = __shfl_sync(0xffffffffu, cur.rec_bytes, i);
          const int first_step = __shfl_sync(0xffffffffu, cur.first_step, i);
          const int nsteps = __shfl_sync(0xffffffffu, cur.nsteps, i);
          const int c = base + i;
          if (lane == 0) {
            // the stage's previous use (phase ph ^ 1) must have been released
            if (g + c >= NS && !mbar_wait(&empty[st], (unsigned)(ph ^ 1), a.err, kSiteEmpty, jslot, c)) {
              abort = true;
            } else {
              const unsigned rhs_bytes = (unsigned)(nsteps * STEP_RHS);
              mbar_expect_tx(&full[st], (unsigned)rec_bytes + rhs_bytes);
              tma_load_1d(rstage + (size_t)st * a.rec_stage, recs + rec_off, (unsigned)rec_bytes, &full[st]);
              tma_load_1d(vstage + (size_t)st * VS, in + (size_t)first_step * STEP_RHS, rhs_bytes, &full[st]);
            }
          }
          abort = __shfl_sync(0xffffffffu, abort, 0);
          if (abort) break;
          ++n_issued;
          if (++st == NS) { st = 0; ph ^= 1; }
        }
        cur = nxt;
        nxt = base + 64 + lane < nch ? chunks[base + 64 + lane] : SoloChunk{};
      }
      if (abort && lane == 0) {  // copies already issued land before the CTA moves on (bounded)
        int dst = st0, dph = ph0;
        for (int k = 0; k < n_issued; ++k) {
          mbar_drain(&full[dst], (unsigned)dph);
          if (++dst == NS) { dst = 0; dph ^= 1; }
        }
      }
    } else {
      // ------------------------------------------------------------- compute
      T* out = reinterpret_cast<T*>(S.out);
      int st = st0, ph = ph0;
      for (int c = 0; c < nch; ++c, (++st == NS ? (st = 0, ph ^= 1) : 0)) {
        // (the wait is voted across the warp, so that abort stays warp-uniform)
        if (!abort) abort = !__all_sync(0xffffffffu, mbar_wait(&full[st], (unsigned)ph, a.err, kSiteFull, jslot, c));
        const unsigned char* stage = rstage + (size_t)st * a.rec_stage;
        const int4 hdr = *reinterpret_cast<const int4*>(stage);
        const int nent = hdr.x;
        const int nst = abort ? 0 : (hdr.y & 0xffff);
        const int rec_sz = 144 + nent * 128 + nent * 32 * BS * SZ + (FWD ? 32 * BS * SZ : 0);
        // a chunk may hold the ends of several narrow levels: lane j reads
        // step j's header (does it close its level, its place in the level)
        int yv = 0, wv = 0;
        if (lane < nst) {
          const int4 hj = *reinterpret_cast<const int4*>(stage + (size_t)lane * rec_sz);
          yv = hj.y;
          wv = hj.w;
        }
        const unsigned closes = __ballot_sync(0xffffffffu, lane < nst && (yv >> 16) != 0);
        // segments of one level each; a segment's steps go to warps by their
        // place in the level, so a level of <= kSoloWarps steps costs each
        // warp one step whatever its chunks
        for (int j0 = 0; j0 < nst;) {
          const unsigned rest = closes >> j0;
          const int j1 = rest ? j0 + __ffs(rest) : nst;
          const int p0 = __shfl_sync(0xffffffffu, wv, j0);
          for (int k = j0 + (warp - p0 % NW + NW) % NW; k < j1; k += NW) {
            const unsigned char* rec = stage + (size_t)k * rec_sz;
            const int s = reinterpret_cast<const int*>(rec)[2];
            const int o = reinterpret_cast<const int*>(rec + 16)[lane];
            const int* code = reinterpret_cast<const int*>(rec + 144);
            const T* blk = reinterpret_cast<const T*>(rec + 144 + nent * 128);
            if (o >= 0) {
              const T* val = reinterpret_cast<const T*>(vstage + (size_t)st * VS + (size_t)k * STEP_RHS);
              T t[B];
#pragma unroll
              for (int d = 0; d < B; ++d) t[d] = val[lane * B + d];
              if constexpr (MAXE > 0) {
                // all dependency values first, then the FMAs.  The codes are
                // loaded together, then every value from the ring together
                // (a global reference reads the ring's zero bytes first), so
                // the step waits on two shared-memory round trips, not two per
                // entry; global references are read after, in a warp-uniform
                // branch that is taken only where the ring does not reach
                int cdv[MAXE];
#pragma unroll
                for (int e = 0; e < MAXE; ++e) cdv[e] = e < nent ? code[e * 32 + lane] : 0;
                T v[MAXE][B];
                bool glob = false;
#pragma unroll
                for (int e = 0; e < MAXE; ++e) {
                  const T* vp = reinterpret_cast<const T*>(ringreg + (cdv[e] >= 0 ? cdv[e] : 0));
#pragma unroll
                  for (int d = 0; d < B; ++d) v[e][d] = vp[d];
                  glob |= cdv[e] < 0;
                }
                if (__any_sync(__activemask(), glob)) {
#pragma unroll
                  for (int e = 0; e < MAXE; ++e) {
                    if (cdv[e] < 0) {
                      const T* gp = out + (size_t)(-cdv[e] - 1) * B;
#pragma unroll
                      for (int d = 0; d < B; ++d) v[e][d] = __ldcg(gp + d);
                    }
                  }
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
                  const int cd = code[e * 32 + lane];
                  T v[B];
                  if (cd >= 0) {
                    const T* vp = reinterpret_cast<const T*>(ringreg + cd);
#pragma unroll
                    for (int d = 0; d < B; ++d) v[d] = vp[d];
                  } else {
                    const T* gp = out + (size_t)(-cd - 1) * B;
#pragma unroll
                    for (int d = 0; d < B; ++d) v[d] = __ldcg(gp + d);
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
              T* rg = reinterpret_cast<T*>(ringreg + 32) + (((s & RM) * 32 + lane) * B);
#pragma unroll
              for (int d = 0; d < B; ++d) {
                rg[d] = y[d];
                out[(size_t)o * B + d] = y[d];
              }
            }
          }
          if (rest) named_sync(1, NW * 32);  // the segment closes its level
          j0 = j1;
        }
        // a warp that gave up waiting takes the chunk's level ends from its
        // table entry, so that every warp passes the same barriers
        if (abort) {
          const int nb = __ldg(&S.chunks[c].nclose);
          for (int i = 0; i < nb; ++i) named_sync(1, NW * 32);
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[st]);
      }
    }
    g += nch;
    if (__any_sync(0xffffffffu, abort)) {
      if (lane == 0) record_fail(a.err, kErrTimeout, kSiteRange, jslot, -1);
    }
    // one read of the error word decides for the whole CTA
    __syncthreads();
    if (threadIdx.x == 0) s_stop = ld_relaxed_int(a.err) != 0;
    __syncthreads();
    if (s_stop) break;
  }
}

template <typename T>
__global__ void k_solo_permute(long long n, int b, const int* __restrict__ pos, const T* __restrict__ in,
                               T* __restrict__ out) {
  const long long m = n * b;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < m; k += (long long)gridDim.x * blockDim.x) {
    const long long row = k / b;
    out[(long long)pos[row] * b + (k - row * b)] = in[k];
  }
}

// ------------------------------------------------------------------ launchers

cudaError_t launch_solo_permute(bool fp32, long long n, int b, const int* pos, const void* in, void* out,
                                cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const int grid = (int)std::min<long long>((n * b + 255) / 256, 1216);
  if (fp32) k_solo_permute<float><<<grid, 256, 0, st>>>(n, b, pos, static_cast<const float*>(in), static_cast<float*>(out));
  else k_solo_permute<double><<<grid, 256, 0, st>>>(n, b, pos, static_cast<const double*>(in), static_cast<double*>(out));
  return cudaGetLastError();
}

template <typename T, int B, bool FWD>
static cudaError_t launch_e(const SoloArgs& a, int grid, size_t smem, cudaStream_t st) {
  constexpr int NT = (kSoloWarps + 1) * 32;
  if (a.max_nent <= 4) k_solo<T, B, FWD, 4><<<grid, NT, smem, st>>>(a);
  else if (a.max_nent <= 8) k_solo<T, B, FWD, 8><<<grid, NT, smem, st>>>(a);
  else k_solo<T, B, FWD, 0><<<grid, NT, smem, st>>>(a);
  return cudaGetLastError();
}

template <typename T, bool FWD>
static cudaError_t launch_b(int B, const SoloArgs& a, int grid, size_t smem, cudaStream_t st) {
  switch (B) {
    case 1: return launch_e<T, 1, FWD>(a, grid, smem, st);
    case 2: return launch_e<T, 2, FWD>(a, grid, smem, st);
    case 3: return launch_e<T, 3, FWD>(a, grid, smem, st);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_solo(bool forward, bool fp32, int B, const SoloArgs& a, int grid, size_t smem, cudaStream_t st) {
  if (fp32) return forward ? launch_b<float, true>(B, a, grid, smem, st) : launch_b<float, false>(B, a, grid, smem, st);
  return forward ? launch_b<double, true>(B, a, grid, smem, st) : launch_b<double, false>(B, a, grid, smem, st);
}

template <typename T, int B, bool FWD>
static cudaError_t set_attr(size_t max_smem) {
  cudaError_t e = cudaFuncSetAttribute(k_solo<T, B, FWD, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_solo<T, B, FWD, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_solo<T, B, FWD, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);
  return e;
}

cudaError_t solo_set_smem_limits(size_t max_smem) {
  cudaError_t e = cudaSuccess;
#define DFG_ATTR(T, B)                                        \
  if (e == cudaSuccess) e = set_attr<T, B, true>(max_smem);   \
  if (e == cudaSuccess) e = set_attr<T, B, false>(max_smem);
  DFG_ATTR(double, 1) DFG_ATTR(double, 2) DFG_ATTR(double, 3)
  DFG_ATTR(float, 1) DFG_ATTR(float, 2) DFG_ATTR(float, 3)
#undef DFG_ATTR
  return e;
}

}  // namespace dfg
