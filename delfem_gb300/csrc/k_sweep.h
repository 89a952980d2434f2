// k_sweep.h -- launch interface of the triangular-sweep kernels.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>

namespace dfg {

// Several independent sweeps in one launch (the serving path): a claimed
// ticket t selects the slot j with range_start[j] <= t < range_start[j+1] and
// its range t - range_start[j]; ranges of a slot whose *done is non-zero are
// skipped.  All slots share the launch's stage sizes (rec_stage, val_stage,
// R, NS), so every slot's records must fit them.
constexpr int kSweepMaxSlots = 256;
struct SweepSlot {
  const unsigned char* rec;
  const long long* rec_off;
  const int* range_steps;
  const void* in;
  void* out;
  const int* done;
};
struct SweepBatch {
  int nslots;
  int range_start[kSweepMaxSlots + 1];
  SweepSlot slot[kSweepMaxSlots];
};

struct SweepArgs {
  const SweepBatch* batch;    // non-null: batched launch (rec .. done below unused)
  const unsigned char* rec;   // packed step records
  const long long* rec_off;   // nsteps+1 byte offsets
  const int* range_steps;     // nranges+1
  int nranges;
  const void* in;             // right-hand side, n*B of T
  void* out;                  // result, n*B of T, pre-filled with the sentinel (+32 B slack)
  int* ticket;                // range ticket counter (0 at launch)
  int* err;                   // device error word
  const int* done;            // optional: skip the launch when *done != 0
  int rec_stage;              // bytes per record slot (>= the largest record)
  int val_stage;              // bytes per value slot
  int R;                      // ring depth in steps
  int NS;                     // pipeline stages
  int max_nent;               // most dependency entries of any step (selects the unrolled variant)
};

// smem bytes a launch needs: mbarriers, NS record slots, NS value slots,
// a 32-byte zero pad and the ring
inline size_t sweep_smem_bytes(int NS, int rec_stage, int val_stage, int R, int B, int elem) {
  return ((size_t)3 * NS * 8 + 127) / 128 * 128 + (size_t)NS * rec_stage + (size_t)NS * val_stage + 32 +
         (size_t)R * B * 32 * elem;
}
// bytes of the right-hand-side part of a value slot
inline int sweep_rhs_bytes(int B, int elem) { return (B * 32 * elem + 15) / 16 * 16; }
// bytes of one value slot: right-hand sides + 32-byte windows per dependency entry
inline int sweep_val_stage(int max_nent, int B, int elem) { return sweep_rhs_bytes(B, elem) + max_nent * 32 * 32; }

// launchers (k_sweep.cu)
// dep: launch as a programmatic dependent of the previous kernel in the stream
cudaError_t launch_sweep(bool forward, bool fp32, int B, const SweepArgs& a, int grid, size_t smem,
                         cudaStream_t st, bool dep = false);
cudaError_t sweep_set_smem_limits(size_t max_smem);
// one bounded wait on a value nothing writes (`never` holds the sentinel)
cudaError_t launch_wait_selftest(const double* never, int* err, cudaStream_t st);

// packing the factor into step records (k_sweep.cu)
struct PackArgs {
  int nsteps;
  unsigned char* rec;
  const long long* rec_off;
  const long long* ent_off;   // nsteps+1
  const int* ent_slot;        // per 32-lane entry
  const int* step_rows;       // nsteps*32
  const double* fdiag;
  const double* foffd;
  int code_bytes;             // bytes of dependency codes per entry: 256 ranged (code + row), 128 solo; 0 = 256
};
cudaError_t launch_pack(bool forward, bool fp32, int B, const PackArgs& a, cudaStream_t st);

// Solo sweeps (k_solo.cu): a CTA owns one solve's whole sweep, level after
// level (solo_sweep_plan / pack_solo_headers in sched.cpp).  The sweep's
// input is stored in its step order (element (step*32 + lane)*B + d), so a
// chunk of steps needs two contiguous bulk copies: its records and its
// right-hand sides.  Batched: a ticket claims the next solve of the batch,
// in batch order.
struct SoloChunk {
  long long rec_off;  // byte offset of the chunk's first record
  int rec_bytes;      // bytes of the chunk's records
  int first_step, nsteps, nent;
  int nclose;         // levels that end inside the chunk
};
struct SoloSlot {
  const unsigned char* rec;
  const SoloChunk* chunks;
  const int* lev_chunks;  // nlevels + 1: the chunk holding each level's first step
  int nlevels, nchunks;
  const void* in;         // right-hand sides in step order (nsteps*32*B of T)
  void* out;              // results at the records' output positions
  const int* done;        // the solve's state: nonzero = skip
};
struct SoloBatch {
  int nslots;
  SoloSlot slot[kSweepMaxSlots];
};
struct SoloArgs {
  const SoloBatch* batch;
  int* ticket;       // 0 at launch
  int* err;          // device error word
  int rec_stage;     // bytes per record stage (>= every chunk's records, 16-aligned)
  int ch_max;        // steps per chunk at most (sizes the right-hand-side stage)
  int NS;            // pipeline stages
  int R;             // ring depth in steps (a power of two)
  int max_nent;      // selects the unrolled variant
};
// compute warps per CTA (plus one producer warp)
constexpr int kSoloWarps = 16;
inline int solo_val_stage(int ch_max, int B, int elem) { return ch_max * 32 * B * elem; }
inline size_t solo_smem_bytes(int NS, int rec_stage, int val_stage, int R, int B, int elem) {
  return ((size_t)2 * NS * 8 + 127) / 128 * 128 + (size_t)NS * rec_stage + (size_t)NS * val_stage + 32 +
         (size_t)R * 32 * B * elem;
}
cudaError_t launch_solo(bool forward, bool fp32, int B, const SoloArgs& a, int grid, size_t smem, cudaStream_t st);
// out[pos[row]*b + c] = in[row*b + c] for rows < n: a vector in row order into
// a solo sweep's step order (elements of T: float when fp32)
cudaError_t launch_solo_permute(bool fp32, long long n, int b, const int* pos, const void* in, void* out,
                                cudaStream_t st);

// Shared-memory shape of a solo sweep CTA for block size b, rows of at most
// maxe lower or upper entries and elem-byte values, in `budget` bytes.  The
// ring: rows with at most 4 entries (triangle meshes) depend on the level
// before theirs only, at most about 20 steps wide on meshes of up to 400k
// nodes, so 64 steps hold every dependency; wider rows (tetrahedral meshes,
// levels of up to ~150 steps reaching two or three levels back) get up to a
// third of the budget (a power of two of steps, at most 512).  The chunk
// stages take the rest -- the bytes in flight that hide HBM latency: up to 64
// of them, each holding up to ch_max steps' records and right-hand sides;
// ch_max (1..16) is the largest (fewest chunk handshakes per level) within
// 10 % of the most steps in flight.  ns == 0 when nothing fits.
struct SoloShape {
  int R = 0, ch_max = 0, rec_stage = 0, ns = 0;
  size_t smem = 0;
};
inline long long solo_record_bytes(int nent, int bs, int sz, bool forward) {
  return 16 + 128 + (long long)nent * 128 + (long long)nent * 32 * bs * sz + (forward ? 32LL * bs * sz : 0);
}
inline SoloShape solo_shape(int b, int maxe, int elem, bool forward, size_t budget) {
  SoloShape sh;
  const size_t step_ring = (size_t)32 * b * elem;
  int R = maxe <= 4 ? 64 : 512;
  while (R > 16 && (size_t)R * step_ring > budget / 3) R /= 2;
  sh.R = R;
  const long long rec1 = solo_record_bytes(maxe, b * b, elem, forward);
  const size_t fixed = solo_smem_bytes(64, 0, 0, R, b, elem);
  // chunks above 8 steps only with at least 4 stages, so that the producer
  // still refills stages while others are consumed
  int ns_of[17] = {}, most = 0;
  auto usable = [&](int ch) { return ns_of[ch] >= (ch <= 8 ? 2 : 4); };
  for (int ch = 1; ch <= 16; ++ch) {
    const size_t per_stage = (size_t)ch * rec1 + (size_t)solo_val_stage(ch, b, elem);
    ns_of[ch] = (int)std::min<size_t>(64, (budget - std::min(budget, fixed)) / per_stage);
    if (usable(ch)) most = ns_of[ch] * ch > most ? ns_of[ch] * ch : most;
  }
  for (int ch = 1; ch <= 16; ++ch)
    if (usable(ch) && 10 * ns_of[ch] * ch >= 9 * most) { sh.ch_max = ch; sh.ns = ns_of[ch]; }
  if (sh.ns > 0) {
    sh.rec_stage = (int)(sh.ch_max * rec1);
    sh.smem = solo_smem_bytes(sh.ns, sh.rec_stage, solo_val_stage(sh.ch_max, b, elem), R, b, elem);
  }
  return sh;
}
cudaError_t solo_set_smem_limits(size_t max_smem);

// Level-scheduled sweep (k_level.cu): the factor in block CRS (values of
// the sweep's type), rows listed level after level; one launch per level.
struct LevelSweepArgs {
  const int4* info;    // per position (rows level after level): {row, first entry, end entry, 0}
  const int* colind;
  const void* fdiag;   // D^-1 blocks (forward)
  const void* foffd;   // L | D^-1 U blocks
  const void* in;
  void* out;
  const int* done;     // nonzero: return at once
  int G;               // lanes per row: level_group_lanes of the widest row
};
// lanes per row of the level-scheduled sweep: the smallest power of two that
// holds `max_entries`, 4 to 32
inline int level_group_lanes(int max_entries) {
  int g = 4;
  while (g < 32 && g < max_entries) g *= 2;
  return g;
}
// dependent: launch as a programmatic dependent of the previous kernel in the
// stream (a previous level of the same sweep; the first level is launched in
// plain stream order)
cudaError_t launch_sweep_level(bool forward, bool fp32, int b, const LevelSweepArgs& a, int first, int cnt,
                               bool dependent, cudaStream_t s);

}  // namespace dfg
