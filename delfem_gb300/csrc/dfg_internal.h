// dfg_internal.h -- host-side structures of libdfg (not part of the ABI).
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/dfg.h"
#include "k_sweep.h"

namespace dfg {

// ------------------------------------------------------------------ errors

struct Error {
  int status;
  std::string msg;
};

// ------------------------------------------------------------ device buffer

struct DBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DBuf() = default;
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  DBuf(DBuf&& o) noexcept : p(o.p), bytes(o.bytes) { o.p = nullptr; o.bytes = 0; }
  DBuf& operator=(DBuf&& o) noexcept {
    if (this != &o) { release(); p = o.p; bytes = o.bytes; o.p = nullptr; o.bytes = 0; }
    return *this;
  }
  ~DBuf() { release(); }
  void release();
  template <class T> T* as() const { return static_cast<T*>(p); }
};

// --------------------------------------------------------------- schedules

// Forward/backward sweep over the rows of a block-triangular factor, cut into
// contiguous "ranges" (one warp each) and, inside a range, into "steps" of up
// to 32 rows whose intra-range dependencies all sit in earlier steps.  Each
// dependency is encoded as
//   src >= 0        : ring slot (step % R)*32 + lane of a row of the same range
//                     finished fewer than R steps ago (read from shared memory)
//   src == kSrcPad  : padding
//   otherwise       : -(row+1), a row read from the global output buffer
//                     (another range, or an old row of the same range)
struct SweepPlan {
  static constexpr int kSrcPad = INT32_MIN;
  bool forward = true;
  int n = 0, b = 1;
  int nranges = 0, nsteps = 0, R = 32, max_nent = 0;
  std::vector<int> range_steps;      // nranges+1
  std::vector<int> step_nent;        // nsteps
  std::vector<long long> ent_off;    // nsteps+1, in units of 32-lane entries
  std::vector<int> step_rows;        // nsteps*32, -1 = empty lane
  std::vector<int> ent_src;          // ent_off[nsteps]*32
  std::vector<int> ent_slot;         // CRS slot of the block (-1 for padding)
  double est_cost = 0.0;             // model makespan (steps), for range-size choice
};

// byte layout of one step record for element size `sz` (k_sweep.cu):
//   [hdr 16][row 32*4][code nent*32*4][grow nent*32*4][blk nent*32*bs*sz][dinv 32*bs*sz (forward only)]
inline long long rec_bytes(int nent, int bs, int sz, bool forward) {
  return 16 + 128 + (long long)nent * 256 + (long long)nent * 32 * bs * sz + (forward ? 32LL * bs * sz : 0);
}

// Host-assembled static parts of the step records of a plan (header, row
// ids, dependency codes, dependency rows) for element size `elem`; the value
// regions stay zero and are filled on the device after each factorisation.
// A code is a byte offset the compute warp adds to one of two bases without
// branching: the ring region for a dependency finished by the same range
// within the last R steps (offset 0 = 32 zero bytes for padding), or -- bit 31
// set -- the step's value slot, where the loader warp gathers the 16-byte
// window holding an out-of-range dependency.
std::vector<unsigned char> pack_record_headers(const SweepPlan& P, int elem, std::vector<long long>& off,
                                               long long& max_rec);

// Plan of one solve's sweep run by a single CTA (k_solo.cu): the SweepPlan
// structure with one "range" per dependency level -- range_steps holds the
// first step of each level, nranges the number of levels -- and steps of <= 32
// rows of one level, in row order.  The steps of a level are cut into chunks
// (at most `ch_max` steps and `stage_bytes` of records each, elem-byte
// values), the unit the kernel copies into shared memory; every step of a
// chunk carries the chunk's largest entry count (padding entries zero), so a
// chunk's records all have one size.  A dependency is a ring slot when its
// step is among the R steps before the end of the consuming step's level
// (the ring is never overwritten while that level runs), else a global read.
struct SoloPlan {
  SweepPlan P;                      // steps, padded entries (ent_off / ent_src / ent_slot)
  std::vector<SoloChunk> chunks;
  std::vector<int> lev_chunks;      // nlevels + 1: the chunk holding each level's first step
  std::vector<int> pos;             // per row: step * 32 + lane (its slot in step order)
};
SoloPlan solo_sweep_plan(int n, int b, const int* rowptr, const int* colind, const int* diaind, bool forward,
                         int R, int elem, int stage_bytes, int ch_max);

// byte layout of one solo step record (k_solo.cu):
//   [hdr int4: nent, chunk steps, step, chunk's first step - its level's first step]
//   [out: 32 int][code nent*32*4][blk nent*32*bs*sz][dinv 32*bs*sz (forward only)]
inline long long solo_rec_bytes(int nent, int bs, int sz, bool forward) {
  return 16 + 128 + (long long)nent * 128 + (long long)nent * 32 * bs * sz + (forward ? 32LL * bs * sz : 0);
}
// Static parts of the solo step records (header, output positions, codes) for
// element size `elem`.  out_pos[row]: where the sweep writes the row's result
// (its position in the vector's storage order); glob_pos[row]: where a global
// dependency read finds a row (the storage order of the sweep's own output).
// code >= 0 is a byte offset into the CTA's ring region (0 = 32 zero bytes,
// for padding); code < 0 is -(glob_pos[row] + 1).  rec_off: nsteps + 1 byte
// offsets (the value packer's view).
std::vector<unsigned char> pack_solo_headers(const SoloPlan& S, int elem, const int* out_pos, const int* glob_pos,
                                             std::vector<long long>& rec_off);

// level sets of the triangular dependency DAG (rows sorted by level, then row)
struct Levels {
  std::vector<int> level;   // per row
  std::vector<int> ptr;     // nlevels+1
  std::vector<int> rows;    // n
};

Levels build_levels(int n, const int* rowptr, const int* colind, const int* diaind, bool forward);
// ILU(lev_fill) factor pattern (AddFracPtn); false beyond max_nnz entries
bool ilu_fill_pattern(int n, const int* rowptr, const int* colind, int lev_fill, std::vector<int>& rowptr_f,
                      std::vector<int>& colind_f, long long max_nnz);
// A's CRS slot -> factor slot of the same block
bool factor_slot_map(int n, const int* rowptr, const int* colind, const int* rowptr_f, const int* colind_f,
                     std::vector<int>& a2f);
SweepPlan build_sweep_plan(int n, int b, const int* rowptr, const int* colind, const int* diaind,
                           bool forward, int range_rows, int R);
SweepPlan choose_sweep_plan(int n, int b, const int* rowptr, const int* colind, const int* diaind,
                            bool forward, int R, int elem_size);
// the plan with the fullest steps among ranges of 8, 16 and 32 typical
// dependency distances (batched launches)
SweepPlan fullest_sweep_plan(int n, int b, const int* rowptr, const int* colind, const int* diaind, bool forward,
                             int R);
// the `keep` plans with the lowest model makespan over range sizes 256, 512, ... rows
std::vector<SweepPlan> candidate_sweep_plans(int n, int b, const int* rowptr, const int* colind, const int* diaind,
                                             bool forward, int R, int keep);

// node-to-node pattern from elements, no diagonal, ascending (MakePattern_FEM)
void pattern_from_elements(int nnode, int nelem, int nnoel, const int* conn,
                           std::vector<int>& rowptr, std::vector<int>& colind);

// Element-to-slot gather map.  Slot s < n is diagonal block s, slot n+c is
// off-diagonal CRS block c.  slot_src lists, in increasing element order,
// the element-matrix block index e*k*k + i*k + j contributing to that slot;
// res_src lists e*k + i for each node.  Summing in this order reproduces the
// reference's CMatDia_BlkCrs::Mearge / CVector_Blk::AddValue order exactly.
struct GatherMap {
  std::vector<long long> slot_ptr;  // n+nnz+1
  std::vector<int> slot_src;
  std::vector<long long> res_ptr;   // n+1
  std::vector<int> res_src;
};
bool build_gather_map(int n, const int* rowptr, const int* colind, int nelem, int nnoel,
                      const int* conn, GatherMap& out, std::string& err);

// Sliced-ELL copy of the block matrix for the PCG products: slice s holds
// rows [32s, 32s+32) and W_s block columns (the longest row of the slice, its
// off-diagonal blocks in CRS order then the diagonal block, then padding).
// Block position k = ptr[s] + w*32 + lane holds row 32s+lane's w-th block;
// col[k] is its column (the row itself for padding) and src[k] its source:
// >= 0 an off-diagonal CRS slot, -1 padding (zero), <= -2 the diagonal block
// of row -src-2.  Values are stored entry-major per position group:
// value (k, e) at (ptr[s]*bs + (w*bs + e)*32 + lane), so 32 lanes reading
// entry e of their w-th block touch 32 consecutive words.
struct SellMap {
  int nslices = 0;
  std::vector<long long> ptr;  // nslices+1, in blocks
  std::vector<int> width;      // nslices
  std::vector<int> col;        // ptr[nslices]
  std::vector<int> src;        // ptr[nslices]
};
SellMap build_sell(int n, const int* rowptr, const int* colind);

// --------------------------------------------------------------- handles

struct Ctx;

struct PcgState;  // device-side solver state (defined in solve.cu)

struct SweepDev {
  bool forward = true;
  // level-scheduled (one launch per level, k_level.cu) instead of ranged
  bool levels = false;
  float t_ranged = -1.f, t_levels = -1.f;  // set-up timings of the two kinds (ms; -1 = not timed)
  Levels lev;
  DBuf lev_info;   // level-scheduled: int4 {row, first entry, end entry, 0} per position
  int lev_G = 4;   // level-scheduled: lanes per row
  // one CTA (k_solo.cu): the input is permuted into the plan's step order
  // first, the output is written in row order; [0] FP64 records, [1] FP32
  bool solo = false;
  float t_solo = -1.f;
  struct SoloDev {
    SoloPlan plan;
    SoloShape shape;
    DBuf rec, rec_off, chunks, lev_chunks, ent_off, ent_slot, step_rows;
  };
  SoloDev sd[2];
  DBuf solo_pos, solo_in;      // row -> position (int); the permuted input (FP64-sized)
  DBuf solo_batch;             // kSoloBatchRing single-slot batches, one per launch set-up in use
  int solo_next = 0;
  int solo_maxe = 0;
  // ranged: one packed record buffer per precision
  DBuf rec64, rec32;
  DBuf rec_off64, rec_off32;       // long long per step (+1)
  DBuf step_nent, range_steps;
  DBuf ent_slot, ent_off, step_rows;
  long long rec_total64 = 0, rec_total32 = 0;
  long long max_rec64 = 0, max_rec32 = 0;
  SweepPlan plan;
};

}  // namespace dfg

struct dfg_ctx_s {
  int device = 0;
  int nsm = 0;
  size_t smem_optin = 0;
  cudaStream_t stream = nullptr;
  std::string last_error;
  long long launches = 0;
  dfg::DBuf err_word;     // int, device error word (dfg::kErr*)
  dfg::DBuf scratch;      // reduction partials + scalars
  int* h_pinned = nullptr;  // small pinned host area for status reads
  int last_timeout_site = 0;  // wait site of the last reported timeout
};

struct dfg_system_s {
  dfg_ctx ctx = nullptr;
  int n = 0, b = 1;
  long long nnz = 0;
  std::vector<int> h_rowptr, h_colind, h_diaind;
  dfg::DBuf rowptr, colind, diaind;
  dfg::DBuf diag, offd;            // FP64 matrix, reference layout
  dfg::DBuf diag32, offd32;        // FP32 copy (mixed precision)
  bool mat32_valid = false;
  // sliced-ELL copies for the PCG products (SellMap), repacked when the
  // matrix changed (mat_version) since the last pack
  int sell_nslices = 0;
  long long sell_blocks = 0;
  dfg::DBuf s_ptr, s_width, s_col, s_src, s_val64, s_val32;
  long long mat_version = 0, sell64_version = -1, sell32_version = -1;
  dfg::DBuf res, upd, rhs0;        // slots -1, -2 and the finalized right-hand side
  bool rhs0_valid = false;
  std::vector<dfg::DBuf> tmp;      // slots >= 0
  dfg::DBuf bcflag;
  bool has_bc = false;
  dfg::DBuf load;                  // resident nodal load added at finalize
  bool has_load = false;
  // mesh
  int ndim = 0, nelem = 0, nnoel = 0;
  dfg::DBuf coords, conn, coef, fu, fv;
  bool has_coef = false, has_u = false, has_v = false;
  dfg::DBuf slot_ptr, slot_src, res_ptr, res_src;
  dfg::DBuf em, er;                // element matrices / residuals (assembly scratch)
  // solver workspace (allocated on first solve)
  dfg::DBuf w_p, w_q, w_z, w_state;          // FP64 PCG
  dfg::DBuf w_rd, w_d, w_r32, w_p32, w_q32, w_z32;  // mixed
  dfg::DBuf w_bicg;                           // BiCGSTAB vectors, state, paired-sum scratch
};

struct dfg_precond_s {
  dfg_ctx ctx = nullptr;
  int lev = 0;
  dfg_system sys = nullptr;        // system of the symbolic set-up
  bool symbolic = false, numeric = false, numeric32 = false;
  int n = 0, b = 1;
  long long nnz = 0;               // off-diagonal blocks of the factor
  // Factor pattern: the system's (own_pattern false) unless fill-in changed it
  bool own_pattern = false;
  std::vector<int> h_rowptr, h_colind, h_diaind;
  dfg::DBuf rowptr, colind, diaind, a2f;  // a2f: A's CRS slot -> factor slot
  int sweep_mode = 0;                     // 0 timed choice, 1 ranged, 2 level-scheduled
  dfg::DBuf fdiag32, foffd32;             // FP32 factor in CRS (level-scheduled FP32 sweeps)
  dfg::DBuf fdiag, foffd;          // factor, reference layout (FP64)
  dfg::Levels lev_fwd;
  dfg::DBuf lev_rows;
  dfg::SweepDev fwd, bwd;
  dfg::DBuf ybuf64, ybuf32;        // forward-sweep outputs
};
