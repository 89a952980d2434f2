// serve.cu -- the serving runtime: a persistent request loop that keeps many
// FE solves resident on the device and advances all of them with batched
// launches replayed from one captured CUDA graph.
//
// Request life cycle:
//   submit      inputs copied; queued for the symbolic workers
//   symbolic    host threads: node pattern (MakePattern_FEM), element-to-slot
//               gather map, ILU level sets, forward/backward sweep schedules
//               and their record headers, and the request's device memory plan
//   admission   one thread, FIFO: once the request's bytes fit the device
//               arena and an in-flight slot is free, it uploads the request and
//               runs assembly (element kernels + gather), Dirichlet rows, the
//               ILU(0) factorisation, record packing and the PCG start on its
//               own low-priority stream; transient buffers are released
//   iteration   the loop thread adds the solve to its size group's slot table;
//               each group has its own graph and streams, so groups iterate
//               concurrently at their own pace; every replay of a group's
//               graph runs `chunk` PCG iterations of all its slots (sweeps
//               per block-size class on parallel branches, then the batched
//               vector kernels), checks converged slots' true residuals, and
//               copies a status array back
//   retire      a finished slot leaves the table; its solution is copied to the
//               caller's buffer and its memory returns to the arena
// Nothing on the loop path allocates or frees device memory: the arena is one
// reservation made at creation.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <atomic>
#include <condition_variable>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "dfg_internal.h"
#include "k_assemble.h"
#include "k_ilu.h"
#include "k_serve.h"
#include "k_solve.h"
#include "k_sweep.h"

using namespace dfg;

namespace {

using Clock = std::chrono::steady_clock;

constexpr int kClasses = 9;         // block size 1..3 x dependency entries <= 4, 8, 16
constexpr int kMaxChunks = 1 << 20; // chunk space of one launch (kSrvRows rows each)
constexpr int kRingSteps = 32;
constexpr int kServeStages = 3;   // sweep pipeline depth in batched launches
// mixed form: a reliable update falls due once the recursive residual norm
// has dropped by 10x since the last one (delta 0.1, as dfg_solve_pcg_mixed)
constexpr double kMixedDelta2 = 0.01;
// Solves are iterated in groups of similar size, each with its own table and
// graph on its own streams (dfg_server_config::size_groups): a batched sweep
// lasts as long as the largest solve's dependency chain, so small solves that
// share a table with large ones idle for most of every iteration.  Measured on
// the 2D serving stream: three groups keep the throughput of one table (41.8
// vs 41.9 solves/s, FP32 factor) and halve the median latency (0.80 vs
// 1.54 s), so three is the default.
// Groups by DOF: < 30k, < 150k, larger (three); < 60k, larger (two).
constexpr int kGroups = 3;
// Admission lanes: requests are admitted (uploads, assembly, Dirichlet, the
// level-by-level ILU, packing) this many at a time, each on its own stream.
constexpr int kAdmLanes = 4;
inline int group_of(long long dof, int ngroups) {
  if (ngroups <= 1) return 0;
  if (ngroups == 2) return dof < 60000 ? 0 : 1;
  return dof < 30000 ? 0 : dof < 150000 ? 1 : 2;
}

struct CudaFail {
  cudaError_t e;
  const char* what;
};
#define SCK(call)                                   \
  do {                                              \
    cudaError_t e_ = (call);                        \
    if (e_ != cudaSuccess) throw CudaFail{e_, #call}; \
  } while (0)

// ------------------------------------------------------------------ arena

// First-fit allocator over one device reservation; offsets and sizes are
// multiples of 256 bytes.
class Arena {
 public:
  void init(size_t bytes) {
    cap_ = bytes / 256 * 256;
    free_.clear();
    if (cap_) free_[0] = cap_;
  }
  bool alloc(size_t bytes, size_t* off) {
    bytes = round(bytes);
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= bytes) {
        *off = it->first;
        const size_t rest = it->second - bytes, o = it->first + bytes;
        free_.erase(it);
        if (rest) free_[o] = rest;
        used_ += bytes;
        peak_ = std::max(peak_, used_);
        return true;
      }
    }
    return false;
  }
  void release(size_t off, size_t bytes) {
    bytes = round(bytes);
    used_ -= bytes;
    auto it = free_.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
  size_t capacity() const { return cap_; }
  size_t peak() const { return peak_; }
  static size_t round(size_t b) { return (std::max<size_t>(b, 1) + 255) / 256 * 256; }

 private:
  std::map<size_t, size_t> free_;
  size_t cap_ = 0, used_ = 0, peak_ = 0;
};

struct Layout {
  size_t total = 0;
  size_t add(size_t bytes) {
    const size_t o = total;
    total += Arena::round(bytes);
    return o;
  }
};

// ---------------------------------------------------------------- requests

struct Req {
  long long id = 0;
  int kind = 0, b = 1, ndim = 2, nnoel = 3, n = 0, nelem = 0;
  std::vector<double> coords, coef, load, params;
  std::vector<int> conn, bcflag;
  double* x_out = nullptr;
  double t_submit = 0, t_admit = 0, t_done = 0;
  // symbolic set-up
  std::vector<int> rowptr, colind, diaind;
  long long nnz = 0;
  GatherMap gm;
  SellMap sell;
  Levels lev;
  SweepPlan pf, pb;
  std::vector<unsigned char> hf, hb;
  std::vector<long long> of, ob;
  long long maxrf = 0, maxrb = 0;
  int cls = -1, maxe = 0, group = 0;
  bool solo = false;  // sweeps by one CTA per solve (k_solo.cu), else ranged (k_sweep.cu)
  // solo: chunk tables, first chunk per level, and the forward plan's
  // position of every row (where the forward input is stored)
  std::vector<SoloChunk> chf, chb;
  std::vector<int> posf;
  // algorithmic bytes of one launch of each batched kernel for this solve:
  // 0 r.z, 1 p update, 2 SpMV, 3 r/x update, then forward and backward sweep
  double alg[6] = {};
  // device memory plan (offsets into the persistent / transient blocks)
  Layout P, T;
  size_t o_sptr, o_swidth, o_scol, o_sval, o_sval32, o_rhs, o_r, o_x, o_p, o_q, o_rd, o_y, o_z, o_r32;
  size_t o_recf, o_offf, o_rsf, o_recb, o_offb, o_rsb, o_st, o_cnt;
  size_t o_chf = 0, o_chb = 0, o_posf = 0, o_rperm = 0;
  size_t t_rowptr, t_colind, t_diag, t_offd, t_ssrc;
  size_t t_coords, t_conn, t_coef, t_bc, t_load, t_em, t_er, t_sp, t_ss, t_rp, t_rs, t_dia, t_lev, t_fd, t_fo;
  size_t t_eof, t_esf, t_srf, t_eob, t_esb, t_srb;
  size_t pbase = 0, tbase = 0;
  bool have_p = false, have_t = false;
  // outcome
  int status = DFG_OK;
  std::string error;
  int iters = 0;
  double conv = 0, rel_true = -1;
  bool finished = false;
};

inline int class_index(int b, int maxe) { return (b - 1) * 3 + (maxe <= 4 ? 0 : maxe <= 8 ? 1 : 2); }
inline int class_maxe(int c) { return (c % 3) == 0 ? 4 : (c % 3) == 1 ? 8 : 16; }
inline int class_b(int c) { return c / 3 + 1; }

// Device tables, streams and graphs of one size group (see kGroups).
struct Group {
  SrvTable* d_tab = nullptr;
  SrvTable* h_tab = nullptr;       // pinned mirror
  SweepBatch* d_sb = nullptr;      // kClasses x 2 (forward, backward): ranged sweeps
  SweepBatch* h_sb = nullptr;
  SoloBatch* d_solo = nullptr;     // kClasses x 2: one-CTA-per-solve sweeps
  SoloBatch* h_solo = nullptr;
  int* d_tickets = nullptr;        // kClasses x 2 ranged, then kClasses x 2 solo
  double* d_partials = nullptr;    // kMaxChunks
  unsigned char* d_chunk_slot = nullptr;  // kMaxChunks: each chunk's slot
  unsigned char* h_chunk_slot = nullptr;
  unsigned char* d_stat = nullptr; // SrvStatus[kSrvMaxSlots] then the error word
  unsigned char* h_stat = nullptr;
  cudaStream_t s_iter = nullptr;
  cudaStream_t s_side[kClasses] = {};
  cudaEvent_t ev_fork = nullptr, ev_done = nullptr, ev_join[kClasses] = {};
  cudaEvent_t ev_prof[2 * DFG_SERVER_NKERNELS] = {};
  cudaGraphExec_t exec = nullptr, exec_prof = nullptr;
  int graph_mask = -1;             // bits 0..8: ranged classes present; 9..17: solo classes
  std::vector<Req*> act;           // table order
  std::deque<Req*> incoming;       // admitted, waiting for a table slot (guarded by the server mutex)
  bool changed = false, in_flight = false, prof = false;
  long long replays = 0;
  Clock::time_point t_launch;
};

}  // namespace

struct dfg_server_s {
  dfg_ctx ctx = nullptr;
  int device = 0, nsm = 0;
  int mode = DFG_PREC_FP32_FACTOR;
  bool fp32 = true;    // FP32 factor and sweeps (both FP32 modes)
  bool mixed = false;  // DFG_PREC_MIXED: FP32 SpMV and Krylov vectors too
  double tol = 1e-8;
  int maxit = 20000, max_inflight = kSrvMaxSlots, chunk = 8, nthreads = 4, ngroups = 1;
  int vec_grid = 0;

  // device resources (made at creation)
  void* arena_base = nullptr;
  Arena arena;
  Group grp[kGroups];
  // admission lanes: each admits one request at a time on its own stream,
  // with its own reduction scratch (partials, counter, result, singular-pivot
  // count) and pinned read-back word
  struct AdmLane {
    cudaStream_t st = nullptr;
    double* d_red = nullptr;
    int* h_nsing = nullptr;
    std::thread th;
  } adm[kAdmLanes];
  cudaStream_t s_copy = nullptr;
  // profiling of every profile_every-th replay of a group (first iteration, per kernel)
  int profile_every = 0;
  double prof_ms[DFG_SERVER_NKERNELS] = {}, prof_bytes[DFG_SERVER_NKERNELS] = {};
  long long prof_n[DFG_SERVER_NKERNELS] = {};
  std::atomic<long long> h2d{0}, d2h{0};
  // per-class sweep launch shape
  int cls_grid[kClasses] = {}, cls_ns[kClasses][2] = {}, cls_rec_stage[kClasses][2] = {}, cls_val_stage[kClasses] = {};
  size_t cls_smem[kClasses][2] = {};
  // per-class solo sweep shape: grid, stages, ring steps, record stage bytes, shared memory
  int solo_grid[kClasses] = {}, solo_ns[kClasses][2] = {}, solo_R[kClasses] = {}, solo_rec_stage[kClasses][2] = {};
  int solo_ch[kClasses][2] = {};
  size_t solo_smem[kClasses][2] = {};
  int sweeps = 0;  // dfg_server_config::sweeps

  // host state
  Clock::time_point t0;
  std::mutex mu;
  std::condition_variable cv_sym, cv_adm, cv_loop, cv_done;
  std::deque<Req*> submitted;          // waiting for symbolic set-up
  std::map<long long, Req*> ready;     // symbolic done, by id (FIFO admission)
  std::unordered_map<long long, std::unique_ptr<Req>> all;
  long long next_id = 0, n_submitted = 0, n_finished = 0;
  int inflight = 0;                    // admitted and not yet released
  bool stopping = false;   // no more submissions; symbolic workers leave when idle
  bool adm_stop = false;   // set once the workers are gone; admission leaves when idle
  bool loop_stop = false;  // set once admission is gone; the loop leaves when idle
  int fatal = DFG_OK;
  std::string fatal_msg;
  std::vector<std::thread> workers;
  std::thread loop_thread;
  // statistics
  long long replays = 0, launches = 0, peak_inflight = 0, graph_builds = 0;
  double busy_s = 0;
  // occupancy of the queues ahead of the device, integrated over time (under mu):
  // backlog = submitted and neither admitted nor finished; ready = set up and
  // waiting for device memory or an in-flight slot
  long long backlog = 0;
  double t_acc = 0, backlog_s = 0, queued_s = 0, full_s = 0, inflight_s = 0;
  bool adm_full = false;  // admission waits for device memory or an in-flight slot
  double symbolic_s = 0, admit_s = 0;

  double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
  // brings the occupancy integrals up to now; called (under mu) before every
  // change of `backlog` or `ready`
  void account_locked() {
    const double t = now();
    if (backlog > 0) backlog_s += t - t_acc;
    if (!ready.empty()) queued_s += t - t_acc;
    if (adm_full) full_s += t - t_acc;
    inflight_s += inflight * (t - t_acc);
    t_acc = t;
  }
};

namespace {

// ---------------------------------------------------------------- symbolic

// Which sweep kernel serves a solve.  One CTA per solve (k_solo.cu) keeps a
// solve's whole dependency chain on one SM, and the in-flight solves fill
// the device; the ranged kernel (k_sweep.cu) spreads one solve over many
// SMs at the price of cross-SM hand-offs (about 0.75 us per dependency level
// in batched launches).  FP32 sweeps take one CTA, except 3x3-block solves
// above 100,000 nodes.  Measured on GB300 over bands of the serving streams
// (FP32 factor, solves/s, ranged -> one CTA).  2D stream: 1x1 blocks
// 231 -> 295 (2k-20k nodes), 58 -> 84, 19 -> 28, 5.5 -> 7.1 (150k-400k);
// 2x2 blocks 142 -> 158, 34 -> 40, 13.0 -> 13.7 (60k-150k), 4.65 -> 5.71
// (150k-250k), 2.07 -> 2.31 (250k-400k).  3D stream: 1x1 blocks
// 52.8 -> 126.0 (< 40k), 13.9 -> 48.1, 12.8 -> 24.8, 6.1 -> 11.5 (> 300k);
// 3x3 blocks 18.1 -> 32.9 (< 40k), 7.8 -> 9.0 (40k-120k), but 4.0 -> 2.4
// (120k-300k) and 2.3 -> 1.1 (> 300k): a wide 3D level of 3x3 blocks is more
// record bytes than one SM streams in a level's time.  FP64 sweeps stay
// ranged: on one SM every level waits on a chain of dependent FP64 FMAs (64
// cycles each on GB300), about twice the ranged kernel's time beyond the
// smallest solves.
constexpr int kSoloMaxNodes3x3 = 100000;
bool use_solo(const dfg_server_s* S, const Req* r) {
  if (S->sweeps == 1) return false;
  if (S->sweeps == 2) return true;
  return S->fp32 && (r->b < 3 || r->n <= kSoloMaxNodes3x3);
}

// Fills the request's host-side set-up; returns false with r->error on failure.
bool symbolic(dfg_server_s* S, Req* r) {
  const int n = r->n;
  pattern_from_elements(n, r->nelem, r->nnoel, r->conn.data(), r->rowptr, r->colind);
  r->nnz = (long long)r->colind.size();
  r->diaind.resize(n);
  for (int i = 0; i < n; ++i) {
    int d = r->rowptr[i + 1];
    for (int c = r->rowptr[i]; c < r->rowptr[i + 1]; ++c)
      if (r->colind[c] > i) { d = c; break; }
    r->diaind[i] = d;
  }
  std::string err;
  if (!build_gather_map(n, r->rowptr.data(), r->colind.data(), r->nelem, r->nnoel, r->conn.data(), r->gm, err)) {
    r->error = err;
    return false;
  }
  r->lev = build_levels(n, r->rowptr.data(), r->colind.data(), r->diaind.data(), true);
  r->sell = build_sell(n, r->rowptr.data(), r->colind.data());
  const int elem = S->fp32 ? 4 : 8;
  r->maxe = 0;
  for (int i = 0; i < n; ++i)
    r->maxe = std::max(r->maxe, std::max(r->diaind[i] - r->rowptr[i], r->rowptr[i + 1] - r->diaind[i]));
  if (r->maxe > 16) {
    r->error = "a row has more than 16 lower or upper neighbours; the serving sweeps take at most 16";
    return false;
  }
  r->cls = class_index(r->b, r->maxe);
  r->group = group_of((long long)n * r->b, S->ngroups);
  r->solo = use_solo(S, r);
  if (r->solo) {
    const int k = r->cls, R = S->solo_R[k];
    SoloPlan sf = solo_sweep_plan(n, r->b, r->rowptr.data(), r->colind.data(), r->diaind.data(), true, R, elem,
                                  S->solo_rec_stage[k][0], S->solo_ch[k][0]);
    SoloPlan sb = solo_sweep_plan(n, r->b, r->rowptr.data(), r->colind.data(), r->diaind.data(), false, R, elem,
                                  S->solo_rec_stage[k][1], S->solo_ch[k][1]);
    // the forward sweep writes y where the backward sweep reads it (its step
    // order); the backward sweep writes z in row order
    std::vector<int> ident(n);
    for (int i = 0; i < n; ++i) ident[i] = i;
    r->hf = pack_solo_headers(sf, elem, sb.pos.data(), sb.pos.data(), r->of);
    r->hb = pack_solo_headers(sb, elem, ident.data(), ident.data(), r->ob);
    r->maxrf = r->maxrb = 0;
    r->chf = std::move(sf.chunks);
    r->chb = std::move(sb.chunks);
    r->posf = std::move(sf.pos);
    r->pf = std::move(sf.P);
    r->pb = std::move(sb.P);
    r->pf.range_steps = std::move(sf.lev_chunks);  // per level: the chunk of its first step
    r->pb.range_steps = std::move(sb.lev_chunks);
  } else {
    r->pf = fullest_sweep_plan(n, r->b, r->rowptr.data(), r->colind.data(), r->diaind.data(), true, kRingSteps);
    r->pb = fullest_sweep_plan(n, r->b, r->rowptr.data(), r->colind.data(), r->diaind.data(), false, kRingSteps);
    r->hf = pack_record_headers(r->pf, elem, r->of, r->maxrf);
    r->hb = pack_record_headers(r->pb, elem, r->ob, r->maxrb);
  }

  const size_t m = (size_t)n * r->b, bs = (size_t)r->b * r->b, Z = (size_t)std::max<long long>(r->nnz, 1);
  const bool mixed = S->mixed;
  {
    const double dm = (double)m, idx = (n + 1) * 4.0 + r->nnz * 4.0, vals = ((double)n + r->nnz) * bs;
    if (mixed) {
      r->alg[0] = dm * 8;                      // r, z
      r->alg[1] = dm * 12;                     // z, p read + write
      r->alg[2] = idx + vals * 4 + dm * 8;     // FP32 values + indices + p read + q write
      r->alg[3] = dm * (8 + 4 + 16 + 4 + 8);   // r r/w, q, d r/w, p, y/z sentinels
    } else {
      r->alg[0] = dm * (8 + elem);
      r->alg[1] = dm * (16 + elem);
      r->alg[2] = idx + vals * 8 + dm * 16;  // values + CRS-equivalent indices + p read + q write
      r->alg[3] = dm * (16 + 8 + 16 + 8 + 2 * elem + (S->fp32 ? 4 : 0));
    }
    r->alg[4] = (double)r->hf.size() + dm * 2 * elem;
    r->alg[5] = (double)r->hb.size() + dm * 2 * elem;
  }
  Layout& P = r->P;
  const size_t sblk = (size_t)std::max<long long>(r->sell.ptr.back(), 1);
  // mixed form: FP32 values beside the FP64 ones (the reliable updates'
  // b - A x), FP32 p and q, and d (the FP64 correction) in rd's place; the
  // FP64 r is not kept
  r->o_sptr = P.add(r->sell.ptr.size() * 8);
  r->o_swidth = P.add(std::max<size_t>(r->sell.width.size(), 1) * 4);
  r->o_scol = P.add(sblk * 4);
  r->o_sval = P.add(sblk * bs * 8);
  r->o_sval32 = P.add(mixed ? sblk * bs * 4 : 16);
  r->o_rhs = P.add(m * 8);
  r->o_r = P.add(mixed ? 16 : m * 8);
  r->o_x = P.add(m * 8);
  r->o_p = P.add(m * (mixed ? 4 : 8));
  r->o_q = P.add(m * (mixed ? 4 : 8));
  r->o_rd = P.add(m * 8);
  // a solo solve's y is stored in the backward plan's step order (padded
  // steps of 32 rows)
  const size_t ystore = r->solo ? std::max<size_t>(m, (size_t)r->pb.nsteps * 32 * r->b) : m;
  r->o_y = P.add(ystore * elem + 64);
  r->o_z = P.add(m * elem + 64);
  r->o_r32 = P.add(S->fp32 ? m * 4 + 64 : 16);
  r->o_recf = P.add(r->hf.size() + 64);
  r->o_offf = P.add(r->of.size() * 8);
  r->o_rsf = P.add(r->pf.range_steps.size() * 4);
  r->o_recb = P.add(r->hb.size() + 64);
  r->o_offb = P.add(r->ob.size() * 8);
  r->o_rsb = P.add(r->pb.range_steps.size() * 4);
  r->o_st = P.add(sizeof(PcgState));
  r->o_cnt = P.add(16);
  if (r->solo) {
    r->o_chf = P.add(r->chf.size() * sizeof(SoloChunk));
    r->o_chb = P.add(r->chb.size() * sizeof(SoloChunk));
    r->o_posf = P.add((size_t)n * 4);
    r->o_rperm = P.add((size_t)r->pf.nsteps * 32 * r->b * elem + 64);
  }
  Layout& T = r->T;
  const size_t k = r->nnoel;
  r->t_rowptr = T.add((n + 1) * 4);
  r->t_colind = T.add(Z * 4);
  r->t_diag = T.add(n * bs * 8);
  r->t_offd = T.add(Z * bs * 8);
  r->t_ssrc = T.add(sblk * 4);
  r->t_coords = T.add(r->coords.size() * 8);
  r->t_conn = T.add(r->conn.size() * 4);
  r->t_coef = T.add(std::max<size_t>(r->coef.size(), 1) * 8);
  r->t_bc = T.add(m * 4);
  r->t_load = T.add(std::max<size_t>(r->load.size(), 1) * 8);
  r->t_em = T.add((size_t)r->nelem * k * k * bs * 8);
  r->t_er = T.add((size_t)r->nelem * k * r->b * 8);
  r->t_sp = T.add(r->gm.slot_ptr.size() * 8);
  r->t_ss = T.add(std::max<size_t>(r->gm.slot_src.size(), 1) * 4);
  r->t_rp = T.add(r->gm.res_ptr.size() * 8);
  r->t_rs = T.add(std::max<size_t>(r->gm.res_src.size(), 1) * 4);
  r->t_dia = T.add((size_t)n * 4);
  r->t_lev = T.add(std::max<size_t>(r->lev.rows.size(), 1) * 4);
  r->t_fd = T.add((size_t)n * bs * 8);
  r->t_fo = T.add(Z * bs * 8);
  r->t_eof = T.add(r->pf.ent_off.size() * 8);
  r->t_esf = T.add(std::max<size_t>(r->pf.ent_slot.size(), 1) * 4);
  r->t_srf = T.add(std::max<size_t>(r->pf.step_rows.size(), 1) * 4);
  r->t_eob = T.add(r->pb.ent_off.size() * 8);
  r->t_esb = T.add(std::max<size_t>(r->pb.ent_slot.size(), 1) * 4);
  r->t_srb = T.add(std::max<size_t>(r->pb.step_rows.size(), 1) * 4);
  return true;
}

template <class T>
T* at(dfg_server_s* S, size_t base, size_t off) {
  return reinterpret_cast<T*>(static_cast<unsigned char*>(S->arena_base) + base + off);
}

template <class T>
void up(dfg_server_s* S, cudaStream_t st, size_t base, size_t off, const std::vector<T>& v) {
  if (v.empty()) return;
  SCK(cudaMemcpyAsync(at<T>(S, base, off), v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st));
  S->h2d += (long long)(v.size() * sizeof(T));
}

SrvSlot slot_of(dfg_server_s* S, Req* r);

// Device work of one admission on an admission lane's stream; returns the
// ILU singular-pivot count.
int admit_device(dfg_server_s* S, Req* r, dfg_server_s::AdmLane& lane) {
  const size_t pb = r->pbase, tb = r->tbase;
  const int n = r->n, b = r->b;
  const long long m = (long long)n * b;
  const size_t bs = (size_t)b * b;
  cudaStream_t st = lane.st;
  up(S, st, tb, r->t_rowptr, r->rowptr);
  up(S, st, tb, r->t_colind, r->colind);
  up(S, st, pb, r->o_sptr, r->sell.ptr);
  up(S, st, pb, r->o_swidth, r->sell.width);
  up(S, st, pb, r->o_scol, r->sell.col);
  up(S, st, tb, r->t_ssrc, r->sell.src);
  up(S, st, tb, r->t_coords, r->coords);
  up(S, st, tb, r->t_conn, r->conn);
  up(S, st, tb, r->t_coef, r->coef);
  up(S, st, tb, r->t_bc, r->bcflag);
  up(S, st, tb, r->t_load, r->load);
  up(S, st, tb, r->t_sp, r->gm.slot_ptr);
  up(S, st, tb, r->t_ss, r->gm.slot_src);
  up(S, st, tb, r->t_rp, r->gm.res_ptr);
  up(S, st, tb, r->t_rs, r->gm.res_src);
  up(S, st, tb, r->t_dia, r->diaind);
  up(S, st, tb, r->t_lev, r->lev.rows);
  up(S, st, pb, r->o_recf, r->hf);
  up(S, st, pb, r->o_offf, r->of);
  up(S, st, pb, r->o_rsf, r->pf.range_steps);
  up(S, st, pb, r->o_recb, r->hb);
  up(S, st, pb, r->o_offb, r->ob);
  up(S, st, pb, r->o_rsb, r->pb.range_steps);
  if (r->solo) {
    up(S, st, pb, r->o_chf, r->chf);
    up(S, st, pb, r->o_chb, r->chb);
    up(S, st, pb, r->o_posf, r->posf);
  }
  up(S, st, tb, r->t_eof, r->pf.ent_off);
  up(S, st, tb, r->t_esf, r->pf.ent_slot);
  up(S, st, tb, r->t_srf, r->pf.step_rows);
  up(S, st, tb, r->t_eob, r->pb.ent_off);
  up(S, st, tb, r->t_esb, r->pb.ent_slot);
  up(S, st, tb, r->t_srb, r->pb.step_rows);
  double* diag = at<double>(S, tb, r->t_diag);
  double* offd = at<double>(S, tb, r->t_offd);
  double* rhs = at<double>(S, pb, r->o_rhs);
  SCK(cudaMemsetAsync(diag, 0, n * bs * 8, st));
  SCK(cudaMemsetAsync(offd, 0, std::max<long long>(r->nnz, 1) * bs * 8, st));
  SCK(cudaMemsetAsync(rhs, 0, m * 8, st));
  SCK(cudaMemsetAsync(at<unsigned>(S, pb, r->o_cnt), 0, 16, st));
  // AddLinSys_*: element kernels, then the gather in element order
  ElemArgs ea{};
  ea.nelem = r->nelem;
  ea.conn = at<int>(S, tb, r->t_conn);
  ea.coords = at<double>(S, tb, r->t_coords);
  ea.coef = r->coef.empty() ? nullptr : at<double>(S, tb, r->t_coef);
  for (int i = 0; i < 8; ++i) ea.p[i] = i < (int)r->params.size() ? r->params[i] : 0.0;
  ea.em = at<double>(S, tb, r->t_em);
  ea.er = at<double>(S, tb, r->t_er);
  SCK(launch_elem(r->kind, ea, st));
  GatherArgs ga{};
  ga.n = n;
  ga.nnz = r->nnz;
  ga.b = b;
  ga.bs = (int)bs;
  ga.slot_ptr = at<long long>(S, tb, r->t_sp);
  ga.slot_src = at<int>(S, tb, r->t_ss);
  ga.res_ptr = at<long long>(S, tb, r->t_rp);
  ga.res_src = at<int>(S, tb, r->t_rs);
  ga.em = ea.em;
  ga.er = ea.er;
  ga.diag = diag;
  ga.offd = offd;
  ga.res = rhs;
  SCK(launch_gather(ga, st));
  int nl = 3;
  // FinalizeMarge: resident load, then Dirichlet rows and columns
  if (!r->load.empty()) {
    SCK(launch_add_vec(m, at<double>(S, tb, r->t_load), rhs, st));
    ++nl;
  }
  BcArgs bc{};
  bc.n = n;
  bc.nnz = r->nnz;
  bc.b = b;
  bc.rowptr = at<int>(S, tb, r->t_rowptr);
  bc.colind = at<int>(S, tb, r->t_colind);
  bc.flag = at<int>(S, tb, r->t_bc);
  bc.diag = diag;
  bc.offd = offd;
  bc.res = rhs;
  SCK(launch_bc(bc, st));
  nl += 2;
  // ILU(0): SetValue_Initialize (copy), then the levels
  double* fd = at<double>(S, tb, r->t_fd);
  double* fo = at<double>(S, tb, r->t_fo);
  SCK(cudaMemcpyAsync(fd, diag, n * bs * 8, cudaMemcpyDeviceToDevice, st));
  if (r->nnz) SCK(cudaMemcpyAsync(fo, offd, r->nnz * bs * 8, cudaMemcpyDeviceToDevice, st));
  int* nsing = reinterpret_cast<int*>(lane.d_red + kRedGrid + 16);
  SCK(cudaMemsetAsync(nsing, 0, sizeof(int), st));
  const int nlev = (int)r->lev.ptr.size() - 1;
  for (int l = 0; l < nlev; ++l)
    SCK(launch_ilu_level(b, at<int>(S, tb, r->t_lev) + r->lev.ptr[l], r->lev.ptr[l + 1] - r->lev.ptr[l],
                         bc.rowptr, bc.colind, at<int>(S, tb, r->t_dia), fd, fo, nsing, st, l > 0));
  nl += nlev;
  // the matrix into its sliced-ELL copy (the only copy that stays resident;
  // the mixed form keeps an FP32 one beside it)
  SCK(sell_pack(r->sell.nslices, b, at<long long>(S, pb, r->o_sptr), at<int>(S, tb, r->t_ssrc), diag, offd,
                at<void>(S, pb, r->o_sval), false, st));
  ++nl;
  if (S->mixed) {
    SCK(sell_pack(r->sell.nslices, b, at<long long>(S, pb, r->o_sptr), at<int>(S, tb, r->t_ssrc), diag, offd,
                  at<void>(S, pb, r->o_sval32), true, st));
    ++nl;
  }
  // the factor into the step records
  for (int dir = 0; dir < 2; ++dir) {
    const SweepPlan& pl = dir == 0 ? r->pf : r->pb;
    PackArgs pa{};
    pa.nsteps = pl.nsteps;
    pa.rec = at<unsigned char>(S, pb, dir == 0 ? r->o_recf : r->o_recb);
    pa.rec_off = at<long long>(S, pb, dir == 0 ? r->o_offf : r->o_offb);
    pa.ent_off = at<long long>(S, tb, dir == 0 ? r->t_eof : r->t_eob);
    pa.ent_slot = at<int>(S, tb, dir == 0 ? r->t_esf : r->t_esb);
    pa.step_rows = at<int>(S, tb, dir == 0 ? r->t_srf : r->t_srb);
    pa.fdiag = fd;
    pa.foffd = fo;
    pa.code_bytes = r->solo ? 128 : 256;
    SCK(launch_pack(dir == 0, S->fp32, b, pa, st));
    ++nl;
  }
  // PCG start: r = b, x = 0, rr0 = r.r
  if (S->mixed)
    SCK(srvm_init_vectors(m, rhs, at<double>(S, pb, r->o_x), at<double>(S, pb, r->o_rd), at<float>(S, pb, r->o_r32),
                          at<float>(S, pb, r->o_p), at<float>(S, pb, r->o_y), at<float>(S, pb, r->o_z), st));
  else
    SCK(srv_init_vectors(m, rhs, at<double>(S, pb, r->o_r), at<double>(S, pb, r->o_x), at<double>(S, pb, r->o_p),
                         at<void>(S, pb, r->o_y), at<void>(S, pb, r->o_z),
                         S->fp32 ? at<float>(S, pb, r->o_r32) : nullptr, S->fp32, st));
  if (r->solo) {  // the first forward input, in the forward plan's step order
    SCK(srv_permute_rhs(slot_of(S, r), S->fp32, st));
    ++nl;
  }
  Red red{lane.d_red, reinterpret_cast<unsigned*>(lane.d_red + kRedGrid), lane.d_red + kRedGrid + 8};
  SCK(api_dot(m, rhs, rhs, red, st));
  SCK(srv_init_state(at<PcgState>(S, pb, r->o_st), red.result, S->tol, S->maxit, S->mixed ? kMixedDelta2 : 0.0, st));
  nl += 3;
  SCK(cudaMemcpyAsync(lane.h_nsing, nsing, sizeof(int), cudaMemcpyDeviceToHost, st));
  SCK(cudaStreamSynchronize(st));
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->launches += nl;
  }
  return *lane.h_nsing;
}

void finish_locked(dfg_server_s* S, Req* r) {
  r->finished = true;
  r->t_done = S->now();
  // host set-up data is no longer needed
  r->coords = {}; r->coef = {}; r->load = {}; r->conn = {}; r->bcflag = {};
  r->rowptr = {}; r->colind = {}; r->diaind = {};
  r->gm = GatherMap{}; r->sell = SellMap{}; r->lev = Levels{}; r->pf = SweepPlan{}; r->pb = SweepPlan{};
  r->hf = {}; r->hb = {}; r->of = {}; r->ob = {};
  r->chf = {}; r->chb = {}; r->posf = {};
  ++S->n_finished;
  S->cv_done.notify_all();
}

void release_locked(dfg_server_s* S, Req* r) {
  if (r->have_p) S->arena.release(r->pbase, r->P.total);
  if (r->have_t) S->arena.release(r->tbase, r->T.total);
  const bool was_admitted = r->have_p;
  r->have_p = r->have_t = false;
  if (was_admitted) {
    S->account_locked();
    --S->inflight;
  }
  S->cv_adm.notify_all();
}

// ------------------------------------------------------------------ threads

void symbolic_worker(dfg_server_s* S) {
  for (;;) {
    Req* r = nullptr;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      S->cv_sym.wait(lk, [&] { return S->stopping || !S->submitted.empty(); });
      if (S->submitted.empty()) return;
      r = S->submitted.front();
      S->submitted.pop_front();
    }
    bool ok = false;
    const Clock::time_point t_sym = Clock::now();
    try {
      ok = symbolic(S, r);
    } catch (const std::bad_alloc&) {
      r->error = "host allocation failed during the symbolic set-up";
    }
    std::lock_guard<std::mutex> lk(S->mu);
    S->symbolic_s += std::chrono::duration<double>(Clock::now() - t_sym).count();
    S->account_locked();
    if (!ok) {
      r->status = DFG_INVALID_ARGUMENT;
      --S->backlog;
      finish_locked(S, r);
      continue;
    }
    if ((size_t)(r->P.total + r->T.total) > S->arena.capacity()) {
      r->status = DFG_OOM_REJECTED;
      r->error = "the request needs " + std::to_string(r->P.total + r->T.total) +
                 " device bytes, more than the whole admission budget";
      --S->backlog;
      finish_locked(S, r);
      continue;
    }
    S->ready[r->id] = r;  // account_locked ran above, before this change
    S->cv_adm.notify_all();
  }
}

void admission_thread(dfg_server_s* S, int li) {
  cudaSetDevice(S->device);
  dfg_server_s::AdmLane& lane = S->adm[li];
  for (;;) {
    Req* r = nullptr;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      for (;;) {
        if (S->fatal != DFG_OK) {
          // drain: everything not admitted fails with the fatal status
          S->account_locked();
          S->backlog -= (long long)S->ready.size();
          for (auto& kv : S->ready) {
            kv.second->status = S->fatal;
            kv.second->error = S->fatal_msg;
            finish_locked(S, kv.second);
          }
          S->ready.clear();
        }
        if (S->adm_stop && S->ready.empty()) return;
        if (!S->ready.empty() && S->inflight < S->max_inflight) {
          Req* h = S->ready.begin()->second;  // lowest id first
          size_t po = 0, to = 0;
          if (S->arena.alloc(h->P.total, &po)) {
            if (S->arena.alloc(h->T.total, &to)) {
              h->pbase = po;
              h->tbase = to;
              h->have_p = h->have_t = true;
              S->account_locked();
              S->adm_full = false;
              --S->backlog;
              S->ready.erase(S->ready.begin());
              ++S->inflight;
              S->peak_inflight = std::max<long long>(S->peak_inflight, S->inflight);
              h->t_admit = S->now();
              r = h;
              break;
            }
            S->arena.release(po, h->P.total);
          }
        }
        if (!S->ready.empty() && !S->adm_full) {
          S->account_locked();
          S->adm_full = true;
        }
        S->cv_adm.wait(lk);
      }
    }
    int nsing = 0;
    const Clock::time_point t_adm = Clock::now();
    try {
      nsing = admit_device(S, r, lane);
      std::lock_guard<std::mutex> lk(S->mu);
      S->admit_s += std::chrono::duration<double>(Clock::now() - t_adm).count();
    } catch (const CudaFail& f) {
      cudaGetLastError();
      std::lock_guard<std::mutex> lk(S->mu);
      r->status = DFG_CUDA_ERROR;
      r->error = std::string("admission: ") + cudaGetErrorString(f.e) + " at " + f.what;
      release_locked(S, r);
      finish_locked(S, r);
      continue;
    }
    std::lock_guard<std::mutex> lk(S->mu);
    S->arena.release(r->tbase, r->T.total);
    r->have_t = false;
    if (S->fatal != DFG_OK) {  // the serving loop has stopped
      r->status = S->fatal;
      r->error = S->fatal_msg;
      release_locked(S, r);
      finish_locked(S, r);
      continue;
    }
    if (nsing > 10) {
      r->status = DFG_SINGULAR_PIVOT;
      r->error = "ILU(0): " + std::to_string(nsing) + " singular pivots (more than 10)";
      release_locked(S, r);
      finish_locked(S, r);
      continue;
    }
    S->grp[r->group].incoming.push_back(r);
    S->cv_loop.notify_all();
  }
}

SrvSlot slot_of(dfg_server_s* S, Req* r) {
  const size_t pb = r->pbase;
  SrvSlot s{};
  s.n = r->n;
  s.b = r->b;
  s.sptr = at<long long>(S, pb, r->o_sptr);
  s.swidth = at<int>(S, pb, r->o_swidth);
  s.scol = at<int>(S, pb, r->o_scol);
  s.sval = at<double>(S, pb, r->o_sval);
  s.rhs = at<double>(S, pb, r->o_rhs);
  s.r = at<double>(S, pb, r->o_r);
  s.x = at<double>(S, pb, r->o_x);
  s.p = at<double>(S, pb, r->o_p);
  s.q = at<double>(S, pb, r->o_q);
  s.rd = at<double>(S, pb, r->o_rd);
  s.y = at<void>(S, pb, r->o_y);
  s.z = at<void>(S, pb, r->o_z);
  s.r32 = S->fp32 ? at<float>(S, pb, r->o_r32) : nullptr;
  s.st = at<PcgState>(S, pb, r->o_st);
  s.cnt = at<unsigned>(S, pb, r->o_cnt);
  if (r->solo) {
    s.posf = at<int>(S, pb, r->o_posf);
    s.rperm = at<void>(S, pb, r->o_rperm);
  }
  if (S->mixed) {
    s.r = s.p = s.q = nullptr;
    s.sval32 = at<float>(S, pb, r->o_sval32);
    s.p32 = at<float>(S, pb, r->o_p);
    s.q32 = at<float>(S, pb, r->o_q);
    s.d = at<double>(S, pb, r->o_rd);
    s.rd = nullptr;
  }
  return s;
}

// Rebuilds a group's pinned table mirrors from its active slots and uploads
// them on its stream; returns the mask of sweep classes present.
int upload_table(dfg_server_s* S, Group& G) {
  const std::vector<Req*>& act = G.act;
  SrvTable* T = G.h_tab;
  T->nslots = (int)act.size();
  int c = 0;
  for (int i = 0; i < (int)act.size(); ++i) {
    SrvSlot s = slot_of(S, act[i]);
    s.chunk0 = c;
    s.nchunks = (act[i]->n + kSrvRows - 1) / kSrvRows;
    T->chunk_start[i] = c;
    T->slot[i] = s;
    std::memset(G.h_chunk_slot + c, i, (size_t)s.nchunks);
    c += s.nchunks;
  }
  T->chunk_start[act.size()] = c;
  T->total_chunks = c;
  T->chunk_slot = G.d_chunk_slot;
  if (c > 0) SCK(cudaMemcpyAsync(G.d_chunk_slot, G.h_chunk_slot, (size_t)c, cudaMemcpyHostToDevice, G.s_iter));
  int mask = 0;
  for (int k = 0; k < kClasses; ++k)
    for (int dir = 0; dir < 2; ++dir) {
      G.h_sb[k * 2 + dir].nslots = 0;
      G.h_sb[k * 2 + dir].range_start[0] = 0;
      G.h_solo[k * 2 + dir].nslots = 0;
    }
  // solo sweeps: largest solves first, so the last CTA to start has the
  // least left to do
  std::vector<int> solo_order;
  for (int i = 0; i < (int)act.size(); ++i)
    if (act[i]->solo) solo_order.push_back(i);
  std::stable_sort(solo_order.begin(), solo_order.end(),
                   [&](int x, int y) { return act[x]->pf.nsteps > act[y]->pf.nsteps; });
  for (int i : solo_order) {
    Req* r = act[i];
    mask |= 1 << (kClasses + r->cls);
    const SrvSlot& sl = T->slot[i];
    for (int dir = 0; dir < 2; ++dir) {
      SoloBatch& B = G.h_solo[r->cls * 2 + dir];
      SoloSlot& w = B.slot[B.nslots++];
      const SweepPlan& pl = dir == 0 ? r->pf : r->pb;
      w.rec = at<unsigned char>(S, r->pbase, dir == 0 ? r->o_recf : r->o_recb);
      w.chunks = at<SoloChunk>(S, r->pbase, dir == 0 ? r->o_chf : r->o_chb);
      w.lev_chunks = at<int>(S, r->pbase, dir == 0 ? r->o_rsf : r->o_rsb);
      w.nlevels = pl.nranges;
      w.nchunks = (int)(dir == 0 ? r->chf.size() : r->chb.size());
      w.in = dir == 0 ? sl.rperm : sl.y;  // both in this sweep's step order
      w.out = dir == 0 ? sl.y : sl.z;     // y in the backward sweep's step order, z in row order
      w.done = &sl.st->done;
    }
  }
  for (int i = 0; i < (int)act.size(); ++i) {
    Req* r = act[i];
    if (r->solo) continue;
    mask |= 1 << r->cls;
    for (int dir = 0; dir < 2; ++dir) {
      SweepBatch& B = G.h_sb[r->cls * 2 + dir];
      const int j = B.nslots++;
      const SweepPlan& pl = dir == 0 ? r->pf : r->pb;
      SweepSlot& w = B.slot[j];
      w.rec = at<unsigned char>(S, r->pbase, dir == 0 ? r->o_recf : r->o_recb);
      w.rec_off = at<long long>(S, r->pbase, dir == 0 ? r->o_offf : r->o_offb);
      w.range_steps = at<int>(S, r->pbase, dir == 0 ? r->o_rsf : r->o_rsb);
      const SrvSlot& sl = T->slot[i];
      w.in = dir == 0 ? (S->fp32 ? (const void*)sl.r32 : (const void*)sl.r) : sl.y;
      w.out = dir == 0 ? sl.y : sl.z;
      w.done = &sl.st->done;
      B.range_start[j + 1] = B.range_start[j] + pl.nranges;
    }
  }
  // only the used prefix of the slot table travels
  const size_t tab_bytes = offsetof(SrvTable, slot) + sizeof(SrvSlot) * std::max<size_t>(act.size(), 1);
  SCK(cudaMemcpyAsync(G.d_tab, G.h_tab, tab_bytes, cudaMemcpyHostToDevice, G.s_iter));
  SCK(cudaMemcpyAsync(G.d_sb, G.h_sb, sizeof(SweepBatch) * kClasses * 2, cudaMemcpyHostToDevice, G.s_iter));
  SCK(cudaMemcpyAsync(G.d_solo, G.h_solo, sizeof(SoloBatch) * kClasses * 2, cudaMemcpyHostToDevice, G.s_iter));
  return mask;
}

SweepArgs class_args(dfg_server_s* S, Group& G, int k, int dir) {
  SweepArgs a{};
  a.batch = G.d_sb + k * 2 + dir;
  a.ticket = G.d_tickets + k * 2 + dir;
  a.err = reinterpret_cast<int*>(G.d_stat + sizeof(SrvStatus) * kSrvMaxSlots);
  a.rec_stage = S->cls_rec_stage[k][dir];
  a.val_stage = S->cls_val_stage[k];
  a.R = kRingSteps;
  a.NS = S->cls_ns[k][dir];
  a.max_nent = class_maxe(k);
  return a;
}

SoloArgs solo_args(dfg_server_s* S, Group& G, int k, int dir) {
  SoloArgs a{};
  a.batch = G.d_solo + k * 2 + dir;
  a.ticket = G.d_tickets + kClasses * 2 + k * 2 + dir;
  a.err = reinterpret_cast<int*>(G.d_stat + sizeof(SrvStatus) * kSrvMaxSlots);
  a.rec_stage = S->solo_rec_stage[k][dir];
  a.ch_max = S->solo_ch[k][dir];
  a.NS = S->solo_ns[k][dir];
  a.R = S->solo_R[k];
  a.max_nent = class_maxe(k);
  return a;
}

// Captures `chunk` iterations of every class in `mask` plus the stop checks
// and the status copy, on the group's streams.  The profiled variant
// brackets each kernel of the first iteration (and the stop checks) with
// timing events.
cudaGraphExec_t capture_graph(dfg_server_s* S, Group& G, int mask, bool prof) {
  cudaGraph_t g = nullptr;
  struct EndOnThrow {  // a failed launch must not leave the stream capturing
    cudaStream_t st;
    bool armed = true;
    ~EndOnThrow() {
      if (armed) {
        cudaGraph_t dead = nullptr;
        cudaStreamEndCapture(st, &dead);
        if (dead) cudaGraphDestroy(dead);
        cudaGetLastError();
      }
    }
  };
  auto mark = [&](int k, int edge, cudaStream_t st) {
    if (prof) SCK(cudaEventRecordWithFlags(G.ev_prof[2 * k + edge], st, cudaEventRecordExternal));
  };
  SCK(cudaStreamBeginCapture(G.s_iter, cudaStreamCaptureModeThreadLocal));
  EndOnThrow guard{G.s_iter};
  const int grid = S->vec_grid;
  // kernels above the six-block register bound run four blocks per SM
  const int grid4 = S->nsm * 4;
  for (int it = 0; it < S->chunk; ++it) {
    const bool pf = prof && it == 0;
    auto mk = [&](int k, int edge, cudaStream_t st) {
      if (pf) mark(k, edge, st);
    };
    SCK(cudaEventRecord(G.ev_fork, G.s_iter));
    for (int k = 0; k < kClasses; ++k) {
      const bool ranged = mask >> k & 1, solo = mask >> (kClasses + k) & 1;
      if (!ranged && !solo) continue;
      SCK(cudaStreamWaitEvent(G.s_side[k], G.ev_fork, 0));
      for (int dir = 0; dir < 2; ++dir) {
        mk(6 + 2 * k + dir, 0, G.s_side[k]);
        if (ranged)
          SCK(launch_sweep(dir == 0, S->fp32, class_b(k), class_args(S, G, k, dir), S->cls_grid[k],
                           S->cls_smem[k][dir], G.s_side[k]));
        if (solo)
          SCK(launch_solo(dir == 0, S->fp32, class_b(k), solo_args(S, G, k, dir), S->solo_grid[k],
                          S->solo_smem[k][dir], G.s_side[k]));
        mk(6 + 2 * k + dir, 1, G.s_side[k]);
      }
      SCK(cudaEventRecord(G.ev_join[k], G.s_side[k]));
      SCK(cudaStreamWaitEvent(G.s_iter, G.ev_join[k], 0));
    }
    mk(0, 0, G.s_iter);
    if (S->mixed) SCK(srvm_rz_beta(G.d_tab, G.d_partials, G.d_tickets, kClasses * 4, grid, G.s_iter));
    else SCK(srv_rz_beta(G.d_tab, G.d_partials, G.d_tickets, kClasses * 4, S->fp32, grid, G.s_iter));
    mk(0, 1, G.s_iter);
    mk(1, 0, G.s_iter);
    if (S->mixed) SCK(srvm_update_p(G.d_tab, grid, G.s_iter));
    else SCK(srv_update_p(G.d_tab, S->fp32, grid, G.s_iter));
    mk(1, 1, G.s_iter);
    mk(2, 0, G.s_iter);
    if (S->mixed) SCK(srvm_spmv_pap(G.d_tab, G.d_partials, grid4, G.s_iter));
    else SCK(srv_spmv_pap(G.d_tab, G.d_partials, grid, G.s_iter));
    mk(2, 1, G.s_iter);
    mk(3, 0, G.s_iter);
    if (S->mixed) SCK(srvm_update_rx(G.d_tab, G.d_partials, grid, G.s_iter));
    else SCK(srv_update_rx(G.d_tab, G.d_partials, S->fp32, grid, G.s_iter));
    mk(3, 1, G.s_iter);
  }
  // end of the replay: true-residual checks (the mixed form: reliable updates)
  if (S->mixed) {
    mark(5, 0, G.s_iter);
    SCK(srvm_fold(G.d_tab, grid, G.s_iter));
    mark(5, 1, G.s_iter);
    mark(4, 0, G.s_iter);
    SCK(srvm_refine(G.d_tab, G.d_partials, grid4, G.s_iter));
    mark(4, 1, G.s_iter);
  } else {
    mark(4, 0, G.s_iter);
    SCK(srv_check_true(G.d_tab, G.d_partials, grid4, G.s_iter));
    mark(4, 1, G.s_iter);
    mark(5, 0, G.s_iter);
    SCK(srv_replace(G.d_tab, G.d_partials, S->fp32, grid, G.s_iter));
    mark(5, 1, G.s_iter);
  }
  SCK(srv_collect(G.d_tab, reinterpret_cast<SrvStatus*>(G.d_stat), G.s_iter));
  SCK(cudaMemcpyAsync(G.h_stat, G.d_stat, sizeof(SrvStatus) * kSrvMaxSlots + 16, cudaMemcpyDeviceToHost, G.s_iter));
  guard.armed = false;
  SCK(cudaStreamEndCapture(G.s_iter, &g));
  cudaGraphExec_t exec = nullptr;
  const cudaError_t e = cudaGraphInstantiate(&exec, g, 0);
  cudaGraphDestroy(g);
  SCK(e);
  return exec;
}

void build_graph(dfg_server_s* S, Group& G, int mask) {
  if (G.exec) cudaGraphExecDestroy(G.exec);
  if (G.exec_prof) cudaGraphExecDestroy(G.exec_prof);
  G.exec = G.exec_prof = nullptr;
  G.exec = capture_graph(S, G, mask, false);
  if (S->profile_every > 0) G.exec_prof = capture_graph(S, G, mask, true);
  G.graph_mask = mask;
  std::lock_guard<std::mutex> lk(S->mu);
  ++S->graph_builds;
}

// Adds a profiled replay's event durations and the algorithmic bytes of the
// solves it ran (all slots of the group at its start) to the totals.
void account_profile(dfg_server_s* S, Group& G) {
  double bytes[DFG_SERVER_NKERNELS] = {};
  for (const Req* r : G.act) {
    for (int k = 0; k < 4; ++k) bytes[k] += r->alg[k];
    bytes[6 + 2 * r->cls] += r->alg[4];
    bytes[7 + 2 * r->cls] += r->alg[5];
  }
  std::lock_guard<std::mutex> lk(S->mu);
  for (int k = 0; k < DFG_SERVER_NKERNELS; ++k) {
    if (k >= 6 && !((G.graph_mask >> ((k - 6) / 2)) & 1) && !((G.graph_mask >> (kClasses + (k - 6) / 2)) & 1))
      continue;
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, G.ev_prof[2 * k], G.ev_prof[2 * k + 1]) != cudaSuccess) {
      cudaGetLastError();
      continue;
    }
    S->prof_ms[k] += ms;
    S->prof_bytes[k] += bytes[k];
    S->prof_n[k] += 1;
  }
}

int kernels_per_replay(dfg_server_s* S, const Group& G) {
  int nc = 0;
  for (int k = 0; k < 2 * kClasses; ++k) nc += (G.graph_mask >> k) & 1;
  // per iteration: the sweeps, four batched kernels, and (outside the mixed
  // form) the three finishing launches of their per-slot reductions
  return S->chunk * (2 * nc + 4 + (S->mixed ? 0 : 3)) + 3;
}

// Reads a finished replay's status array: finished solves leave the table
// (into `retiring`), the rest stay.
void harvest(dfg_server_s* S, Group& G, std::vector<Req*>& retiring) {
  const int* errw = reinterpret_cast<const int*>(G.h_stat + sizeof(SrvStatus) * kSrvMaxSlots);
  const int err = errw[0];
  const SrvStatus* stv = reinterpret_cast<const SrvStatus*>(G.h_stat);
  std::vector<Req*> keep;
  for (int i = 0; i < (int)G.act.size(); ++i) {
    Req* r = G.act[i];
    const SrvStatus& st = stv[i];
    const bool fin = err != 0 || (st.done != 0 && st.done != 6 && (st.done != 1 || st.verified));
    if (!fin) {
      keep.push_back(r);
      continue;
    }
    r->iters = st.iter_out;
    r->conv = st.conv;
    r->rel_true = st.rel_true;
    if (err != 0) {
      r->status = DFG_TIMEOUT;
      r->error = "a triangular-sweep wait gave up (site " + std::to_string(errw[1]) + ", table slot " +
                 std::to_string(errw[2]) + ", range/row " + std::to_string(errw[3]) + ")";
    } else if (st.done == 1) {
      r->status = DFG_OK;
    } else if (st.done == 3) {
      r->status = DFG_NAN_DETECTED;
    } else {
      r->status = DFG_NOT_CONVERGED;
    }
    retiring.push_back(r);
    G.changed = true;
  }
  G.act.swap(keep);
  if (err != 0) {
    SCK(cudaMemsetAsync(G.d_stat + sizeof(SrvStatus) * kSrvMaxSlots, 0, 16, G.s_iter));
    SCK(cudaMemsetAsync(G.d_tickets, 0, sizeof(int) * kClasses * 4, G.s_iter));
    SCK(cudaStreamSynchronize(G.s_iter));
  }
}

// Copies the retired solves' solutions to their callers, then returns their
// memory and completes them.
void retire(dfg_server_s* S, std::vector<Req*>& retiring) {
  if (retiring.empty()) return;
  for (Req* r : retiring) {
    SCK(cudaMemcpyAsync(r->x_out, at<double>(S, r->pbase, r->o_x), (size_t)r->n * r->b * 8, cudaMemcpyDeviceToHost,
                        S->s_copy));
    S->d2h += (long long)r->n * r->b * 8;
  }
  SCK(cudaStreamSynchronize(S->s_copy));
  std::lock_guard<std::mutex> lk(S->mu);
  for (Req* r : retiring) {
    release_locked(S, r);
    finish_locked(S, r);
  }
  retiring.clear();
}

void loop_thread(dfg_server_s* S) {
  cudaSetDevice(S->device);
  std::vector<Req*> retiring;
  try {
    for (;;) {
      bool idle_all = true;
      {
        std::unique_lock<std::mutex> lk(S->mu);
        auto has_work = [&] {
          for (int g = 0; g < S->ngroups; ++g) {
            const Group& G = S->grp[g];
            if (!G.act.empty() || !G.incoming.empty() || G.in_flight) return true;
          }
          return !retiring.empty();
        };
        if (!has_work()) {
          if (S->loop_stop) return;
          S->cv_loop.wait(lk, [&] { return has_work() || S->loop_stop; });
          continue;
        }
      }
      // replays that have finished: statuses, profiles, retirements
      for (int g = 0; g < S->ngroups; ++g) {
        Group& G = S->grp[g];
        if (!G.in_flight) continue;
        const cudaError_t q = cudaEventQuery(G.ev_done);
        if (q == cudaErrorNotReady) continue;
        SCK(q);
        G.in_flight = false;
        idle_all = false;
        S->busy_s += std::chrono::duration<double>(Clock::now() - G.t_launch).count();
        if (G.prof) account_profile(S, G);
        harvest(S, G, retiring);
      }
      // groups with no replay in flight take the solves admitted meanwhile
      // (a group's table changes only between its replays: the status array
      // of a replay in flight describes the slots it was launched with), then
      // start their next replay
      for (int g = 0; g < S->ngroups; ++g) {
        Group& G = S->grp[g];
        if (G.in_flight) continue;
        {
          std::lock_guard<std::mutex> lk(S->mu);
          while (!G.incoming.empty() && (int)G.act.size() < kSrvMaxSlots) {
            G.act.push_back(G.incoming.front());
            G.incoming.pop_front();
            G.changed = true;
          }
        }
        if (G.act.empty()) continue;
        if (G.changed) {
          const int mask = upload_table(S, G);
          if (mask != G.graph_mask) build_graph(S, G, mask);
          G.changed = false;
        }
        G.prof = G.exec_prof && G.replays % S->profile_every == 0;
        SCK(cudaGraphLaunch(G.prof ? G.exec_prof : G.exec, G.s_iter));
        SCK(cudaEventRecord(G.ev_done, G.s_iter));
        G.t_launch = Clock::now();
        G.in_flight = true;
        ++G.replays;
        idle_all = false;
        std::lock_guard<std::mutex> lk(S->mu);
        ++S->replays;
        S->launches += kernels_per_replay(S, G);
      }
      // solutions of finished solves go out while the replays run
      if (!retiring.empty()) {
        retire(S, retiring);
        idle_all = false;
      }
      if (idle_all) std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
  } catch (const CudaFail& f) {
    cudaGetLastError();
    std::lock_guard<std::mutex> lk(S->mu);
    S->fatal = DFG_CUDA_ERROR;
    S->fatal_msg = std::string("serving loop: ") + cudaGetErrorString(f.e) + " at " + f.what;
    auto fail = [&](Req* r) {
      r->status = S->fatal;
      r->error = S->fatal_msg;
      release_locked(S, r);
      finish_locked(S, r);
    };
    for (Req* r : retiring) fail(r);
    for (Group& G : S->grp) {
      for (Req* r : G.act) fail(r);
      for (Req* r : G.incoming) fail(r);
      G.act.clear();
      G.incoming.clear();
    }
    S->cv_adm.notify_all();
  }
}

// Sweep launch shape per class.  A batched sweep has many independent
// ranges in flight, so it trades pipeline depth for CTAs: three stages per
// CTA and as many CTAs per SM as shared memory allows (measured on GB300 over
// 150-request streams: depth 3 beat depths 2 and 5-16 in both precisions).
void class_shapes(dfg_server_s* S) {
  const int elem = S->fp32 ? 4 : 8;
  int per_sm_bytes = 0;
  cudaDeviceGetAttribute(&per_sm_bytes, cudaDevAttrMaxSharedMemoryPerMultiprocessor, S->device);
  for (int k = 0; k < kClasses; ++k) {
    const int b = class_b(k), maxe = class_maxe(k);
    S->cls_val_stage[k] = sweep_val_stage(maxe, b, elem);
    size_t worst = 0;
    for (int dir = 0; dir < 2; ++dir) {
      const int rs = (int)((rec_bytes(maxe, b * b, elem, dir == 0) + 15) / 16 * 16);
      S->cls_rec_stage[k][dir] = rs;
      S->cls_ns[k][dir] = kServeStages;
      S->cls_smem[k][dir] = sweep_smem_bytes(kServeStages, rs, S->cls_val_stage[k], kRingSteps, b, elem);
      worst = std::max(worst, S->cls_smem[k][dir]);
    }
    const int per_sm = std::max(1, std::min(16, (int)(per_sm_bytes / (worst + 1024))));
    S->cls_grid[k] = S->nsm * per_sm;
  }
  // solo sweeps: one CTA per SM (solo_shape)
  for (int k = 0; k < kClasses; ++k) {
    const int b = class_b(k), maxe = class_maxe(k);
    const size_t budget = std::min<size_t>(S->ctx->smem_optin, (size_t)per_sm_bytes) - 4096;
    size_t worst = 0;
    for (int dir = 0; dir < 2; ++dir) {
      const SoloShape sh = solo_shape(b, maxe, elem, dir == 0, budget);
      if (sh.ns < 2) throw CudaFail{cudaErrorInvalidValue, "solo sweep stages do not fit in shared memory"};
      S->solo_R[k] = sh.R;
      S->solo_ch[k][dir] = sh.ch_max;
      S->solo_rec_stage[k][dir] = sh.rec_stage;
      S->solo_ns[k][dir] = sh.ns;
      S->solo_smem[k][dir] = sh.smem;
      worst = std::max(worst, sh.smem);
    }
    if (worst > S->ctx->smem_optin) throw CudaFail{cudaErrorInvalidValue, "solo sweep shared memory"};
    S->solo_grid[k] = S->nsm;
  }
}

int server_error(dfg_ctx ctx, int status, const std::string& m) {
  if (ctx) ctx->last_error = m;
  return status;
}

}  // namespace

// ====================================================================== C ABI

extern "C" int dfg_server_create(dfg_ctx ctx, const dfg_server_config* cfg, dfg_server* out) {
  if (!ctx || !cfg || !out) return DFG_INVALID_ARGUMENT;
  *out = nullptr;
  if (cfg->mode != DFG_PREC_FP64 && cfg->mode != DFG_PREC_FP32_FACTOR && cfg->mode != DFG_PREC_MIXED)
    return server_error(ctx, DFG_INVALID_ARGUMENT,
                        "serving modes: DFG_PREC_FP64, DFG_PREC_FP32_FACTOR or DFG_PREC_MIXED");
  if (cfg->max_inflight < 0 || cfg->max_inflight > kSrvMaxSlots || cfg->chunk_iters < 0 || cfg->chunk_iters > 64 ||
      !(cfg->tol > 0.0) || cfg->maxit < 0 || cfg->budget_bytes < 0 || cfg->size_groups < 0 || cfg->size_groups > kGroups ||
      cfg->sweeps < 0 || cfg->sweeps > 2)
    return server_error(ctx, DFG_INVALID_ARGUMENT, "server configuration out of range");
  std::unique_ptr<dfg_server_s> S(new (std::nothrow) dfg_server_s);
  if (!S) return DFG_OOM_REJECTED;
  S->ctx = ctx;
  S->device = ctx->device;
  S->nsm = ctx->nsm;
  S->mode = cfg->mode;
  S->fp32 = cfg->mode != DFG_PREC_FP64;
  S->mixed = cfg->mode == DFG_PREC_MIXED;
  S->tol = cfg->tol;
  S->maxit = cfg->maxit > 0 ? cfg->maxit : 20000;
  // more solves in flight fill the one-CTA sweeps' SMs and the batched
  // kernels better: 62.6 / 68.8 / 71.7 solves/s at 128 / 192 / 256 on the
  // saturated 2D stream (FP32 factor; FP64 40.1 -> 44.2 from 128 to 256)
  S->max_inflight = cfg->max_inflight > 0 ? cfg->max_inflight : kSrvMaxSlots;
  S->chunk = cfg->chunk_iters > 0 ? cfg->chunk_iters : 8;
  const int hw = (int)std::thread::hardware_concurrency();
  S->nthreads = cfg->host_threads > 0 ? cfg->host_threads : std::max(1, hw - 2);
  S->vec_grid = S->nsm * 6;  // blocks of the batched kernels (k_serve.cu kSrvVecBlocks)
  S->profile_every = std::max(0, cfg->profile_every);
  S->ngroups = cfg->size_groups > 0 ? cfg->size_groups : kGroups;
  S->sweeps = cfg->sweeps;
  S->t0 = Clock::now();
  try {
    SCK(cudaSetDevice(S->device));
    size_t fre = 0, tot = 0;
    SCK(cudaMemGetInfo(&fre, &tot));
    size_t budget = cfg->budget_bytes > 0 ? (size_t)cfg->budget_bytes : (size_t)(fre * 0.85);
    if (budget + (64u << 20) > fre)
      return server_error(ctx, DFG_OOM_REJECTED,
                          "admission budget of " + std::to_string(budget) + " bytes exceeds free device memory (" +
                              std::to_string(fre) + ")");
    SCK(cudaMalloc(&S->arena_base, budget));
    S->arena.init(budget);
    int lo = 0, hi = 0;
    SCK(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    for (auto& a : S->adm) {
      SCK(cudaMalloc(&a.d_red, sizeof(double) * (kRedGrid + 32)));
      SCK(cudaMemset(a.d_red, 0, sizeof(double) * (kRedGrid + 32)));
      SCK(cudaHostAlloc(&a.h_nsing, 64, cudaHostAllocDefault));
      SCK(cudaStreamCreateWithPriority(&a.st, cudaStreamNonBlocking, lo));
    }
    SCK(cudaStreamCreateWithPriority(&S->s_copy, cudaStreamNonBlocking, lo));
    for (int g = 0; g < S->ngroups; ++g) {
      Group& G = S->grp[g];
      SCK(cudaMalloc(&G.d_tab, sizeof(SrvTable)));
      SCK(cudaMalloc(&G.d_sb, sizeof(SweepBatch) * kClasses * 2));
      SCK(cudaMalloc(&G.d_solo, sizeof(SoloBatch) * kClasses * 2));
      SCK(cudaMalloc(&G.d_tickets, sizeof(int) * kClasses * 4));
      SCK(cudaMalloc(&G.d_partials, sizeof(double) * kMaxChunks));
      SCK(cudaMalloc(&G.d_chunk_slot, kMaxChunks));
      SCK(cudaHostAlloc(&G.h_chunk_slot, kMaxChunks, cudaHostAllocDefault));
      SCK(cudaMalloc(&G.d_stat, sizeof(SrvStatus) * kSrvMaxSlots + 64));
      SCK(cudaMemset(G.d_tickets, 0, sizeof(int) * kClasses * 4));
      SCK(cudaMemset(G.d_solo, 0, sizeof(SoloBatch) * kClasses * 2));
      SCK(cudaMemset(G.d_stat, 0, sizeof(SrvStatus) * kSrvMaxSlots + 64));
      SCK(cudaMemset(G.d_sb, 0, sizeof(SweepBatch) * kClasses * 2));
      SCK(cudaHostAlloc(&G.h_tab, sizeof(SrvTable), cudaHostAllocDefault));
      SCK(cudaHostAlloc(&G.h_sb, sizeof(SweepBatch) * kClasses * 2, cudaHostAllocDefault));
      SCK(cudaHostAlloc(&G.h_solo, sizeof(SoloBatch) * kClasses * 2, cudaHostAllocDefault));
      SCK(cudaHostAlloc(&G.h_stat, sizeof(SrvStatus) * kSrvMaxSlots + 64, cudaHostAllocDefault));
      std::memset(G.h_tab, 0, sizeof(SrvTable));
      std::memset(G.h_sb, 0, sizeof(SweepBatch) * kClasses * 2);
      std::memset(G.h_solo, 0, sizeof(SoloBatch) * kClasses * 2);
      std::memset(G.h_stat, 0, sizeof(SrvStatus) * kSrvMaxSlots + 64);
      SCK(cudaStreamCreateWithPriority(&G.s_iter, cudaStreamNonBlocking, hi));
      for (int k = 0; k < kClasses; ++k) {
        SCK(cudaStreamCreateWithPriority(&G.s_side[k], cudaStreamNonBlocking, hi));
        SCK(cudaEventCreateWithFlags(&G.ev_join[k], cudaEventDisableTiming));
      }
      SCK(cudaEventCreateWithFlags(&G.ev_fork, cudaEventDisableTiming));
      SCK(cudaEventCreateWithFlags(&G.ev_done, cudaEventDisableTiming));
      if (S->profile_every > 0)
        for (int k = 0; k < 2 * DFG_SERVER_NKERNELS; ++k) SCK(cudaEventCreate(&G.ev_prof[k]));
    }
    SCK(sweep_set_smem_limits(ctx->smem_optin));
    SCK(solo_set_smem_limits(ctx->smem_optin));
    class_shapes(S.get());
  } catch (const CudaFail& f) {
    cudaGetLastError();
    const int st = f.e == cudaErrorMemoryAllocation ? DFG_OOM_REJECTED : DFG_CUDA_ERROR;
    const std::string m = std::string("dfg_server_create: ") + cudaGetErrorString(f.e) + " at " + f.what;
    dfg_server raw = S.release();
    dfg_server_destroy(raw);
    return server_error(ctx, st, m);
  }
  dfg_server s = S.release();
  for (int i = 0; i < s->nthreads; ++i) s->workers.emplace_back(symbolic_worker, s);
  for (int i = 0; i < kAdmLanes; ++i) s->adm[i].th = std::thread(admission_thread, s, i);
  s->loop_thread = std::thread(loop_thread, s);
  *out = s;
  return DFG_OK;
}

extern "C" int dfg_server_submit(dfg_server s, const dfg_request* q, long long* id) {
  if (!s || !q || !id) return DFG_INVALID_ARGUMENT;
  dfg_ctx ctx = s->ctx;
  if (q->kind < 1 || q->kind > 5 || q->nnode <= 0 || q->nelem < 0 || !q->coords || (q->nelem > 0 && !q->conn) ||
      !q->params || q->nparams < 0 || q->nparams > 8 || !q->bcflag || !q->x_out)
    return server_error(ctx, DFG_INVALID_ARGUMENT, "dfg_server_submit: malformed request");
  std::unique_ptr<Req> r(new (std::nothrow) Req);
  if (!r) return DFG_OOM_REJECTED;
  const bool three = q->kind == 2 || q->kind == 5;
  r->kind = q->kind;
  r->ndim = three ? 3 : 2;
  r->nnoel = three ? 4 : 3;
  r->b = q->kind == 4 ? 2 : q->kind == 5 ? 3 : 1;
  r->n = q->nnode;
  r->nelem = q->nelem;
  const size_t m = (size_t)r->n * r->b;
  try {
    r->coords.assign(q->coords, q->coords + (size_t)r->n * r->ndim);
    r->conn.assign(q->conn, q->conn + (size_t)r->nelem * r->nnoel);
    if (q->coef) r->coef.assign(q->coef, q->coef + r->nelem);
    r->params.assign(q->params, q->params + q->nparams);
    r->bcflag.assign(q->bcflag, q->bcflag + m);
    if (q->load) r->load.assign(q->load, q->load + m);
  } catch (const std::bad_alloc&) {
    return server_error(ctx, DFG_OOM_REJECTED, "dfg_server_submit: host allocation failed");
  }
  for (int v : r->conn)
    if (v < 0 || v >= r->n) return server_error(ctx, DFG_INVALID_ARGUMENT, "dfg_server_submit: node index out of range");
  r->x_out = q->x_out;
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->stopping) return server_error(ctx, DFG_NOT_READY, "the server is shutting down");
  r->id = s->next_id++;
  r->t_submit = s->now();
  *id = r->id;
  Req* raw = r.get();
  s->all[raw->id] = std::move(r);
  ++s->n_submitted;
  s->account_locked();
  if (s->fatal != DFG_OK) {
    raw->status = s->fatal;
    raw->error = s->fatal_msg;
    finish_locked(s, raw);
    return DFG_OK;
  }
  ++s->backlog;
  s->submitted.push_back(raw);
  s->cv_sym.notify_one();
  return DFG_OK;
}

static void fill_result(const Req* r, dfg_result* out) {
  out->id = r->id;
  out->status = r->status;
  out->iterations = r->iters;
  out->conv = r->conv;
  out->rel_true = r->rel_true;
  out->t_submit = r->t_submit;
  out->t_admit = r->t_admit;
  out->t_done = r->t_done;
  out->device_bytes = (long long)(r->P.total + r->T.total);
}

extern "C" int dfg_server_wait(dfg_server s, long long id, dfg_result* out) {
  if (!s || !out) return DFG_INVALID_ARGUMENT;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->all.find(id);
  if (it == s->all.end()) return server_error(s->ctx, DFG_INVALID_ARGUMENT, "unknown request id");
  Req* r = it->second.get();
  s->cv_done.wait(lk, [&] { return r->finished; });
  fill_result(r, out);
  return DFG_OK;
}

extern "C" int dfg_server_error_text(dfg_server s, long long id, char* buf, int len) {
  if (!s || !buf || len <= 0) return DFG_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->all.find(id);
  if (it == s->all.end()) return DFG_INVALID_ARGUMENT;
  std::snprintf(buf, (size_t)len, "%s", it->second->error.c_str());
  return DFG_OK;
}

extern "C" int dfg_server_drain(dfg_server s) {
  if (!s) return DFG_INVALID_ARGUMENT;
  std::unique_lock<std::mutex> lk(s->mu);
  s->cv_done.wait(lk, [&] { return s->n_finished == s->n_submitted; });
  return s->fatal;
}

extern "C" int dfg_server_stats(dfg_server s, dfg_server_counters* out) {
  if (!s || !out) return DFG_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(s->mu);
  out->submitted = s->n_submitted;
  out->finished = s->n_finished;
  out->replays = s->replays;
  out->kernel_launches = s->launches;
  out->graph_builds = s->graph_builds;
  out->peak_inflight = s->peak_inflight;
  out->budget_bytes = (long long)s->arena.capacity();
  out->peak_bytes = (long long)s->arena.peak();
  out->h2d_bytes = s->h2d.load();
  out->d2h_bytes = s->d2h.load();
  out->busy_seconds = s->busy_s;
  s->account_locked();
  out->backlog_seconds = s->backlog_s;
  out->queued_seconds = s->queued_s;
  out->full_seconds = s->full_s;
  out->inflight_seconds = s->inflight_s;
  out->symbolic_seconds = s->symbolic_s;
  out->admit_seconds = s->admit_s;
  out->now_seconds = s->now();
  return DFG_OK;
}

extern "C" int dfg_server_profile(dfg_server s, dfg_server_profile_t* out) {
  if (!s || !out) return DFG_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(s->mu);
  for (int k = 0; k < DFG_SERVER_NKERNELS; ++k) {
    out->ms[k] = s->prof_ms[k];
    out->bytes[k] = s->prof_bytes[k];
    out->n[k] = s->prof_n[k];
  }
  return DFG_OK;
}

extern "C" int dfg_server_destroy(dfg_server s) {
  if (!s) return DFG_INVALID_ARGUMENT;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stopping = true;
  }
  s->cv_sym.notify_all();
  s->cv_adm.notify_all();
  s->cv_loop.notify_all();
  for (auto& t : s->workers)
    if (t.joinable()) t.join();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->adm_stop = true;
    s->cv_adm.notify_all();
  }
  for (auto& a : s->adm)
    if (a.th.joinable()) a.th.join();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->loop_stop = true;
    s->cv_loop.notify_all();
  }
  if (s->loop_thread.joinable()) s->loop_thread.join();
  cudaSetDevice(s->device);
  for (Group& G : s->grp) {
    if (G.s_iter) cudaStreamSynchronize(G.s_iter);
    if (G.exec) cudaGraphExecDestroy(G.exec);
    if (G.exec_prof) cudaGraphExecDestroy(G.exec_prof);
    for (cudaEvent_t e : G.ev_prof)
      if (e) cudaEventDestroy(e);
    for (int k = 0; k < kClasses; ++k) {
      if (G.s_side[k]) cudaStreamDestroy(G.s_side[k]);
      if (G.ev_join[k]) cudaEventDestroy(G.ev_join[k]);
    }
    for (cudaEvent_t e : {G.ev_fork, G.ev_done})
      if (e) cudaEventDestroy(e);
    if (G.s_iter) cudaStreamDestroy(G.s_iter);
    for (void* p : {(void*)G.d_tab, (void*)G.d_sb, (void*)G.d_solo, (void*)G.d_tickets, (void*)G.d_partials,
                    (void*)G.d_stat, (void*)G.d_chunk_slot})
      if (p) cudaFree(p);
    for (void* p : {(void*)G.h_tab, (void*)G.h_sb, (void*)G.h_solo, (void*)G.h_stat, (void*)G.h_chunk_slot})
      if (p) cudaFreeHost(p);
  }
  for (auto& a : s->adm) {
    if (a.st) cudaStreamDestroy(a.st);
    if (a.d_red) cudaFree(a.d_red);
    if (a.h_nsing) cudaFreeHost(a.h_nsing);
  }
  if (s->s_copy) cudaStreamDestroy(s->s_copy);
  if (s->arena_base) cudaFree(s->arena_base);
  delete s;
  return DFG_OK;
}
