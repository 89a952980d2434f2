// sweep_emul.cpp -- TEST INFRASTRUCTURE: executes a sweep schedule built by
// the library's host scheduler (delfem_gb300/csrc/sched.cpp) sequentially on
// the CPU, with exactly the dependency encoding the GPU kernel decodes
// (ring slots for recent same-range rows, global reads otherwise), and
// checks the properties the kernel relies on:
//   * every row is scheduled exactly once;
//   * a ring reference points at the slot the dependency was written to and
//     that slot has not been overwritten since;
//   * a global reference points at a row that an earlier range (or an older
//     step of the same range) has finished -- so ranges claimed in order
//     can never wait on a range that has not started (no deadlock).
// It also executes the level schedule of the level-scheduled sweep
// (emul_level_sweep) with the same checks in their level form.
// Built by tests/test_cpu_schedule.py with g++; never part of libdfg.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../delfem_gb300/csrc/dfg_internal.h"
#include "../../delfem_gb300/csrc/k_sweep.h"

using namespace dfg;

extern "C" int emul_sweep(int n, int b, const int* rowptr, const int* colind, int forward, int range_rows, int R,
                          const double* fdiag, const double* foffd, const double* rhs, double* out, long long* info) {
  std::vector<int> diaind(n);
  for (int i = 0; i < n; ++i) {
    int d = rowptr[i + 1];
    for (int c = rowptr[i]; c < rowptr[i + 1]; ++c)
      if (colind[c] > i) { d = c; break; }
    diaind[i] = d;
  }
  SweepPlan P = range_rows > 0    ? build_sweep_plan(n, b, rowptr, colind, diaind.data(), forward != 0, range_rows, R)
                : range_rows == 0 ? choose_sweep_plan(n, b, rowptr, colind, diaind.data(), forward != 0, R, 8)
                                  : fullest_sweep_plan(n, b, rowptr, colind, diaind.data(), forward != 0, R);
  const int bs = b * b;
  info[0] = P.nranges;
  info[1] = P.nsteps;
  info[2] = P.max_nent;
  info[3] = 0;  // errors
  std::vector<int> seen(n, 0), done(n, 0), range_of(n, -1);
  for (int r = 0; r < P.nranges; ++r)
    for (int s = P.range_steps[r]; s < P.range_steps[r + 1]; ++s)
      for (int l = 0; l < 32; ++l) {
        const int row = P.step_rows[(size_t)s * 32 + l];
        if (row >= 0) { seen[row]++; range_of[row] = r; }
      }
  for (int i = 0; i < n; ++i)
    if (seen[i] != 1) { info[3] = 1; return 1; }
  std::vector<double> ring((size_t)P.R * 32 * b, NAN);
  std::vector<int> ring_row((size_t)P.R * 32, -1);
  for (int r = 0; r < P.nranges; ++r) {
    std::fill(ring_row.begin(), ring_row.end(), -1);
    for (int s = P.range_steps[r]; s < P.range_steps[r + 1]; ++s) {
      const int loc = s - P.range_steps[r];
      const int nent = P.step_nent[s];
      // rows of one step are computed from state before the step (as on the GPU)
      std::vector<double> yv(32 * b, 0.0);
      std::vector<int> rows(32, -1);
      for (int l = 0; l < 32; ++l) {
        const int row = P.step_rows[(size_t)s * 32 + l];
        rows[l] = row;
        if (row < 0) continue;
        double t[3];
        for (int d = 0; d < b; ++d) t[d] = rhs[(size_t)row * b + d];
        int c0 = forward ? rowptr[row] : diaind[row];
        int c1 = forward ? diaind[row] : rowptr[row + 1];
        if (c1 - c0 > nent) { info[3] = 2; return 2; }
        for (int e = 0; e < nent; ++e) {
          const int src = P.ent_src[(size_t)(P.ent_off[s] + e) * 32 + l];
          const int slot = P.ent_slot[(size_t)(P.ent_off[s] + e) * 32 + l];
          if (src == SweepPlan::kSrcPad) {
            if (e < c1 - c0) { info[3] = 3; return 3; }
            continue;
          }
          if (slot != c0 + e) { info[3] = 4; return 4; }
          const int k = colind[slot];
          double v[3];
          if (src >= 0) {
            const int ss = src >> 5, ln = src & 31;
            if (ss >= P.R || ring_row[(size_t)ss * 32 + ln] != k) { info[3] = 5; return 5; }
            for (int d = 0; d < b; ++d) v[d] = ring[((size_t)ss * b + d) * 32 + ln];
          } else {
            if (-src - 1 != k) { info[3] = 6; return 6; }
            if (!done[k]) { info[3] = 7; return 7; }          // would spin forever
            if (range_of[k] > r) { info[3] = 8; return 8; }   // waits on a later range
            for (int d = 0; d < b; ++d) v[d] = out[(size_t)k * b + d];
          }
          const double* L = foffd + (size_t)slot * bs;
          for (int p = 0; p < b; ++p)
            for (int q = 0; q < b; ++q) t[p] -= L[p * b + q] * v[q];
        }
        if (forward) {
          const double* D = fdiag + (size_t)row * bs;
          for (int p = 0; p < b; ++p) {
            double acc = 0.0;
            for (int q = 0; q < b; ++q) acc += D[p * b + q] * t[q];
            yv[l * b + p] = acc;
          }
        } else {
          for (int p = 0; p < b; ++p) yv[l * b + p] = t[p];
        }
      }
      const int rs = loc % P.R;
      for (int l = 0; l < 32; ++l) {
        const int row = rows[l];
        ring_row[(size_t)rs * 32 + l] = row;
        if (row < 0) continue;
        for (int d = 0; d < b; ++d) {
          ring[((size_t)rs * b + d) * 32 + l] = yv[l * b + d];
          out[(size_t)row * b + d] = yv[l * b + d];
        }
        done[row] = 1;
      }
    }
  }
  info[4] = (long long)P.est_cost;
  // decode the packed record headers the GPU kernel reads, for both element
  // sizes, and check every code against the plan
  for (int elem = 4; elem <= 8; elem += 4) {
    std::vector<long long> off;
    long long max_rec = 0;
    const std::vector<unsigned char> h = pack_record_headers(P, elem, off, max_rec);
    const int rhs_bytes = sweep_rhs_bytes(b, elem);
    const int val_stage = sweep_val_stage(P.max_nent, b, elem);
    for (int r = 0; r < P.nranges; ++r)
      for (int s = P.range_steps[r]; s < P.range_steps[r + 1]; ++s) {
        const unsigned char* rec = h.data() + off[s];
        const int nent = *reinterpret_cast<const int*>(rec);
        if (nent != P.step_nent[s] || off[s + 1] - off[s] > max_rec || (off[s + 1] - off[s]) % 16) { info[3] = 20; return 20; }
        const int* rows = reinterpret_cast<const int*>(rec + 16);
        const int* code = reinterpret_cast<const int*>(rec + 144);
        const int* grow = code + nent * 32;
        const int loc = s - P.range_steps[r];
        for (int l = 0; l < 32; ++l) {
          if (rows[l] != P.step_rows[(size_t)s * 32 + l]) { info[3] = 21; return 21; }
          for (int e = 0; e < nent; ++e) {
            const int src = P.ent_src[(size_t)(P.ent_off[s] + e) * 32 + l];
            const int c = code[e * 32 + l], g = grow[e * 32 + l];
            if (src == SweepPlan::kSrcPad) {
              if (c != 0 || g != -1) { info[3] = 22; return 22; }
            } else if (src >= 0) {
              const int off_ring = c - 32;
              if (c < 32 || g != -1 || off_ring % (b * elem)) { info[3] = 23; return 23; }
              const int slot = off_ring / (b * elem), ss = slot / 32, ln = slot % 32;
              if (ss >= P.R || ss * 32 + ln != src || (loc - ss) % P.R < 0) { info[3] = 24; return 24; }
            } else {
              const unsigned o = (unsigned)c & 0x7fffffffu;
              if (c >= 0 || g != -src - 1) { info[3] = 25; return 25; }
              if ((int)(o & ~15u) != rhs_bytes + (e * 32 + l) * 32 || (int)(o & 15) != (int)(((long long)g * b * elem) & 15) ||
                  (int)o + b * elem > val_stage) { info[3] = 26; return 26; }
            }
          }
        }
      }
  }
  return 0;
}

// Sliced-ELL map (build_sell) and value layout: emulates the packing kernel
// (k_sell_pack) and the thread-per-row product (sell_row_mv) sequentially and
// compares with the row-order CRS product (off-diagonal blocks in CRS order,
// then the diagonal block): the same operation sequence, so the results must
// be bitwise equal.  Returns 0 on success.
extern "C" int emul_sell(int n, int b, const int* rowptr, const int* colind, const double* diag, const double* offd,
                         const double* x, double* y_sell, double* y_crs, long long* info) {
  const SellMap M = build_sell(n, rowptr, colind);
  const int bs = b * b;
  info[0] = M.nslices;
  info[1] = M.ptr.back();
  // packing
  std::vector<double> val((size_t)M.ptr.back() * bs, 0.0);
  for (int s = 0; s < M.nslices; ++s) {
    const long long k0 = M.ptr[s];
    const int nval = (int)(M.ptr[s + 1] - k0) * bs;
    for (int o = 0; o < nval; ++o) {
      const int lane = o & 31, e = (o >> 5) % bs, w = (o >> 5) / bs;
      const int v = M.src[k0 + w * 32 + lane];
      val[k0 * bs + o] = v >= 0 ? offd[(size_t)v * bs + e] : v == -1 ? 0.0 : diag[(size_t)(-v - 2) * bs + e];
    }
  }
  // coverage: every CRS slot and every diagonal block exactly once
  std::vector<int> seen_off(rowptr[n], 0), seen_dia(n, 0);
  for (long long k = 0; k < M.ptr.back(); ++k) {
    const int v = M.src[k];
    if (v >= 0) seen_off[v]++;
    else if (v <= -2) seen_dia[-v - 2]++;
  }
  for (int c = 0; c < rowptr[n]; ++c) if (seen_off[c] != 1) return 1;
  for (int i = 0; i < n; ++i) if (seen_dia[i] != 1) return 2;
  for (int i = 0; i < n; ++i) {
    // SELL thread-per-row
    const int s = i >> 5, lane = i & 31;
    const long long k0 = M.ptr[s];
    double acc[3] = {0, 0, 0};
    for (int w = 0; w < M.width[s]; ++w) {
      const int j = M.col[k0 + w * 32 + lane];
      for (int p = 0; p < b; ++p)
        for (int q = 0; q < b; ++q) acc[p] += val[k0 * bs + (w * bs + p * b + q) * 32 + lane] * x[(size_t)j * b + q];
    }
    for (int p = 0; p < b; ++p) y_sell[(size_t)i * b + p] = acc[p];
    // CRS row order
    double ref[3] = {0, 0, 0};
    for (int c = rowptr[i]; c < rowptr[i + 1]; ++c)
      for (int p = 0; p < b; ++p)
        for (int q = 0; q < b; ++q) ref[p] += offd[(size_t)c * bs + p * b + q] * x[(size_t)colind[c] * b + q];
    for (int p = 0; p < b; ++p)
      for (int q = 0; q < b; ++q) ref[p] += diag[(size_t)i * bs + p * b + q] * x[(size_t)i * b + q];
    for (int p = 0; p < b; ++p) y_crs[(size_t)i * b + p] = ref[p];
  }
  return 0;
}

// The library's ILU(k) fill pattern (sched.cpp ilu_fill_pattern) for the CPU
// tests: returns the factor's nnz, writing rowptr_f/colind_f when it fits cap.
extern "C" long long emul_ilu_pattern(int n, const int* rowptr, const int* colind, int lev, int* rowptr_f,
                                      int* colind_f, long long cap) {
  std::vector<int> rp, ci;
  if (!ilu_fill_pattern(n, rowptr, colind, lev, rp, ci, (long long)1 << 40)) return -1;
  if ((long long)ci.size() <= cap) {
    std::memcpy(rowptr_f, rp.data(), sizeof(int) * rp.size());
    if (!ci.empty()) std::memcpy(colind_f, ci.data(), sizeof(int) * ci.size());
  }
  return (long long)ci.size();
}

// The level schedule of the level-scheduled sweep (sched.cpp build_levels),
// checked and executed level by level: rows form a permutation grouped by
// level, every dependency of a row lies in an earlier level and a row's level
// is one above its deepest dependency (the longest-path levels, so no launch
// is wasted).  Each row is computed as k_sweep_level computes it: lane l of
// the row's group of G lanes sums entries l, l+G, ... in order, the G
// partials meet in the xor butterfly, and the group's lanes finish the row's
// components.  Rows of later levels are NaN until written, so a read ahead
// of the schedule shows in the result.  info[0] = number of levels,
// info[1] = widest level, info[2] = error code, info[3] = G.
extern "C" int emul_level_sweep(int n, int b, const int* rowptr, const int* colind, int forward, const double* fdiag,
                                const double* foffd, const double* in, double* out, long long* info) {
  std::vector<int> diaind(n);
  for (int i = 0; i < n; ++i) {
    int d = rowptr[i + 1];
    for (int c = rowptr[i]; c < rowptr[i + 1]; ++c)
      if (colind[c] > i) { d = c; break; }
    diaind[i] = d;
  }
  const Levels V = build_levels(n, rowptr, colind, diaind.data(), forward != 0);
  const int nl = (int)V.ptr.size() - 1;
  info[0] = nl;
  info[1] = 0;
  info[2] = 0;
  auto fail = [&](int code) { info[2] = code; return code; };
  if (nl < 0 || V.ptr[0] != 0 || V.ptr[nl] != n || (int)V.rows.size() != n) return fail(1);
  std::vector<int> seen(n, 0);
  for (int l = 0; l < nl; ++l) {
    if (V.ptr[l + 1] <= V.ptr[l]) return fail(2);  // an empty level is a wasted launch
    info[1] = std::max<long long>(info[1], V.ptr[l + 1] - V.ptr[l]);
    for (int k = V.ptr[l]; k < V.ptr[l + 1]; ++k) {
      const int row = V.rows[k];
      if (row < 0 || row >= n || seen[row]++ || V.level[row] != l) return fail(3);
    }
  }
  const int bs = b * b;
  int widest = 0;
  for (int i = 0; i < n; ++i)
    widest = std::max(widest, forward ? diaind[i] - rowptr[i] : rowptr[i + 1] - diaind[i]);
  const int G = level_group_lanes(widest);  // lanes per row, as the library launches the kernel
  info[3] = G;
  for (int i = 0; i < n * b; ++i) out[i] = NAN;
  for (int l = 0; l < nl; ++l) {
    for (int k = V.ptr[l]; k < V.ptr[l + 1]; ++k) {
      const int i = V.rows[k];
      const int c0 = forward ? rowptr[i] : diaind[i];
      const int c1 = forward ? diaind[i] : rowptr[i + 1];
      int deepest = -1;
      for (int c = c0; c < c1; ++c) deepest = std::max(deepest, V.level[colind[c]]);
      if (deepest >= l || deepest + 1 != l) return fail(4);
      double part[32][3] = {};
      for (int lane = 0; lane < G; ++lane)
        for (int c = c0 + lane; c < c1; c += G) {
          const double* blk = foffd + (size_t)c * bs;
          for (int p = 0; p < b; ++p)
            for (int q = 0; q < b; ++q) part[lane][p] += blk[p * b + q] * out[(size_t)colind[c] * b + q];
        }
      for (int o = G / 2; o > 0; o >>= 1) {
        double nxt[32][3];
        for (int lane = 0; lane < G; ++lane)
          for (int p = 0; p < b; ++p) nxt[lane][p] = part[lane][p] + part[lane ^ o][p];
        std::memcpy(part, nxt, sizeof(part));
      }
      double acc[3];
      for (int p = 0; p < b; ++p) acc[p] = in[(size_t)i * b + p] - part[0][p];
      for (int p = 0; p < b; ++p) {
        double y = acc[p];
        if (forward) {
          const double* dv = fdiag + (size_t)i * bs;
          y = dv[p * b] * acc[0];
          for (int q = 1; q < b; ++q) y += dv[p * b + q] * acc[q];
        }
        out[(size_t)i * b + p] = y;
      }
    }
  }
  for (int i = 0; i < n * b; ++i)
    if (std::isnan(out[i])) return fail(5);
  return 0;
}

// Executes the one-CTA-per-solve schedules (solo_sweep_plan + the records of
// pack_solo_headers) the way k_solo.cu runs them, forward then backward, with
// the storage orders the server uses: the forward input in the forward
// plan's step order, y written in the backward plan's step order (where the
// backward sweep reads its input and the forward sweep its global
// dependencies), z in row order.  Per direction: levels in order, a level's
// chunks and steps concurrently (each step reads the ring and the output as
// they stood when the level began), every step writing its ring slot (step
// mod R) and its output position.  Checks: every row once; chunks tile each
// level, hold at most ch_max steps and stage_bytes of records, and carry one
// entry count; a ring code decodes to the slot its dependency was written to,
// that slot is not rewritten by any step of the consuming level, and holds
// the dependency's row; a global code names a row finished in an earlier
// level, at its storage position.  z receives the result (the kernel's
// summation order).  info: [0] forward levels, [1] forward steps, [2] largest
// entry count, [3] error code, [4] ring references, [5] global references,
// [6] chunks (forward + backward).
extern "C" int emul_solo_precond(int n, int b, const int* rowptr, const int* colind, int R, int elem,
                                 int stage_bytes, int ch_max, const double* fdiag, const double* foffd,
                                 const double* rhs, double* z, long long* info) {
  std::vector<int> diaind(n);
  for (int i = 0; i < n; ++i) {
    int d = rowptr[i + 1];
    for (int c = rowptr[i]; c < rowptr[i + 1]; ++c)
      if (colind[c] > i) { d = c; break; }
    diaind[i] = d;
  }
  const SoloPlan SF = solo_sweep_plan(n, b, rowptr, colind, diaind.data(), true, R, elem, stage_bytes, ch_max);
  const SoloPlan SB = solo_sweep_plan(n, b, rowptr, colind, diaind.data(), false, R, elem, stage_bytes, ch_max);
  std::vector<int> ident(n);
  for (int i = 0; i < n; ++i) ident[i] = i;
  const int bs = b * b;
  for (int k = 0; k < 7; ++k) info[k] = 0;
  info[0] = SF.P.nranges;
  info[1] = SF.P.nsteps;
  info[2] = std::max(SF.P.max_nent, SB.P.max_nent);
  info[6] = (long long)(SF.chunks.size() + SB.chunks.size());
  // storage: forward input and y in step order (padded), z in row order
  std::vector<double> xin((size_t)SF.P.nsteps * 32 * b, NAN), y((size_t)SB.P.nsteps * 32 * b, NAN);
  for (int i = 0; i < n; ++i)
    for (int d = 0; d < b; ++d) xin[(size_t)SF.pos[i] * b + d] = rhs[(size_t)i * b + d];
  for (int i = 0; i < n * b; ++i) z[i] = NAN;
  for (int dir = 0; dir < 2; ++dir) {
    const bool forward = dir == 0;
    const SoloPlan& S = forward ? SF : SB;
    const SweepPlan& P = S.P;
    const int* out_pos = forward ? SB.pos.data() : ident.data();
    std::vector<long long> off;
    const std::vector<unsigned char> h = pack_solo_headers(S, elem, out_pos, out_pos, off);
    const double* in = forward ? xin.data() : y.data();
    double* out = forward ? y.data() : z;
    std::vector<int> seen(n, 0), level_of(n, -1);
    for (int l = 0; l < P.nranges; ++l)
      for (int s = P.range_steps[l]; s < P.range_steps[l + 1]; ++s)
        for (int ln = 0; ln < 32; ++ln) {
          const int row = P.step_rows[(size_t)s * 32 + ln];
          if (row >= 0) { seen[row]++; level_of[row] = l; }
        }
    for (int i = 0; i < n; ++i)
      if (seen[i] != 1) { info[3] = 1; return 1; }
    // chunks: tile the steps in order (across level ends), bounded, one size
    // per chunk, with the count of levels ending inside; lev_chunks names the
    // chunk holding each level's first step
    if ((int)S.lev_chunks.size() != P.nranges + 1) { info[3] = 8; return 8; }
    std::vector<int> chunk_of(P.nsteps, -1);
    {
      int next = 0;
      for (size_t c = 0; c < S.chunks.size(); ++c) {
        const SoloChunk& ch = S.chunks[c];
        if (ch.first_step != next || ch.nsteps < 1 || ch.nsteps > ch_max || ch.rec_off != off[ch.first_step] ||
            ch.rec_bytes != off[ch.first_step + ch.nsteps] - off[ch.first_step] ||
            (ch.nsteps > 1 && ch.rec_bytes > stage_bytes)) { info[3] = 9; return 9; }
        int ends = 0;
        for (int s = ch.first_step; s < ch.first_step + ch.nsteps; ++s) {
          if (P.step_nent[s] != ch.nent) { info[3] = 10; return 10; }
          chunk_of[s] = (int)c;
        }
        for (int l = 0; l < P.nranges; ++l)
          if (P.range_steps[l + 1] > ch.first_step && P.range_steps[l + 1] <= ch.first_step + ch.nsteps) ++ends;
        if (ends != ch.nclose) { info[3] = 11; return 11; }
        next += ch.nsteps;
      }
      if (next != P.nsteps) { info[3] = 11; return 11; }
      for (int l = 0; l < P.nranges; ++l)
        if (P.range_steps[l] < P.nsteps && S.lev_chunks[l] != chunk_of[P.range_steps[l]]) { info[3] = 8; return 8; }
    }
    std::vector<int> ring_row((size_t)R * 32, -1);
    std::vector<double> ring((size_t)R * 32 * b, NAN);
    std::vector<char> done(n, 0), written_now(R, 0);
    for (int l = 0; l < P.nranges; ++l) {
      std::fill(written_now.begin(), written_now.end(), 0);
      for (int s = P.range_steps[l]; s < P.range_steps[l + 1]; ++s) written_now[s % R] = 1;
      struct W { int row, o, slot; double y[3]; };
      std::vector<W> writes;
      for (int s = P.range_steps[l]; s < P.range_steps[l + 1]; ++s) {
        const unsigned char* rec = h.data() + off[s];
        int hdr[4];
        std::memcpy(hdr, rec, 16);
        const int nent = hdr[0];
        if (nent != P.step_nent[s] || hdr[2] != s) { info[3] = 2; return 2; }
        {  // the step's chunk size, whether it closes its level, its place in
           // the level (the kernel distributes a level's steps by it)
          const SoloChunk& ch = S.chunks[chunk_of[s]];
          const int closes = s + 1 == P.range_steps[l + 1] ? 1 << 16 : 0;
          if (hdr[1] != (ch.nsteps | closes) || hdr[3] != s - P.range_steps[l]) {
            info[3] = 12;
            return 12;
          }
        }
        const int* outv = reinterpret_cast<const int*>(rec + 16);
        const int* code = reinterpret_cast<const int*>(rec + 144);
        for (int ln = 0; ln < 32; ++ln) {
          const int row = P.step_rows[(size_t)s * 32 + ln];
          if (outv[ln] != (row >= 0 ? out_pos[row] : -1)) { info[3] = 3; return 3; }
          if (row < 0) continue;
          const int c0 = forward ? rowptr[row] : diaind[row];
          const int c1 = forward ? diaind[row] : rowptr[row + 1];
          double t[3];
          for (int d = 0; d < b; ++d) t[d] = in[((size_t)s * 32 + ln) * b + d];
          for (int e = 0; e < nent; ++e) {
            const int c = code[e * 32 + ln];
            if (e >= c1 - c0) {
              if (c != 0) { info[3] = 4; return 4; }
              continue;
            }
            const int k = colind[c0 + e];
            double v[3];
            if (c >= 0) {
              if (c < 32 || (c - 32) % (b * elem) != 0) { info[3] = 5; return 5; }
              const int idx = (c - 32) / (b * elem);
              if (idx >= R * 32 || ring_row[idx] != k || written_now[idx / 32]) { info[3] = 6; return 6; }
              for (int d = 0; d < b; ++d) v[d] = ring[(size_t)idx * b + d];
              info[4]++;
            } else {
              if (-c - 1 != out_pos[k] || !done[k] || level_of[k] >= l) { info[3] = 7; return 7; }
              for (int d = 0; d < b; ++d) v[d] = out[(size_t)(-c - 1) * b + d];
              info[5]++;
            }
            const double* blk = foffd + (size_t)(c0 + e) * bs;
            for (int p = 0; p < b; ++p) {
              double acc = t[p];
              for (int q = 0; q < b; ++q) acc -= blk[p * b + q] * v[q];
              t[p] = acc;
            }
          }
          W w{row, outv[ln], (s % R) * 32 + ln, {0, 0, 0}};
          if (forward) {
            const double* dv = fdiag + (size_t)row * bs;
            for (int p = 0; p < b; ++p) {
              double acc = dv[p * b] * t[0];
              for (int q = 1; q < b; ++q) acc += dv[p * b + q] * t[q];
              w.y[p] = acc;
            }
          } else {
            for (int p = 0; p < b; ++p) w.y[p] = t[p];
          }
          writes.push_back(w);
        }
      }
      for (const W& w : writes) {
        for (int d = 0; d < b; ++d) {
          out[(size_t)w.o * b + d] = w.y[d];
          ring[(size_t)w.slot * b + d] = w.y[d];
        }
        ring_row[w.slot] = w.row;
        done[w.row] = 1;
      }
    }
  }
  return 0;
}

// The one-CTA sweep's launch shape for a class (solo_shape, k_sweep.h):
// out = {R, ch_max, rec_stage, ns, smem}.
extern "C" void emul_solo_shape(int b, int maxe, int elem, int forward, long long budget, long long* out) {
  const SoloShape s = solo_shape(b, maxe, elem, forward != 0, (size_t)budget);
  out[0] = s.R;
  out[1] = s.ch_max;
  out[2] = s.rec_stage;
  out[3] = s.ns;
  out[4] = (long long)s.smem;
}
