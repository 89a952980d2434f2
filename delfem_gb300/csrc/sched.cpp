// sched.cpp -- host-side symbolic work: patterns, level sets, sweep
// schedules and the assembly gather map.  Runs once per mesh / pattern.
#include <algorithm>
#include <climits>
#include <cstring>
#include <numeric>

#include "dfg_internal.h"
#include "k_sweep.h"

namespace dfg {

// CElemAry::MakePattern_FEM (src/femfield/elem_ary.cpp:225-245): elements
// surrounding each point, then the points of those elements except the point
// itself, sorted ascending (Com::CIndexedArray::Sort).
void pattern_from_elements(int nnode, int nelem, int nnoel, const int* conn,
                           std::vector<int>& rowptr, std::vector<int>& colind) {
  std::vector<int> esup_ptr(nnode + 1, 0);
  for (long long k = 0; k < (long long)nelem * nnoel; ++k) esup_ptr[conn[k] + 1]++;
  for (int i = 0; i < nnode; ++i) esup_ptr[i + 1] += esup_ptr[i];
  std::vector<int> esup(esup_ptr[nnode]);
  std::vector<int> fill(esup_ptr.begin(), esup_ptr.end() - 1);
  for (int e = 0; e < nelem; ++e)
    for (int k = 0; k < nnoel; ++k) esup[fill[conn[(long long)e * nnoel + k]]++] = e;
  std::vector<int> mark(nnode, -1);
  rowptr.assign(nnode + 1, 0);
  colind.clear();
  colind.reserve((size_t)nnode * 8);
  std::vector<int> tmp;
  for (int i = 0; i < nnode; ++i) {
    tmp.clear();
    for (int p = esup_ptr[i]; p < esup_ptr[i + 1]; ++p) {
      const int e = esup[p];
      for (int k = 0; k < nnoel; ++k) {
        const int j = conn[(long long)e * nnoel + k];
        if (j == i || mark[j] == i) continue;
        mark[j] = i;
        tmp.push_back(j);
      }
    }
    std::sort(tmp.begin(), tmp.end());
    colind.insert(colind.end(), tmp.begin(), tmp.end());
    rowptr[i + 1] = (int)colind.size();
  }
}

// Block pattern of the ILU(lev_fill) factor: CMatDiaFrac_BlkCrs::AddFracPtn
// (src/matvec/matdiafrac_blkcrs.cpp:1254-1382) as CPreconditioner_ILU::
// SetLinearSystem calls it for one segment (src/ls/preconditioner.cpp:96-157).
// Row i starts as A's row at level 0.  Its entries k < i are taken in
// ascending column order, fill found on the way included; an entry of level
// L spawns only while L + 1 <= lev_fill (always for lev_fill == -1): every
// entry (k, j), j > k, of the finished factor row k whose level M passes the
// same test adds (i, j) at level max(L, M) + 1, unless j == i or (i, j) is
// already present (its level then stays).  Level 0, an empty off-diagonal
// pattern and a full one leave the pattern as it is.  False when the factor
// would exceed `max_nnz` entries.
bool ilu_fill_pattern(int n, const int* rowptr, const int* colind, int lev_fill, std::vector<int>& rowptr_f,
                      std::vector<int>& colind_f, long long max_nnz) {
  const long long nnz = rowptr[n];
  if (lev_fill == 0 || nnz == 0 || nnz == (long long)n * (n - 1)) {
    rowptr_f.assign(rowptr, rowptr + n + 1);
    colind_f.assign(colind, colind + nnz);
    return true;
  }
  const auto spawns = [lev_fill](int l) { return lev_fill < 0 || l + 1 <= lev_fill; };
  constexpr int kEnd = -1;
  std::vector<int> succ(n + 1), lev(n), seen(n, -1), upper(n);  // succ[n]: first column of the row
  std::vector<int> flev;
  rowptr_f.assign(n + 1, 0);
  colind_f.clear();
  colind_f.reserve((size_t)nnz * 2);
  flev.reserve((size_t)nnz * 2);
  for (int i = 0; i < n; ++i) {
    int last = n;
    for (int c = rowptr[i]; c < rowptr[i + 1]; ++c) {
      const int j = colind[c];
      succ[last] = j;
      last = j;
      lev[j] = 0;
      seen[j] = i;
    }
    succ[last] = kEnd;
    for (int k = succ[n]; k != kEnd; k = succ[k]) {
      if (!spawns(lev[k])) continue;
      if (k >= i) break;
      int at = k;  // new columns are > k and ascend with the loop below
      for (int q = upper[k]; q < rowptr_f[k + 1]; ++q) {
        if (!spawns(flev[q])) continue;
        const int j = colind_f[q];
        if (j == i || seen[j] == i) continue;
        while (succ[at] != kEnd && succ[at] < j) at = succ[at];
        succ[j] = succ[at];
        succ[at] = j;
        lev[j] = std::max(lev[k], flev[q]) + 1;
        seen[j] = i;
        at = j;
      }
    }
    upper[i] = -1;
    for (int j = succ[n]; j != kEnd; j = succ[j]) {
      if (upper[i] < 0 && j > i) upper[i] = (int)colind_f.size();
      colind_f.push_back(j);
      flev.push_back(lev[j]);
    }
    if ((long long)colind_f.size() > max_nnz) return false;
    if (upper[i] < 0) upper[i] = (int)colind_f.size();
    rowptr_f[i + 1] = (int)colind_f.size();
  }
  return true;
}

// For every CRS slot of A, the slot of the same block in the factor pattern
// (which contains A's); false if some block is missing.
bool factor_slot_map(int n, const int* rowptr, const int* colind, const int* rowptr_f, const int* colind_f,
                     std::vector<int>& a2f) {
  a2f.assign((size_t)rowptr[n], -1);
  for (int i = 0; i < n; ++i) {
    int q = rowptr_f[i];
    for (int c = rowptr[i]; c < rowptr[i + 1]; ++c) {
      while (q < rowptr_f[i + 1] && colind_f[q] < colind[c]) ++q;
      if (q == rowptr_f[i + 1] || colind_f[q] != colind[c]) return false;
      a2f[c] = q;
    }
  }
  return true;
}

static inline void deps_of(int row, bool forward, const int* rowptr, const int* diaind, int& c0, int& c1) {
  if (forward) { c0 = rowptr[row]; c1 = diaind[row]; }
  else { c0 = diaind[row]; c1 = rowptr[row + 1]; }
}

Levels build_levels(int n, const int* rowptr, const int* colind, const int* diaind, bool forward) {
  Levels L;
  L.level.assign(n, 0);
  int maxlev = -1;
  for (int p = 0; p < n; ++p) {
    const int row = forward ? p : n - 1 - p;
    int c0, c1;
    deps_of(row, forward, rowptr, diaind, c0, c1);
    int lv = 0;
    for (int c = c0; c < c1; ++c) lv = std::max(lv, L.level[colind[c]] + 1);
    L.level[row] = lv;
    maxlev = std::max(maxlev, lv);
  }
  const int nl = maxlev + 1;
  L.ptr.assign(nl + 1, 0);
  for (int i = 0; i < n; ++i) L.ptr[L.level[i] + 1]++;
  for (int l = 0; l < nl; ++l) L.ptr[l + 1] += L.ptr[l];
  L.rows.assign(n, 0);
  std::vector<int> fill(L.ptr.begin(), L.ptr.end() - 1);
  for (int p = 0; p < n; ++p) {
    const int row = forward ? p : n - 1 - p;
    L.rows[fill[L.level[row]]++] = row;
  }
  return L;
}

// Range boundaries.  A cut right after a row that the next rows depend on
// makes the next range wait for the end of this one, so a cut goes where the
// row at the cut depends on no row close before it: between half and twice
// the target size, the candidate whose nearest dependency lies furthest back
// wins (a plane start beats a line start in a structured 3D mesh), ties going
// to the candidate closest to the target.
static std::vector<int> range_cuts(int n, const int* rowptr, const int* colind, const int* diaind, bool forward,
                                   int target) {
  std::vector<int> dist(n + 1, 0);  // position distance to the nearest dependency
  for (int p = 0; p < n; ++p) {
    const int row = forward ? p : n - 1 - p;
    int c0, c1;
    deps_of(row, forward, rowptr, diaind, c0, c1);
    int nearest = -1;
    for (int c = c0; c < c1; ++c) {
      const int k = colind[c];
      nearest = std::max(nearest, forward ? k : n - 1 - k);
    }
    dist[p] = nearest < 0 ? n : p - nearest;
  }
  std::vector<int> cuts{0};
  int a = 0;
  const int g = 2;
  while (a < n) {
    const int want = a + target;
    if (want >= n) break;
    const int lo = std::max(a + 1, a + target / 2), hi = std::min(n - 1, a + 2 * target);
    int pick = -1, best_d = g, best_off = 0;
    for (int p = lo; p <= hi; ++p) {
      const int d = dist[p], off = std::abs(p - want);
      if (d > best_d || (d == best_d && pick >= 0 && off < best_off)) {
        if (d > g) { pick = p; best_d = d; best_off = off; }
      }
    }
    if (pick < 0) pick = want;
    cuts.push_back(pick);
    a = pick;
  }
  cuts.push_back(n);
  return cuts;
}

SweepPlan build_sweep_plan(int n, int b, const int* rowptr, const int* colind, const int* diaind,
                           bool forward, int range_rows, int R) {
  SweepPlan P;
  P.forward = forward;
  P.n = n;
  P.b = b;
  P.R = R;
  range_rows = std::max(1, range_rows);
  const std::vector<int> cuts = range_cuts(n, rowptr, colind, diaind, forward, range_rows);
  P.nranges = (int)cuts.size() - 1;
  P.range_steps.assign(P.nranges + 1, 0);
  std::vector<int> llev(n, 0);          // local level per row
  std::vector<int> row_step(n, 0), row_lane(n, 0), row_range(n, 0);
  std::vector<int> cnt;
  // pass 1: steps per range
  for (int r = 0; r < P.nranges; ++r) {
    const int p0 = cuts[r], p1 = cuts[r + 1];
    int maxl = 0;
    for (int p = p0; p < p1; ++p) {
      const int row = forward ? p : n - 1 - p;
      int c0, c1;
      deps_of(row, forward, rowptr, diaind, c0, c1);
      int lv = 0;
      for (int c = c0; c < c1; ++c) {
        const int k = colind[c];
        const int pk = forward ? k : n - 1 - k;
        if (pk >= p0) lv = std::max(lv, llev[k] + 1);
      }
      llev[row] = lv;
      row_range[row] = r;
      maxl = std::max(maxl, lv);
    }
    cnt.assign(maxl + 2, 0);
    for (int p = p0; p < p1; ++p) cnt[llev[forward ? p : n - 1 - p] + 1]++;
    // steps: ceil(level size / 32) per level, in level order, rows in position order
    int s = P.nsteps;
    std::vector<int> lvl_first_step(maxl + 1), lvl_fill(maxl + 1, 0);
    for (int l = 0; l <= maxl; ++l) {
      lvl_first_step[l] = s;
      s += (cnt[l + 1] + 31) / 32;
    }
    for (int p = p0; p < p1; ++p) {
      const int row = forward ? p : n - 1 - p;
      const int l = llev[row];
      const int q = lvl_fill[l]++;
      row_step[row] = lvl_first_step[l] + q / 32;
      row_lane[row] = q % 32;
    }
    P.range_steps[r] = P.nsteps;
    P.nsteps = s;
  }
  P.range_steps[P.nranges] = P.nsteps;
  // pass 2: rows per step and entry counts
  P.step_rows.assign((size_t)P.nsteps * 32, -1);
  P.step_nent.assign(P.nsteps, 0);
  for (int row = 0; row < n; ++row) {
    P.step_rows[(size_t)row_step[row] * 32 + row_lane[row]] = row;
    int c0, c1;
    deps_of(row, forward, rowptr, diaind, c0, c1);
    P.step_nent[row_step[row]] = std::max(P.step_nent[row_step[row]], c1 - c0);
  }
  P.ent_off.assign(P.nsteps + 1, 0);
  for (int s = 0; s < P.nsteps; ++s) {
    P.ent_off[s + 1] = P.ent_off[s] + P.step_nent[s];
    P.max_nent = std::max(P.max_nent, P.step_nent[s]);
  }
  const long long nent_total = P.ent_off[P.nsteps];
  P.ent_src.assign((size_t)nent_total * 32, SweepPlan::kSrcPad);
  P.ent_slot.assign((size_t)nent_total * 32, -1);
  for (int row = 0; row < n; ++row) {
    const int s = row_step[row], lane = row_lane[row], r = row_range[row];
    const int local = s - P.range_steps[r];
    int c0, c1;
    deps_of(row, forward, rowptr, diaind, c0, c1);
    for (int c = c0; c < c1; ++c) {
      const int k = colind[c];
      const long long e = P.ent_off[s] + (c - c0);
      int src;
      if (row_range[k] == r && local - (row_step[k] - P.range_steps[r]) < R) {
        const int lk = row_step[k] - P.range_steps[r];
        src = (lk % R) * 32 + row_lane[k];
      } else {
        src = -(k + 1);
      }
      P.ent_src[(size_t)e * 32 + lane] = src;
      P.ent_slot[(size_t)e * 32 + lane] = c;
    }
  }
  // makespan model: a step takes one unit once its range's previous step and
  // every producer step (+ a hop of kHop units between ranges) are done
  {
    const double kHop = 40.0;
    std::vector<double> step_end(P.nsteps, 0.0);
    double makespan = 0.0;
    for (int r = 0; r < P.nranges; ++r) {
      double t = 0.0;
      for (int s = P.range_steps[r]; s < P.range_steps[r + 1]; ++s) {
        double start = t;
        for (long long e = P.ent_off[s]; e < P.ent_off[s + 1]; ++e)
          for (int lane = 0; lane < 32; ++lane) {
            const int src = P.ent_src[(size_t)e * 32 + lane];
            if (src == SweepPlan::kSrcPad || src >= 0) continue;
            const int k = -src - 1;
            const double ready = step_end[row_step[k]] + (row_range[k] == r ? 0.0 : kHop);
            start = std::max(start, ready);
          }
        int nrow = 0;
        for (int lane = 0; lane < 32; ++lane) nrow += P.step_rows[(size_t)s * 32 + lane] >= 0;
        t = start + 1.0 + 0.0005 * nrow * (P.step_nent[s] + 1) * b * b;
        step_end[s] = t;
      }
      makespan = std::max(makespan, t);
    }
    P.est_cost = makespan;
  }
  return P;
}

std::vector<SweepPlan> candidate_sweep_plans(int n, int b, const int* rowptr, const int* colind, const int* diaind,
                                             bool forward, int R, int keep) {
  std::vector<SweepPlan> all;
  for (long long rr = 256;; rr *= 2) {
    const int range_rows = (int)std::min<long long>(rr, std::max(n, 1));
    SweepPlan P = build_sweep_plan(n, b, rowptr, colind, diaind, forward, range_rows, R);
    bool dup = false;
    for (const SweepPlan& Q : all) dup |= (Q.nranges == P.nranges && Q.nsteps == P.nsteps);
    if (!dup) all.push_back(std::move(P));
    if (range_rows >= n) break;
  }
  std::stable_sort(all.begin(), all.end(), [](const SweepPlan& x, const SweepPlan& y) { return x.est_cost < y.est_cost; });
  if ((int)all.size() > keep) all.resize(keep);
  return all;
}

SweepPlan choose_sweep_plan(int n, int b, const int* rowptr, const int* colind, const int* diaind,
                            bool forward, int R, int /*elem_size*/) {
  std::vector<SweepPlan> c = candidate_sweep_plans(n, b, rowptr, colind, diaind, forward, R, 1);
  return std::move(c.front());
}

std::vector<unsigned char> pack_record_headers(const SweepPlan& P, int elem, std::vector<long long>& off,
                                               long long& max_rec) {
  const int b = P.b, bs = b * b;
  const int rhs_bytes = sweep_rhs_bytes(b, elem);
  off.assign(P.nsteps + 1, 0);
  max_rec = 0;
  for (int s = 0; s < P.nsteps; ++s) {
    const long long rb = rec_bytes(P.step_nent[s], bs, elem, P.forward);
    off[s + 1] = off[s] + rb;
    max_rec = std::max(max_rec, rb);
  }
  std::vector<unsigned char> h((size_t)off[P.nsteps], 0);
  for (int s = 0; s < P.nsteps; ++s) {
    unsigned char* r = h.data() + off[s];
    const int nent = P.step_nent[s];
    std::memcpy(r, &nent, 4);
    std::memcpy(r + 16, &P.step_rows[(size_t)s * 32], 128);
    int* code = reinterpret_cast<int*>(r + 144);
    int* grow = code + nent * 32;
    for (int e = 0; e < nent; ++e)
      for (int lane = 0; lane < 32; ++lane) {
        const int src = P.ent_src[(size_t)(P.ent_off[s] + e) * 32 + lane];
        int c = 0, gr = -1;
        if (src == SweepPlan::kSrcPad) {
          c = 0;
        } else if (src >= 0) {
          const int ss = src >> 5, ln = src & 31;
          c = 32 + (ss * 32 + ln) * b * elem;
        } else {
          const long long k = -(long long)src - 1;
          gr = (int)k;
          c = (int)(0x80000000u | (unsigned)(rhs_bytes + (e * 32 + lane) * 32 + (int)((k * b * elem) & 15)));
        }
        code[e * 32 + lane] = c;
        grow[e * 32 + lane] = gr;
      }
  }
  return h;
}

SoloPlan solo_sweep_plan(int n, int b, const int* rowptr, const int* colind, const int* diaind, bool forward,
                         int R, int elem, int stage_bytes, int ch_max) {
  SoloPlan S;
  SweepPlan& P = S.P;
  P.forward = forward;
  P.n = n;
  P.b = b;
  P.R = R;
  const int bs = b * b;
  const Levels L = build_levels(n, rowptr, colind, diaind, forward);
  const int nl = (int)L.ptr.size() - 1;
  P.nranges = std::max(nl, 0);
  P.range_steps.assign(P.nranges + 1, 0);
  std::vector<int> row_step(n, 0), row_lane(n, 0);
  for (int l = 0; l < nl; ++l) {
    P.range_steps[l] = P.nsteps;
    const int cnt = L.ptr[l + 1] - L.ptr[l];
    for (int q = 0; q < cnt; ++q) {
      const int row = L.rows[L.ptr[l] + q];
      row_step[row] = P.nsteps + q / 32;
      row_lane[row] = q % 32;
    }
    P.nsteps += (cnt + 31) / 32;
  }
  P.range_steps[P.nranges] = P.nsteps;
  std::vector<int> step_level(P.nsteps, 0);
  for (int l = 0; l < nl; ++l)
    for (int s = P.range_steps[l]; s < P.range_steps[l + 1]; ++s) step_level[s] = l;
  P.step_rows.assign((size_t)P.nsteps * 32, -1);
  std::vector<int> own(P.nsteps, 0);  // the step's own largest entry count
  S.pos.assign(n, 0);
  for (int row = 0; row < n; ++row) {
    P.step_rows[(size_t)row_step[row] * 32 + row_lane[row]] = row;
    S.pos[row] = row_step[row] * 32 + row_lane[row];
    int c0, c1;
    deps_of(row, forward, rowptr, diaind, c0, c1);
    own[row_step[row]] = std::max(own[row_step[row]], c1 - c0);
  }
  // chunks: consecutive steps, across level ends, at most ch_max of them and
  // stage_bytes of records (a chunk holds at least one step); a narrow level
  // shares its chunk with the next ones, so the copies and the handshake of
  // one chunk serve several levels
  S.lev_chunks.assign(P.nranges + 1, 0);
  P.step_nent.assign(P.nsteps, 0);
  {
    int s = 0, l = 0;
    while (s < P.nsteps) {
      SoloChunk c{0, 0, s, 0, 0, 0};
      while (s < P.nsteps && c.nsteps < ch_max) {
        const int ne = std::max(c.nent, own[s]);
        if (c.nsteps > 0 && (c.nsteps + 1) * solo_rec_bytes(ne, bs, elem, forward) > stage_bytes) break;
        c.nent = ne;
        ++c.nsteps;
        ++s;
      }
      for (int t = c.first_step; t < c.first_step + c.nsteps; ++t) P.step_nent[t] = c.nent;
      // levels ending inside the chunk; the next level's first step is in
      // this chunk unless the chunk ends with the level
      for (; l < nl && P.range_steps[l + 1] <= s; ++l) {
        ++c.nclose;
        S.lev_chunks[l + 1] = (int)S.chunks.size() + (P.range_steps[l + 1] < s ? 0 : 1);
      }
      S.chunks.push_back(c);
    }
  }
  S.lev_chunks[P.nranges] = (int)S.chunks.size();
  P.ent_off.assign(P.nsteps + 1, 0);
  for (int s = 0; s < P.nsteps; ++s) {
    P.ent_off[s + 1] = P.ent_off[s] + P.step_nent[s];
    P.max_nent = std::max(P.max_nent, P.step_nent[s]);
  }
  const long long nent_total = P.ent_off[P.nsteps];
  P.ent_src.assign((size_t)nent_total * 32, SweepPlan::kSrcPad);
  P.ent_slot.assign((size_t)nent_total * 32, -1);
  for (int row = 0; row < n; ++row) {
    const int s = row_step[row], lane = row_lane[row];
    const int level_end = P.range_steps[step_level[s] + 1];
    int c0, c1;
    deps_of(row, forward, rowptr, diaind, c0, c1);
    for (int c = c0; c < c1; ++c) {
      const int k = colind[c];
      const long long e = P.ent_off[s] + (c - c0);
      const int sk = row_step[k];
      P.ent_src[(size_t)e * 32 + lane] = (sk >= level_end - R) ? (sk % R) * 32 + row_lane[k] : -(k + 1);
      P.ent_slot[(size_t)e * 32 + lane] = c;
    }
  }
  long long off = 0;
  for (SoloChunk& c : S.chunks) {
    c.rec_off = off;
    c.rec_bytes = (int)(c.nsteps * solo_rec_bytes(c.nent, bs, elem, forward));
    off += c.rec_bytes;
  }
  P.est_cost = (double)P.nranges;
  return S;
}

std::vector<unsigned char> pack_solo_headers(const SoloPlan& S, int elem, const int* out_pos, const int* glob_pos,
                                             std::vector<long long>& off) {
  const SweepPlan& P = S.P;
  const int b = P.b, bs = b * b;
  off.assign(P.nsteps + 1, 0);
  for (int s = 0; s < P.nsteps; ++s) off[s + 1] = off[s] + solo_rec_bytes(P.step_nent[s], bs, elem, P.forward);
  std::vector<unsigned char> h((size_t)off[P.nsteps], 0);
  std::vector<int> level_first(P.nsteps, 0), level_end(P.nsteps, 0);
  for (int l = 0; l < P.nranges; ++l)
    for (int s = P.range_steps[l]; s < P.range_steps[l + 1]; ++s) {
      level_first[s] = P.range_steps[l];
      level_end[s] = P.range_steps[l + 1];
    }
  for (const SoloChunk& c : S.chunks)
    for (int s = c.first_step; s < c.first_step + c.nsteps; ++s) {
      unsigned char* r = h.data() + off[s];
      // steps in the chunk, plus 1 << 16 when this step closes its level; the
      // step's place in its level
      const int closes = s + 1 == level_end[s] ? 1 << 16 : 0;
      const int hdr[4] = {P.step_nent[s], c.nsteps | closes, s, s - level_first[s]};
      std::memcpy(r, hdr, 16);
      int* outv = reinterpret_cast<int*>(r + 16);
      int* code = reinterpret_cast<int*>(r + 144);
      for (int lane = 0; lane < 32; ++lane) {
        const int row = P.step_rows[(size_t)s * 32 + lane];
        outv[lane] = row >= 0 ? out_pos[row] : -1;
      }
      for (int e = 0; e < P.step_nent[s]; ++e)
        for (int lane = 0; lane < 32; ++lane) {
          const int src = P.ent_src[(size_t)(P.ent_off[s] + e) * 32 + lane];
          int cd = 0;
          if (src == SweepPlan::kSrcPad) cd = 0;
          else if (src >= 0) cd = 32 + src * b * elem;
          else cd = -(glob_pos[-src - 1] + 1);
          code[e * 32 + lane] = cd;
        }
    }
  return h;
}

bool build_gather_map(int n, const int* rowptr, const int* colind, int nelem, int nnoel,
                      const int* conn, GatherMap& G, std::string& err) {
  const long long nnz = rowptr[n];
  const int k = nnoel;
  G.slot_ptr.assign(n + nnz + 1, 0);
  G.res_ptr.assign(n + 1, 0);
  // count
  for (int e = 0; e < nelem; ++e) {
    const int* no = conn + (long long)e * k;
    for (int i = 0; i < k; ++i) {
      if (no[i] < 0 || no[i] >= n) { err = "connectivity index out of range"; return false; }
      G.res_ptr[no[i] + 1]++;
      for (int j = 0; j < k; ++j) {
        if (i == j) { G.slot_ptr[no[i] + 1]++; continue; }
        const int* b0 = colind + rowptr[no[i]];
        const int* b1 = colind + rowptr[no[i] + 1];
        const int* f = std::lower_bound(b0, b1, no[j]);
        if (f == b1 || *f != no[j]) continue;  // Mearge skips blocks outside the pattern
        G.slot_ptr[n + (f - colind) + 1]++;
      }
    }
  }
  for (long long s = 0; s < n + nnz; ++s) G.slot_ptr[s + 1] += G.slot_ptr[s];
  for (int i = 0; i < n; ++i) G.res_ptr[i + 1] += G.res_ptr[i];
  if (G.slot_ptr[n + nnz] > INT32_MAX || (long long)nelem * k * k > INT32_MAX) {
    err = "mesh too large for 32-bit element-block indices";
    return false;
  }
  G.slot_src.assign(G.slot_ptr[n + nnz], 0);
  G.res_src.assign(G.res_ptr[n], 0);
  std::vector<long long> sf(G.slot_ptr.begin(), G.slot_ptr.end() - 1);
  std::vector<long long> rf(G.res_ptr.begin(), G.res_ptr.end() - 1);
  // fill in element order, so each list is sorted by element
  for (int e = 0; e < nelem; ++e) {
    const int* no = conn + (long long)e * k;
    for (int i = 0; i < k; ++i) {
      G.res_src[rf[no[i]]++] = e * k + i;
      for (int j = 0; j < k; ++j) {
        const int blk = (e * k + i) * k + j;
        if (i == j) { G.slot_src[sf[no[i]]++] = blk; continue; }
        const int* b0 = colind + rowptr[no[i]];
        const int* b1 = colind + rowptr[no[i] + 1];
        const int* f = std::lower_bound(b0, b1, no[j]);
        if (f == b1 || *f != no[j]) continue;
        G.slot_src[sf[n + (f - colind)]++] = blk;
      }
    }
  }
  return true;
}

// Schedule for batched launches, where many solves fill the device and a
// CTA's steps are the scarce resource: the fullest steps (rows per step)
// rather than the shortest single-solve makespan.  Candidate ranges hold
// 8, 16 or 32 times the median distance from a row to its farthest dependency
// (a grid line of a structured mesh), so a range spans up to 32 lines and a
// step up to 32 rows; a larger range is taken only when its steps are at
// least 10 % fuller (it also makes the solve's own critical path longer).
SweepPlan fullest_sweep_plan(int n, int b, const int* rowptr, const int* colind, const int* diaind, bool forward,
                             int R) {
  std::vector<int> dist;
  dist.reserve(n);
  for (int i = 0; i < n; ++i) {
    if (forward) {
      if (diaind[i] > rowptr[i]) dist.push_back(i - colind[rowptr[i]]);
    } else {
      if (rowptr[i + 1] > diaind[i]) dist.push_back(colind[rowptr[i + 1] - 1] - i);
    }
  }
  long long D = 1;
  if (!dist.empty()) {
    std::nth_element(dist.begin(), dist.begin() + dist.size() / 2, dist.end());
    D = std::max(1, dist[dist.size() / 2]);
  }
  SweepPlan best;
  double best_fill = -1.0;
  for (int mult : {8, 16, 32}) {
    const int range_rows = (int)std::min<long long>(std::max<long long>(256, mult * D), std::max(n, 1));
    SweepPlan P = build_sweep_plan(n, b, rowptr, colind, diaind, forward, range_rows, R);
    const double fill = P.nsteps ? (double)n / P.nsteps : 0.0;
    if (fill > best_fill * 1.10) {
      best_fill = fill;
      best = std::move(P);
    }
    if (range_rows >= n) break;
  }
  return best;
}

SellMap build_sell(int n, const int* rowptr, const int* colind) {
  SellMap M;
  M.nslices = (n + 31) / 32;
  M.ptr.assign(M.nslices + 1, 0);
  M.width.assign(M.nslices, 0);
  for (int s = 0; s < M.nslices; ++s) {
    int w = 0;
    for (int i = 32 * s; i < std::min(n, 32 * s + 32); ++i) w = std::max(w, rowptr[i + 1] - rowptr[i] + 1);
    M.width[s] = w;
    M.ptr[s + 1] = M.ptr[s] + 32LL * w;
  }
  M.col.assign(M.ptr[M.nslices], 0);
  M.src.assign(M.ptr[M.nslices], -1);
  for (int s = 0; s < M.nslices; ++s)
    for (int lane = 0; lane < 32; ++lane) {
      const int i = 32 * s + lane;
      const long long base = M.ptr[s] + lane;
      if (i >= n) {
        for (int w = 0; w < M.width[s]; ++w) M.col[base + 32LL * w] = 0;  // padding rows read x[0] * 0
        continue;
      }
      const int nb = rowptr[i + 1] - rowptr[i];
      for (int w = 0; w < M.width[s]; ++w) {
        const long long k = base + 32LL * w;
        if (w < nb) {
          M.col[k] = colind[rowptr[i] + w];
          M.src[k] = rowptr[i] + w;
        } else if (w == nb) {
          M.col[k] = i;
          M.src[k] = -2 - i;
        } else {
          M.col[k] = i;
          M.src[k] = -1;
        }
      }
    }
  return M;
}

}  // namespace dfg
