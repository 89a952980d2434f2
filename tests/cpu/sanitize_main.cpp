// sanitize_main.cpp -- TEST INFRASTRUCTURE: the library's host code (the
// pattern, fill-in, level, sweep-schedule, record and gather-map builders of
// delfem_gb300/csrc/sched.cpp and the GiD reader of meshio.cpp) run under
// AddressSanitizer and UndefinedBehaviorSanitizer beside the oracle, on
// small structured, permuted, high-valence and empty meshes.  Built and run
// by tests/test_cpu_sanitizers.py; the sanitizers abort on their first
// report, and every result is also checked against the oracle.  Exit status
// 0 = all checks passed, otherwise the number of the failed check.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "../../delfem_gb300/csrc/dfg_internal.h"
#include "../../oracle/dfg_oracle.h"

using namespace dfg;

extern "C" int emul_sweep(int n, int b, const int* rowptr, const int* colind, int forward, int range_rows, int R,
                          const double* fdiag, const double* foffd, const double* rhs, double* out, long long* info);
extern "C" int emul_level_sweep(int n, int b, const int* rowptr, const int* colind, int forward, const double* fdiag,
                                const double* foffd, const double* in, double* out, long long* info);

// meshio.cpp reports errors through the library's context-free error slot
// (defined in capi.cu, which this program does not link); kept here instead
namespace dfg {
static std::string g_noctx_error;
void set_noctx_error(const std::string& msg) { g_noctx_error = msg; }
}  // namespace dfg

static int g_checks = 0;
static char g_where[96] = "";  // the case being checked, for the failure message
#define CHECK(cond)                                                              \
  do {                                                                           \
    ++g_checks;                                                                  \
    if (!(cond)) {                                                               \
      std::fprintf(stderr, "check %d (%s) failed at line %d: %s\n", g_checks, g_where, __LINE__, #cond); \
      std::exit(g_checks > 250 ? 250 : g_checks);                                \
    }                                                                            \
  } while (0)

struct Mesh {
  int ndim = 2, nnoel = 3, nnode = 0, nelem = 0;
  std::vector<double> coords;
  std::vector<int> conn;
  std::vector<int> boundary;  // 1 on nodes fixed by the load case
};

// (nx x ny) cells, two triangles each, interior nodes jittered; optionally
// the node numbering is a random permutation (irregular bandwidth)
static Mesh tri_grid(int nx, int ny, unsigned seed, bool permute) {
  Mesh m;
  m.nnode = (nx + 1) * (ny + 1);
  std::mt19937 rng(seed);
  std::uniform_real_distribution<double> jit(-0.2, 0.2);
  std::vector<int> perm(m.nnode);
  for (int i = 0; i < m.nnode; ++i) perm[i] = i;
  if (permute) std::shuffle(perm.begin(), perm.end(), rng);
  m.coords.assign((size_t)m.nnode * 2, 0.0);
  m.boundary.assign(m.nnode, 0);
  for (int j = 0; j <= ny; ++j)
    for (int i = 0; i <= nx; ++i) {
      const int v = perm[j * (nx + 1) + i];
      const bool edge = i == 0 || j == 0 || i == nx || j == ny;
      m.coords[v * 2 + 0] = (i + (edge ? 0.0 : jit(rng))) / nx;
      m.coords[v * 2 + 1] = (j + (edge ? 0.0 : jit(rng))) / ny;
      m.boundary[v] = i == 0;  // clamped / Dirichlet on the left side
    }
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      const int a = perm[j * (nx + 1) + i], b = perm[j * (nx + 1) + i + 1];
      const int c = perm[(j + 1) * (nx + 1) + i + 1], d = perm[(j + 1) * (nx + 1) + i];
      const int t[6] = {a, b, c, a, c, d};
      m.conn.insert(m.conn.end(), t, t + 6);
    }
  m.nelem = (int)m.conn.size() / 3;
  return m;
}

// n^3 cells, six tetrahedra each around the (0,0,0)-(1,1,1) diagonal, every
// one oriented positively (TetVolume is signed: a negative one would enter
// the matrix with the wrong sign)
static Mesh tet_grid(int n) {
  Mesh m;
  m.ndim = 3;
  m.nnoel = 4;
  const int s = n + 1;
  m.nnode = s * s * s;
  m.boundary.assign(m.nnode, 0);
  for (int k = 0; k <= n; ++k)
    for (int j = 0; j <= n; ++j)
      for (int i = 0; i <= n; ++i) {
        m.coords.push_back((double)i / n);
        m.coords.push_back((double)j / n);
        m.coords.push_back((double)k / n);
        m.boundary[(k * s + j) * s + i] = k == 0;
      }
  auto id = [&](int i, int j, int k) { return (k * s + j) * s + i; };
  static const int paths[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i)
        for (const auto& p : paths) {
          int c[3] = {i, j, k};
          int t[4];
          t[0] = id(c[0], c[1], c[2]);
          for (int q = 0; q < 3; ++q) {
            ++c[p[q]];
            t[q + 1] = id(c[0], c[1], c[2]);
          }
          double e[3][3];
          for (int q = 0; q < 3; ++q)
            for (int d = 0; d < 3; ++d) e[q][d] = m.coords[(size_t)t[q + 1] * 3 + d] - m.coords[(size_t)t[0] * 3 + d];
          const double vol = e[0][0] * (e[1][1] * e[2][2] - e[1][2] * e[2][1]) -
                             e[0][1] * (e[1][0] * e[2][2] - e[1][2] * e[2][0]) +
                             e[0][2] * (e[1][0] * e[2][1] - e[1][1] * e[2][0]);
          if (vol < 0) std::swap(t[2], t[3]);
          m.conn.insert(m.conn.end(), t, t + 4);
        }
  m.nelem = (int)m.conn.size() / 4;
  return m;
}

// a disc of nfan triangles around node 0 (one node of valence nfan)
static Mesh fan(int nfan) {
  Mesh m;
  m.nnode = nfan + 1;
  m.coords = {0.0, 0.0};
  m.boundary.assign(m.nnode, 1);
  m.boundary[0] = 0;
  for (int i = 0; i < nfan; ++i) {
    const double a = 2.0 * M_PI * i / nfan;
    m.coords.push_back(std::cos(a));
    m.coords.push_back(std::sin(a));
    const int t[3] = {0, 1 + i, 1 + (i + 1) % nfan};
    m.conn.insert(m.conn.end(), t, t + 3);
  }
  m.nelem = nfan;
  return m;
}

static bool close_to(const std::vector<double>& a, const std::vector<double>& r, double rtol) {
  double mx = 0.0, err = 0.0;
  for (size_t i = 0; i < r.size(); ++i) {
    mx = std::max(mx, std::fabs(r[i]));
    err = std::max(err, std::fabs(a[i] - r[i]));
  }
  return a.size() == r.size() && err <= rtol * std::max(mx, 1e-300);
}

// pattern and gather map of a mesh against the oracle's pattern
static void check_pattern(const Mesh& m, std::vector<int>& rp, std::vector<int>& ci) {
  const int n = m.nnode, k = m.nnoel;
  const int* conn = m.conn.empty() ? nullptr : m.conn.data();
  pattern_from_elements(n, m.nelem, k, conn, rp, ci);
  CHECK((int)rp.size() == n + 1 && rp[n] == (int)ci.size());
  const long nz = dfo_pattern(n, m.nelem, k, conn, nullptr, nullptr);
  CHECK(nz == (long)ci.size());
  std::vector<int> orp(n + 1), oci(std::max<long>(nz, 1));
  CHECK(dfo_pattern(n, m.nelem, k, conn, orp.data(), oci.data()) == nz);
  CHECK(std::equal(rp.begin(), rp.end(), orp.begin()) && std::equal(ci.begin(), ci.end(), oci.begin()));
  GatherMap G;
  std::string err;
  const int* cc = ci.empty() ? rp.data() : ci.data();
  CHECK(build_gather_map(n, rp.data(), cc, m.nelem, k, conn, G, err));
  const size_t nslot = (size_t)n + ci.size();
  CHECK(G.slot_ptr.size() == nslot + 1 && G.slot_ptr[nslot] == (long long)m.nelem * k * k);
  CHECK(G.res_ptr.size() == (size_t)n + 1 && G.res_ptr[n] == (long long)m.nelem * k);
  std::vector<int> seen((size_t)m.nelem * k * k, 0);
  std::vector<int> row_of(ci.size());
  for (int i = 0; i < n; ++i)
    for (int c = rp[i]; c < rp[i + 1]; ++c) row_of[c] = i;
  for (size_t s = 0; s < nslot; ++s) {
    int last_e = -1;
    for (long long q = G.slot_ptr[s]; q < G.slot_ptr[s + 1]; ++q) {
      const int src = G.slot_src[q];
      CHECK(src >= 0 && src < (int)seen.size());
      ++seen[src];
      const int e = src / (k * k), i = (src / k) % k, j = src % k;
      CHECK(e >= last_e);  // element order, as Mearge adds them
      last_e = e;
      const int gi = m.conn[(size_t)e * k + i], gj = m.conn[(size_t)e * k + j];
      if (s < (size_t)n) CHECK(gi == (int)s && gj == (int)s);
      else CHECK(gi == row_of[s - n] && gj == ci[s - n]);
    }
  }
  for (int c : seen) CHECK(c == 1);
  for (int i = 0; i < n; ++i)
    for (long long q = G.res_ptr[i]; q < G.res_ptr[i + 1]; ++q) CHECK(m.conn[G.res_src[q]] == i);
}

// records of every candidate plan: sizes, headers and code offsets in bounds
static void check_records(int n, int b, const int* rp, const int* ci, const int* dia) {
  for (int fwd = 0; fwd < 2; ++fwd) {
    const std::vector<SweepPlan> plans = candidate_sweep_plans(n, b, rp, ci, dia, fwd != 0, 32, 3);
    for (const SweepPlan& P : plans) {
      CHECK((int)P.range_steps.size() == P.nranges + 1 && P.range_steps[P.nranges] == P.nsteps);
      for (int elem : {4, 8}) {
        std::vector<long long> off;
        long long max_rec = 0;
        const std::vector<unsigned char> h = pack_record_headers(P, elem, off, max_rec);
        CHECK((int)off.size() == P.nsteps + 1 && (long long)h.size() == off[P.nsteps]);
        const long long ring_end = 32 + (long long)P.R * 32 * b * elem;
        for (int s = 0; s < P.nsteps; ++s) {
          int nent = -1;
          std::memcpy(&nent, h.data() + off[s], 4);
          CHECK(nent == P.step_nent[s] && off[s + 1] - off[s] <= max_rec);
          const int* code = reinterpret_cast<const int*>(h.data() + off[s] + 144);
          const int* grow = code + nent * 32;
          for (int q = 0; q < nent * 32; ++q) {
            const unsigned c = (unsigned)code[q];
            if (c & 0x80000000u) CHECK(grow[q] >= 0 && grow[q] < n);
            else CHECK(grow[q] == -1 && (long long)c < ring_end);
          }
        }
      }
    }
  }
}

// kind: 1 Poisson 2D, 2 Poisson 3D, 4 solid 2D, 5 solid 3D (the oracle's
// assembly); then every fill level, both sweep schedules against the oracle's
// substitutions, the step records, and with each factor PCG (solve >= 1) and
// BiCGSTAB (solve >= 2)
static void check_case(const Mesh& m, int kind, int b, int solve) {
  std::vector<int> rp, ci;
  check_pattern(m, rp, ci);
  const int n = m.nnode;
  const size_t bs = (size_t)b * b, nnz = ci.size();
  const int* cci = ci.empty() ? rp.data() : ci.data();
  std::vector<double> diag(n * bs), offd(std::max<size_t>(nnz, 1) * bs), res((size_t)n * b);
  std::vector<double> coef(m.nelem);
  std::mt19937 rng(7 + kind);
  std::lognormal_distribution<double> ln(0.0, 0.5);
  for (double& c : coef) c = ln(rng);
  const double E = 1.0, nu = 0.3, lam = E * nu / ((1 + nu) * (1 - 2 * nu)), myu = E / (2 * (1 + nu));
  int rc = -1;
  const int* conn = m.conn.data();
  const double* xy = m.coords.data();
  if (kind == 1) rc = dfo_assemble_poisson2d(n, rp.data(), cci, m.nelem, conn, xy, coef.data(), 1.0, 1.0, nullptr, diag.data(), offd.data(), res.data());
  if (kind == 2) rc = dfo_assemble_poisson3d(n, rp.data(), cci, m.nelem, conn, xy, coef.data(), 1.0, 1.0, nullptr, diag.data(), offd.data(), res.data());
  if (kind == 4) rc = dfo_assemble_solid2d(n, rp.data(), cci, m.nelem, conn, xy, coef.data(), lam, myu, 1.0, 0.0, -1e-3, nullptr, diag.data(), offd.data(), res.data());
  if (kind == 5) rc = dfo_assemble_solid3d(n, rp.data(), cci, m.nelem, conn, xy, coef.data(), lam, myu, 1.0, 0.0, 0.0, -1e-3, nullptr, diag.data(), offd.data(), res.data());
  CHECK(rc == 0);
  std::vector<int> flag((size_t)n * b);
  for (int i = 0; i < n; ++i)
    for (int d = 0; d < b; ++d) flag[(size_t)i * b + d] = m.boundary[i];
  const double norm = dfo_finalize(n, b, rp.data(), cci, flag.data(), diag.data(), offd.data(), res.data());
  CHECK(norm > 0.0);
  for (int lev : {0, 1, 2, -1}) {
    std::snprintf(g_where, sizeof g_where, "kind %d, b %d, %d nodes, fill level %d", kind, b, n, lev);
    std::vector<int> frp, fci;
    CHECK(ilu_fill_pattern(n, rp.data(), cci, lev, frp, fci, 1LL << 40));
    const long fnz = dfo_ilu_pattern(n, rp.data(), cci, lev, nullptr, nullptr, 0);
    CHECK(fnz == (long)fci.size());
    std::vector<int> orf(n + 1), ocf(std::max<long>(fnz, 1));
    CHECK(dfo_ilu_pattern(n, rp.data(), cci, lev, orf.data(), ocf.data(), fnz) == fnz);
    CHECK(std::equal(frp.begin(), frp.end(), orf.begin()) && std::equal(fci.begin(), fci.end(), ocf.begin()));
    const int* fcc = fci.empty() ? frp.data() : fci.data();
    std::vector<int> a2f;
    CHECK(factor_slot_map(n, rp.data(), cci, frp.data(), fcc, a2f));
    CHECK(a2f.size() == nnz);
    for (size_t c = 0; c < nnz; ++c) CHECK(a2f[c] >= 0 && a2f[c] < fnz && fci[a2f[c]] == ci[c]);
    std::vector<double> fdiag(n * bs), foffd(std::max<long>(fnz, 1) * bs);
    CHECK(dfo_ilu_init(n, b, rp.data(), cci, diag.data(), offd.data(), frp.data(), fcc, fdiag.data(), foffd.data()) == 0);
    std::vector<int> fdi(n);
    dfo_diaind(n, frp.data(), fcc, fdi.data());
    CHECK(dfo_ilu0(n, b, frp.data(), fcc, fdi.data(), fdiag.data(), foffd.data()) >= 0);
    std::vector<double> rhs((size_t)n * b), yref, zref;
    std::normal_distribution<double> nd;
    for (double& v : rhs) v = nd(rng);
    yref = rhs;
    dfo_forward(n, b, frp.data(), fcc, fdi.data(), fdiag.data(), foffd.data(), yref.data());
    zref = yref;
    dfo_backward(n, b, frp.data(), fcc, fdi.data(), foffd.data(), zref.data());
    long long info[8];
    std::vector<double> y((size_t)n * b), z((size_t)n * b);
    for (int range_rows : {-1, 0, 1, 37, 256})
      for (int R : {2, 32}) {
        CHECK(emul_sweep(n, b, frp.data(), fcc, 1, range_rows, R, fdiag.data(), foffd.data(), rhs.data(), y.data(), info) == 0);
        CHECK(emul_sweep(n, b, frp.data(), fcc, 0, range_rows, R, fdiag.data(), foffd.data(), y.data(), z.data(), info) == 0);
        CHECK(close_to(y, yref, 1e-11) && close_to(z, zref, 1e-11));
      }
    CHECK(emul_level_sweep(n, b, frp.data(), fcc, 1, fdiag.data(), foffd.data(), rhs.data(), y.data(), info) == 0);
    CHECK(emul_level_sweep(n, b, frp.data(), fcc, 0, fdiag.data(), foffd.data(), y.data(), z.data(), info) == 0);
    CHECK(close_to(y, yref, 1e-11) && close_to(z, zref, 1e-11));
    check_records(n, b, frp.data(), fcc, fdi.data());
    if (solve < 1) continue;
    std::vector<double> r = res, x((size_t)n * b), work((size_t)7 * n * b);
    double conv = 1e-8;
    unsigned it = 20000;
    CHECK(dfo_pcg_f(n, b, rp.data(), cci, diag.data(), offd.data(), frp.data(), fcc, fdi.data(), fdiag.data(),
                    foffd.data(), r.data(), x.data(), &conv, &it, work.data()) == 1);
    if (solve < 2) continue;
    r = res;
    conv = 1e-8;
    it = 20000;
    const int ok = dfo_bicgstab(n, b, rp.data(), cci, diag.data(), offd.data(), frp.data(), fcc, fdi.data(),
                                fdiag.data(), foffd.data(), r.data(), x.data(), &conv, &it, work.data());
    if (!ok) std::fprintf(stderr, "bicgstab: conv %g after %u\n", conv, it);
    CHECK(ok == 1);
  }
}

// pattern, fill-in, levels and schedules of a matrix without elements (no
// off-diagonal blocks) and of an empty one
static void check_degenerate() {
  for (int n : {0, 1, 40}) {
    Mesh m;
    m.nnode = n;
    std::vector<int> rp, ci;
    check_pattern(m, rp, ci);
    CHECK(ci.empty());
    std::vector<int> frp, fci;
    CHECK(ilu_fill_pattern(n, rp.data(), rp.data(), 1, frp, fci, 1LL << 40) && fci.empty());
    std::vector<int> dia(n);
    for (int i = 0; i < n; ++i) dia[i] = rp[i];
    for (int fwd = 0; fwd < 2; ++fwd) {
      const Levels V = build_levels(n, rp.data(), rp.data(), dia.data(), fwd != 0);
      CHECK((int)V.ptr.size() == (n ? 2 : 1) && (int)V.rows.size() == n);
    }
    if (n) check_records(n, 2, rp.data(), rp.data(), dia.data());
    std::vector<double> fdiag((size_t)std::max(n, 1) * 4, 0.5), foffd(4, 0.0), in((size_t)std::max(n, 1) * 2, 1.0),
        out(in.size());
    long long info[8];
    CHECK(emul_level_sweep(n, 2, rp.data(), rp.data(), 1, fdiag.data(), foffd.data(), in.data(), out.data(), info) == 0);
    if (n) CHECK(emul_sweep(n, 2, rp.data(), rp.data(), 1, 0, 32, fdiag.data(), foffd.data(), in.data(), out.data(), info) == 0);
  }
}

static std::string write_file(const std::string& dir, const char* name, const std::string& text) {
  const std::string p = dir + "/" + name;
  FILE* f = std::fopen(p.c_str(), "w");
  CHECK(f != nullptr);
  std::fputs(text.c_str(), f);
  std::fclose(f);
  return p;
}

// the GiD reader on a planar triangle mesh, a tetrahedron mesh and malformed files
static void check_meshio(const std::string& dir) {
  const std::string head = "MESH    dimension 3 ElemType ";
  const std::string tri = write_file(dir, "tri.msh", head + "Triangle  Nnode 3\nCoordinates\n"
      "1 0 0 0.5\n2 1 0 0.5\n3 1 1 0.5\n4 0 1 0.5\nend coordinates\n\nElements\n1 1 2 3\n2 1 3 4\nend elements\n");
  int ndim = 0, nnoel = 0, nnode = 0, nelem = 0;
  CHECK(dfg_mesh_read_gid(tri.c_str(), &ndim, &nnoel, &nnode, &nelem, nullptr, nullptr) == DFG_OK);
  CHECK(ndim == 2 && nnoel == 3 && nnode == 4 && nelem == 2);
  std::vector<double> co(8);
  std::vector<int> cn(6);
  CHECK(dfg_mesh_read_gid(tri.c_str(), &ndim, &nnoel, &nnode, &nelem, co.data(), cn.data()) == DFG_OK);
  CHECK(cn == std::vector<int>({0, 1, 2, 0, 2, 3}));
  CHECK(co == std::vector<double>({0, 0, 1, 0, 1, 1, 0, 1}));  // z (no variance) dropped, x and y kept
  const std::string tet = write_file(dir, "tet.msh", head + "Tetrahedra  Nnode 4\nCoordinates\n"
      "1 0 0 0\n2 1 0 0\n3 0 1 0\n4 0 0 1\n5 1 1 1\nend coordinates\n\nElements\n1 1 2 3 4\n2 2 3 4 5\nend elements\n");
  CHECK(dfg_mesh_read_gid(tet.c_str(), &ndim, &nnoel, &nnode, &nelem, nullptr, nullptr) == DFG_OK);
  CHECK(ndim == 3 && nnoel == 4 && nnode == 5 && nelem == 2);
  std::vector<double> c3(15);
  std::vector<int> n3(8);
  CHECK(dfg_mesh_read_gid(tet.c_str(), &ndim, &nnoel, &nnode, &nelem, c3.data(), n3.data()) == DFG_OK);
  CHECK(n3 == std::vector<int>({0, 1, 2, 3, 1, 2, 3, 4}) && c3[12] == 1.0 && c3[14] == 1.0);
  const char* bad[] = {
      "",
      "MESH    dimension 3 ElemType Quadrilateral  Nnode 4\nCoordinates\nend coordinates\n",
      "MESH    dimension 3 ElemType Triangle  Nnode 3\nCoordinates\n1 0 0 0\n2 1 0",
      "MESH    dimension 3 ElemType Triangle  Nnode 3\nCoordinates\n1 0 0 0\n3 1 0 0\nend coordinates\n",
      "MESH    dimension 3 ElemType Triangle  Nnode 3\nCoordinates\n1 0 0 0\n2 1 0 0\n3 0 1 0\nend coordinates\n"
      "\nElements\n1 1 2 9\nend elements\n",
      "MESH    dimension 3 ElemType Tetrahedra  Nnode 4\nCoordinates\n1 0 0 0\n2 1 0 0\n3 0 1 0\n4 0 0 1\n"
      "end coordinates\n\nElements\n1 1 2 3\n",
  };
  for (const char* text : bad) {
    const std::string p = write_file(dir, "bad.msh", text);
    dfg::g_noctx_error.clear();
    CHECK(dfg_mesh_read_gid(p.c_str(), &ndim, &nnoel, &nnode, &nelem, nullptr, nullptr) != DFG_OK);
    CHECK(!dfg::g_noctx_error.empty());
  }
  CHECK(dfg_mesh_read_gid((dir + "/missing.msh").c_str(), &ndim, &nnoel, &nnode, &nelem, nullptr, nullptr) != DFG_OK);
}

int main(int argc, char** argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: %s <scratch directory>\n", argv[0]);
    return 2;
  }
  check_degenerate();
  check_case(tri_grid(9, 6, 1, false), 1, 1, 2);
  check_case(tri_grid(9, 6, 2, true), 4, 2, 2);
  check_case(tri_grid(40, 3, 3, false), 4, 2, 0);
  check_case(tet_grid(3), 2, 1, 2);
  check_case(tet_grid(3), 5, 3, 2);
  // one free unknown: BiCGSTAB's half step solves it exactly, s = 0 and
  // omega = 0/0 (the reference's loop has no guard), so PCG only
  check_case(fan(40), 1, 1, 1);
  check_meshio(argv[1]);
  std::printf("%d checks passed\n", g_checks);
  return 0;
}
