// ref_harness.cpp -- drives the reference DelFEM code (compiled headless from
// its own sources by oracle/Makefile into oracle/_ref/) on one problem file
// and dumps every intermediate of the hot path.  TEST INFRASTRUCTURE ONLY:
// it is how the golden fixtures in tests/golden/ are produced and how the
// C restatement in dfg_oracle.c is pinned.  It follows the low-level driver
// flow of test_glut_lowlev/solid2d/main.cpp:186-298:
//   IMesh -> CFieldWorld::AddMesh -> MakeField_FieldElemDim ->
//   CLinearSystem_Field::AddPattern_Field -> BC flags -> InitializeMarge ->
//   AddLinSys_* (or the per-element-coefficient restatement feeding the
//   reference's own Mearge) -> extra loads -> FinalizeMarge ->
//   CPreconditioner_ILU(fill level, 0 by default) -> LsSol::Solve_PCG.
//
// Usage: ref_harness problem.bin out.bin [fill_level [pcg|bicgstab]]
// (the solver is LsSol::Solve_PCG by default, LsSol::Solve_PBiCGSTAB on request)
//        ref_harness --mesh2d|--mesh3d file.msh out.bin
// (loads a GiD mesh file with the reference's reader, Msh::CMesher2D or
// Msh::CMesh3D ::ReadFromFile_GiDMsh, and dumps the nodes and elements:
// int32 magic 0x44464D31, ndim, nnoel, nnode, nelem; f64 coords; i32 conn)
// Input / output formats are described in tests/golden/make_golden.py.
#include <cassert>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "delfem/mesh_interface.h"
#include "delfem/field_world.h"
#include "delfem/field.h"
#include "delfem/femls/linearsystem_field.h"
#include "delfem/ls/preconditioner.h"
#include "delfem/ls/solver_ls_iter.h"
#include "delfem/matvec/matdia_blkcrs.h"
#include "delfem/matvec/matdiafrac_blkcrs.h"
#include "delfem/matvec/vector_blk.h"
#include "delfem/matvec/bcflag_blk.h"
#include "delfem/femeqn/eqn_poisson.h"
#include "delfem/femeqn/eqn_diffusion.h"
#include "delfem/femeqn/eqn_linear_solid2d.h"
#include "delfem/femeqn/eqn_linear_solid3d.h"
#include "delfem/femeqn/ker_emat_tri.h"
#include "delfem/femeqn/ker_emat_tet.h"
#include "delfem/mesher2d.h"
#include "delfem/mesh3d.h"

using namespace Fem::Field;

enum { K_POISSON2D = 1, K_POISSON3D = 2, K_DIFFUSION2D = 3, K_SOLID2D = 4, K_SOLID3D = 5 };

struct Problem {
  int kind, nnode, ndim, nelem, nnoel, b;
  std::vector<double> coords, coef, load, u, v;
  std::vector<int> conn, bcflag;
  double prm[8];
  double tol;
  int maxit;
};

class GridMesh : public Msh::IMesh {
 public:
  explicit GridMesh(const Problem& p) : p_(p) {}
  unsigned int GetDimention() const { return p_.ndim; }
  void GetInfo(unsigned int, unsigned int& id_cad, unsigned int& id_msh_before_ext,
               unsigned int& inum_ext, int& ilayer) const {
    id_cad = 1; id_msh_before_ext = 0; inum_ext = 0; ilayer = 0;
  }
  void GetCoord(std::vector<double>& coord) const { coord = p_.coords; }
  Msh::MSH_TYPE GetConnectivity(unsigned int, std::vector<int>& lnods) const {
    lnods = p_.conn;
    return p_.ndim == 2 ? Msh::TRI : Msh::TET;
  }
  std::vector<unsigned int> GetAry_ID() const { return std::vector<unsigned int>(1, 1u); }
  std::vector<unsigned int> GetIncludeElemIDAry(unsigned int) const { return std::vector<unsigned int>(); }
 private:
  const Problem& p_;
};

static void rd(FILE* f, void* p, size_t n) {
  if (n && fread(p, 1, n, f) != n) { fprintf(stderr, "short read\n"); exit(2); }
}
static int rdi(FILE* f) { int v; rd(f, &v, 4); return v; }

static Problem load(const char* path) {
  FILE* f = fopen(path, "rb");
  if (!f) { perror(path); exit(2); }
  Problem p;
  if (rdi(f) != 0x44464731) { fprintf(stderr, "bad magic\n"); exit(2); }
  p.kind = rdi(f); p.nnode = rdi(f); p.ndim = rdi(f); p.nelem = rdi(f); p.nnoel = rdi(f); p.b = rdi(f);
  p.coords.resize((size_t)p.nnode * p.ndim); rd(f, p.coords.data(), p.coords.size() * 8);
  p.conn.resize((size_t)p.nelem * p.nnoel); rd(f, p.conn.data(), p.conn.size() * 4);
  if (rdi(f)) { p.coef.resize(p.nelem); rd(f, p.coef.data(), p.coef.size() * 8); }
  rd(f, p.prm, sizeof(p.prm));
  p.bcflag.resize((size_t)p.nnode * p.b); rd(f, p.bcflag.data(), p.bcflag.size() * 4);
  if (rdi(f)) { p.load.resize((size_t)p.nnode * p.b); rd(f, p.load.data(), p.load.size() * 8); }
  if (rdi(f)) { p.u.resize((size_t)p.nnode * p.b); rd(f, p.u.data(), p.u.size() * 8); }
  if (rdi(f)) { p.v.resize((size_t)p.nnode * p.b); rd(f, p.v.data(), p.v.size() * 8); }
  rd(f, &p.tol, 8); p.maxit = rdi(f);
  fclose(f);
  return p;
}

// Per-element-coefficient restatement of the reference element loops; the
// emat expressions are the reference's (eqn_poisson.cpp:99-119,
// eqn_linear_solid2d.cpp:565-591, eqn_linear_solid3d.cpp:297-325) with
// alpha / lambda / myu scaled per element; the scatter is the reference's own
// CMatDia_BlkCrs::Mearge and CVector_Blk::AddValue.
static void assemble_coef(const Problem& p, MatVec::CMatDia_BlkCrs& A, MatVec::CVector_Blk& r) {
  const double* P = p.prm;
  for (int e = 0; e < p.nelem; ++e) {
    const double m = p.coef[e];
    unsigned int no[4];
    for (int k = 0; k < p.nnoel; ++k) no[k] = (unsigned)p.conn[(size_t)e * p.nnoel + k];
    if (p.kind == K_POISSON2D) {
      const double alpha = P[0] * m, source = P[1];
      double c[3][2], val[3];
      for (int k = 0; k < 3; ++k) {
        c[k][0] = p.coords[no[k] * 2]; c[k][1] = p.coords[no[k] * 2 + 1];
        val[k] = p.u.empty() ? 0.0 : p.u[no[k]];
      }
      const double area = TriArea(c[0], c[1], c[2]);
      double dldx[3][2], ct[3];
      TriDlDx(dldx, ct, c[0], c[1], c[2]);
      double emat[3][3], eres[3];
      for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j)
        emat[i][j] = alpha * area * (dldx[i][0] * dldx[j][0] + dldx[i][1] * dldx[j][1]);
      for (int i = 0; i < 3; ++i) eres[i] = source * area * 0.33333333333333333;
      for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) eres[i] -= emat[i][j] * val[j];
      A.Mearge(3, no, 3, no, 1, &emat[0][0]);
      for (int i = 0; i < 3; ++i) r.AddValue(no[i], 0, eres[i]);
    } else if (p.kind == K_POISSON3D) {
      const double alpha = P[0] * m, source = P[1];
      double c[4][3], val[4];
      for (int k = 0; k < 4; ++k) {
        for (int a = 0; a < 3; ++a) c[k][a] = p.coords[no[k] * 3 + a];
        val[k] = p.u.empty() ? 0.0 : p.u[no[k]];
      }
      const double vol = TetVolume(c[0], c[1], c[2], c[3]);
      double dldx[4][3], ct[4];
      TetDlDx(dldx, ct, c[0], c[1], c[2], c[3]);
      double emat[4][4], eres[4];
      for (int i = 0; i < 4; ++i) for (int j = 0; j < 4; ++j)
        emat[i][j] = alpha * vol * (dldx[i][0] * dldx[j][0] + dldx[i][1] * dldx[j][1] + dldx[i][2] * dldx[j][2]);
      for (int i = 0; i < 4; ++i) eres[i] = source * vol * 0.25;
      for (int i = 0; i < 4; ++i) for (int j = 0; j < 4; ++j) eres[i] -= emat[i][j] * val[j];
      A.Mearge(4, no, 4, no, 1, &emat[0][0]);
      for (int i = 0; i < 4; ++i) r.AddValue(no[i], 0, eres[i]);
    } else if (p.kind == K_SOLID2D) {
      const double lambda = P[0] * m, myu = P[1] * m, rho = P[2], g_x = P[3], g_y = P[4];
      double c[3][2], disp[3][2];
      for (int k = 0; k < 3; ++k)
        for (int a = 0; a < 2; ++a) {
          c[k][a] = p.coords[no[k] * 2 + a];
          disp[k][a] = p.u.empty() ? 0.0 : p.u[no[k] * 2 + a];
        }
      const double area = TriArea(c[0], c[1], c[2]);
      double dldx[3][2], ct[3];
      TriDlDx(dldx, ct, c[0], c[1], c[2]);
      double emat[3][3][2][2], eres[3][2];
      for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) {
        emat[i][j][0][0] = area * (lambda + myu) * dldx[i][0] * dldx[j][0];
        emat[i][j][0][1] = area * (lambda * dldx[i][0] * dldx[j][1] + myu * dldx[j][0] * dldx[i][1]);
        emat[i][j][1][0] = area * (lambda * dldx[i][1] * dldx[j][0] + myu * dldx[j][1] * dldx[i][0]);
        emat[i][j][1][1] = area * (lambda + myu) * dldx[i][1] * dldx[j][1];
        const double dtmp1 = (dldx[i][1] * dldx[j][1] + dldx[i][0] * dldx[j][0]) * area * myu;
        emat[i][j][0][0] += dtmp1;
        emat[i][j][1][1] += dtmp1;
      }
      for (int i = 0; i < 3; ++i) {
        eres[i][0] = area * rho * g_x * 0.33333333333333333;
        eres[i][1] = area * rho * g_y * 0.33333333333333333;
      }
      for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) {
        eres[i][0] -= emat[i][j][0][0] * disp[j][0] + emat[i][j][0][1] * disp[j][1];
        eres[i][1] -= emat[i][j][1][0] * disp[j][0] + emat[i][j][1][1] * disp[j][1];
      }
      A.Mearge(3, no, 3, no, 4, &emat[0][0][0][0]);
      for (int i = 0; i < 3; ++i) { r.AddValue(no[i], 0, eres[i][0]); r.AddValue(no[i], 1, eres[i][1]); }
    } else if (p.kind == K_SOLID3D) {
      const double lambda = P[0] * m, myu = P[1] * m, rho = P[2], g_x = P[3], g_y = P[4], g_z = P[5];
      double c[4][3], disp[4][3];
      for (int k = 0; k < 4; ++k)
        for (int a = 0; a < 3; ++a) {
          c[k][a] = p.coords[no[k] * 3 + a];
          disp[k][a] = p.u.empty() ? 0.0 : p.u[no[k] * 3 + a];
        }
      const double vol = TetVolume(c[0], c[1], c[2], c[3]);
      double dldx[4][3], ct[4];
      TetDlDx(dldx, ct, c[0], c[1], c[2], c[3]);
      double emat[4][4][3][3], eres[4][3];
      for (int i = 0; i < 4; ++i) for (int j = 0; j < 4; ++j) {
        for (int a = 0; a < 3; ++a) for (int q = 0; q < 3; ++q)
          emat[i][j][a][q] = vol * (lambda * dldx[i][a] * dldx[j][q] + myu * dldx[j][a] * dldx[i][q]);
        const double dtmp1 = dldx[i][0] * dldx[j][0] + dldx[i][1] * dldx[j][1] + dldx[i][2] * dldx[j][2];
        emat[i][j][0][0] += vol * myu * dtmp1;
        emat[i][j][1][1] += vol * myu * dtmp1;
        emat[i][j][2][2] += vol * myu * dtmp1;
      }
      for (int i = 0; i < 4; ++i) {
        eres[i][0] = vol * rho * g_x * 0.25;
        eres[i][1] = vol * rho * g_y * 0.25;
        eres[i][2] = vol * rho * g_z * 0.25;
        for (int j = 0; j < 4; ++j)
          for (int a = 0; a < 3; ++a)
            eres[i][a] -= emat[i][j][a][0] * disp[j][0] + emat[i][j][a][1] * disp[j][1] + emat[i][j][a][2] * disp[j][2];
      }
      A.Mearge(4, no, 4, no, 9, &emat[0][0][0][0]);
      for (int i = 0; i < 4; ++i) for (int a = 0; a < 3; ++a) r.AddValue(no[i], a, eres[i][a]);
    } else {
      fprintf(stderr, "per-element coefficients not supported for kind %d\n", p.kind);
      exit(2);
    }
  }
}

static void wr(FILE* f, const void* p, size_t n) { if (n) fwrite(p, 1, n, f); }
static void wri(FILE* f, int v) { wr(f, &v, 4); }

static int dump_mesh(const char* kind, const char* in, const char* out) {
  std::vector<double> co;
  std::vector<int> cn;
  int ndim = 0, nnoel = 0;
  if (strcmp(kind, "--mesh2d") == 0) {
    Msh::CMesher2D m;
    if (!m.ReadFromFile_GiDMsh(in)) return 3;
    for (const Com::CVector2D& v : m.GetVectorAry()) { co.push_back(v.x); co.push_back(v.y); }
    for (const Msh::CTriAry2D& a : m.GetTriArySet())
      for (const Msh::STri2D& t : a.m_aTri) for (int k = 0; k < 3; ++k) cn.push_back((int)t.v[k]);
    ndim = 2; nnoel = 3;
  } else {
    Msh::CMesh3D m;
    if (!m.ReadFromFile_GiDMsh(in)) return 3;
    for (const Com::CVector3D& v : m.GetVectorAry()) { co.push_back(v.x); co.push_back(v.y); co.push_back(v.z); }
    for (const Msh::CTetAry& a : m.GetTetArySet())
      for (const Msh::STet& t : a.m_aTet) for (int k = 0; k < 4; ++k) cn.push_back((int)t.v[k]);
    ndim = 3; nnoel = 4;
  }
  FILE* f = fopen(out, "wb");
  if (!f) return 2;
  const int hdr[5] = {0x44464D31, ndim, nnoel, (int)(co.size() / ndim), (int)(cn.size() / nnoel)};
  fwrite(hdr, 4, 5, f);
  fwrite(co.data(), 8, co.size(), f);
  fwrite(cn.data(), 4, cn.size(), f);
  fclose(f);
  return 0;
}

int main(int argc, char** argv) {
  if (argc == 4 && strncmp(argv[1], "--mesh", 6) == 0) return dump_mesh(argv[1], argv[2], argv[3]);
  if (argc < 3 || argc > 5) {
    fprintf(stderr, "usage: %s problem.bin out.bin [fill_level [pcg|bicgstab]]\n", argv[0]);
    return 2;
  }
  Problem p = load(argv[1]);
  const int fill_level = argc >= 4 ? atoi(argv[3]) : 0;
  const bool bicgstab = argc == 5 && strcmp(argv[4], "bicgstab") == 0;
  const int b = p.b;
  CFieldWorld world;
  GridMesh mesh(p);
  const unsigned int id_base = world.AddMesh(mesh);
  FIELD_TYPE ft = (b == 1) ? SCALAR : (b == 2 ? VECTOR2 : VECTOR3);
  const int deriv = (p.kind == K_DIFFUSION2D) ? (VALUE | VELOCITY) : VALUE;
  const unsigned int id_field = world.MakeField_FieldElemDim(id_base, p.ndim, ft, deriv, CORNER);
  if (!p.u.empty()) {
    CNodeAry::CNodeSeg& ns = world.GetField(id_field).GetNodeSeg(CORNER, true, world, VALUE);
    for (int i = 0; i < p.nnode; ++i) for (int d = 0; d < b; ++d) ns.SetValue(i, d, p.u[(size_t)i * b + d]);
  }
  if (!p.v.empty()) {
    CNodeAry::CNodeSeg& ns = world.GetField(id_field).GetNodeSeg(CORNER, true, world, VELOCITY);
    for (int i = 0; i < p.nnode; ++i) for (int d = 0; d < b; ++d) ns.SetValue(i, d, p.v[(size_t)i * b + d]);
  }
  Fem::Ls::CLinearSystem_Field ls;
  ls.AddPattern_Field(id_field, world);
  {
    MatVec::CBCFlag& bc = ls.m_ls.GetBCFlag(0);
    for (int i = 0; i < p.nnode; ++i)
      for (int d = 0; d < b; ++d)
        if (p.bcflag[(size_t)i * b + d]) bc.SetBC(i, d);
  }
  LsSol::CPreconditioner_ILU prec;
  prec.SetFillInLevel(fill_level);
  prec.SetLinearSystem(ls.m_ls);

  ls.InitializeMarge();
  MatVec::CMatDia_BlkCrs& A = ls.GetMatrix(id_field, CORNER, world);
  MatVec::CVector_Blk& res = ls.GetResidual(id_field, CORNER, world);
  const double* P = p.prm;
  if (!p.coef.empty()) {
    assemble_coef(p, A, res);
  } else if (p.kind == K_POISSON2D || p.kind == K_POISSON3D) {
    Fem::Eqn::AddLinSys_Poisson(ls, P[0], P[1], world, id_field);
  } else if (p.kind == K_DIFFUSION2D) {
    // AddLinSys_Diffusion(dt, gamma, ls, rho, alpha, source, world, id_field)
    Fem::Eqn::AddLinSys_Diffusion(P[4], P[3], ls, P[0], P[1], P[2], world, id_field);
  } else if (p.kind == K_SOLID2D) {
    Fem::Eqn::AddLinSys_LinearSolid2D_Static(ls, P[0], P[1], P[2], P[3], P[4], world, id_field);
  } else if (p.kind == K_SOLID3D) {
    Fem::Eqn::AddLinSys_LinearSolid3D_Static(ls, P[0], P[1], P[2], P[3], P[4], P[5], world, id_field);
  }
  if (!p.load.empty())
    for (int i = 0; i < p.nnode; ++i)
      for (int d = 0; d < b; ++d) res.AddValue(i, d, p.load[(size_t)i * b + d]);
  const double norm_res = ls.FinalizeMarge();

  const int n = p.nnode, bs = b * b;
  std::vector<int> rowptr(n + 1, 0), colind;
  std::vector<double> diag((size_t)n * bs), offd, rhs((size_t)n * b);
  for (int i = 0; i < n; ++i) {
    unsigned int np = 0;
    const unsigned int* ci = A.GetPtrIndPSuP(i, np);
    const double* cv = A.GetPtrValPSuP(i, np);
    for (unsigned k = 0; k < np; ++k) {
      colind.push_back((int)ci[k]);
      for (int q = 0; q < bs; ++q) offd.push_back(cv[k * bs + q]);
    }
    rowptr[i + 1] = (int)colind.size();
    const double* dv = A.GetPtrValDia(i);
    for (int q = 0; q < bs; ++q) diag[(size_t)i * bs + q] = dv[q];
    for (int d = 0; d < b; ++d) rhs[(size_t)i * b + d] = res.GetValue(i, d);
  }
  // ILU factor, computed through the same calls the preconditioner makes for
  // one segment: the level-0 copy of the pattern, then for a non-zero level
  // AddFracPtn + MakePatternFinalize (preconditioner.cpp:96-157), then
  // SetValue_Initialize + DoILUDecomp (preconditioner.cpp:229-272).
  MatVec::CMatDiaFrac_BlkCrs frac(0, A);
  if (fill_level != 0) {
    frac.AddFracPtn(fill_level);
    frac.MakePatternFinalize();
  }
  frac.SetValue_Initialize(A);
  const bool ilu_ok = frac.DoILUDecomp();
  std::vector<int> rowptr_f(n + 1, 0), colind_f;
  for (int i = 0; i < n; ++i) {
    unsigned int np = 0;
    const unsigned int* ci = frac.GetPtrIndPSuP(i, np);
    for (unsigned k = 0; k < np; ++k) colind_f.push_back((int)ci[k]);
    rowptr_f[i + 1] = (int)colind_f.size();
  }
  const int nnz_f = rowptr_f[n];
  std::vector<double> fdiag((size_t)n * bs), foffd((size_t)nnz_f * bs);
  for (int i = 0; i < n; ++i) {
    const double* dv = frac.GetValDiaPtr(i);
    for (int q = 0; q < bs; ++q) fdiag[(size_t)i * bs + q] = dv[q];
  }
  for (int c = 0; c < nnz_f; ++c) {
    const double* cv = frac.GetValCrsPtr(c);
    for (int q = 0; q < bs; ++q) foffd[(size_t)c * bs + q] = cv[q];
  }
  // the real solve path
  bool prec_ok = prec.SetValue(ls.m_ls);
  double conv = p.tol;
  unsigned int iter = (unsigned)p.maxit;
  bool converged = false;
  {
    LsSol::CLinearSystemPreconditioner lsp(ls.m_ls, prec);
    converged = bicgstab ? LsSol::Solve_PBiCGSTAB(conv, iter, lsp) : LsSol::Solve_PCG(conv, iter, lsp);
  }
  MatVec::CVector_Blk& upd = ls.GetUpdate(id_field, CORNER, world);
  std::vector<double> x((size_t)n * b);
  for (int i = 0; i < n; ++i) for (int d = 0; d < b; ++d) x[(size_t)i * b + d] = upd.GetValue(i, d);

  FILE* f = fopen(argv[2], "wb");
  if (!f) { perror(argv[2]); return 2; }
  wri(f, 0x44464733); wri(f, n); wri(f, b); wri(f, rowptr[n]);
  wr(f, rowptr.data(), rowptr.size() * 4);
  wr(f, colind.data(), colind.size() * 4);
  wr(f, diag.data(), diag.size() * 8);
  wr(f, offd.data(), offd.size() * 8);
  wr(f, rhs.data(), rhs.size() * 8);
  wr(f, &norm_res, 8);
  wri(f, ilu_ok ? 1 : 0); wri(f, prec_ok ? 1 : 0);
  wri(f, fill_level); wri(f, nnz_f);
  wr(f, rowptr_f.data(), rowptr_f.size() * 4);
  wr(f, colind_f.data(), colind_f.size() * 4);
  wr(f, fdiag.data(), fdiag.size() * 8);
  wr(f, foffd.data(), foffd.size() * 8);
  wri(f, converged ? 1 : 0); wri(f, (int)iter); wr(f, &conv, 8);
  wr(f, x.data(), x.size() * 8);
  fclose(f);
  return 0;
}
