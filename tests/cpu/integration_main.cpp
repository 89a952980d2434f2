// integration_main.cpp -- TEST INFRASTRUCTURE: a DelFEM-side program that
// uses include/dfg_delfem.hpp exactly as a maintainer would: mesh through
// Msh::IMesh into CFieldWorld, the GPU linear system from the field, the
// reference's own LsSol::Solve_PCG and LsSol::Solve_PBiCGSTAB driving it
// through the virtual interface, the device-resident fast paths, and the
// matrix-level MatVec::Sol::Solve_PCG beside CMatSolverGPU on the same matrix,
// and the reference's host linear system with CPreconditioner_ILU_GPU.
// Compiled (and, where a GPU exists, run) by tests/test_integration_adapter.py
// against the reference's headers.
#include <algorithm>
#include <cassert>
#include <cmath>
#include <cstdio>
#include <vector>

#include "delfem/mesh_interface.h"
#include "delfem/field_world.h"
#include "delfem/femeqn/eqn_poisson.h"
#include "delfem/femls/linearsystem_field.h"
#include "delfem/ls/preconditioner.h"
#include "delfem/ls/solver_ls_iter.h"
#include "delfem/matvec/bcflag_blk.h"
#include "delfem/matvec/matdiafrac_blkcrs.h"
#include "delfem/matvec/solver_mat_iter.h"
#include "dfg_delfem.hpp"

class Square : public Msh::IMesh {
 public:
  explicit Square(int n) : n_(n) {}
  unsigned int GetDimention() const { return 2; }
  void GetInfo(unsigned int, unsigned int& a, unsigned int& b, unsigned int& c, int& d) const { a = 1; b = 0; c = 0; d = 0; }
  void GetCoord(std::vector<double>& co) const {
    co.clear();
    for (int j = 0; j <= n_; ++j) for (int i = 0; i <= n_; ++i) { co.push_back((double)i / n_); co.push_back((double)j / n_); }
  }
  Msh::MSH_TYPE GetConnectivity(unsigned int, std::vector<int>& l) const {
    l.clear();
    for (int j = 0; j < n_; ++j) for (int i = 0; i < n_; ++i) {
      int a = j * (n_ + 1) + i, b = a + 1, c = a + n_ + 2, d = a + n_ + 1;
      int t[6] = {a, b, c, a, c, d};
      l.insert(l.end(), t, t + 6);
    }
    return Msh::TRI;
  }
  std::vector<unsigned int> GetAry_ID() const { return std::vector<unsigned int>(1, 1u); }
  std::vector<unsigned int> GetIncludeElemIDAry(unsigned int) const { return std::vector<unsigned int>(); }
 private:
  int n_;
};

// The finalized system of `ls` as a reference CMatDia_BlkCrs; the reference's
// matrix-level PCG with its ILU(0) CMatDiaFrac_BlkCrs against CMatSolverGPU:
// both converge, iterations within 2, solutions within 1e-6 (relative L2).
static int matrix_level_check(dfg_ctx ctx, DfgDelFEM::CLinearSystem_FieldGPU& ls) {
  dfg_system sys = ls.system();
  int n = 0, b = 0;
  long long nnz = 0;
  if (dfg_system_info(sys, &n, &b, &nnz) != DFG_OK) return 10;
  const size_t bs = (size_t)b * b;
  std::vector<int> rowptr(n + 1), colind(nnz > 0 ? nnz : 1);
  std::vector<double> diag(n * bs), offd((nnz > 0 ? nnz : 1) * bs), rhs((size_t)n * b);
  if (dfg_system_get_pattern(sys, rowptr.data(), colind.data()) != DFG_OK ||
      dfg_get_matrix(sys, diag.data(), offd.data()) != DFG_OK || dfg_get_vector(sys, -1, rhs.data()) != DFG_OK)
    return 11;
  Com::CIndexedArray crs;
  crs.InitializeSize(n);
  for (int i = 0; i <= n; ++i) crs.index[i] = rowptr[i];
  crs.array.assign(colind.begin(), colind.begin() + nnz);
  MatVec::CMatDia_BlkCrs mat(n, b);
  if (!mat.AddPattern(crs)) return 12;
  mat.SetZero();  // allocates the value arrays (the reference allocates them lazily here)
  for (int i = 0; i < n; ++i) {
    std::copy(diag.begin() + i * bs, diag.begin() + (i + 1) * bs, mat.GetPtrValDia(i));
    unsigned int np = 0;
    const unsigned int* c = static_cast<const MatVec::CMatDia_BlkCrs&>(mat).GetPtrIndPSuP(i, np);
    if ((int)np != rowptr[i + 1] - rowptr[i]) return 13;
    for (unsigned int k = 0; k < np; ++k)
      if ((int)c[k] != colind[rowptr[i] + k]) return 13;
    double* v = mat.GetPtrValPSuP(i, np);
    std::copy(offd.begin() + rowptr[i] * bs, offd.begin() + rowptr[i + 1] * bs, v);
  }
  MatVec::CVector_Blk r_ref(n, b), u_ref(n, b), r_gpu(n, b), u_gpu(n, b);
  for (int i = 0; i < n; ++i)
    for (int p = 0; p < b; ++p) {
      r_ref.SetValue(i, p, rhs[(size_t)i * b + p]);
      r_gpu.SetValue(i, p, rhs[(size_t)i * b + p]);
    }
  MatVec::CMatDiaFrac_BlkCrs frac(0, mat);
  if (!frac.SetValue(mat)) return 14;
  double conv_ref = 1e-8, conv_gpu = 1e-8;
  unsigned int it_ref = 1000, it_gpu = 1000;
  const bool ok_ref = MatVec::Sol::Solve_PCG(conv_ref, it_ref, mat, r_ref, u_ref, frac, mat);
  DfgDelFEM::CMatSolverGPU solver(ctx, mat, 0);
  if (!solver.IsValid() || !solver.SetValue(mat)) return 15;
  const bool ok_gpu = solver.Solve_PCG(conv_gpu, it_gpu, r_gpu, u_gpu);
  double d2 = 0.0, x2 = 0.0;
  for (int i = 0; i < n; ++i)
    for (int p = 0; p < b; ++p) {
      const double d = u_gpu.GetValue(i, p) - u_ref.GetValue(i, p);
      d2 += d * d;
      x2 += u_ref.GetValue(i, p) * u_ref.GetValue(i, p);
    }
  std::printf("matrix-level PCG reference: %d iter %u conv %.3e; device: %d iter %u conv %.3e; |du|/|u| %.2e\n",
              ok_ref, it_ref, conv_ref, ok_gpu, it_gpu, conv_gpu, x2 > 0 ? std::sqrt(d2 / x2) : std::sqrt(d2));
  // the iteration limit: false, conv_ratio left as given, iteration = the limit
  MatVec::CVector_Blk r_lim(n, b), u_lim(n, b);
  for (int i = 0; i < n; ++i)
    for (int p = 0; p < b; ++p) r_lim.SetValue(i, p, rhs[(size_t)i * b + p]);
  double conv_lim = 1e-8;
  unsigned int it_lim = 3;
  const bool ok_lim = solver.Solve_PCG(conv_lim, it_lim, r_lim, u_lim);
  if (ok_lim || conv_lim != 1e-8 || it_lim != 3) return 16;
  const unsigned int di = it_ref > it_gpu ? it_ref - it_gpu : it_gpu - it_ref;
  return (ok_ref && ok_gpu && di <= 2 && d2 <= 1e-12 * x2) ? 0 : 17;
}

// The reference's own host CLinearSystem_Field, assembled by the reference's
// AddLinSys_Poisson and solved by the reference's Solve_PCG twice: with its
// CPreconditioner_ILU and with CPreconditioner_ILU_GPU swapped in.  Both
// converge, iterations within 2, solutions within 1e-6 (relative L2).
static int host_system_check(dfg_ctx ctx, Fem::Field::CFieldWorld& world, unsigned int id_field,
                             const std::vector<int>& fixed) {
  Fem::Ls::CLinearSystem_Field ls;
  if (!ls.AddPattern_Field(id_field, world)) return 20;
  MatVec::CBCFlag& bc = ls.m_ls.GetBCFlag(0);
  for (size_t i = 0; i < fixed.size(); ++i)
    if (fixed[i]) bc.SetBC((unsigned)i, 0);
  LsSol::CPreconditioner_ILU prec_cpu;
  prec_cpu.SetFillInLevel(0);
  prec_cpu.SetLinearSystem(ls.m_ls);
  DfgDelFEM::CPreconditioner_ILU_GPU prec_gpu(ctx);
  prec_gpu.SetFillInLevel(0);
  prec_gpu.SetLinearSystem(ls.m_ls);
  if (!prec_gpu.IsValid()) return 21;
  ls.InitializeMarge();
  Fem::Eqn::AddLinSys_Poisson(ls, 1.0, 1.0, world, id_field);
  ls.FinalizeMarge();
  if (!prec_cpu.SetValue(ls.m_ls) || !prec_gpu.SetValue(ls.m_ls)) return 22;
  const MatVec::CVector_Blk rhs = ls.m_ls.GetVector(-1, 0);
  double conv[2] = {1e-8, 1e-8};
  unsigned int it[2] = {1000, 1000};
  std::vector<double> x[2];
  for (int k = 0; k < 2; ++k) {
    ls.m_ls.GetVector(-1, 0) = rhs;
    LsSol::CPreconditioner& prec = k == 0 ? static_cast<LsSol::CPreconditioner&>(prec_cpu) : prec_gpu;
    LsSol::CLinearSystemPreconditioner lsp(ls.m_ls, prec);
    if (!LsSol::Solve_PCG(conv[k], it[k], lsp)) return 23 + k;
    const MatVec::CVector_Blk& u = ls.m_ls.GetVector(-2, 0);
    for (unsigned int i = 0; i < u.NBlk(); ++i) x[k].push_back(u.GetValue(i, 0));
  }
  double d2 = 0.0, x2 = 0.0;
  for (size_t i = 0; i < x[0].size(); ++i) {
    d2 += (x[1][i] - x[0][i]) * (x[1][i] - x[0][i]);
    x2 += x[0][i] * x[0][i];
  }
  std::printf("host system, reference Solve_PCG: CPU ILU iter %u conv %.3e; GPU ILU iter %u conv %.3e; |du|/|u| %.2e\n",
              it[0], conv[0], it[1], conv[1], std::sqrt(d2 / x2));
  const unsigned int di = it[0] > it[1] ? it[0] - it[1] : it[1] - it[0];
  return (di <= 2 && d2 <= 1e-12 * x2) ? 0 : 25;
}

int main() {
  std::setvbuf(stdout, nullptr, _IOLBF, 0);  // each report line reaches the log even if a later step fails
  dfg_ctx ctx = nullptr;
  if (dfg_ctx_create(0, &ctx) != DFG_OK) {
    std::printf("no CUDA device: adapter compiled and linked\n");
    return 0;
  }
  const int nside = 16;
  Fem::Field::CFieldWorld world;
  const unsigned int id_base = world.AddMesh(Square(nside));
  const unsigned int id_field = world.MakeField_FieldElemDim(id_base, 2, Fem::Field::SCALAR, Fem::Field::VALUE, Fem::Field::CORNER);
  // u = 0 on the square's four sides (node j*(nside+1)+i at (i, j)/nside)
  std::vector<int> fixed((nside + 1) * (nside + 1), 0);
  for (int j = 0; j <= nside; ++j)
    for (int i = 0; i <= nside; ++i) fixed[j * (nside + 1) + i] = i == 0 || j == 0 || i == nside || j == nside;
  const int host_rc = host_system_check(ctx, world, id_field, fixed);
  if (host_rc != 0) {
    dfg_ctx_destroy(ctx);
    return host_rc;
  }
  DfgDelFEM::CLinearSystem_FieldGPU ls(ctx);
  if (!ls.AddPattern_Field(id_field, world)) return 1;
  if (dfg_set_bcflags(ls.system(), fixed.data()) != DFG_OK) return 1;
  ls.SetFillInLevel(0);
  ls.SetPreconditionerLinearSystem();
  ls.InitializeMarge();
  DfgDelFEM::AddLinSys_Poisson(ls, 1.0, 1.0);
  ls.FinalizeMarge();
  ls.SetPreconditionerValue();
  double conv = 1e-8;
  unsigned int iter = 1000;
  const bool ok_ref = LsSol::Solve_PCG(conv, iter, ls);  // the reference's solver over the GPU system
  // the reference's loop leaves its final residual in the residual vector:
  // assemble again so that the device loop solves the same system
  ls.InitializeMarge();
  DfgDelFEM::AddLinSys_Poisson(ls, 1.0, 1.0);
  ls.FinalizeMarge();
  double conv2 = 1e-8;
  unsigned int iter2 = 1000;
  const bool ok_fast = DfgDelFEM::Solve_PCG(conv2, iter2, ls);
  std::printf("reference loop: %d iter %u conv %.3e; device loop: %d iter %u conv %.3e\n", ok_ref, iter, conv, ok_fast,
              iter2, conv2);
  // BiCGSTAB, the reference's loop and the device one, on a fresh right-hand side each
  ls.InitializeMarge();
  DfgDelFEM::AddLinSys_Poisson(ls, 1.0, 1.0);
  ls.FinalizeMarge();
  double conv3 = 1e-8;
  unsigned int iter3 = 1000;
  const bool ok_ref_b = LsSol::Solve_PBiCGSTAB(conv3, iter3, ls);
  ls.InitializeMarge();
  DfgDelFEM::AddLinSys_Poisson(ls, 1.0, 1.0);
  ls.FinalizeMarge();
  double conv4 = 1e-8;
  unsigned int iter4 = 1000;
  const bool ok_fast_b = DfgDelFEM::Solve_PBiCGSTAB(conv4, iter4, ls);
  std::printf("BiCGSTAB reference loop: %d iter %u conv %.3e; device loop: %d iter %u conv %.3e\n", ok_ref_b, iter3,
              conv3, ok_fast_b, iter4, conv4);
  ls.UpdateValueOfField(id_field, world);
  ls.InitializeMarge();
  DfgDelFEM::AddLinSys_Poisson(ls, 1.0, 1.0);
  ls.FinalizeMarge();
  const int mat_rc = matrix_level_check(ctx, ls);
  dfg_ctx_destroy(ctx);
  if (mat_rc != 0) return mat_rc;
  const bool pcg_ok = ok_ref && ok_fast && (iter > iter2 ? iter - iter2 : iter2 - iter) <= 2;
  const bool bicg_ok = ok_ref_b && ok_fast_b && iter3 < 1000 && (iter3 > iter4 ? iter3 - iter4 : iter4 - iter3) <= 2;
  return (pcg_ok && bicg_ok) ? 0 : 2;
}
