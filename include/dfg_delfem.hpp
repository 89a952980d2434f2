// dfg_delfem.hpp -- C++ adapter for DelFEM code that drives libdfg.
//
// Header-only; include it in a DelFEM build (it needs DelFEM's headers on the
// include path) and link libdfg.so.  It is the reference-side binding of the
// C ABI in dfg.h:
//
//  * CLinearSystem_FieldGPU mirrors Fem::Ls::CLinearSystem_Field
//    (include/delfem/femls/linearsystem_field.h:67-172) for one field: the
//    pattern and the mesh come from the same CFieldWorld segments the
//    reference's AddPattern_Field and AddLinSys_* read, and it implements
//    LsSol::ILinearSystemPreconditioner_Sol
//    (include/delfem/ls/linearsystem_interface_solver.h:61-82), so the
//    reference's own LsSol::Solve_PCG can drive it unchanged (strict drop-in);
//  * the AddLinSys_* overloads take the GPU system with the reference's
//    parameter lists (eqn_poisson.h:71-76, eqn_diffusion.h:68-73,
//    eqn_linear_solid2d.h:68-72, eqn_linear_solid3d.h:59-64);
//  * DfgDelFEM::Solve_PCG and DfgDelFEM::Solve_PBiCGSTAB are the
//    device-resident fast paths with the in/out semantics of LsSol::Solve_PCG
//    and LsSol::Solve_PBiCGSTAB (solver_ls_iter.h:38-45);
//  * CMatSolverGPU is the matrix-level MatVec::Sol::Solve_PCG
//    (include/delfem/matvec/solver_mat_iter.h:47-51) over a host
//    CMatDia_BlkCrs and CVector_Blk pair;
//  * CPreconditioner_ILU_GPU is an LsSol::CPreconditioner for the
//    reference's own host CLinearSystem: only the ILU factor and its
//    application move to the device.
#ifndef DFG_DELFEM_HPP
#define DFG_DELFEM_HPP

#include <algorithm>
#include <cassert>
#include <memory>
#include <string>
#include <vector>

#include "dfg.h"
#include "delfem/elem_ary.h"
#include "delfem/field.h"
#include "delfem/field_world.h"
#include "delfem/ls/linearsystem.h"
#include "delfem/ls/linearsystem_interface_solver.h"
#include "delfem/ls/preconditioner.h"
#include "delfem/matvec/matdia_blkcrs.h"
#include "delfem/matvec/vector_blk.h"
#include "delfem/node_ary.h"

namespace DfgDelFEM {

class CLinearSystem_FieldGPU : public LsSol::ILinearSystemPreconditioner_Sol {
 public:
  explicit CLinearSystem_FieldGPU(dfg_ctx ctx) : ctx_(ctx) {}
  virtual ~CLinearSystem_FieldGPU() {
    if (prec_) dfg_precond_destroy(prec_);
    if (sys_) dfg_system_destroy(sys_);
  }

  // CLinearSystem_Field::AddPattern_Field (linearsystem_field.cpp:196-280):
  // node-to-node pattern of the field's corner segments, plus the mesh the
  // element routines read (CElemSeg::GetNodes / CNodeSeg::GetValue).
  bool AddPattern_Field(unsigned int id_field, const Fem::Field::CFieldWorld& world) {
    using namespace Fem::Field;
    if (!world.IsIdField(id_field)) return false;
    const CField& f = world.GetField(id_field);
    const CNodeAry::CNodeSeg& ns_co = f.GetNodeSeg(CORNER, false, world);
    const CNodeAry::CNodeSeg& ns_va = f.GetNodeSeg(CORNER, true, world);
    const unsigned int nnode = ns_co.Size(), ndim = ns_co.Length();
    blklen_ = (int)ns_va.Length();
    nnode_ = (int)nnode;
    std::vector<double> coords((size_t)nnode * ndim);
    for (unsigned int i = 0; i < nnode; ++i) ns_co.GetValue(i, &coords[(size_t)i * ndim]);
    std::vector<int> conn;
    int nnoel = 0;
    const std::vector<unsigned int> aIdEA = f.GetAryIdEA();
    for (unsigned int k = 0; k < aIdEA.size(); ++k) {
      const CElemAry::CElemSeg& es = f.GetElemSeg(aIdEA[k], CORNER, true, world);
      nnoel = (int)es.Length();
      std::vector<unsigned int> no(nnoel);
      for (unsigned int e = 0; e < es.Size(); ++e) {
        es.GetNodes(e, no.data());
        for (int q = 0; q < nnoel; ++q) conn.push_back((int)no[q]);
      }
    }
    nelem_ = nnoel ? (int)(conn.size() / nnoel) : 0;
    if (dfg_system_create_from_elements(ctx_, nnode_, blklen_, nelem_, nnoel, conn.data(), &sys_) != DFG_OK) return false;
    return dfg_system_set_mesh(sys_, (int)ndim, coords.data(), nelem_, nnoel, conn.data()) == DFG_OK;
  }

  // SetFixedBoundaryCondition_Field (linearsystem_field.cpp:618-710): every
  // DOF of every node of the partial field's element segments is fixed.
  bool SetFixedBoundaryCondition_Field(unsigned int id_field_fix, const Fem::Field::CFieldWorld& world) {
    using namespace Fem::Field;
    if (!sys_ || !world.IsIdField(id_field_fix)) return false;
    if (flags_.empty()) flags_.assign((size_t)nnode_ * blklen_, 0);
    const CField& f = world.GetField(id_field_fix);
    const std::vector<unsigned int> aIdEA = f.GetAryIdEA();
    for (unsigned int k = 0; k < aIdEA.size(); ++k) {
      const CElemAry::CElemSeg& es = f.GetElemSeg(aIdEA[k], CORNER, true, world);
      std::vector<unsigned int> no(es.Length());
      for (unsigned int e = 0; e < es.Size(); ++e) {
        es.GetNodes(e, no.data());
        for (unsigned int q = 0; q < no.size(); ++q)
          for (int d = 0; d < blklen_; ++d) flags_[(size_t)no[q] * blklen_ + d] = 1;
      }
    }
    return dfg_set_bcflags(sys_, flags_.data()) == DFG_OK;
  }

  void InitializeMarge() { dfg_initialize_marge(sys_); }
  double FinalizeMarge() {
    double r = 0.0;
    dfg_finalize_marge(sys_, &r);
    return r;
  }

  // UpdateValueOfField (linearsystem_field.cpp:716-794): field += update
  bool UpdateValueOfField(unsigned int id_field, Fem::Field::CFieldWorld& world,
                          Fem::Field::FIELD_DERIVATION_TYPE fdt = Fem::Field::VALUE) {
    using namespace Fem::Field;
    std::vector<double> x((size_t)nnode_ * blklen_);
    if (dfg_get_vector(sys_, -2, x.data()) != DFG_OK) return false;
    CNodeAry::CNodeSeg& ns = world.GetField(id_field).GetNodeSeg(CORNER, true, world, fdt);
    for (int i = 0; i < nnode_; ++i)
      for (int d = 0; d < blklen_; ++d) ns.AddValue(i, d, x[(size_t)i * blklen_ + d]);
    return true;
  }

  // ---- CPreconditioner_ILU (preconditioner.h:59-108), owned by the system
  bool SetFillInLevel(int lev) {
    if (!prec_ && dfg_precond_create(ctx_, &prec_) != DFG_OK) return false;
    return dfg_precond_set_fill_level(prec_, lev) == DFG_OK;
  }
  bool SetPreconditionerLinearSystem() {
    if (!prec_ && dfg_precond_create(ctx_, &prec_) != DFG_OK) return false;
    return dfg_precond_set_linear_system(prec_, sys_) == DFG_OK;
  }
  bool SetPreconditionerValue() { return dfg_precond_set_value(prec_, sys_) == DFG_OK; }

  // ---- LsSol::ILinearSystemPreconditioner_Sol
  unsigned int GetTmpVectorArySize() const {
    unsigned int n = 0;
    dfg_get_tmp_vector_size(sys_, &n);
    return n;
  }
  bool ReSizeTmpVecSolver(unsigned int size_new) { return dfg_resize_tmp_vec(sys_, size_new) == DFG_OK; }
  double DOT(int iv1, int iv2) {
    double r = 0.0;
    dfg_dot(sys_, iv1, iv2, &r);
    return r;
  }
  bool COPY(int iv1, int iv2) { return dfg_copy(sys_, iv1, iv2) == DFG_OK; }
  bool SCAL(double alpha, int iv1) { return dfg_scal(sys_, alpha, iv1) == DFG_OK; }
  bool AXPY(double alpha, int iv1, int iv2) { return dfg_axpy(sys_, alpha, iv1, iv2) == DFG_OK; }
  bool MATVEC(double alpha, int iv1, double beta, int iv2) { return dfg_matvec(sys_, alpha, iv1, beta, iv2) == DFG_OK; }
  bool SolvePrecond(int iv) { return dfg_precond_solve(prec_, sys_, iv) == DFG_OK; }

  dfg_system system() const { return sys_; }
  dfg_precond preconditioner() const { return prec_; }
  int BlockLength() const { return blklen_; }

 private:
  dfg_ctx ctx_ = nullptr;
  dfg_system sys_ = nullptr;
  dfg_precond prec_ = nullptr;
  int nnode_ = 0, blklen_ = 0, nelem_ = 0;
  std::vector<int> flags_;
};

// ---- Fem::Eqn element routines with the reference's parameter lists
inline bool AddLinSys_Poisson(CLinearSystem_FieldGPU& ls, double alpha, double source) {
  return dfg_assemble_poisson(ls.system(), alpha, source) == DFG_OK;
}
inline bool AddLinSys_Diffusion(double dt, double gamma, CLinearSystem_FieldGPU& ls, double rho, double alpha,
                                double source) {
  return dfg_assemble_diffusion(ls.system(), dt, gamma, rho, alpha, source) == DFG_OK;
}
inline bool AddLinSys_LinearSolid2D_Static(CLinearSystem_FieldGPU& ls, double lambda, double myu, double rho,
                                           double g_x, double g_y) {
  return dfg_assemble_solid2d(ls.system(), lambda, myu, rho, g_x, g_y) == DFG_OK;
}
inline bool AddLinSys_LinearSolid3D_Static(CLinearSystem_FieldGPU& ls, double lambda, double myu, double rho,
                                           double g_x, double g_y, double g_z) {
  return dfg_assemble_solid3d(ls.system(), lambda, myu, rho, g_x, g_y, g_z) == DFG_OK;
}

// ---- device-resident LsSol::Solve_PCG
inline bool Solve_PCG(double& conv_ratio, unsigned int& iteration, CLinearSystem_FieldGPU& ls) {
  return dfg_solve_pcg(ls.system(), ls.preconditioner(), &conv_ratio, &iteration) == DFG_OK;
}
inline bool Solve_PCG_Mixed(double& conv_ratio, unsigned int& iteration, CLinearSystem_FieldGPU& ls) {
  unsigned int outer = 0;
  return dfg_solve_pcg_mixed(ls.system(), ls.preconditioner(), &conv_ratio, &iteration, &outer) == DFG_OK;
}

// ---- device-resident LsSol::Solve_PBiCGSTAB (solver_ls_iter.cpp:291-408);
// like the reference it returns true at the iteration limit too, with
// num_iter = the limit and conv_ratio left as given
inline bool Solve_PBiCGSTAB(double& conv_ratio, unsigned int& num_iter, CLinearSystem_FieldGPU& ls) {
  const int st = dfg_solve_pbicgstab(ls.system(), ls.preconditioner(), DFG_PREC_FP64, &conv_ratio, &num_iter);
  return st == DFG_OK || st == DFG_NOT_CONVERGED;
}

// ---- MatVec::Sol::Solve_PCG (src/matvec/solver_mat_iter.cpp:115-189), the
// matrix-level PCG.  The reference passes the matrix, the residual and update
// vectors, and a CPrecond_Blk with its factor matrix (a CMatDiaFrac_BlkCrs
// made from the same matrix).  Here one object holds the matrix's device copy
// and its ILU(fill_level) factor, so the call keeps the matrix and vector
// arguments and the preconditioner pair becomes SetValue.  Same arithmetic as
// LsSol::Solve_PCG; at the iteration limit it returns false with conv_ratio
// left as given and iteration = the limit, as the matrix-level loop does.
// The pattern must be the reference's own: columns sorted per row, no
// diagonal (CMatDia_BlkCrs::AddPattern builds it so); block lengths 1-3.
class CMatSolverGPU {
 public:
  // symbolic: the block pattern (GetPtrIndPSuP per row) and the factor's
  CMatSolverGPU(dfg_ctx ctx, const MatVec::CMatDia_BlkCrs& mat, int fill_level = 0)
      : n_((int)mat.NBlkMatCol()), b_(mat.LenBlkCol()) {
    std::vector<int> rowptr(n_ + 1, 0);
    for (int i = 0; i < n_; ++i) {
      unsigned int np = 0;
      const unsigned int* c = mat.GetPtrIndPSuP(i, np);
      for (unsigned int k = 0; k < np; ++k) colind_.push_back((int)c[k]);
      rowptr[i + 1] = (int)colind_.size();
    }
    const int* ci = colind_.empty() ? rowptr.data() : colind_.data();
    ok_ = dfg_system_create(ctx, n_, b_, rowptr.data(), ci, &sys_) == DFG_OK &&
          dfg_precond_create(ctx, &prec_) == DFG_OK && dfg_precond_set_fill_level(prec_, fill_level) == DFG_OK &&
          dfg_precond_set_linear_system(prec_, sys_) == DFG_OK;
  }
  ~CMatSolverGPU() {
    if (prec_) dfg_precond_destroy(prec_);
    if (sys_) dfg_system_destroy(sys_);
  }
  CMatSolverGPU(const CMatSolverGPU&) = delete;
  CMatSolverGPU& operator=(const CMatSolverGPU&) = delete;
  bool IsValid() const { return ok_; }

  // numeric: the matrix values (GetPtrValDia / GetPtrValPSuP) and the factor
  // (CMatDiaFrac_BlkCrs::SetValue + DoILUDecomp); false on a singular pivot
  bool SetValue(const MatVec::CMatDia_BlkCrs& mat) {
    if (!ok_ || (int)mat.NBlkMatCol() != n_ || mat.LenBlkCol() != b_ || mat.NCrs() != colind_.size()) return false;
    const size_t bs = (size_t)b_ * b_;
    std::vector<double> diag(n_ * bs + 1), offd(colind_.size() * bs + 1);
    size_t o = 0;
    for (int i = 0; i < n_; ++i) {
      const double* d = mat.GetPtrValDia(i);
      std::copy(d, d + bs, diag.begin() + i * bs);
      unsigned int np = 0;
      const double* v = mat.GetPtrValPSuP(i, np);
      std::copy(v, v + np * bs, offd.begin() + o);
      o += np * bs;
    }
    return dfg_set_matrix(sys_, diag.data(), offd.data()) == DFG_OK && dfg_precond_set_value(prec_, sys_) == DFG_OK;
  }

  // vec := (LU)^-1 vec, the factor's forward and backward substitution
  // (CMatDiaFrac_BlkCrs::ForwardSubstitution / BackwardSubstitution,
  // src/matvec/matdiafrac_blkcrs.cpp:332-669) on the device
  bool SolvePrecond(MatVec::CVector_Blk& vec) {
    if (!ok_ || (int)vec.NBlk() != n_ || vec.Len() != b_) return false;
    if (n_ == 0) return true;
    unsigned ntmp = 0;
    if (dfg_get_tmp_vector_size(sys_, &ntmp) != DFG_OK || (ntmp < 1 && dfg_resize_tmp_vec(sys_, 1) != DFG_OK))
      return false;
    return dfg_set_vector(sys_, 0, vec.GetValuePtr(0)) == DFG_OK && dfg_precond_solve(prec_, sys_, 0) == DFG_OK &&
           dfg_get_vector(sys_, 0, vec.GetValuePtr(0)) == DFG_OK;
  }

  // r_vec: right-hand side in, recursive residual out; u_vec: solution out
  bool Solve_PCG(double& conv_ratio, unsigned int& iteration, MatVec::CVector_Blk& r_vec, MatVec::CVector_Blk& u_vec) {
    if (!ok_ || (int)r_vec.NBlk() != n_ || r_vec.Len() != b_ || (int)u_vec.NBlk() != n_ || u_vec.Len() != b_)
      return false;
    if (n_ == 0) {  // ||r||^2 = 0 < 1e-30: the reference's early return
      conv_ratio = 0.0;
      iteration = 0;
      return true;
    }
    const double tol = conv_ratio;
    const unsigned int mx = iteration;
    if (dfg_set_vector(sys_, -1, r_vec.GetValuePtr(0)) != DFG_OK) return false;
    const int st = dfg_solve_pcg(sys_, prec_, &conv_ratio, &iteration);
    if ((st != DFG_OK && st != DFG_NOT_CONVERGED) || dfg_get_vector(sys_, -1, r_vec.GetValuePtr(0)) != DFG_OK ||
        dfg_get_vector(sys_, -2, u_vec.GetValuePtr(0)) != DFG_OK)
      return false;
    if (st == DFG_NOT_CONVERGED) {
      conv_ratio = tol;
      iteration = mx;
      return false;
    }
    return true;
  }

 private:
  int n_, b_;
  std::vector<int> colind_;
  dfg_system sys_ = nullptr;
  dfg_precond prec_ = nullptr;
  bool ok_ = false;
};

// ---- LsSol::CPreconditioner_ILU (include/delfem/ls/preconditioner.h:55-97,
// src/ls/preconditioner.cpp) for the reference's own host CLinearSystem: the
// factor is built and applied on the device, everything else stays on the
// host.  A DelFEM program swaps the one declaration
//     LsSol::CPreconditioner_ILU prec;   ->   DfgDelFEM::CPreconditioner_ILU_GPU prec(ctx);
// and keeps SetFillInLevel / SetLinearSystem(ls.m_ls) / SetValue(ls.m_ls),
// LsSol::CLinearSystemPreconditioner lsp(ls.m_ls, prec) and the reference's
// own LsSol::Solve_PCG.  One linear-system segment (one field), block length
// 1-3; every apply copies the vector to the device and back.
class CPreconditioner_ILU_GPU : public LsSol::CPreconditioner {
 public:
  explicit CPreconditioner_ILU_GPU(dfg_ctx ctx) : ctx_(ctx) {}
  // CPreconditioner_ILU::SetFillInLevel (preconditioner.h:75): one segment,
  // so ilss0 is -1 (all) or 0
  void SetFillInLevel(int lev, int ilss0 = -1) {
    if (ilss0 <= 0) lev_ = lev;
  }
  // symbolic: the segment's pattern and the factor's (preconditioner.cpp:57-211)
  virtual void SetLinearSystem(const LsSol::CLinearSystem& ls) {
    core_.reset();
    if (ls.GetNLinSysSeg() != 1) return;
    core_.reset(new CMatSolverGPU(ctx_, ls.GetMatrix(0), lev_));
  }
  // numeric factorisation (preconditioner.cpp:217-297); false on more than
  // 10 singular pivots, as DoILUDecomp
  virtual bool SetValue(const LsSol::CLinearSystem& ls) {
    return core_ && core_->IsValid() && ls.GetNLinSysSeg() == 1 && core_->SetValue(ls.GetMatrix(0));
  }
  // forward then backward substitution of vector iv (preconditioner.cpp:301-335)
  virtual bool SolvePrecond(LsSol::CLinearSystem& ls, unsigned int iv) {
    return core_ && ls.GetNLinSysSeg() == 1 && core_->SolvePrecond(ls.GetVector((int)iv, 0));
  }
  bool IsValid() const { return core_ && core_->IsValid(); }

 private:
  dfg_ctx ctx_;
  int lev_ = 0;
  std::unique_ptr<CMatSolverGPU> core_;
};

}  // namespace DfgDelFEM

#endif  // DFG_DELFEM_HPP
