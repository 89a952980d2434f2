// integration_main.cpp -- TEST INFRASTRUCTURE: a DelFEM-side program that
// uses include/dfg_delfem.hpp exactly as a maintainer would: mesh through
// Msh::IMesh into CFieldWorld, the GPU linear system from the field, the
// reference's own LsSol::Solve_PCG and LsSol::Solve_PBiCGSTAB driving it
// through the virtual interface, and the device-resident fast paths.  Compiled (and, where a GPU exists, run)
// by tests/test_integration_adapter.py against the reference's headers.
#include <cassert>
#include <cstdio>
#include <vector>

#include "delfem/mesh_interface.h"
#include "delfem/field_world.h"
#include "delfem/ls/solver_ls_iter.h"
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

int main() {
  dfg_ctx ctx = nullptr;
  if (dfg_ctx_create(0, &ctx) != DFG_OK) {
    std::printf("no CUDA device: adapter compiled and linked\n");
    return 0;
  }
  Fem::Field::CFieldWorld world;
  const unsigned int id_base = world.AddMesh(Square(16));
  const unsigned int id_field = world.MakeField_FieldElemDim(id_base, 2, Fem::Field::SCALAR, Fem::Field::VALUE, Fem::Field::CORNER);
  DfgDelFEM::CLinearSystem_FieldGPU ls(ctx);
  if (!ls.AddPattern_Field(id_field, world)) return 1;
  ls.SetFillInLevel(0);
  ls.SetPreconditionerLinearSystem();
  ls.InitializeMarge();
  DfgDelFEM::AddLinSys_Poisson(ls, 1.0, 1.0);
  ls.FinalizeMarge();
  ls.SetPreconditionerValue();
  double conv = 1e-8;
  unsigned int iter = 1000;
  const bool ok_ref = LsSol::Solve_PCG(conv, iter, ls);  // the reference's solver over the GPU system
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
  dfg_ctx_destroy(ctx);
  const bool pcg_ok = ok_ref && ok_fast && (iter > iter2 ? iter - iter2 : iter2 - iter) <= 2;
  const bool bicg_ok = ok_ref_b && ok_fast_b && iter3 < 1000 && (iter3 > iter4 ? iter3 - iter4 : iter4 - iter3) <= 2;
  return (pcg_ok && bicg_ok) ? 0 : 2;
}
