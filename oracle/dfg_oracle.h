/*
 * dfg_oracle.h -- CPU oracle for the DelFEM assembly + ILU-PCG path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithm; tests/ and __graft_entry__.smoke() check the library's results
 * against it, and bench.py times it as the CPU baseline.  The product
 * library (libdfg) never links, loads or calls it.
 *
 * Parity pin: every function here is checked bit-for-bit against the
 * reference code itself (compiled headless from its sources by
 * oracle/Makefile into oracle/_ref/) through the golden fixtures in
 * tests/golden/, which tests/golden/make_golden.py generates from that
 * build.
 *
 * Matrix layout follows CMatDia_BlkCrs (matvec/matdia_blkcrs.h:118-123):
 * diagonal blocks stored apart from the off-diagonal CRS blocks, each block
 * b x b row-major doubles; rowptr[n+1] / colind[nnz] hold the block pattern
 * (the reference calls these m_colInd_Blk / m_rowPtr_Blk).
 */
#ifndef DFG_ORACLE_H
#define DFG_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Node-to-node block pattern without the diagonal, columns ascending per row.
 * Mirrors CElemAry::MakePattern_FEM (femfield/elem_ary.cpp:225-245) followed by
 * CMatDia_BlkCrs::AddPattern on an empty matrix (matvec/matdia_blkcrs.cpp:383-402).
 * Call with colind == NULL to get the count; returns nnz or -1 on bad input. */
long dfo_pattern(int nnode, int nelem, int nnoel, const int* conn,
                 int* rowptr, int* colind);

/* ILU(0) split index: first CRS slot of row i whose column is > i
 * (matvec/matdiafrac_blkcrs.cpp:203-218). */
void dfo_diaind(int n, const int* rowptr, const int* colind, int* diaind);

/* Block pattern of the ILU(lev_fill) factor, without the diagonal, columns
 * ascending per row (CMatDiaFrac_BlkCrs::AddFracPtn, matvec/matdiafrac_blkcrs.cpp:
 * 1254-1382; lev_fill -1 = no level limit).  Returns the factor's nnz; when it
 * exceeds cap nothing is written. */
long dfo_ilu_pattern(int n, const int* rowptr, const int* colind, int lev_fill,
                     int* rowptr_f, int* colind_f, long cap);

/* A's values into the factor pattern, zero elsewhere (SetValue_Initialize,
 * matvec/matdiafrac_blkcrs.h:90-96).  Returns -1 when A's pattern is not a
 * subset of the factor's. */
int dfo_ilu_init(int n, int b, const int* rowptr, const int* colind, const double* diag, const double* offd,
                 const int* rowptr_f, const int* colind_f, double* fdiag, double* foffd);

/* Element assembly (scatter follows CMatDia_BlkCrs::Mearge,
 * matvec/matdia_blkcrs.cpp:165-258, in element order).
 * coef: per-element multiplier or NULL (== all 1.0).  u: current field value
 * per node (n*b) or NULL (== zero).  res receives the element residuals. */
int dfo_assemble_poisson2d(int n, const int* rowptr, const int* colind,
                           int nelem, const int* conn, const double* coords,
                           const double* coef, double alpha, double source,
                           const double* u, double* diag, double* offd, double* res);
int dfo_assemble_poisson3d(int n, const int* rowptr, const int* colind,
                           int nelem, const int* conn, const double* coords,
                           const double* coef, double alpha, double source,
                           const double* u, double* diag, double* offd, double* res);
int dfo_assemble_diffusion2d(int n, const int* rowptr, const int* colind,
                             int nelem, const int* conn, const double* coords,
                             const double* coef, double rho, double alpha, double source,
                             double gamma, double dt, const double* u, const double* v,
                             double* diag, double* offd, double* res);
int dfo_assemble_solid2d(int n, const int* rowptr, const int* colind,
                         int nelem, const int* conn, const double* coords,
                         const double* coef, double lambda, double myu,
                         double rho, double gx, double gy,
                         const double* u, double* diag, double* offd, double* res);
int dfo_assemble_solid3d(int n, const int* rowptr, const int* colind,
                         int nelem, const int* conn, const double* coords,
                         const double* coef, double lambda, double myu,
                         double rho, double gx, double gy, double gz,
                         const double* u, double* diag, double* offd, double* res);

/* Dirichlet rows/columns + zeroed residual; returns ||res||_2
 * (CLinearSystem::FinalizeMarge, ls/linearsystem.cpp:92-128). */
double dfo_finalize(int n, int b, const int* rowptr, const int* colind,
                    const int* bcflag, double* diag, double* offd, double* res);

/* In-place block ILU(0): diag <- D^-1, strictly lower <- L, strictly upper <- D^-1 U.
 * Returns the number of singular pivots (>=0), or -1 when it exceeds 10
 * (CMatDiaFrac_BlkCrs::DoILUDecomp, matvec/matdiafrac_blkcrs.cpp:774-1107). */
int dfo_ilu0(int n, int b, const int* rowptr, const int* colind, const int* diaind,
             double* diag, double* offd);

void dfo_forward(int n, int b, const int* rowptr, const int* colind, const int* diaind,
                 const double* fdiag, const double* foffd, double* vec);
void dfo_backward(int n, int b, const int* rowptr, const int* colind, const int* diaind,
                  const double* foffd, double* vec);

/* y = alpha*A*x + beta*y (CMatDia_BlkCrs::MatVec, matvec/matdia_blkcrs.cpp:921-1094). */
void dfo_matvec(int n, int b, const int* rowptr, const int* colind,
                const double* diag, const double* offd,
                double alpha, const double* x, double beta, double* y);

/* LsSol::Solve_PCG (ls/solver_ls_iter.cpp:100-172).  r: residual in, recursive
 * residual out; x: solution out.  *conv in = tolerance, out = achieved ratio;
 * *iter in = max iterations, out = 0-based iteration count.  Returns 1 when
 * converged.  work: 2*n*b doubles. */
int dfo_pcg(int n, int b, const int* rowptr, const int* colind, const int* diaind,
            const double* diag, const double* offd,
            const double* fdiag, const double* foffd,
            double* r, double* x, double* conv, unsigned* iter, double* work);

/* dfo_pcg with the factor in its own pattern (ILU(k), k != 0). */
int dfo_pcg_f(int n, int b, const int* rowptr, const int* colind, const double* diag, const double* offd,
              const int* rowptr_f, const int* colind_f, const int* diaind_f,
              const double* fdiag, const double* foffd,
              double* r, double* x, double* conv, unsigned* iter, double* work);

/* LsSol::Solve_PBiCGSTAB (ls/solver_ls_iter.cpp:291-408) with the ILU factor
 * in its own pattern.  r: residual in, residual out; x: solution out.  *conv
 * in = tolerance, out = achieved ratio when converged (untouched otherwise,
 * as in the reference); *iter in = max iterations, out = the 1-based
 * iteration of convergence (max iterations otherwise).  A residual with
 * ||r||^2 < 1e-60 returns at once with *conv = ||r|| and x untouched.
 * Returns 1 when converged (the reference returns true in both cases).
 * work: 7*n*b doubles. */
int dfo_bicgstab(int n, int b, const int* rowptr, const int* colind, const double* diag, const double* offd,
                 const int* rowptr_f, const int* colind_f, const int* diaind_f,
                 const double* fdiag, const double* foffd,
                 double* r, double* x, double* conv, unsigned* iter, double* work);
/* dfo_bicgstab recording hist[it] = ||r||^2 / ||r0||^2 after iteration it
 * (hist: max iterations doubles). */
int dfo_bicgstab_hist(int n, int b, const int* rowptr, const int* colind, const double* diag, const double* offd,
                      const int* rowptr_f, const int* colind_f, const int* diaind_f,
                      const double* fdiag, const double* foffd,
                      double* r, double* x, double* conv, unsigned* iter, double* work, double* hist);

/* Wall-time helpers for the CPU baseline. */
double dfo_now(void);

#ifdef __cplusplus
}
#endif
#endif
