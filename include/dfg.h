/*
 * dfg.h -- C ABI of libdfg, the GB300 (sm_103a) implementation of DelFEM's
 * finite-element assembly + block ILU(0) preconditioned CG hot path.
 *
 * Every entry point is extern "C", takes plain pointers and sizes, and
 * returns an int status (DFG_OK == 0).  Host pointers passed in are copied
 * before the call returns and never retained.  Device memory is owned by
 * the handles.  All work of one context is ordered on that context's CUDA
 * stream; calls that hand data back to the host synchronise that stream.
 * A context is used from one host thread at a time.
 *
 * Conventions follow the reference (paths relative to the DelFEM tree):
 *  - block-CRS with the diagonal blocks kept apart from the off-diagonal CRS
 *    blocks, each block b x b row-major (include/delfem/matvec/matdia_blkcrs.h:118-123);
 *    rowptr[nblk+1] / colind[nnz] are what the reference calls m_colInd_Blk /
 *    m_rowPtr_Blk; columns ascending within a row, no diagonal entry;
 *  - vector slots of the solver interface: -1 = residual (right-hand side in,
 *    recursive residual out), -2 = update (solution), >= 0 = work vectors
 *    (include/delfem/ls/linearsystem_interface_solver.h:39-82);
 *  - the ILU factor keeps D^-1 in the diagonal slots, the unscaled L in the
 *    strictly lower part and D^-1 U in the strictly upper part
 *    (src/matvec/matdiafrac_blkcrs.cpp:862-1046).
 */
#ifndef DFG_H
#define DFG_H

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
enum {
  DFG_OK = 0,
  DFG_NOT_CONVERGED = 1,   /* Solve_PCG returned false (solver_ls_iter.cpp:168-171) */
  DFG_SINGULAR_PIVOT = 2,  /* more than 10 pivots below 1e-30 (matdiafrac_blkcrs.cpp:779-780) */
  DFG_NAN_DETECTED = 3,
  DFG_OOM_REJECTED = 4,    /* device allocation refused */
  DFG_TIMEOUT = 5,         /* a bounded device-side wait gave up */
  DFG_INVALID_ARGUMENT = 6,
  DFG_CUDA_ERROR = 7,
  DFG_NOT_READY = 8        /* call order violated (e.g. solve before the preconditioner value) */
};

/* vector precision / solver modes */
enum {
  DFG_PREC_FP64 = 0,        /* plain FP64 path */
  DFG_PREC_MIXED = 1,       /* FP32 factor, sweeps, SpMV and Krylov vectors inside FP64 refinement */
  DFG_PREC_FP32_FACTOR = 2  /* FP32 factor and sweeps; FP64 SpMV, vectors and reductions */
};

typedef struct dfg_ctx_s* dfg_ctx;
typedef struct dfg_system_s* dfg_system;
typedef struct dfg_precond_s* dfg_precond;

/* ---------------------------------------------------------------- context */

/* Creates a context on CUDA device `device` with its own stream. */
int dfg_ctx_create(int device, dfg_ctx* out);
/* Destroys the context; systems, preconditioners and servers made on it
 * must be destroyed first (they use its stream and device). */
int dfg_ctx_destroy(dfg_ctx ctx);
/* Text of the last error raised through this context (never NULL); with
 * ctx == NULL, the reason the last dfg_ctx_create or dfg_dot_noalloc of this
 * thread failed. */
const char* dfg_last_error(dfg_ctx ctx);
/* Library version string. */
const char* dfg_version(void);
/* Blocks until all work queued on the context's stream has finished. */
int dfg_ctx_synchronize(dfg_ctx ctx);
/* Number of kernels this library has launched through the context. */
long long dfg_ctx_kernel_launches(dfg_ctx ctx);
/* The context's CUDA stream (a cudaStream_t), for callers that time or order
 * their own work against the library's. */
int dfg_ctx_get_stream(dfg_ctx ctx, void** stream);

/* ------------------------------------------------- linear system (pattern) */

/* Square block-CRS system with a caller-supplied pattern.
 * Replaces CLinearSystem::AddLinSysSeg + CMatDia_BlkCrs::AddPattern
 * (src/ls/linearsystem.cpp:138-167, src/matvec/matdia_blkcrs.cpp:346-505). */
int dfg_system_create(dfg_ctx ctx, int nblk, int blklen,
                      const int* rowptr, const int* colind, dfg_system* out);
/* Same, with the node-to-node pattern built from element connectivity
 * (CElemAry::MakePattern_FEM, src/femfield/elem_ary.cpp:225-245, through
 * CLinearSystem_Field::AddPattern_Field, src/femls/linearsystem_field.cpp:196-280). */
int dfg_system_create_from_elements(dfg_ctx ctx, int nblk, int blklen, int nelem, int nnoel,
                                    const int* conn, dfg_system* out);
int dfg_system_destroy(dfg_system sys);
/* nblk, block length and number of off-diagonal blocks. */
int dfg_system_info(dfg_system sys, int* nblk, int* blklen, long long* nnz);
/* Copies the pattern out (rowptr: nblk+1 ints, colind: nnz ints). */
int dfg_system_get_pattern(dfg_system sys, int* rowptr, int* colind);

/* Mesh the element routines read: coordinates (nnode x ndim doubles, node
 * order == block order) and connectivity (nelem x nnoel ints; 3 = P1
 * triangle, 4 = P1 tetrahedron).  Builds the element-to-slot gather map.
 * Stands in for the CFieldWorld node / element segments the reference's
 * AddLinSys_* routines read (CElemSeg::GetNodes, CNodeSeg::GetValue). */
int dfg_system_set_mesh(dfg_system sys, int ndim, const double* coords,
                        int nelem, int nnoel, const int* conn);
/* Per-element coefficient multiplier (nelem doubles) or NULL for none.
 * The reference has one scalar per element array; with a multiplier, alpha
 * (Poisson/diffusion) or lambda and myu (elasticity) become value*coef[e].
 * A multiplier of exactly 1.0 reproduces the reference bit-for-bit. */
int dfg_system_set_coef(dfg_system sys, const double* coef);
/* Current field values u and velocities v (nblk*blklen doubles each, NULL = 0),
 * read by the element routines as the reference reads the field node segments. */
int dfg_system_set_field(dfg_system sys, const double* u, const double* v);
/* CLinearSystem_Field::UpdateValueOfField (src/femls/linearsystem_field.cpp:
 * 716-794) on the resident field: field += 1.0 * update slot, for the
 * field's value (fdt 0, VALUE) or velocity (fdt 1, VELOCITY), on the device
 * -- the next assembly reads it without a host round trip.  A field not set
 * before starts from zero, as a fresh reference field does. */
int dfg_system_update_field(dfg_system sys, int fdt);
/* Host copy of the resident field (u and/or v, nblk*blklen doubles each;
 * NULL skips one; zeros for a field never set). */
int dfg_system_get_field(dfg_system sys, double* u, double* v);
/* Dirichlet flags, one int per DOF (1 = fixed).  Replaces
 * CLinearSystem_Field::SetFixedBoundaryCondition_Field -> CBCFlag::SetBC
 * (src/femls/linearsystem_field.cpp:618-710, include/delfem/matvec/bcflag_blk.h:153-164). */
int dfg_set_bcflags(dfg_system sys, const int* flags);

/* --------------------------------------------------------------- assembly */

/* Zeroes matrix, residual and update (CLinearSystem::InitializeMarge,
 * src/ls/linearsystem.cpp:74-88). */
int dfg_initialize_marge(dfg_system sys);
/* Fem::Eqn::AddLinSys_Poisson (src/femeqn/eqn_poisson.cpp:428-470): P1 triangle
 * (:49-125) or P1 tetrahedron (:249-323) according to the mesh. */
int dfg_assemble_poisson(dfg_system sys, double alpha, double source);
/* Fem::Eqn::AddLinSys_Diffusion (src/femeqn/eqn_diffusion.cpp:348-400), P1 triangle (:240-347).
 * The CLinearSystem_Field overload takes triangles only; a tetrahedral mesh is
 * DFG_INVALID_ARGUMENT, where the reference prints "NotImplimented" and asserts.  (The 3D
 * P1 routine at :662-768 serves the CLinearSystem_SaveDiaM_Newmark overload.) */
int dfg_assemble_diffusion(dfg_system sys, double dt, double gamma,
                           double rho, double alpha, double source);
/* Fem::Eqn::AddLinSys_LinearSolid2D_Static (src/femeqn/eqn_linear_solid2d.cpp:215-266),
 * P1 triangle (:505-598). */
int dfg_assemble_solid2d(dfg_system sys, double lambda, double myu,
                         double rho, double g_x, double g_y);
/* Fem::Eqn::AddLinSys_LinearSolid3D_Static (src/femeqn/eqn_linear_solid3d.cpp:162-194),
 * P1 tetrahedron (:241-334). */
int dfg_assemble_solid3d(dfg_system sys, double lambda, double myu,
                         double rho, double g_x, double g_y, double g_z);
/* residual += f (nblk*blklen doubles): extra nodal loads such as the traction
 * CEqnSystem_Solid2D::SetLoad stores (src/femeqn/eqnsys_solid.cpp:894-907);
 * equivalent to CVector_Blk::AddValue on every DOF. */
int dfg_add_residual(dfg_system sys, const double* f);
/* Stores a nodal load (nblk*blklen doubles, NULL clears it) on the device;
 * every later dfg_finalize_marge adds it to the residual before the
 * Dirichlet rows are applied, so a fixed load stays resident across solves.
 * Counterpart of CEqnSystem_Solid2D::SetLoad (src/femeqn/eqnsys_solid.cpp:894-907),
 * which keeps the load with the equation system; the addition is the
 * element-wise one of dfg_add_residual. */
int dfg_system_set_load(dfg_system sys, const double* f);
/* Dirichlet rows/columns, residual zeroed on fixed DOFs; *norm_res = ||r||_2
 * (CLinearSystem::FinalizeMarge, src/ls/linearsystem.cpp:92-128). */
int dfg_finalize_marge(dfg_system sys, double* norm_res);

/* Host copies of the matrix (diag: nblk*b*b, offd: nnz*b*b doubles) and of the
 * solver vectors (CLinearSystem_Field::GetMatrix / GetResidual / GetUpdate,
 * src/femls/linearsystem_field.cpp:577-616). */
int dfg_get_matrix(dfg_system sys, double* diag, double* offd);
int dfg_set_matrix(dfg_system sys, const double* diag, const double* offd);
int dfg_get_vector(dfg_system sys, int iv, double* out);
int dfg_set_vector(dfg_system sys, int iv, const double* in);

/* ---------------------------------------- solver interface (ILinearSystem_Sol) */

/* Number of work vectors (slots >= 0) and resizing them
 * (ILinearSystem_Sol::GetTmpVectorArySize / ReSizeTmpVecSolver,
 * include/delfem/ls/linearsystem_interface_solver.h:71-73,
 * src/ls/linearsystem.cpp:208-245); new slots start at zero. */
int dfg_get_tmp_vector_size(dfg_system sys, unsigned* size);
int dfg_resize_tmp_vec(dfg_system sys, unsigned size);
/* *out = {v1}.{v2} (CLinearSystem::DOT, src/ls/linearsystem.cpp:335-360) */
int dfg_dot(dfg_system sys, int iv1, int iv2, double* out);
/* Allocation-free dot product.  No counterpart in the reference (its DOT,
 * src/ls/linearsystem.cpp:335-360, is dfg_dot above).
 *
 * *out = x.y for m doubles in device memory of the calling thread's current
 * CUDA device, computed on `stream` (a cudaStream_t; NULL = the default
 * stream); the call returns once the result is on the host.  Same
 * deterministic two-pass sum as dfg_dot (fixed-shape block trees, then the
 * per-block partials in index order), with 4096-element blocks: the same
 * inputs give the same bits on every call, and the value agrees with
 * dfg_dot's to rounding.
 *
 * For callers that may not allocate device memory: a serving loop whose
 * device budget is fully reserved at admission while other solves run
 * (cudaMalloc could exceed the budget, cudaFree waits for the whole device),
 * and callers holding vectors in their own device memory without a dfg
 * context (creating one allocates).  Nothing is allocated: the reduction
 * scratch is a fixed file-scope device array of 8192 partial sums plus two
 * words (65,552 bytes per device), so m > DFG_DOT_NOALLOC_MAX_LEN is rejected
 * with DFG_INVALID_ARGUMENT (reason in dfg_last_error(NULL)).  The arrival
 * counter is cleared on `stream` before each launch.
 *
 * The first call in each CUDA context (the device's primary context, or a
 * context the caller made current) looks up the array's address
 * (cudaGetSymbolAddress) with that context current, and later calls in the
 * same context reuse it; make that first call before any stream capture
 * begins.  The address is kept per context ID, so after a device reset the
 * next call looks it up again.  All calls on one device share the one
 * array: calls that overlap (several host threads, or several streams at
 * once) race, and the caller must serialise them. */
#define DFG_DOT_NOALLOC_MAX_LEN 33554432LL /* 8192 blocks x 4096 elements */
int dfg_dot_noalloc(const double* x, const double* y, long long m, double* out, void* stream);
/* {v2} := {v1} (COPY :366-392) */
int dfg_copy(dfg_system sys, int iv1, int iv2);
/* {v1} := alpha*{v1} (SCAL :398-415) */
int dfg_scal(dfg_system sys, double alpha, int iv1);
/* {v2} := alpha*{v1} + {v2} (AXPY :298-329; no-op when alpha == 0) */
int dfg_axpy(dfg_system sys, double alpha, int iv1, int iv2);
/* {v2} := alpha*[A]{v1} + beta*{v2} (MATVEC :250-292 -> CMatDia_BlkCrs::MatVec,
 * src/matvec/matdia_blkcrs.cpp:921-1094) */
int dfg_matvec(dfg_system sys, double alpha, int iv1, double beta, int iv2);

/* ---------------------------------------------------------- ILU preconditioner */

/* LsSol::CPreconditioner_ILU (include/delfem/ls/preconditioner.h:59-108). */
int dfg_precond_create(dfg_ctx ctx, dfg_precond* out);
int dfg_precond_destroy(dfg_precond prec);
/* SetFillInLevel (preconditioner.h:77): 0 (the default) = ILU(0), k > 0 =
 * level-of-fill ILU(k), -1 = no level limit (complete LU in natural order).
 * Takes effect at the next dfg_precond_set_linear_system; < -1 is rejected. */
int dfg_precond_set_fill_level(dfg_precond prec, int lev);
/* Symbolic set-up: the factor's block pattern (A's for level 0; with the
 * fill-in of CMatDiaFrac_BlkCrs::AddFracPtn, src/matvec/matdiafrac_blkcrs.cpp:
 * 1254-1382, otherwise), split index, level sets and sweep schedules
 * (CPreconditioner_ILU::SetLinearSystem, src/ls/preconditioner.cpp:57-211;
 * CMatDiaFrac_BlkCrs(0,A), src/matvec/matdiafrac_blkcrs.cpp:171-225). */
int dfg_precond_set_linear_system(dfg_precond prec, dfg_system sys);
/* How the triangular sweeps are scheduled (no counterpart in the reference,
 * whose substitutions are sequential loops): 0 (default) times the kinds
 * on the device at the symbolic set-up and keeps the fastest per direction;
 * 1 = ranged (contiguous row ranges pipelined across CTAs, good for the long
 * thin wavefronts of large 2D meshes); 2 = level-scheduled (one launch per
 * dependency level, good for the wide levels of 3D meshes); 3 = one CTA
 * (the whole sweep on one SM, level after level, its input first permuted
 * into the schedule's order: good for small 2D meshes, whose sweeps are
 * bound by the latency of each level).  Takes effect at the next
 * dfg_precond_set_linear_system; results agree to rounding. */
int dfg_precond_set_sweep_mode(dfg_precond prec, int mode);
/* The kind chosen per direction after the symbolic set-up (1, 2 or 3). */
int dfg_precond_get_sweep_mode(dfg_precond prec, int* fwd, int* bwd);
/* The set-up's timings behind that choice, ms per FP32 sweep: ms[0..3] =
 * forward ranged, forward level-scheduled, backward ranged, backward
 * level-scheduled (-1 where a kind was not timed). */
int dfg_precond_get_sweep_timing(dfg_precond prec, float* ms);
/* The set-up's timings of the one-CTA kind, ms per FP32 sweep: ms[0] forward,
 * ms[1] backward (-1 where it was not timed). */
int dfg_precond_get_solo_timing(dfg_precond prec, float* ms);
/* The factor's block pattern after the symbolic set-up: *nnz off-diagonal
 * blocks; rowptr (n+1) and colind (nnz) in the layout of
 * dfg_system_get_pattern, each written when non-NULL. */
int dfg_precond_get_pattern(dfg_precond prec, long long* nnz, int* rowptr, int* colind);
/* Numeric factorisation of the system's current matrix
 * (CPreconditioner_ILU::SetValue, src/ls/preconditioner.cpp:217-297 ->
 * DoILUDecomp, src/matvec/matdiafrac_blkcrs.cpp:774-1107).  Returns
 * DFG_SINGULAR_PIVOT when the reference would return false. */
int dfg_precond_set_value(dfg_precond prec, dfg_system sys);
/* {iv} := (LU)^-1 {iv} (CPreconditioner_ILU::SolvePrecond, src/ls/preconditioner.cpp:301-335). */
int dfg_precond_solve(dfg_precond prec, dfg_system sys, int iv);
/* Host copy of the factor in the reference layout: fdiag n*b*b, foffd
 * nnz*b*b with nnz and the block order of dfg_precond_get_pattern. */
int dfg_precond_get_factor(dfg_precond prec, double* fdiag, double* foffd);

/* ------------------------------------------------------------- mesh input */

/* Reads a GiD mesh file (".msh", the format of the reference's input meshes,
 * test_glut/input_file/) as Msh::CMesher2D::ReadFromFile_GiDMsh
 * (src/msh/mesher2d.cpp:2463) reads triangles and Msh::CMesh3D::
 * ReadFromFile_GiDMsh (src/msh/mesh3d.cpp:601) tetrahedra: *ndim = 2 with
 * *nnoel = 3 (triangles; three-coordinate nodes in a coordinate plane are
 * projected on it, dropping the axis of smallest variance) or *ndim = 3 with
 * *nnoel = 4.  coords: nnode*ndim doubles, conn: nelem*nnoel 0-based node
 * ids, in file order; call with both NULL to get the sizes first.  Needs no
 * device.  Other element types and malformed files: DFG_INVALID_ARGUMENT,
 * reason in dfg_last_error(NULL). */
int dfg_mesh_read_gid(const char* path, int* ndim, int* nnoel, int* nnode, int* nelem, double* coords, int* conn);

/* ------------------------------------------------------------------- solvers */

/* LsSol::Solve_PCG (src/ls/solver_ls_iter.cpp:100-172) run device-resident:
 * residual slot in = right-hand side, out = recursive residual; update slot
 * out = solution.  *conv_ratio: tolerance in, achieved ||r||/||r0|| out;
 * *iteration: maximum in, 0-based iteration of convergence out.
 * Returns DFG_OK when converged, DFG_NOT_CONVERGED otherwise. */
int dfg_solve_pcg(dfg_system sys, dfg_precond prec, double* conv_ratio, unsigned* iteration);

/* General form of the device-resident PCG.  `mode` is one of DFG_PREC_*.
 * With target_true != 0 the solve also requires the true relative residual
 * ||b - A x|| / ||b|| (b = the finalized right-hand side) to be <= the
 * tolerance: when the recursive residual says converged but the true one does
 * not, the recursion continues from the true residual.  With target_true == 0
 * and DFG_PREC_FP64 this is exactly dfg_solve_pcg.  *conv_ratio: tolerance in,
 * achieved ratio out (the true one when target_true != 0); *iteration: maximum
 * in, iterations out; *refinements: true-residual recomputations (may be NULL). */
int dfg_solve_pcg_ex(dfg_system sys, dfg_precond prec, int mode, int target_true, double* conv_ratio,
                     unsigned* iteration, unsigned* refinements);

/* LsSol::Solve_PBiCGSTAB (src/ls/solver_ls_iter.cpp:291-408) run
 * device-resident, for non-symmetric systems (SPD ones too); the same slots
 * as dfg_solve_pcg.  mode: DFG_PREC_FP64 (other modes are rejected with
 * DFG_INVALID_ARGUMENT: BiCGSTAB does not tolerate a preconditioner applied
 * in FP32, whose rounding differs at every application; on ill-conditioned
 * systems its iteration then diverges).  *conv_ratio: tolerance in, achieved
 * ||r||/||r0|| out when converged (left as given otherwise, as the reference
 * does); *iteration: maximum in, 1-based iteration of convergence out (the
 * maximum when it did not converge).  A residual with ||r||^2 < 1e-60 returns
 * at once with *conv_ratio = ||r||, *iteration = 0 and the update slot
 * untouched.  Returns DFG_OK when converged and DFG_NOT_CONVERGED when the
 * limit was reached (the reference returns true in both cases). */
int dfg_solve_pbicgstab(dfg_system sys, dfg_precond prec, int mode, double* conv_ratio, unsigned* iteration);

/* Mixed-precision form of the same solve: FP32 factor, sweeps and SpMV
 * inside FP64 iterative refinement (FP64 outer residual r = b - A x, FP64
 * alpha/beta reductions and FP64 solution accumulation).  *conv_ratio: target
 * true relative residual ||b - A x|| / ||b|| in, achieved out; *iteration:
 * maximum total inner iterations in, total inner iterations out;
 * *outer: number of refinement passes out (may be NULL). */
int dfg_solve_pcg_mixed(dfg_system sys, dfg_precond prec, double* conv_ratio,
                        unsigned* iteration, unsigned* outer);

/* Times each kernel of one PCG iteration on its own (CUDA events on the
 * context's stream, averaged over `reps` launches) with the system's current
 * matrix, factor and solver vectors; call after a solve of the same mode.
 * mode: DFG_PREC_FP64 or DFG_PREC_MIXED.  ms[0..5] = SpMV + p.Ap, forward
 * sweep, backward sweep, r/x update + r.r, r.z + beta, p update (ms per launch);
 * bytes[0..2] = algorithmic bytes of one SpMV, forward and backward sweep. */
int dfg_profile_kernels(dfg_system sys, dfg_precond prec, int mode, int reps, double* ms, double* bytes);

/* Self-test of the device-side bounded waits (no counterpart in the
 * reference): launches one wait, with the sweep kernels' own poll, on a value
 * that nothing writes.  The wait gives up after its budget (about 2 s of SM
 * clock), records the failure in the context's error word and returns; this
 * call then reads and clears the record and returns DFG_TIMEOUT with the
 * recorded wait site in *site (3 = poll of a dependency value).  Nothing
 * faults, traps or hangs, and the context stays usable afterwards. */
int dfg_selftest_wait_timeout(dfg_ctx ctx, int* site);

/* ||b - A x||_2 / ||b||_2 in FP64 for the system's current matrix, with
 * b = the given host right-hand side and x = the update slot. */
int dfg_true_residual(dfg_system sys, const double* b, double* rel);

/* --------------------------------------------------------------- serving
 *
 * No counterpart in the reference (its solves run one at a time on the
 * caller's thread).  A server keeps many independent FE solves resident on
 * one device: requests are admitted first-come first-served as device memory
 * (a fixed admission budget reserved at creation) and in-flight slots free
 * up, assembled and factorised on a low-priority stream, and iterated
 * together -- every replay of one captured CUDA graph runs `chunk_iters` PCG
 * iterations of all in-flight solves through batched launches.  Each solve
 * follows the reference path (AddLinSys_* -> FinalizeMarge -> ILU(0) ->
 * Solve_PCG) and stops when its TRUE relative residual ||b-Ax||/||b|| is
 * <= tol (the recursion continues from the true residual when they disagree).
 * A solve's arithmetic does not depend on the other solves in flight: the
 * same request gives the same bits alone and in any mix. */

typedef struct dfg_server_s* dfg_server;

typedef struct {
  int mode;               /* DFG_PREC_FP64, DFG_PREC_FP32_FACTOR, or DFG_PREC_MIXED (FP32 SpMV on
                             FP32-stored values, FP32 Krylov vectors, FP32 factor and sweeps; FP64
                             dot reductions, solution and reliable-update residual b - A x) */
  double tol;             /* true relative residual target */
  int maxit;              /* iteration limit per solve; 0 = 20000 */
  long long budget_bytes; /* device bytes reserved for admitted solves; 0 = 85% of free memory */
  int max_inflight;       /* solves resident at once, <= 256; 0 = 256 */
  int chunk_iters;        /* PCG iterations per graph replay, <= 64; 0 = 8 */
  int host_threads;       /* symbolic set-up threads; 0 = hardware threads - 2 */
  int profile_every;      /* every n-th replay times its first iteration per kernel; 0 = never */
  int size_groups;        /* solves grouped by size, each group iterating at its own pace on its own
                             streams: 1 = one table for all, 2-3 groups; 0 = 3 */
  int sweeps;             /* triangular-sweep kernel: 0 = per solve (FP32 sweeps one CTA per solve
                             except 3x3-block solves above 100,000 nodes; FP64 sweeps ranged over
                             several CTAs), 1 = ranged, 2 = one CTA per solve; the same bits either way */
} dfg_server_config;

/* kind: 1 Poisson 2D (P1 triangles), 2 Poisson 3D (P1 tetrahedra),
 * 3 diffusion 2D, 4 linear solid 2D, 5 linear solid 3D.  params as the
 * matching dfg_assemble_* takes them, in its argument order (Poisson: alpha,
 * source; solid 2D: lambda, myu, rho, g_x, g_y; solid 3D: + g_z; diffusion:
 * rho, alpha, source, gamma, dt).  Block length: 1, 1, 1, 2, 3. */
typedef struct {
  int kind;
  int nnode, nelem;
  const double* coords;   /* nnode x dim */
  const int* conn;        /* nelem x (3 or 4) */
  const double* coef;     /* per-element multiplier, or NULL */
  const double* params;
  int nparams;            /* <= 8 */
  const int* bcflag;      /* per DOF: != 0 fixed at 0 */
  const double* load;     /* per DOF nodal load added at FinalizeMarge, or NULL */
  double* x_out;          /* host buffer, nnode x block length: the solution */
} dfg_request;

typedef struct {
  long long id;
  int status;             /* DFG_OK, DFG_NOT_CONVERGED, DFG_SINGULAR_PIVOT, DFG_NAN_DETECTED,
                             DFG_OOM_REJECTED (larger than the whole budget), DFG_TIMEOUT, ... */
  int iterations;         /* 0-based iteration of the stop, as Solve_PCG reports it */
  double conv;            /* recursive residual ratio at the stop */
  double rel_true;        /* ||b - A x|| / ||b|| of the returned x (-1 if not checked) */
  double t_submit, t_admit, t_done;  /* seconds since the server was created */
  long long device_bytes; /* device bytes the solve reserved while admitted */
} dfg_result;

typedef struct {
  long long submitted, finished, replays, kernel_launches, graph_builds, peak_inflight;
  long long budget_bytes, peak_bytes;
  long long h2d_bytes;    /* request data uploaded (inputs and derived set-up) */
  long long d2h_bytes;    /* solutions copied back */
  double busy_seconds;    /* loop-thread time with a replay in flight */
  double now_seconds;     /* on the clock of dfg_result's times */
  double backlog_seconds; /* time with at least one request submitted and not yet admitted */
  double queued_seconds;  /* time with at least one request set up and waiting for device
                             admission (behind another admission, or the device was full) */
  double full_seconds;    /* time with a request set up and no device memory or in-flight
                             slot free for it */
  double inflight_seconds; /* solves admitted and not yet released, integrated over time */
  double symbolic_seconds; /* host symbolic set-up, summed over requests */
  double admit_seconds;   /* device admission (uploads, assembly, ILU, packing), summed */
} dfg_server_counters;

/* Per-kernel timing of profiled replays (dfg_server_config::profile_every):
 * for kernel k, ms[k] sums the CUDA-event durations of its launches and
 * bytes[k] their algorithmic bytes (the solves in flight at that launch),
 * over n[k] launches.  k: 0 r.z + beta, 1 p update, 2 SpMV + p.Ap,
 * 3 r/x update + r.r, 4 true-residual check, 5 residual replacement,
 * 6 + 2*c forward sweep of class c, 7 + 2*c backward sweep of class c, where
 * class c holds block length c/3 + 1 and at most 4, 8 or 16 (c % 3)
 * dependency entries per row. */
#define DFG_SERVER_NKERNELS 24
typedef struct {
  double ms[DFG_SERVER_NKERNELS];
  double bytes[DFG_SERVER_NKERNELS];
  long long n[DFG_SERVER_NKERNELS];
} dfg_server_profile_t;

/* Creates a server on the context's device (its own streams and threads). */
int dfg_server_create(dfg_ctx ctx, const dfg_server_config* cfg, dfg_server* out);
/* Queues one solve (all inputs copied; x_out is written before the request
 * completes).  Thread-safe. */
int dfg_server_submit(dfg_server s, const dfg_request* req, long long* id);
/* Blocks until request `id` has completed and reports its outcome. */
int dfg_server_wait(dfg_server s, long long id, dfg_result* out);
/* Text of a failed request's error ("" when it succeeded). */
int dfg_server_error_text(dfg_server s, long long id, char* buf, int len);
/* Blocks until every submitted request has completed. */
int dfg_server_drain(dfg_server s);
/* Counters since creation (dfg_server_counters): requests submitted and
 * finished, replays, kernel launches, graph builds, peak solves in flight,
 * device bytes reserved and at peak, bytes moved each way, busy time. */
int dfg_server_stats(dfg_server s, dfg_server_counters* out);
/* Per-kernel device time and algorithmic bytes summed over the profiled
 * replays (dfg_server_config::profile_every). */
int dfg_server_profile(dfg_server s, dfg_server_profile_t* out);
/* Completes the requests in flight, then releases the server. */
int dfg_server_destroy(dfg_server s);

#ifdef __cplusplus
}
#endif
#endif /* DFG_H */
