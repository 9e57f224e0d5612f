/*
 * gbfe.h -- C ABI of the GB300 FE-operator / ChFSI library (libgbfe.so).
 *
 * One process, one GPU.  Every entry point returns an int status
 * (GBFE_OK == 0); the message of the last failure on a context is read with
 * gbfe_last_error().  No C++ exception crosses this boundary.
 *
 * Data layouts are the reference's (dft-efe):
 *   - block vectors ("MultiVector") are row-major [n_dofs][m], vector index
 *     fastest (linearAlgebra/MultiVector.h:133, data()[iDof*m + iVec]);
 *   - cell dof ids are cell-major and flat (basis/FEBasisManager.h,
 *     locallyOwnedCellLocalDofIdsBegin), size_type = uint32;
 *   - cell matrices are column-major nd_c x nd_c, cells concatenated
 *     (ksdft/KohnShamOperatorContextFE.h:141-155, d_hamiltonianInAllCells);
 *   - constraints are the CSR arrays of basis/ConstraintsInternal.h
 *     (rowConstraintsIdsLocal, rowConstraintsSizes, columnConstraintsIdsLocal,
 *     columnConstraintsAccumulated, columnConstraintsValues,
 *     constraintsInhomogenities).
 */
#ifndef GBFE_H
#define GBFE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (mirror linearAlgebra/LinearAlgebraTypes.h error enums) */
enum {
  GBFE_OK = 0,
  GBFE_ERR_ARG = 1,            /* invalid argument / contract violation       */
  GBFE_ERR_CUDA = 2,           /* CUDA runtime / library failure              */
  GBFE_ERR_ALLOC = 3,          /* device allocation failed / over budget      */
  GBFE_ERR_NOT_ORTHONORMALIZABLE = 4, /* Cholesky-GS: globalSize < m or
                                   near-zero L diagonal
                                   (OrthonormalizationFunctions.t.cpp:274-306) */
  GBFE_ERR_LAPACK = 5,         /* potrf / trtri / syevd failure               */
  GBFE_ERR_NOT_CONVERGED = 6,  /* CG FAILED_TO_CONVERGE, KS_MAX_PASS_ERROR     */
  GBFE_ERR_DIVERGED = 7,       /* CG RESIDUAL_DIVERGENCE                      */
  GBFE_ERR_TIMEOUT = 8,        /* a bounded device wait gave up               */
  GBFE_ERR_CANCELLED = 9       /* serving request cancelled                   */
};

enum { GBFE_F64 = 0, GBFE_F32 = 1 };

/* cell-matrix precision variants an operator carries */
enum {
  GBFE_PREC_FP64 = 1,          /* FP64 matrices (always present)               */
  GBFE_PREC_MIXED = 2,         /* + split-BF16 hi/lo copies for the FP32 path   */
  GBFE_PREC_FP64_TENSOR = 4    /* + 8-slice integer copies for the FP64-accurate
                                  tensor-core product (cells up to 256 dofs)    */
};

typedef struct gbfe_ctx gbfe_ctx;
typedef struct gbfe_mesh gbfe_mesh;
typedef struct gbfe_cons gbfe_cons;
typedef struct gbfe_op gbfe_op;
typedef struct gbfe_mv gbfe_mv;
typedef struct gbfe_nl gbfe_nl;

/* ---- lifecycle ------------------------------------------------------------
 * Replaces the LinAlgOpContext<DEVICE> / BlasQueue / LapackQueue bundle
 * (linearAlgebra/LinAlgOpContext.h:148-176). */
int gbfe_ctx_create(int device, gbfe_ctx **out);
int gbfe_ctx_destroy(gbfe_ctx *ctx);
int gbfe_last_error(const gbfe_ctx *ctx, char *buf, size_t len);
/* cudaStream_t as void*; NULL selects the context's own stream */
int gbfe_ctx_set_stream(gbfe_ctx *ctx, void *stream);
int gbfe_ctx_synchronize(gbfe_ctx *ctx);
/* Reads and clears the device status word that the tensor-core kernels set
 * when one of their bounded waits gives up: GBFE_OK or GBFE_ERR_TIMEOUT. */
int gbfe_ctx_check_status(gbfe_ctx *ctx);
/* Check of that failure path (no counterpart in the reference): launches one
 * thread that waits, through the same bounded-wait routine, on a barrier that
 * nothing completes, giving up after limit_s seconds (0 to 1).  Afterwards
 * gbfe_ctx_check_status returns GBFE_ERR_TIMEOUT once and the context stays
 * usable.  Nothing else is in flight in that kernel, so no GPU fault is
 * involved. */
int gbfe_ctx_check_wait_timeout(gbfe_ctx *ctx, double limit_s);
/* Cell product of the FP32 apply: 2 (default) the persistent warp-specialised
 * split-BF16 tcgen05 kernel (16-byte row gathers when m % 4 == 0); 3 the same
 * kernel with one 4-byte element per gather load; 1 the one-CTA-per-cell
 * tcgen05 kernel; 0 the FP32 SIMT kernel.  The environment variable
 * GBFE_TENSOR_CORES=0|1 sets the initial mode of a new context. */
int gbfe_ctx_set_tensor_cores(gbfe_ctx *ctx, int mode);
/* 1 (default): the size groups of a split-BF16 cell product (cells needing one
 * or two 128-row tiles) run concurrently on a second stream when one of them
 * does not read the enrichment rows computed just before (profiling off);
 * 0: one after the other on the context's stream. */
int gbfe_ctx_set_split_groups(gbfe_ctx *ctx, int on);
/* Size the grids of this context's kernels (persistent kernels: CTAs per SM x
 * this count; strided kernels: their block counts) for `sms` multiprocessors
 * instead of all of them (0: all).  Concurrent contexts on one GPU -- the
 * serving slots -- then leave room on every SM for each other's kernels. */
int gbfe_ctx_set_sm_budget(gbfe_ctx *ctx, int sms);
/* ---- nonlocal pseudopotential part ---------------------------------------
 * Replaces basis::AtomCenterNonLocalOpContextFE
 * (basis/AtomCenterNonLocalOpContextFE.h:47-179): Y = sum_atoms C^T V C X.
 * The arrays are what its constructor computes from the atom data
 * (AtomCenterNonLocalOpContextFE.t.cpp:410-632):
 *   n_proj              projectors on this mesh (d_CX rows)
 *   proj_per_cell[C]    d_numProjsInCells
 *   proj_ids[sum np_c]  d_locallyOwnedCellLocalProjectorIds (projector of each
 *                       (cell, local projector) slot, cell-major)
 *   cell_c[sum np_c*nd_c] d_cellWiseC: per cell np_c x nd_c, column-major
 *                       (projector index fastest), cells concatenated
 *   coupling[n_proj]    d_V, the diagonal coupling constant of each projector
 * Cells with np_c = 0 take no work. */
int gbfe_nonlocal_upload(gbfe_mesh *mesh, uint32_t n_proj, const uint32_t *proj_per_cell, const uint32_t *proj_ids,
                         const double *cell_c, const double *coupling, gbfe_nl **out);
int gbfe_nonlocal_destroy(gbfe_nl *nl);
/* Standalone AtomCenterNonLocalOpContextFE::apply (.t.cpp:715-849): X gets the
 * parent-to-child constraints, Y = assembled C^T V C X with child-to-parent. */
int gbfe_nonlocal_apply(const gbfe_nl *nl, const gbfe_cons *cons, gbfe_mv *X, gbfe_mv *Y);
/* Fuse the nonlocal part into a cell operator's apply (FP64 and FP32 paths):
 * the Kohn-Sham apply with an ONCV component
 * (ksdft/KohnShamOperatorContextFE.t.cpp:1022-1080, 1177-1180) adds C_c^T W
 * into each cell's block before the scatter.  nl = NULL detaches; the
 * operator keeps a pointer, so nl must outlive it or be detached first. */
int gbfe_op_attach_nonlocal(gbfe_op *op, const gbfe_nl *nl);

/* Autotuner of the persistent split-BF16 tensor-core kernel: times every
 * (vector tile, pipeline stages, CTAs per SM, TMEM buffers, X-row prefetch,
 * orientation) shape on `op` (built with GBFE_PREC_MIXED) with m vectors, per
 * launch group of cell sizes, and keeps the fastest on the context.  `report`
 * receives one line per group ("tc2 nd_max tiles m N stages occupancy ms
 * tmem_buffers prefetch swapped"; tmem_buffers 1: one accumulator, which
 * leaves TMEM for another CTA per SM; 0: two where they fit; prefetch 0-3:
 * chunks of X rows copied ahead into shared memory, 0 = gathered into
 * registers; swapped 1: 128 vectors on the MMA's M extent and the cell's
 * rows on N, 0: cell rows on M).  With
 * GBFE_AUTOTUNE_CACHE=<file> in the environment, new
 * contexts load earlier lines from that file and tuning appends to it; a
 * group whose shape the context already holds is reported, not re-timed. */
int gbfe_autotune(const gbfe_op *op, uint32_t m, char *report, size_t report_len);
/* 1 (default): inside gbfe_ks_eigen_solve the d-1 steps of the Chebyshev
 * recurrence are captured once into a CUDA graph (second pass) and replayed
 * on every later pass; 0: launched one by one. */
int gbfe_ctx_set_graphs(gbfe_ctx *ctx, int on);
/* 1 (default): each step of the mixed-precision Chebyshev recurrence runs as
 * two launches -- the split-BF16 cell product with the diagonal of B^-1 folded
 * into A's tiles (A diag(B^-1), built on first use; rows of a dense
 * enrichment block of B^-1 are computed beforehand and substituted in the
 * gather) and the assembly that also computes the recurrence update -- where
 * the operators allow it (homogeneous Dirichlet rows); 0: B^-1 apply, A apply
 * and the update as separate launches.  The two agree to the split-BF16
 * rounding. */
int gbfe_ctx_set_fused_filter(gbfe_ctx *ctx, int on);
/* The m x m symmetric eigenproblems of Rayleigh-Ritz (syevd('V','L') in
 * RayleighRitzEigenSolver.t.cpp:233-301): 1 (default) on the host for
 * m <= 128 (Householder tridiagonalization + implicit QR, one copy each way);
 * 0 cuSOLVER syevd on the device. */
int gbfe_ctx_set_small_eig(gbfe_ctx *ctx, int mode);
/* FP64 arithmetic of the applies and subspace stages:
 *   0 (default) FP64 FMA cell products, DGEMM Gram matrices and rotations;
 *   1 FP64-accurate sliced tensor-core products (Ozaki-style splitting into
 *     eight balanced 7-bit slices, exact FP32 accumulation per level): the
 *     cell products of operators built with GBFE_PREC_FP64_TENSOR and the
 *     Gram matrices / rotations of the fused ChFSI pass (m <= 512);
 *   2 as 1 for the cell products only (Gram / rotations stay DGEMM). */
int gbfe_ctx_set_fp64_apply(gbfe_ctx *ctx, int mode);
/* number of kernels this context has launched so far */
int gbfe_ctx_kernel_launches(const gbfe_ctx *ctx, uint64_t *count);
/* Per-kernel timing (no counterpart in the reference, whose Profiler times
 * host sections: utils/Profiler.h:44-85).  With profiling on, each launch of
 * the cell-product kernels ("cell_apply_f64", "cell_apply_mixed") is bracketed
 * by CUDA events on the launching stream; stats report launches, total device
 * milliseconds and the algorithmic flops / bytes of those launches. */
int gbfe_ctx_set_profiling(gbfe_ctx *ctx, int on);
/* Restrict profiling to the comma-separated scope names (NULL or "": every
 * scope), so a timed run pays for the events of the kernels it reports only. */
int gbfe_ctx_set_profile_filter(gbfe_ctx *ctx, const char *names);
int gbfe_ctx_kernel_stats(gbfe_ctx *ctx, const char *name, uint64_t *launches, double *total_ms,
                          double *flops, double *bytes);
int gbfe_ctx_reset_kernel_stats(gbfe_ctx *ctx);
/* Measured FP64 FMA throughput of this GPU (GFLOP/s), the roofline
 * denominator of the FP64 cell product. */
int gbfe_probe_fp64_peak(gbfe_ctx *ctx, double *gflops);

/* ---- mesh: cell -> dof map ------------------------------------------------
 * Replaces FEBasisManager::nLocallyOwnedCells / nLocallyOwnedCellDofs /
 * locallyOwnedCellLocalDofIdsBegin (basis/FEBasisManager.h) as consumed by
 * KohnShamOperatorContextFE.t.cpp:1334-1356. */
int gbfe_mesh_upload(gbfe_ctx *ctx, uint32_t n_cells, const uint32_t *nd_per_cell,
                     const uint32_t *cell_dof_ids, uint64_t n_dofs, gbfe_mesh **out);
int gbfe_mesh_destroy(gbfe_mesh *mesh);

/* ---- constraints ------------------------------------------------------------
 * Replaces ConstraintsLocal<...,DEVICE> built from CFEConstraintsLocalDealii
 * (basis/CFEConstraintsLocalDealii.t.cpp:360-460, ConstraintsInternal.h).
 * The constraint set must be closed (no column is itself a constrained row). */
int gbfe_constraints_upload(gbfe_mesh *mesh, uint32_t n_rows, const uint32_t *row_ids,
                            const uint32_t *row_sizes, const uint32_t *col_ids,
                            const uint32_t *row_acc, const double *col_values,
                            const double *inhomogeneities, gbfe_cons **out);
int gbfe_constraints_destroy(gbfe_cons *cons);
/* ConstraintsInternal<DEVICE>::constraintsDistributeParentToChild
 * (basis/ConstraintsInternal.cpp:37-107; .cu:39) */
int gbfe_constraints_distribute_parent_to_child(const gbfe_cons *cons, gbfe_mv *x);
/* ConstraintsInternal<DEVICE>::constraintsDistributeChildToParent
 * (basis/ConstraintsInternal.cpp:112-170; .cu:85) -- deterministic, no atomics */
int gbfe_constraints_distribute_child_to_parent(const gbfe_cons *cons, gbfe_mv *x);

/* ---- operators --------------------------------------------------------------
 * Cell-matrix operator: KohnShamOperatorContextFE (H), CFEOverlapOperatorContext
 * (consistent M) and LaplaceOperatorContextFE (K) all reduce to this
 * (KohnShamOperatorContextFE.t.cpp:1326-1443, CFEOverlapOperatorContext.t.cpp:
 * 587-640, LaplaceOperatorContextFE.t.cpp:397-467).  `cons` may be NULL.
 * `prec_flags` is a mask of GBFE_PREC_*. */
int gbfe_cellmat_upload(gbfe_mesh *mesh, const gbfe_cons *cons, const double *mats,
                        int prec_flags, gbfe_op **out);
/* Cell-matrix operator whose cells share stored matrices: `mats` holds n_mats
 * matrices (column-major, concatenated in index order; matrix u has nd x nd
 * entries where nd is the size of the cells that name it) and cell_to_mat[c]
 * names cell c's matrix.  On a uniform mesh (every cell's Laplace or mass
 * matrix identical) this stores one matrix instead of one per cell; the
 * apply is the same as gbfe_cellmat_upload with the matrices expanded. */
int gbfe_cellmat_upload_indexed(gbfe_mesh *mesh, const gbfe_cons *cons, uint32_t n_mats,
                                const double *mats, const uint32_t *cell_to_mat, int prec_flags,
                                gbfe_op **out);
/* Diagonal operator with constraints: CFEOverlapInverseOpContextGLL
 * (CFEOverlapInverseOpContextGLL.t.cpp:528-559) or the lumped
 * CFEOverlapOperatorContext (:546-582).  `diag` holds the diagonal entries
 * (already inverted for an inverse operator). */
int gbfe_diag_upload(gbfe_mesh *mesh, const gbfe_cons *cons, const double *diag, gbfe_op **out);
/* OrthoEFE inverse overlap (basis/OrthoEFEOverlapInverseOpContextGLL.t.cpp:
 * 1182-1270): Y = diag o X on every dof, then the rows [blk_begin, blk_begin +
 * blk_n) (the enrichment dofs) are replaced by blk * X[those rows] (blk is the
 * column-major blk_n x blk_n inverse of the enrichment overlap block), then
 * child-to-parent constraints. */
int gbfe_diag_block_upload(gbfe_mesh *mesh, const gbfe_cons *cons, const double *diag,
                           uint64_t blk_begin, uint64_t blk_n, const double *blk, gbfe_op **out);
/* Jacobi preconditioner: Y = diagInv o X, no constraints
 * (linearAlgebra/PreconditionerJacobi.t.cpp:23-80; the reciprocal is taken
 * here from `diagonal` exactly as the reference constructor does). */
int gbfe_jacobi_upload(gbfe_mesh *mesh, const double *diagonal, gbfe_op **out);
int gbfe_op_destroy(gbfe_op *op);
/* Rebuild a cell operator's matrices on the device (uniform nd):
 *   A_c = alpha * F_c + B^T diag(w_c) B
 * B: basis values at the nq quadrature points of the reference cell, row-major
 * [nq][nd]; weights: [n_cells][nq] quadrature weight times Jacobian times the
 * field (e.g. the local potential); fixed_mats: cell-concatenated column-major
 * F_c (e.g. the Laplace matrices, alpha = 0.5 for the kinetic part) or NULL.
 * This is KohnShamOperatorContextFE::reinit (KohnShamOperatorContextFE.t.cpp:
 * 1253-1311) with KineticFE (KineticFE.t.cpp:90-97) and ElectrostaticLocalFE
 * (ElectrostaticLocalFE.t.cpp:1625-1660) getLocal on the device.  The derived
 * FP32, split-BF16 and sliced copies are rebuilt. */
int gbfe_op_assemble_local(gbfe_op *op, uint32_t nq, const double *basis_values, const double *weights,
                           const double *fixed_mats, double alpha);

/* ---- block vectors (MultiVector) -------------------------------------------- */
int gbfe_mv_create(gbfe_mesh *mesh, uint32_t m, int dtype, gbfe_mv **out);
/* Wrap a caller-owned device buffer [n_dofs][m] (e.g. the data() of a
 * reference MultiVector<..., MemorySpace::DEVICE>, MultiVector.h:133) without
 * copying; gbfe_mv_destroy then releases only the handle. */
int gbfe_mv_wrap(gbfe_mesh *mesh, uint32_t m, int dtype, void *device_ptr, gbfe_mv **out);
int gbfe_mv_destroy(gbfe_mv *mv);
int gbfe_mv_copy_in(gbfe_mv *mv, const void *host_rowmajor);
int gbfe_mv_copy_out(const gbfe_mv *mv, void *host_rowmajor);
int gbfe_mv_copy(const gbfe_mv *src, gbfe_mv *dst); /* same shape; converts dtype */
int gbfe_mv_set_value(gbfe_mv *mv, double value);
int gbfe_mv_device_ptr(const gbfe_mv *mv, void **ptr);
/* MultiVector::l2Norms (MultiVector.t.cpp:553-578); deterministic reduction */
int gbfe_mv_l2_norms(const gbfe_mv *mv, double *norms_host);
/* blasLapack::dotMultiVector: per-column sum_i x_i y_i */
int gbfe_mv_dots(const gbfe_mv *x, const gbfe_mv *y, double *dots_host);

/* ---- the apply -------------------------------------------------------------
 * OperatorContext::apply(X, Y, updateGhostX, updateGhostY)
 * (linearAlgebra/OperatorContext.h:104-108).  Y is overwritten.  X is modified
 * by distributeParentToChild exactly as the reference documents
 * (OperatorContext.h:79-83).  On one GPU the ghost flags are no-ops.
 * X and Y may be F64 (FP64 path) or both F32 (mixed path: split-BF16 tensor
 * products accumulated in FP32; needs an operator built with GBFE_PREC_MIXED). */
int gbfe_apply(const gbfe_op *op, gbfe_mv *X, gbfe_mv *Y);

/* FP64 apply that allocates nothing.  No counterpart in the reference: it is
 * for callers that cannot call cudaMalloc while they apply an operator -- a
 * process whose device memory is all reserved by another component's pool,
 * or a latency-critical loop that must not take the device-wide
 * synchronisation a cudaMalloc can cause.  The caller passes device buffers
 * X and Y ([n_dofs][m] row-major FP64, X is modified by the constraints as in
 * gbfe_apply) and an operator built earlier with gbfe_cellmat_upload.  The
 * cell-wise intermediate lives in a fixed library array of 8,388,608 doubles
 * (64 MiB) that every GPU loading the library keeps until the process exits;
 * calls with sum over cells of nd_c times m above that return GBFE_ERR_ARG.
 * The first call on a device looks up that array's device address (with the
 * context's device current), so make the first call before any stream
 * capture.  All calls share the one array and every element of it is
 * rewritten by each call: calls whose work overlaps on the GPU (other streams,
 * other contexts) race and must be serialised by the caller. */
int gbfe_apply_f64_noalloc(const gbfe_op *op, double *X_dev, double *Y_dev, uint32_t m);

/* Cell matrices of cells of any size and quadrature rule (enriched cells carry
 * extra basis functions and a finer rule): A_c = alpha F_c + B_c^T diag(w_c)
 * B_c with B_c the cell's nq_c x nd_c basis values (row-major, cells
 * concatenated) and w_c its nq_c weights (cells concatenated); the rest as
 * gbfe_op_assemble_local (KohnShamOperatorContextFE.t.cpp:1253-1311). */
int gbfe_op_assemble_cells(gbfe_op *op, const uint32_t *nq_per_cell, const double *basis_values,
                           const double *weights, const double *fixed_mats, double alpha);
/* Electron density for cells of any size and quadrature rule
 * (DensityCalculator.t.cpp:37-100, 283-345): rho at the nq_c points of each
 * cell (rho_host: sum nq_c values, cells concatenated), basis values as in
 * gbfe_op_assemble_cells.  FP64. */
int gbfe_density_cells(const gbfe_mv *Psi, const double *occupation, const uint32_t *nq_per_cell,
                       const double *basis_values, double *rho_host);
/* The same density with the interpolation psi_c = B_c Psi_c run as the cell
 * product of `basis_op`: a cell operator on Psi's mesh, built without
 * constraints from each cell's basis values B_c (nd_c points x nd_c
 * functions, row-major, uploaded as the cell's "matrix" by
 * gbfe_cellmat_upload), so rho has nd_c points per cell (rho_host: sum nd_c).
 * With GBFE_PREC_FP64_TENSOR and FP64 mode 1 or 2 the product is the sliced
 * FP64-accurate tensor-core kernel; else the FP64 FMA kernel. */
int gbfe_density_op(const gbfe_op *basis_op, gbfe_mv *Psi, const double *occupation, double *rho_host);

/* ---- Chebyshev filters -----------------------------------------------------
 * ResidualChebyshevFilterGEP (linearAlgebra/ChebyshevFilter.t.cpp:242-444).
 * eigenvalues: host array of length m.  X is the input subspace, Y the output.
 * precision: GBFE_F64 runs the recurrence in FP64; GBFE_F32 runs it in FP32
 * with split-BF16 tensor-core cell products (the initial residual and the
 * final reconstruction stay FP64). */
int gbfe_residual_chebyshev_filter(const gbfe_op *A, const gbfe_op *B, const gbfe_op *BInv,
                                   const double *eigenvalues, gbfe_mv *X, uint32_t degree,
                                   double wanted_lower, double wanted_upper,
                                   double unwanted_upper, int precision, gbfe_mv *Y);
/* ChebyshevFilter (ChebyshevFilter.t.cpp:39-135); result in Y (and X). */
int gbfe_chebyshev_filter(const gbfe_op *A, const gbfe_op *BInv, gbfe_mv *X, uint32_t degree,
                          double wanted_lower, double wanted_upper, double unwanted_upper,
                          gbfe_mv *Y);

/* ---- FP64 dense stages -------------------------------------------------------
 * OrthonormalizationFunctions::CholeskyGramSchmidt, serial LAPACK branch
 * (OrthonormalizationFunctions.t.cpp:356-415): S = X^T B X, potrf('L'),
 * trtri('L'), X_o = X S^T (row-major view). */
int gbfe_cholesky_gram_schmidt(const gbfe_op *B, gbfe_mv *X, gbfe_mv *X_ortho);
/* RayleighRitzEigenSolver::solve, LAPACK branch
 * (RayleighRitzEigenSolver.t.cpp:233-301): X^T A X, syevd('V','L'), X Q. */
int gbfe_rayleigh_ritz(const gbfe_op *A, gbfe_mv *X, double *eigenvalues_host, gbfe_mv *X_out);
/* The two dense shapes of those stages, as building blocks:
 * S = X^T Y (X: N x mx, Y: N x my; S mx x my column-major, host) -- the GEMM
 * of computeXTransOpX (RayleighRitzEigenSolver.t.cpp:488-680) -- and
 * Y = X T (T: m x mo column-major, host) -- the rotation gemm of
 * RayleighRitzEigenSolver.t.cpp:233-301.  DGEMM, or with FP64 mode 1
 * (gbfe_ctx_set_fp64_apply) the sliced tensor-core products (m <= 512). */
int gbfe_mv_gram(const gbfe_mv *X, const gbfe_mv *Y, double *S_host);
int gbfe_mv_rotate(const gbfe_mv *X, const double *T_host, gbfe_mv *Y);
/* KohnShamEigenSolver::getLinearEigenSolveResidual
 * (KohnShamEigenSolver.t.cpp:574-684): ||A x_i - eps_i B x_i||_2. */
int gbfe_eigen_residual_norms(const gbfe_op *A, const gbfe_op *B, gbfe_mv *X,
                              const double *eigenvalues, double *norms_host);

/* Electron density at the quadrature points (uniform nd):
 * rho[c][q] = sum_i 2 f_i (sum_a B[q][a] Psi[ids_c[a]][i])^2 with B row-major
 * [nq][nd] (DensityCalculator::computeRho, ksdft/DensityCalculator.t.cpp:
 * 37-100, 283-345).  rho_host: [n_cells][nq]. */
int gbfe_density(const gbfe_mv *Psi, const double *occupation, uint32_t nq, const double *basis_values,
                 double *rho_host);

/* ---- ChFSI ---------------------------------------------------------------- */
typedef struct {
  uint32_t degree;              /* Chebyshev polynomial degree                */
  uint32_t max_passes;          /* maxChebyshevFilterPass                     */
  uint32_t n_wanted;            /* eigenpairs checked for convergence         */
  int      filter_precision;    /* GBFE_F64 or GBFE_F32 (mixed)               */
  double   residual_tol;        /* eigenSolveResidualTolerance               */
  double   wanted_lower;        /* bounds; set use_lanczos=1 to estimate them */
  double   wanted_upper;
  double   unwanted_upper;
  int      use_lanczos;         /* 1: LanczosExtremeEigenSolver-style bounds  */
  uint32_t lanczos_steps;       /* Krylov dimension (reference default 20)    */
  uint64_t lanczos_seed;
  int      fixed_passes;        /* 1: run exactly max_passes passes           */
  int      fp64_apply;          /* as gbfe_ctx_set_fp64_apply, for this solve:
                                   0 FP64 FMA / DGEMM; 1 sliced tensor-core
                                   cell products, Gram matrices and rotations;
                                   2 sliced cell products only                */
  int      faithful_passes;     /* 1: every pass repeats the reference's call
                                   sequence (filter with its own A X, B X;
                                   Cholesky-GS; Rayleigh-Ritz; residual with
                                   fresh H X, M X: six FP64 applies per pass).
                                   0: H X and M X are carried through the
                                   m x m rotations (two FP64 applies per pass). */
  const double *lanczos_start;  /* with use_lanczos: the Lanczos start vector
                                   (n_dofs values, host or device memory; read
                                   once per solve), or NULL for a seeded
                                   uniform [0, 1) vector (lanczos_seed)       */
} gbfe_ks_params;

/* ChebyshevFilteredEigenSolver::solve (ChebyshevFilteredEigenSolver.t.cpp:
 * 194-437): filter -> Cholesky-GS -> Rayleigh-Ritz, one pass.
 * eigenvalues (host, length m) in: previous Ritz values; out: new ones. */
int gbfe_chfsi_pass(const gbfe_op *A, const gbfe_op *B, const gbfe_op *BInv, gbfe_mv *X,
                    double *eigenvalues, uint32_t degree, double wanted_lower,
                    double wanted_upper, double unwanted_upper, int filter_precision);
/* KohnShamEigenSolver::solve pass loop (KohnShamEigenSolver.t.cpp:214-536)
 * without the Fermi-level / occupancy step: bounds, up to max_passes ChFSI
 * passes, residual check on the first n_wanted pairs.  X in: initial block,
 * out: eigenvectors.  eigenvalues/residuals: host arrays of length m. */
int gbfe_ks_eigen_solve(const gbfe_op *A, const gbfe_op *B, const gbfe_op *BInv, gbfe_mv *X,
                        const gbfe_ks_params *params, double *eigenvalues, double *residuals,
                        uint32_t *passes_out);
/* LanczosExtremeEigenSolver-style spectrum bounds of B^-1 A
 * (LanczosExtremeEigenSolver.t.cpp:296-440): out[0] = smallest, out[1] =
 * largest Ritz value, out[2] = last beta (residual). */
int gbfe_lanczos_bounds(const gbfe_op *A, const gbfe_op *B, const gbfe_op *BInv,
                        uint32_t steps, uint64_t seed, double *out3);
/* The same from a given start vector (n_dofs values, host or device memory):
 * the initialGuess constructor argument of LanczosExtremeEigenSolver
 * (LanczosExtremeEigenSolver.t.cpp:94-112). */
int gbfe_lanczos_bounds_from(const gbfe_op *A, const gbfe_op *B, const gbfe_op *BInv,
                             uint32_t steps, const double *start, double *out3);

/* ---- CG -------------------------------------------------------------------
 * CGLinearSolver::solve (linearAlgebra/CGLinearSolver.t.cpp:68-313) with
 * per-component convergence.  x: in initial guess, out solution.
 * Returns GBFE_OK, GBFE_ERR_NOT_CONVERGED or GBFE_ERR_DIVERGED. */
int gbfe_cg_solve(const gbfe_op *A, const gbfe_op *PC, const gbfe_mv *b, gbfe_mv *x,
                  uint32_t max_iter, double abs_tol, double rel_tol, double div_tol,
                  uint32_t *iters_out, double *rnorm_host);

/* Batched CG over independent instances stored as one block-diagonal system
 * (instance i owns dofs [inst_dof_off[i], inst_dof_off[i+1]) of b and x, and
 * A / PC act block-diagonally).  Per instance this is CGLinearSolver::solve
 * (CGLinearSolver.t.cpp:68-313) with one component; all instances advance in
 * the same kernels, their scalars stay on the device, and `iters_chunk`
 * iterations are replayed as one captured CUDA graph between host checks.
 * Outputs per instance (host arrays of n_inst): iterations, status
 * (GBFE_OK / GBFE_ERR_NOT_CONVERGED / GBFE_ERR_DIVERGED) and final residual
 * norm.  Returns GBFE_OK when the call itself succeeded. */
int gbfe_pcg_solve_batched(const gbfe_op *A, const gbfe_op *PC, const gbfe_mv *b, gbfe_mv *x,
                           uint32_t n_inst, const uint64_t *inst_dof_off, uint32_t max_iter,
                           double abs_tol, double rel_tol, double div_tol, uint32_t iters_chunk,
                           uint32_t *iters_out, int *status_out, double *rnorm_out);

/* ---- serving ---------------------------------------------------------------
 * A continuous-batching request loop (no counterpart in the reference, which
 * solves one problem per process).  The server owns `slots` contexts, each with
 * its own CUDA stream and worker thread.  Requests (KS eigen solves or Poisson
 * solves, each on its own mesh) are admitted in arrival order as soon as a slot
 * is free and their estimated HBM footprint fits `hbm_budget_bytes` beside the
 * resident requests; a request that can never fit finishes with
 * GBFE_ERR_ALLOC.  An admitted request keeps its mesh, matrices and vectors
 * resident until it finishes; the kernels of concurrently admitted requests
 * overlap on the device.  A request's result does not depend on the mix. */
typedef struct gbfe_server gbfe_server;

typedef struct {
  uint32_t n_cells;
  const uint32_t *nd_per_cell;
  const uint32_t *cell_dof_ids;
  uint64_t n_dofs;
  uint32_t n_cons_rows;
  const uint32_t *row_ids, *row_sizes, *col_ids, *row_acc;
  const double *col_values, *inhomogeneities;
} gbfe_mesh_desc;

typedef struct {
  int status;              /* the solve's status (GBFE_OK, ..._NOT_CONVERGED, ..._ALLOC, ..._CANCELLED) */
  double t_submit, t_admit, t_done;  /* seconds, steady clock */
  uint32_t passes_or_iters;
  uint64_t footprint_bytes;
  char message[256];
} gbfe_request_info;

int gbfe_server_create(int device, uint32_t slots, uint64_t hbm_budget_bytes, gbfe_server **out);
int gbfe_server_destroy(gbfe_server *server);
/* KS request: H, M cell matrices (gbfe_cellmat_upload layout), the inverse
 * GLL diagonal (and, for enriched meshes, the dense enrichment block of
 * gbfe_diag_block_upload; blk_n = 0 otherwise), the initial block X0 and the
 * solve parameters.  All arrays are copied; the caller may free them. */
int gbfe_server_submit_ks(gbfe_server *server, const gbfe_mesh_desc *mesh, const double *H, const double *M,
                          const double *minv_diag, uint64_t blk_begin, uint64_t blk_n, const double *blk,
                          const double *X0, uint32_t m, const gbfe_ks_params *params, uint64_t *id_out);
/* Poisson request: indexed Laplace matrices (gbfe_cellmat_upload_indexed),
 * the Jacobi diagonal, the right-hand side and the CG tolerances. */
int gbfe_server_submit_poisson(gbfe_server *server, const gbfe_mesh_desc *mesh, uint32_t n_mats,
                               const double *mats, const uint32_t *cell_to_mat, const double *jacobi_diag,
                               const double *b, uint32_t max_iter, double abs_tol, double rel_tol,
                               double div_tol, uint64_t *id_out);
/* Queued requests are dropped; running ones stop at their next pass/iteration
 * boundary with GBFE_ERR_CANCELLED. */
int gbfe_server_cancel(gbfe_server *server, uint64_t id);
/* Blocks until request `id` finishes or `timeout_s` passes (GBFE_ERR_TIMEOUT). */
int gbfe_server_wait(gbfe_server *server, uint64_t id, double timeout_s, gbfe_request_info *info);
/* KS: eigenvalues and residual norms (m each); Poisson: the solution (n_dofs). */
int gbfe_server_result(gbfe_server *server, uint64_t id, double *values, double *residuals);
int gbfe_server_release(gbfe_server *server, uint64_t id);
int gbfe_server_stats(gbfe_server *server, uint64_t *admitted, uint64_t *completed, uint64_t *rejected,
                      uint64_t *used_bytes, uint32_t *queued);
/* Continuous batching of Poisson requests: when a Poisson request is admitted,
 * the queued Poisson requests with the same iteration limit and tolerances
 * join it (up to the batch limit, default 32, and the HBM budget) and all run
 * as one batched solve (gbfe_pcg_solve_batched over the concatenated meshes).
 * Each instance's arithmetic is that of a solve of its own, so results do not
 * depend on the batch; a running batch is not cancellable.  Counters: batches
 * of two or more requests, and the requests they carried. */
int gbfe_server_batch_stats(gbfe_server *server, uint64_t *poisson_batches, uint64_t *poisson_batched_requests);
/* Largest Poisson batch (1 turns batching off). */
int gbfe_server_set_max_batch(gbfe_server *server, uint32_t max_poisson_batch);
/* Fault injection for tests (host side): the next `count` admitted requests
 * (a batch counts as one) fail their device upload with GBFE_ERR_ALLOC. */
int gbfe_server_inject_alloc_failures(gbfe_server *server, int count);

#ifdef __cplusplus
}
#endif
#endif /* GBFE_H */
