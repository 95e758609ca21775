/*
 * mpdok_gb300 — C ABI of the GB300-native dense-operator Krylov solvers.
 *
 * Two layers are exported:
 *
 *  1. The reference's own ctypes ABI (the symbols MPDOK's mpdok_ops.py binds
 *     to mpdok.so / lu_ir.so).  Same names, argument order, argument meaning
 *     and out-parameter conventions: device (or managed) pointers, A in
 *     column-major (Fortran) order, void return, status through int*
 *     out-parameters, the caller synchronises the null stream afterwards.
 *     Like the reference these keep one process-wide saved factorization.
 *
 *  2. The handle-free mpdok_* API: explicit cudaStream_t, caller-owned
 *     workspace sized by *_workspace_size(), int status return
 *     (0 ok, <0 error, >0 numerical information), no hidden globals.
 *
 * All compute runs in hand-written sm_103a kernels; nothing here falls back
 * to the CPU.
 */
#ifndef MPDOK_GB300_H
#define MPDOK_GB300_H

#include <stddef.h>
#include <cuda_runtime.h>

#if defined(__GNUC__)
#define MPDOK_API __attribute__((visibility("default")))
#else
#define MPDOK_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
enum {
  MPDOK_OK = 0,
  MPDOK_ERR_INVALID_ARG = -1,
  MPDOK_ERR_CUDA = -2,
  MPDOK_ERR_ALLOC = -3,
  MPDOK_ERR_NOT_FACTORED = -4,
  MPDOK_ERR_TIMEOUT = -5,     /* a bounded device-side wait gave up */
  MPDOK_ERR_UNSUPPORTED = -6,
  MPDOK_ERR_IO = -7,
  MPDOK_ERR_NONFINITE = -8    /* NaN / Inf met in a residual or pivot */
};

/* element types */
enum { MPDOK_F64 = 0, MPDOK_F32 = 1, MPDOK_BF16 = 2, MPDOK_F16 = 3 };
/* radial basis functions: Gaussian exp(-gamma r^2), multiquadric sqrt(1 + gamma r^2) */
enum { MPDOK_KERNEL_GAUSSIAN = 0, MPDOK_KERNEL_MQ = 1 };

#define MPDOK_HISTORY_MAX 256

/* Per-solve report: outer FP64 relative residual history and counters. */
typedef struct mpdok_solve_info {
  int converged;          /* 1 when the FP64 relative residual fell below tol */
  int outer_iters;        /* outer refinement steps (or restarts / CG checks) */
  int inner_iters;        /* total inner matvecs */
  int stagnated;          /* 1: the 1 % stagnation rule stopped the solve; 2: the residual diverged and the
                             best iterate was restored (mpdok_lu_gmres_ir) */
  double relres;          /* final FP64 ||b - A x|| / ||b|| */
  double bnorm;           /* ||b|| */
  int n_history;          /* entries used in history[] */
  int hist_iter[MPDOK_HISTORY_MAX];   /* iteration index of each entry */
  double history[MPDOK_HISTORY_MAX];  /* FP64 relative residual of each entry */
} mpdok_solve_info;

MPDOK_API int mpdok_version(void);
MPDOK_API const char* mpdok_status_string(int status);
/* Message of the last error raised on the calling host thread. */
MPDOK_API const char* mpdok_last_error(void);
/* Empty that message, so that a caller can tell whether the next call (for
 * example a py_* entry point, which returns no status) raised an error. */
MPDOK_API void mpdok_clear_error(void);

/* Test hooks for the failure paths; no counterpart in the reference.
 * MPDOK_DEBUG_WAIT_LIMIT: iteration limit of the triangular solves' bounded
 *   waits on a predecessor block, on the current device (value <= 0 restores
 *   the default).
 * MPDOK_DEBUG_TRSV_FIRST_TICKET: first ticket that the next triangular solves
 *   of this process hand out (0 = normal).  With a value above 0 no block ever
 *   solves block 0, so the blocks that depend on it wait until their limit
 *   runs out, return, and the solve reports MPDOK_ERR_TIMEOUT; the device
 *   stays usable.  Returns a status. */
enum { MPDOK_DEBUG_WAIT_LIMIT = 1, MPDOK_DEBUG_TRSV_FIRST_TICKET = 2 };
MPDOK_API int mpdok_debug_set(int key, long long value);

/* ------------------------------------------------------------ assembly
 * out(i, j) = phi(||rows_i - cols_j||) + reg * [i + diag_offset == j]
 * rows: (n_rows, dim) and cols: (n_cols, dim) FP64, row-major (C order).
 * out: column-major with leading dimension ld (col_major != 0) or row-major.
 * Replaces rbf_kernel.py:158-227 (build_rbf_kernel) and mpdok_ooc.py:39-46
 * (_build_fp32_tile).  FP64 output computes in FP64; FP32/BF16/FP16 in FP32. */
MPDOK_API int mpdok_rbf_assemble(const double* rows, long long n_rows, const double* cols, long long n_cols,
                       int dim, int kernel, double gamma, double reg, long long diag_offset,
                       int out_dtype, void* out, long long ld, int col_major, cudaStream_t stream);

/* Elementwise type conversion of n contiguous elements (the FP64 -> FP32
 * copy of A that py_gmres_ir makes, mpdok_ops.py:329-333 / dense_krylov.py:47). */
MPDOK_API int mpdok_convert(const void* src, int src_dtype, void* dst, int dst_dtype, long long n, cudaStream_t stream);

/* ---------------------------------------------------------------- GEMV
 * Y = alpha * op(A) X + beta * Y, A column-major (m x n, lda), op = A or A^T.
 * X / Y are FP64 when A is FP64 and FP32 otherwise; nrhs columns.
 * Replaces cp.matmul(A_fp32, x) (dense_krylov.py:61-63). */
MPDOK_API size_t mpdok_gemv_workspace_size(int a_dtype, long long m, long long n, int nrhs, int trans);
MPDOK_API int mpdok_gemv(int a_dtype, int trans, const void* A, long long lda, long long m, long long n,
               const void* X, long long ldx, int nrhs, void* Y, long long ldy, double alpha, double beta,
               void* work, size_t work_bytes, cudaStream_t stream);

/* Same product as mpdok_gemv for callers that cannot allocate device memory
 * (their GPU memory is already committed to another pool, or they must not
 * cause the device synchronisation an allocation can bring).  No counterpart
 * in the reference.  The scratch is a built-in device array of
 * MPDOK_NOALLOC_SCRATCH_BYTES, held by every GPU that loads the library until
 * the process exits; products that need more return MPDOK_ERR_INVALID_ARG.
 * The first call on a device looks up that array's device address (with the
 * device current), so make it before any stream capture.  The address is kept
 * for the life of the process: after a cudaDeviceReset in the same process it
 * is stale, so do not call this entry point again after a reset.  All calls share
 * the array: calls that overlap on the GPU (concurrent streams, or other host
 * threads) race on it and must be serialised by the caller.  Nothing is
 * allocated or freed. */
#define MPDOK_NOALLOC_SCRATCH_BYTES (16u << 20)
MPDOK_API int mpdok_gemv_noalloc(int a_dtype, int trans, const void* A, long long lda, long long m, long long n,
                                 const void* X, long long ldx, int nrhs, void* Y, long long ldy, double alpha,
                                 double beta, cudaStream_t stream);

/* r = b - A x in FP64 and *rnorm2 = ||r||^2 (device scalar); workspace as
 * mpdok_gemv_workspace_size(MPDOK_F64, n, n, 1, 0).
 * Replaces DenseLinearOperator.residual_norm (dense_krylov.py:65-79). */
MPDOK_API int mpdok_residual(const double* A, long long lda, long long n, const double* b, const double* x,
                   double* r, double* rnorm2, void* work, size_t work_bytes, cudaStream_t stream);

/* ------------------------------------------------------- Krylov drivers
 * All vectors are device pointers; A32 is the FP32 copy of A (column-major,
 * lda32), A64 the FP64 matrix used for residuals.  The solve stays on the
 * device; the host reads one scalar per outer step. */
MPDOK_API size_t mpdok_krylov_workspace_size(long long n, int restart);

/* GMRES-IR, the algorithm of mpdok_ooc.py:315-373 with the inner solve of
 * mpdok_ooc.py:231-311 (Arnoldi, two-pass classical Gram-Schmidt, FP64
 * Givens rotations, early stop |g_{k+1}|/beta < inner_tol), which the
 * reference labels as its port of the native py_gmres_ir.
 * x holds the initial guess on entry and the FP64 solution on exit.
 * a32_ready != 0 skips the FP64 -> FP32 conversion into A32. */
MPDOK_API int mpdok_gmres_ir(const double* A64, long long lda, float* A32, long long lda32, int a32_ready,
                   long long n, const double* b, double* x, double tol, int maxiter_outer, int restart,
                   double inner_tol, void* work, size_t work_bytes, mpdok_solve_info* info,
                   cudaStream_t stream);

/* Restarted FP32 GMRES(m) of dense_krylov.py:212-331 (single Gram-Schmidt
 * pass, FP64 residual check at each restart, 1 % stagnation stop).
 * x: FP64 initial guess in, FP64 (promoted FP32 iterate) out. */
MPDOK_API int mpdok_gmres(const float* A32, long long lda32, const double* A64, long long lda, long long n,
                const double* b, double* x, double tol, int maxiter, int restart, void* work,
                size_t work_bytes, mpdok_solve_info* info, cudaStream_t stream);

/* GMRES-IR of dense_krylov.py:338-421: FP64 residual, inner restarted FP32
 * GMRES (tol 1e-6, maxiter_inner), FP64 update, final residual. */
MPDOK_API int mpdok_dense_gmres_ir(const float* A32, long long lda32, const double* A64, long long lda, long long n,
                         const double* b, double* x, double tol, int maxiter_outer, int restart,
                         int maxiter_inner, void* work, size_t work_bytes, mpdok_solve_info* info,
                         cudaStream_t stream);

/* FP32 conjugate gradients of dense_krylov.py:119-205 (FP64 residual check
 * every check_every iterations, 1 % stagnation stop). */
MPDOK_API int mpdok_cg(const float* A32, long long lda32, const double* A64, long long lda, long long n,
             const double* b, double* x, double tol, int maxiter, int check_every, void* work,
             size_t work_bytes, mpdok_solve_info* info, cudaStream_t stream);

/* -------------------------------------------------- matrix-free RBF operator
 * Y = K(rows, cols) X + reg X[diag_offset:] where K(i, j) = phi(||r_i - c_j||),
 * recomputed on the fly (A never stored): FP32 (X, Y float; column tiles
 * staged by TMA, exp2 / rsqrt on the special-function pipe) or FP64 (X, Y
 * double; residual accuracy).  Replaces mpdok_ooc.py:205-227 (matrix-free
 * FP64 residual) and the stored FP32 operator of the inner solves.
 * FP32 X must be 16-byte aligned with ldx % 4 == 0.  nrhs in 1..8. */
MPDOK_API size_t mpdok_matfree_workspace_size(long long n_rows, long long n_cols, int nrhs, int precision);
MPDOK_API int mpdok_matfree_apply(const double* rows, long long n_rows, const double* cols, long long n_cols, int dim,
                                  int kernel, double gamma, double reg, long long diag_offset, int precision,
                                  const void* X, long long ldx, int nrhs, void* Y, long long ldy, void* work,
                                  size_t work_bytes, cudaStream_t stream);
/* GMRES-IR (inner tol, restart as mpdok_gmres_ir) and CG (as mpdok_cg) on the
 * matrix-free operator of one RBF system (coords (n, dim) FP64): FP32
 * evaluate-and-multiply inside, FP64 evaluate-and-multiply residuals. */
MPDOK_API size_t mpdok_mf_krylov_workspace_size(long long n, int restart);
MPDOK_API int mpdok_mf_gmres_ir(const double* coords, long long n, int dim, int kernel, double gamma, double reg,
                                const double* b, double* x, double tol, int maxiter_outer, int restart,
                                double inner_tol, void* work, size_t work_bytes, mpdok_solve_info* info,
                                cudaStream_t stream);
MPDOK_API int mpdok_mf_cg(const double* coords, long long n, int dim, int kernel, double gamma, double reg,
                          const double* b, double* x, double tol, int maxiter, int check_every, void* work,
                          size_t work_bytes, mpdok_solve_info* info, cudaStream_t stream);

/* ------------------------------------------------ split operator and CG-IR
 * Split A = A_hi + A_lo into two FP32 slices (hi = fl32(a), lo = fl32(a - hi));
 * mpdok_split_gemv forms Y = alpha (A_hi + A_lo) X + beta B with error-free
 * FP32 products and double-float sums (FP64-level accuracy on the FP32 pipe;
 * X, Y, B FP64; slices 16-byte aligned with ld % 4 == 0). */
MPDOK_API int mpdok_split_matrix(const double* A, long long lda, long long m, long long n, float* hi, float* lo,
                                 long long ld, cudaStream_t stream);
MPDOK_API size_t mpdok_split_gemv_workspace_size(long long m, long long n, int nrhs);
MPDOK_API int mpdok_split_gemv(const float* hi, const float* lo, long long ld, long long m, long long n,
                               const double* X, long long ldx, int nrhs, double* Y, long long ldy, double alpha,
                               double beta, const double* B, long long ldb, void* work, size_t work_bytes,
                               cudaStream_t stream);
/* Multi-RHS CG-IR (C2 family): FP64 residual R = B - A X, inner FP32 CG on
 * A E = R for all nrhs (<= 8) columns in lockstep, X += E in FP64.  mode 0:
 * FP32 copy of A inside + native FP64 residual; mode 1: split A for both.
 * opbuf holds the FP32 copy or the two slices (mpdok_cg_ir_operator_size);
 * op_ready != 0 reuses it.  info->history holds the worst column's relres. */
MPDOK_API size_t mpdok_cg_ir_operator_size(long long n, int mode);
MPDOK_API size_t mpdok_cg_ir_workspace_size(long long n, int nrhs, int mode);
MPDOK_API int mpdok_cg_ir(const double* A64, long long lda, long long n, int mode, void* opbuf, int op_ready,
                          int nrhs, const double* B, long long ldb, double* X, long long ldx, double tol,
                          int maxiter_outer, double inner_tol, int inner_maxiter, void* work, size_t work_bytes,
                          mpdok_solve_info* info, cudaStream_t stream);
MPDOK_API size_t mpdok_mf_cg_ir_workspace_size(long long n, int nrhs);
MPDOK_API int mpdok_mf_cg_ir(const double* coords, long long n, int dim, int kernel, double gamma, double reg,
                             int nrhs, const double* B, long long ldb, double* X, long long ldx, double tol,
                             int maxiter_outer, double inner_tol, int inner_maxiter, void* work, size_t work_bytes,
                             mpdok_solve_info* info, cudaStream_t stream);

/* CG-IR whose inner CG is preconditioned by an FP64-accurate Cholesky factor:
 * a batch plan (below) of one system of size n with nrhs equal to this
 * solve's nrhs, loaded and factored (mpdok_batch_factor).  For SPD systems
 * too ill-conditioned for any FP32 CG body (kappa * 6e-8 > 1, the C2
 * family) the inner PCG keeps FP64 vectors (an FP32 correction would move the
 * residual by up to kappa * 6e-8), converges in a few steps and the FP64
 * refinement reaches the FP64 floor.  mode 0: stored FP64 A64 (opbuf
 * unused); 1: the inner products from split A64 (two FP32 slices in opbuf,
 * mpdok_cg_ir_operator_size(n, 1); error-free FP32 products, about 2^-48 on
 * the FP32 pipe), the FP64 residual from A64; 2: matrix-free from coords
 * (dim, kernel, gamma, reg; A64 / opbuf unused).
 * The reference's cg (dense_krylov.py:119-205) with its FP64 residual check,
 * made convergent on this family by the preconditioner. */
MPDOK_API size_t mpdok_chol_cg_ir_workspace_size(long long n, int nrhs, int mode);
MPDOK_API int mpdok_chol_cg_ir(void* plan, const double* A64, long long lda, const double* coords, int dim,
                               int kernel, double gamma, double reg, long long n, int mode, void* opbuf, int op_ready,
                               int nrhs, const double* B, long long ldb, double* X, long long ldx, double tol,
                               int maxiter_outer, double inner_tol, int inner_maxiter, void* work, size_t work_bytes,
                               mpdok_solve_info* info, cudaStream_t stream);

/* ----------------------------------------------------------- LU (tensor cores)
 * Blocked right-looking LU with FP32 panels and a trailing update
 * W22 -= L21 U12 whose operands are rounded to the factor type: BF16 / FP16
 * run on tcgen05 tensor cores (FP32 accumulation in tensor memory), FP32 on
 * CUDA cores (the reference's Sgetrf precision, benchmark_mpdok.ipynb:982-993).
 *
 * pivoting = 0: W = D A D (D = diag(1/sqrt|a_ii|), symmetric scaling), no row
 *   exchanges (SPD / diagonally dominant systems, e.g. Gaussian RBF); pivots
 *   below 1e-6 in magnitude are replaced by +-1e-6.  Return: 0 ok, > 0 the
 *   number of pivots that had to be perturbed (still a usable preconditioner).
 * pivoting = 1: W = Dr A Dc (power-of-two row and column equilibration),
 *   P W = L U with partial pivoting by rows, as cusolverDnSgetrf / LAPACK
 *   getrf (the reference's lu_ir.so, benchmark_mpdok.ipynb:989-990).  Return:
 *   LAPACK's info, 0 ok or i > 0 when U(i, i) is exactly zero (1-based; the
 *   factors are then singular).  n is limited by the panel factorization,
 *   which keeps the panel's rows in the shared memory of co-resident CTAs
 *   (about 65000 rows on a GB300): larger n returns MPDOK_ERR_UNSUPPORTED.
 * Both: < 0 error.
 *
 * Factors live in a caller-owned device buffer of mpdok_lu_factor_size()
 * bytes; factorization scratch is mpdok_lu_work_size() bytes. */
enum { MPDOK_ENGINE_TENSOR = 0, MPDOK_ENGINE_SIMT = 1 };

MPDOK_API int mpdok_gemm_update(float* C, long long ldc, const void* A, const void* B, int M, int N, int K,
                                int fdtype, int engine, int* err, cudaStream_t stream);
MPDOK_API size_t mpdok_lu_factor_size(long long n, int fdtype);
MPDOK_API size_t mpdok_lu_work_size(long long n, int fdtype);
MPDOK_API int mpdok_lu_factor(const double* A, long long lda, long long n, int fdtype, int pivoting, void* factors,
                              size_t factor_bytes, void* work, size_t work_bytes, cudaStream_t stream);
/* The launch schedule of mpdok_lu_factor for n and fdtype, host only (no
 * device call): every launch, event record and event wait across its three
 * streams (0 caller's, 1 chain, 2 strip), in issue order.  12 integers per
 * step: kind (0 diagonal LU, 1 panel solve, 2 trailing update, 3 event record,
 * 4 event wait, 5 / 6 profiling window start / stop), stream, J (super-panel
 * start), jp (panel start), a, b (solve: rows and columns [a, b); update:
 * first C row and column), m, nn (update extent), K, koff (update depth and
 * operand K-slot), rb (solve rows per block), event.  Writes at most
 * max_steps steps (out may be NULL); returns the number of steps or a
 * negative status. */
MPDOK_API long long mpdok_lu_schedule(long long n, int fdtype, long long* out, long long max_steps);
/* The factors in plain form (device outputs, each may be NULL): L\U as an
 * n x n column-major FP32 matrix (unit L below the diagonal), the 0-based
 * pivot rows (LAPACK's ipiv; the identity for unpivoted factors), the row
 * permutation as a gather ((P x)_i = x_perm[i]) and the scalings Dr, Dc,
 * with P (Dr A Dc) = L U. */
MPDOK_API int mpdok_lu_export(const void* factors, long long n, int fdtype, float* lu, long long ldo, int* ipiv,
                              int* perm, float* dr, float* dc, cudaStream_t stream);
/* z = (Dc U^-1 L^-1 P Dr) v: one application of the factorization (FP32 vectors). */
MPDOK_API size_t mpdok_lu_apply_work_size(long long n);
MPDOK_API int mpdok_lu_apply(const void* factors, long long n, int fdtype, const float* v, float* z, void* work,
                             size_t work_bytes, cudaStream_t stream);
/* LU-IR (benchmark_mpdok.ipynb:982-993): x = LU^-1 b, then FP64 residual,
 * correction solve with the factors, FP64 update, until relres < tol. */
MPDOK_API size_t mpdok_lu_ir_work_size(long long n);
MPDOK_API int mpdok_lu_ir_solve(const double* A, long long lda, long long n, const void* factors, int fdtype,
                                const double* b, double* x, double tol, int maxiter_outer, void* work,
                                size_t work_bytes, mpdok_solve_info* info, cudaStream_t stream);
/* Three-precision GMRES-IR: the LU (BF16/FP16) preconditions FP32 GMRES on
 * the FP32 copy of A (right preconditioning), FP64 residual r = b - A x and
 * FP64 update x += d, FP64 Hessenberg / Givens. */
/* LU-IR on nrhs <= 8 right-hand sides together (the reference's
 * LUIRSolver.solve_factored, mpdok_ops.py:280-320, batched over the fields of
 * its time-series use): X = LU^-1 B, then R = B - A X in FP64 (one multi-RHS
 * GEMV) and X += LU^-1 R (one multi-RHS triangular sweep pair, each factor
 * tile read once for all columns) until max_k ||R_k|| / ||B_k|| < tol or
 * maxiter_outer corrections.  info->relres is the worst column. */
MPDOK_API size_t mpdok_lu_ir_multi_work_size(long long n, int nrhs);
MPDOK_API int mpdok_lu_ir_solve_multi(const double* A, long long lda, long long n, const void* factors, int fdtype,
                                      int nrhs, const double* B, long long ldb, double* X, long long ldx, double tol,
                                      int maxiter_outer, void* work, size_t work_bytes, mpdok_solve_info* info,
                                      cudaStream_t stream);
MPDOK_API size_t mpdok_lu_gmres_ir_work_size(long long n, int restart);
MPDOK_API int mpdok_lu_gmres_ir(const double* A64, long long lda, const float* A32, long long lda32, long long n,
                                const void* factors, int fdtype, const double* b, double* x, double tol,
                                int maxiter_outer, int restart, double inner_tol, void* work, size_t work_bytes,
                                mpdok_solve_info* info, cudaStream_t stream);

/* CG-IR preconditioned by the factors (PCG inner, z = (LU)^-1 r per column),
 * for SPD systems too ill-conditioned for an unpreconditioned FP32 CG body.
 * op_mode 0 / 1 as mpdok_cg_ir; mpdok_mf_lu_cg_ir applies A matrix-free.
 * Workspace: mpdok_lu_cg_ir_workspace_size(n, nrhs, op_mode) with op_mode 2
 * for the matrix-free entry. */
MPDOK_API size_t mpdok_lu_cg_ir_workspace_size(long long n, int nrhs, int op_mode);
MPDOK_API int mpdok_lu_cg_ir(const double* A64, long long lda, long long n, int op_mode, void* opbuf, int op_ready,
                             const void* factors, int fdtype, int nrhs, const double* B, long long ldb, double* X,
                             long long ldx, double tol, int maxiter_outer, double inner_tol, int inner_maxiter,
                             void* work, size_t work_bytes, mpdok_solve_info* info, cudaStream_t stream);
MPDOK_API int mpdok_mf_lu_cg_ir(const double* coords, long long n, int dim, int kernel, double gamma, double reg,
                                const void* factors, int fdtype, int nrhs, const double* B, long long ldb, double* X,
                                long long ldx, double tol, int maxiter_outer, double inner_tol, int inner_maxiter,
                                void* work, size_t work_bytes, mpdok_solve_info* info, cudaStream_t stream);

/* -------------------------------------------------------- out-of-core (OOC)
 * FP32 A of an RBF system kept outside HBM and streamed per product
 * (mpdok_ooc.py:51-383).  store 0: pinned host RAM (N*N*4 bytes, allocated
 * here); store 1: raw row-major FP32 file without a header at `path` (the
 * reference's SSD format), read through pinned staging.  Tiles of tile_rows
 * rows are copied on a side stream into a ring of device buffers while the
 * previous tile is multiplied.  The handle owns its device buffers. */
MPDOK_API int mpdok_ooc_create(long long n, int tile_rows, int store, const char* path, void** handle);
MPDOK_API int mpdok_ooc_destroy(void* handle);
MPDOK_API int mpdok_ooc_build(void* handle, const double* coords, int dim, int kernel, double gamma, double reg,
                              cudaStream_t stream);
MPDOK_API int mpdok_ooc_matvec(void* handle, const float* x, float* y, cudaStream_t stream);
MPDOK_API double mpdok_ooc_bytes_moved(void* handle);
/* Host copy of rows [row0, row0 + rows) of the stored matrix (row-major FP32). */
MPDOK_API int mpdok_ooc_read_rows(void* handle, long long row0, long long rows, float* dst);
/* GMRES-IR of MPDOKOOCSolver.solve: outer FP64 residual recomputed matrix-free
 * from coords, inner FP32 GMRES on the streamed operator. */
MPDOK_API size_t mpdok_ooc_workspace_size(long long n, int restart);
MPDOK_API int mpdok_ooc_gmres_ir(void* handle, const double* coords, int dim, int kernel, double gamma, double reg,
                                 const double* b, double* x, double tol, int maxiter_outer, int restart,
                                 double inner_tol, void* work, size_t work_bytes, mpdok_solve_info* info,
                                 cudaStream_t stream);

/* ------------------------------------------------------------------ batched
 * Many SPD RBF systems of uneven size, each with nrhs <= 8 right-hand sides:
 * A_s = phi(eps_s * ||c_i - c_j||) + reg_s I (gamma = eps^2).  A plan holds
 * the FP64 matrices (lower triangle overwritten by the Cholesky factor, upper
 * triangle kept for the FP64 residual), the diagonal-block inverses and the
 * level schedule (systems sorted by N; one launch per level covers every
 * active system).  arith 1 runs the O(N^3) trailing update in double-float
 * on the FP32 pipe, arith 0 in FP64; everything else is FP64.  grid_mult
 * scales the persistent trailing-update grid (resident CTAs x SMs x mult).
 * Packing (caller order): coords = concatenated (n_s x dim) row-major;
 * B / X = concatenated (n_s x nrhs) column-major blocks.  All device
 * pointers.  Not in the reference; the batched workload of the Python layer. */
MPDOK_API int mpdok_batch_create(int nsys, const long long* n, int dim, int nrhs, int kernel, int arith,
                                 int grid_mult, void** plan);
MPDOK_API int mpdok_batch_destroy(void* plan);
MPDOK_API size_t mpdok_batch_bytes(void* plan);
/* coords on the device; eps, reg on the host (nsys each). */
MPDOK_API int mpdok_batch_load(void* plan, const double* coords, const double* eps, const double* reg,
                               cudaStream_t stream);
/* Assemble and factor every system (no host synchronisation). */
MPDOK_API int mpdok_batch_factor(void* plan, cudaStream_t stream);
/* X = A^{-1} B with `refine` FP64 refinement steps (no host synchronisation). */
MPDOK_API int mpdok_batch_solve(void* plan, const double* B, double* X, int refine, cudaStream_t stream);
/* relres[s] = max over RHS of ||B - A X|| / ||B|| (device array, caller order). */
MPDOK_API int mpdok_batch_relres(void* plan, const double* B, const double* X, double* relres, cudaStream_t stream);
/* Gradients of a loss L(X) from Lam = A^{-1} dL/dX: grad_coords packed like
 * coords, grad_eps and grad_reg (nsys, device).  phi recomputed in FP64. */
MPDOK_API int mpdok_batch_adjoint(void* plan, const double* X, const double* Lam, double* grad_coords,
                                  double* grad_eps, double* grad_reg, cudaStream_t stream);
/* The gradient contraction of ONE system (the in-core solvers' adjoint):
 * with A = phi_eps(||c_i - c_j||) + reg I (gamma = eps^2), X the solution and
 * Lam = A^-1 dL/dX (n x nrhs column-major, ld n, nrhs <= 8):
 *   grad_coords (n x dim row-major) = dL/dc,  *grad_eps = dL/deps,
 *   *grad_reg = dL/dreg  (= -sum Lam .* X),
 * phi and its derivatives recomputed in FP64 from the coordinates (dA is
 * never stored).  Workspace: mpdok_rbf_adjoint_workspace_size(n) bytes.
 * Synchronises the stream. */
MPDOK_API size_t mpdok_rbf_adjoint_workspace_size(long long n);
MPDOK_API int mpdok_rbf_adjoint(const double* coords, long long n, int dim, int kernel, double eps, int nrhs,
                                const double* X, const double* Lam, double* grad_coords, double* grad_eps,
                                double* grad_reg, void* work, size_t work_bytes, cudaStream_t stream);
/* Pivots perturbed by the last factorization (synchronises the stream). */
MPDOK_API int mpdok_batch_perturbed(void* plan, cudaStream_t stream);
/* Capture factor + solve (+ refine) on fixed B / X into one CUDA graph, then
 * replay it with one launch. */
MPDOK_API int mpdok_batch_graph_build(void* plan, const double* B, double* X, int refine);
MPDOK_API int mpdok_batch_graph_launch(void* plan, cudaStream_t stream);
MPDOK_API long long mpdok_batch_graph_nodes(void* plan);
/* Schedule of mpdok_batch_step and of the captured graph.  0: level
 * synchronous, three launches per 64-column block level (diagonal factor,
 * panel solve, trailing update over every active system) plus the level
 * scheduled solves.  1: the whole step as ONE persistent launch of
 * ctas_per_sm (1..3) CTAs per SM that take tile tasks (assembly, Cholesky,
 * solve, FP64 refinement) from a queue in a topological order and start each
 * one as soon as its inputs are final; results are bit-identical to 0. */
MPDOK_API int mpdok_batch_schedule(void* plan, int schedule, int ctas_per_sm);
/* One step on B / X: assembly + factor + solve + `refine` refinement steps
 * under the plan's schedule (no host synchronisation). */
MPDOK_API int mpdok_batch_step(void* plan, const double* B, double* X, int refine, cudaStream_t stream);
/* MPDOK_ERR_TIMEOUT when a task of the last task-graph step gave up waiting
 * on its inputs (synchronises the stream), else 0. */
MPDOK_API int mpdok_batch_dag_status(void* plan, cudaStream_t stream);

/* --------------------------------------------------------- instrumentation
 * mpdok_launch_count: kernels launched by this library since load.
 * mpdok_profile_enable(1) clears and starts per-launch CUDA-event timing of
 * the kernel classes below (on the launching stream); mpdok_profile_query
 * sums, after the work has completed, the device time, the number of
 * launches and the algorithmic work (bytes or flops) of one class. */
enum {
  MPDOK_PROF_GEMV_F32 = 0,   /* stored FP32 / 16-bit GEMV stage (bytes)  */
  MPDOK_PROF_GEMV_F64 = 1,   /* stored FP64 GEMV stage (bytes)           */
  MPDOK_PROF_ASSEMBLE = 2,   /* RBF assembly (bytes written)             */
  MPDOK_PROF_LU_GEMM = 3,    /* LU trailing-update GEMM, K < 128 or the
                                SIMT engine, and the FP32-factor update
                                (flops)                                  */
  MPDOK_PROF_TRSV = 4,       /* triangular solves (bytes)                */
  MPDOK_PROF_MATFREE = 5,    /* matrix-free evaluate-and-multiply (entries) */
  MPDOK_PROF_OOC_COPY = 6,   /* host -> device tile copies (bytes)       */
  MPDOK_PROF_LU_PANEL = 7,   /* LU panel factorization (flops)           */
  MPDOK_PROF_LU_GEMM_DEEP = 8 /* LU trailing-update GEMM with K >= 128: the
                                warp-specialised tensor-core kernel (flops) */
};
MPDOK_API long long mpdok_launch_count(void);
MPDOK_API int mpdok_profile_enable(int on);
MPDOK_API int mpdok_profile_query(int kernel_class, double* total_ms, long long* launches, double* work);
/* Launches of the class that a device skip flag turned off (a finished
 * Arnoldi cycle): excluded from mpdok_profile_query's totals. */
MPDOK_API long long mpdok_profile_skipped(int kernel_class);
/* Algorithmic bytes of a class whose work counts flops (MPDOK_PROF_LU_GEMM*:
 * the FP32 C tile read and written plus the operands), for its HBM roofline. */
MPDOK_API double mpdok_profile_bytes(int kernel_class);
/* Timeline of every timed launch since mpdok_profile_enable, in launch order:
 * out[4 i .. 4 i + 3] = (class, start ms, end ms, work), times relative to the
 * first launch's start event, each on its own stream.  Writes at most
 * max_records records (out may be NULL) and returns the number of records,
 * or a negative MPDOK status. */
MPDOK_API long long mpdok_profile_timeline(double* out, long long max_records);

/* ------------------------------------------- reference ctypes ABI (mpdok.so)
 * mpdok_ops.py:362-373: A (N x N FP64, Fortran order), b, x (FP64, x is the
 * output and starts as zeros), A_fp32 caller-owned FP32 scratch (N x N,
 * Fortran order) that receives the FP32 copy of A; converged_out = 1 / 0. */
MPDOK_API void py_gmres_ir(double* A, double* b, double* x, float* A_fp32, int N, double tol, int maxiter_outer,
                 int restart, int* converged_out);
/* mpdok_ops.py:375-382: (N, N) FP64 managed allocation, kept until
 * py_free_managed(). */
/* Placement of the last py_alloc_managed / py_lu_alloc_managed buffer: 0 device
 * memory (the normal case on GB300), 1 managed memory placed on the device
 * (when a device allocation of that size failed), -1 failure. */
MPDOK_API int mpdok_managed_kind(void);
MPDOK_API void py_alloc_managed(int N, void** ptr_out);
MPDOK_API void py_free_managed(void);

/* ------------------------------------------- reference ctypes ABI (lu_ir.so)
 * mpdok_ops.py:101-141.  A FP64 N x N Fortran order (device or managed),
 * b / x FP64 (x output).  py_lu_factor stores one process-wide FP32
 * factorization (info_out: 0 ok, > 0 pivots perturbed, < 0 error);
 * py_lu_solve_factored refines with it (converged_out = 1 / 0, -1 when no
 * factorization of size N exists); py_lu_ir = factor + solve. */
MPDOK_API void py_lu_ir(double* A, double* b, double* x, int N, double tol, int maxiter_outer, int* converged_out);
MPDOK_API void py_lu_factor(double* A, int N, int* info_out);
MPDOK_API void py_lu_solve_factored(double* A, double* b, double* x, int N, double tol, int maxiter_outer,
                                    int* converged_out);
MPDOK_API void py_lu_free_factored(void);
MPDOK_API void py_lu_alloc_managed(int N, void** ptr_out);
MPDOK_API void py_lu_free_managed(void);

#ifdef __cplusplus
}
#endif

#endif /* MPDOK_GB300_H */
