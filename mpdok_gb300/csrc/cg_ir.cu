// Multi-right-hand-side CG with FP64 iterative refinement (CG-IR).
//
// The reference's cg (dense_krylov.py:119-205) is plain FP32 CG, capped near
// 1e-6 by its FP32 iterate.  CG-IR keeps the FP32 CG body as the inner solver
// of the correction equation A E = R and refines X in FP64 with an FP64
// residual R = B - A X (the structure of dense_krylov.py:338-421 with CG
// inside), all right-hand sides in lockstep so that one pass over A serves
// every column.  Operators:
//   mode 0  stored FP32 copy of A inside, native FP64 residual;
//   mode 1  split A = A_hi + A_lo (two FP32 slices, double-float products) for
//           both the inner operator and the residual: FP64-accurate products on
//           the FP32 pipe, needed when kappa(A) * 6e-8 >= 1;
//   matrix-free (mpdok_mf_cg_ir) FP32 evaluate-and-multiply inside, FP64
//           evaluate-and-multiply residual.
#include "krylov.cuh"
#include "matfree.cuh"
#include "split.cuh"

#include <cstring>

namespace mpdok {

static size_t op_bytes(long long n, int mode) {
  const long long ld = (long long)align_up((size_t)std::max(1LL, n), 4);
  if (mode == 0) return align_up((size_t)ld * n * sizeof(float), 256);
  return 2 * align_up((size_t)ld * n * sizeof(float), 256);
}

}  // namespace mpdok

using namespace mpdok;

extern "C" size_t mpdok_cg_ir_operator_size(long long n, int mode) {
  if (n < 0 || (mode != 0 && mode != 1)) return 0;
  return op_bytes(n, mode);
}

extern "C" size_t mpdok_cg_ir_workspace_size(long long n, int nrhs, int mode) {
  if (n < 0 || nrhs < 1 || nrhs > 8) return 0;
  size_t g = 0;
  if (mode == 0)
    g = std::max(gemv_workspace_bytes(MPDOK_F32, n, n, nrhs, false), gemv_workspace_bytes(MPDOK_F64, n, n, nrhs, false));
  else
    g = split_gemv_work_bytes(n, n, nrhs);
  return cgir_layout(n, nrhs, nullptr).total + align_up(g, 256) + 256;
}

extern "C" int mpdok_cg_ir(const double* A64, long long lda, long long n, int mode, void* opbuf, int op_ready,
                           int nrhs, const double* B, long long ldb, double* X, long long ldx, double tol,
                           int maxiter_outer, double inner_tol, int inner_maxiter, void* work, size_t work_bytes,
                           mpdok_solve_info* info, cudaStream_t s) {
  if (info) std::memset(info, 0, sizeof(*info));
  MPDOK_ARG_CHECK(n >= 0, "negative n");
  MPDOK_ARG_CHECK(mode == 0 || mode == 1, "mode must be 0 (FP32 copy) or 1 (split)");
  MPDOK_ARG_CHECK(nrhs >= 1 && nrhs <= 8, "nrhs must be in 1..8");
  if (n == 0) { if (info) info->converged = 1; return MPDOK_OK; }
  MPDOK_ARG_CHECK(A64 && opbuf && B && X && work, "null pointer");
  MPDOK_ARG_CHECK(lda >= n && ldb >= n && ldx >= n, "leading dimension too small");
  MPDOK_ARG_CHECK(work_bytes >= mpdok_cg_ir_workspace_size(n, nrhs, mode), "CG-IR workspace too small");
  const long long ld = (long long)align_up((size_t)n, 4);
  CgIrWs w = cgir_layout(n, nrhs, work);
  char* gw = (char*)work + align_up(w.total, 256);
  const size_t gbytes = work_bytes - align_up(w.total, 256);
  if (mode == 0) {
    float* A32 = (float*)opbuf;
    if (!op_ready) MPDOK_TRY(convert_matrix_f64_f32(A64, lda, A32, ld, n, n, s));
    StoredCtx c;
    c.A32 = A32;
    c.lda32 = ld;
    c.A64 = A64;
    c.lda64 = lda;
    c.n = n;
    c.gw = gw;
    c.gbytes = gbytes;
    return cg_ir_core(w, stored_op32(&c), stored_res64(&c), B, ldb, X, ldx, tol, maxiter_outer, inner_tol,
                      inner_maxiter, nullptr, info, s);
  }
  float* hi = (float*)opbuf;
  float* lo = (float*)((char*)opbuf + align_up((size_t)ld * n * sizeof(float), 256));
  if (!op_ready) MPDOK_TRY(split_matrix(A64, lda, n, n, hi, lo, ld, s));
  SplitCtx c;
  c.hi = hi;
  c.lo = lo;
  c.ld = ld;
  c.n = n;
  c.work = gw;
  c.work_bytes = gbytes;
  return cg_ir_core(w, split_op32(&c), split_res64(&c), B, ldb, X, ldx, tol, maxiter_outer, inner_tol, inner_maxiter,
                    nullptr, info, s);
}

extern "C" size_t mpdok_mf_cg_ir_workspace_size(long long n, int nrhs) {
  if (n < 0 || nrhs < 1 || nrhs > 8) return 0;
  return cgir_layout(n, nrhs, nullptr).total + matfree_work_bytes(n, n, nrhs, MPDOK_F32) +
         matfree_work_bytes(n, n, nrhs, MPDOK_F64) + 1024;
}

extern "C" int mpdok_mf_cg_ir(const double* coords, long long n, int dim, int kernel, double gamma, double reg,
                              int nrhs, const double* B, long long ldb, double* X, long long ldx, double tol,
                              int maxiter_outer, double inner_tol, int inner_maxiter, void* work, size_t work_bytes,
                              mpdok_solve_info* info, cudaStream_t s) {
  if (info) std::memset(info, 0, sizeof(*info));
  MPDOK_ARG_CHECK(n >= 0, "negative n");
  MPDOK_ARG_CHECK(nrhs >= 1 && nrhs <= 8, "nrhs must be in 1..8");
  if (n == 0) { if (info) info->converged = 1; return MPDOK_OK; }
  MPDOK_ARG_CHECK(coords && B && X && work, "null pointer");
  MPDOK_ARG_CHECK(work_bytes >= mpdok_mf_cg_ir_workspace_size(n, nrhs), "workspace too small");
  CgIrWs w = cgir_layout(n, nrhs, work);
  char* base = (char*)work + align_up(w.total, 256);
  MfCtx c;
  c.op.rows = coords;
  c.op.cols = coords;
  c.op.nrows = n;
  c.op.ncols = n;
  c.op.dim = dim;
  c.op.kernel = kernel;
  c.op.gamma = gamma;
  c.op.reg = reg;
  c.w32 = base;
  c.w32_bytes = matfree_work_bytes(n, n, nrhs, MPDOK_F32);
  c.w64 = base + align_up(c.w32_bytes, 256);
  c.w64_bytes = matfree_work_bytes(n, n, nrhs, MPDOK_F64);
  MPDOK_TRY(mf_timeout_clear(&c, s));
  return mf_timeout_finish(&c, cg_ir_core(w, mf_op32(&c), mf_res64(&c), B, ldb, X, ldx, tol, maxiter_outer, inner_tol,
                                          inner_maxiter, nullptr, info, s), s);
}

// ------------------------------------------------ Cholesky-preconditioned CG-IR
// CG-IR for SPD systems whose kappa puts every FP32 CG body out of reach (the
// C2 family: kappa ~ 1e8, so kappa * 6e-8 > 1): the inner CG is preconditioned
// by an FP64-accurate Cholesky factor (a batch plan of one system, trailing
// update in double-float), z = (L L^T)^-1 r for all columns at once.  The FP32
// products of the inner PCG and the FP64 residual come from the operator of
// `mode`: 0 stored FP32 copy + native FP64 residual, 1 split (two FP32 slices,
// double-float products, FP64-level accuracy on the FP32 pipe) for both,
// 2 matrix-free (coords; FP32 evaluate-and-multiply, FP64 residual).
extern "C" size_t mpdok_chol_cg_ir_workspace_size(long long n, int nrhs, int mode) {
  if (n < 0 || nrhs < 1 || nrhs > 8 || mode < 0 || mode > 2) return 0;
  const size_t tmp = align_up((size_t)std::max(1LL, n) * nrhs * sizeof(double), 256);
  const size_t base = mode == 2 ? mpdok_mf_cg_ir_workspace_size(n, nrhs) : mpdok_cg_ir_workspace_size(n, nrhs, mode);
  return base + tmp + 256;
}

extern "C" int mpdok_chol_cg_ir(void* plan, const double* A64, long long lda, const double* coords, int dim,
                                int kernel, double gamma, double reg, long long n, int mode, void* opbuf,
                                int op_ready, int nrhs, const double* B, long long ldb, double* X, long long ldx,
                                double tol, int maxiter_outer, double inner_tol, int inner_maxiter, void* work,
                                size_t work_bytes, mpdok_solve_info* info, cudaStream_t s) {
  if (info) std::memset(info, 0, sizeof(*info));
  MPDOK_ARG_CHECK(n >= 0, "negative n");
  MPDOK_ARG_CHECK(mode >= 0 && mode <= 2, "mode must be 0 (FP32 copy), 1 (split) or 2 (matrix-free)");
  MPDOK_ARG_CHECK(nrhs >= 1 && nrhs <= 8, "nrhs must be in 1..8");
  if (n == 0) { if (info) info->converged = 1; return MPDOK_OK; }
  MPDOK_ARG_CHECK(plan && B && X && work, "null pointer");
  MPDOK_ARG_CHECK(mode == 2 ? coords != nullptr : (A64 != nullptr && opbuf != nullptr), "operator inputs missing");
  MPDOK_ARG_CHECK(ldb >= n && ldx >= n && (mode == 2 || lda >= n), "leading dimension too small");
  MPDOK_ARG_CHECK(work_bytes >= mpdok_chol_cg_ir_workspace_size(n, nrhs, mode), "workspace too small");
  const size_t tmp_bytes = align_up((size_t)n * nrhs * sizeof(double), 256);
  double* tmp = (double*)work;
  char* rest = (char*)work + tmp_bytes;
  const size_t rest_bytes = work_bytes - tmp_bytes;
  BatchPcCtx pctx;
  Precond pc;
  MPDOK_TRY(batch_precond(plan, n, nrhs, tmp, &pctx, &pc));
  CgIrWs w = cgir_layout(n, nrhs, rest);
  char* gw = rest + align_up(w.total, 256);
  const size_t gbytes = rest_bytes - align_up(w.total, 256);
  const long long ld = (long long)align_up((size_t)n, 4);
  if (mode == 0) {
    float* A32 = (float*)opbuf;
    if (!op_ready) MPDOK_TRY(convert_matrix_f64_f32(A64, lda, A32, ld, n, n, s));
    StoredCtx c;
    c.A32 = A32;
    c.lda32 = ld;
    c.A64 = A64;
    c.lda64 = lda;
    c.n = n;
    c.gw = gw;
    c.gbytes = gbytes;
    return cg_ir_core(w, stored_op32(&c), stored_res64(&c), B, ldb, X, ldx, tol, maxiter_outer, inner_tol,
                      inner_maxiter, &pc, info, s);
  }
  if (mode == 1) {
    float* hi = (float*)opbuf;
    float* lo = (float*)((char*)opbuf + align_up((size_t)ld * n * sizeof(float), 256));
    if (!op_ready) MPDOK_TRY(split_matrix(A64, lda, n, n, hi, lo, ld, s));
    SplitCtx c;
    c.hi = hi;
    c.lo = lo;
    c.ld = ld;
    c.n = n;
    c.work = gw;
    c.work_bytes = gbytes;
    return cg_ir_core(w, split_op32(&c), split_res64(&c), B, ldb, X, ldx, tol, maxiter_outer, inner_tol,
                      inner_maxiter, &pc, info, s);
  }
  MfCtx c;
  c.op.rows = coords;
  c.op.cols = coords;
  c.op.nrows = n;
  c.op.ncols = n;
  c.op.dim = dim;
  c.op.kernel = kernel;
  c.op.gamma = gamma;
  c.op.reg = reg;
  c.w32 = gw;
  c.w32_bytes = matfree_work_bytes(n, n, nrhs, MPDOK_F32);
  c.w64 = gw + align_up(c.w32_bytes, 256);
  c.w64_bytes = matfree_work_bytes(n, n, nrhs, MPDOK_F64);
  MPDOK_TRY(mf_timeout_clear(&c, s));
  return mf_timeout_finish(&c, cg_ir_core(w, mf_op32(&c), mf_res64(&c), B, ldb, X, ldx, tol, maxiter_outer, inner_tol,
                                          inner_maxiter, &pc, info, s), s);
}
