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

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

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
// C2 family, kappa ~ 1e8: kappa * 6e-8 > 1).  Two things have to change
// against the FP32 CG-IR above, and the GPU measurements show each one is
// needed: the inner CG is preconditioned by an FP64-accurate Cholesky factor
// (a batch plan of one system, trailing update in double-float), and the
// inner recurrence keeps its vectors in FP64, because a correction rounded to
// FP32 changes the residual by up to kappa * 6e-8 relative, more than it
// removes.  The products come from the operator of `mode`: 0 the stored FP64
// matrix (FP64 pipe), 1 the split matrix for the inner products (two FP32
// slices, error-free FP32 products and double-float sums: about 2^-48 on the
// FP32 pipe, the Ozaki-style split matvec) with the outer residual from the
// FP64 matrix, 2 matrix-free (FP64 evaluate-and-multiply from the
// coordinates).  Every column runs its own PCG; the host reads the K dot
// products per step.
namespace mpdok {

__global__ void k_cdot_part(const double* __restrict__ a, const double* __restrict__ b, long long n, int K,
                            double* __restrict__ parts) {
  __shared__ double red[32];
  const int c = blockIdx.y;
  double v = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    v = fma(a[c * n + i], b[c * n + i], v);
  v = block_sum(v, red);
  if (threadIdx.x == 0) parts[(long long)c * gridDim.x + blockIdx.x] = v;
}

__global__ void k_cdot_final(const double* __restrict__ parts, int nb, int K, double* __restrict__ out) {
  const int c = threadIdx.x;
  if (c >= K) return;
  double s = 0.0;
  for (int i = 0; i < nb; ++i) s += parts[(long long)c * nb + i];  // fixed order
  out[c] = s;
}

// y[:, c] += coef[c] * x[:, c]
__global__ void k_caxpy(double* __restrict__ y, const double* __restrict__ x, const double* __restrict__ coef, long long n,
                        int K) {
  const long long total = n * K;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x)
    y[e] = fma(coef[e / n], x[e], y[e]);
}

// p[:, c] = z[:, c] + coef[c] * p[:, c]
__global__ void k_cxpby(double* __restrict__ p, const double* __restrict__ z, const double* __restrict__ coef, long long n,
                        int K) {
  const long long total = n * K;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x)
    p[e] = fma(coef[e / n], p[e], z[e]);
}

__global__ void k_ccopy_in(const double* __restrict__ src, long long lds, double* __restrict__ dst, long long n, int K) {
  const long long total = n * K;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x)
    dst[e] = src[(e / n) * lds + e % n];
}

__global__ void k_ccopy_out(const double* __restrict__ src, double* __restrict__ dst, long long ldd, long long n, int K) {
  const long long total = n * K;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x)
    dst[(e / n) * ldd + e % n] = src[e];
}

struct CholPcgWs {
  double *B, *X, *R, *E, *r, *z, *p, *q, *zero, *parts, *coef, *dots;
  int nb;
  size_t total;
};

static void hist_push_info(mpdok_solve_info* info, int it, double rel) {
  if (!info) return;
  const int i = std::min(info->n_history, MPDOK_HISTORY_MAX - 1);
  info->hist_iter[i] = it;
  info->history[i] = rel;
  info->n_history = std::min(info->n_history + 1, MPDOK_HISTORY_MAX);
  info->relres = rel;
}

static CholPcgWs chol_layout(long long n, int K, void* base) {
  CholPcgWs w{};
  w.nb = (int)std::min<long long>(std::max(1LL, (n + 255) / 256), 256);
  size_t off = 0;
  auto take = [&](size_t b) { size_t o = off; off = align_up(off + b, 256); return o; };
  const size_t vec = (size_t)std::max(1LL, n) * K * sizeof(double);
  const size_t oB = take(vec), oX = take(vec), oR = take(vec), oE = take(vec), or_ = take(vec), oz = take(vec),
               op = take(vec), oq = take(vec), o0 = take(vec), oparts = take((size_t)K * w.nb * sizeof(double)),
               ocoef = take(8 * sizeof(double)), odots = take(8 * sizeof(double));
  w.total = off;
  if (base) {
    char* b = (char*)base;
    w.B = (double*)(b + oB); w.X = (double*)(b + oX); w.R = (double*)(b + oR); w.E = (double*)(b + oE);
    w.r = (double*)(b + or_); w.z = (double*)(b + oz); w.p = (double*)(b + op); w.q = (double*)(b + oq);
    w.zero = (double*)(b + o0); w.parts = (double*)(b + oparts); w.coef = (double*)(b + ocoef);
    w.dots = (double*)(b + odots);
  }
  return w;
}

static size_t chol_op_bytes(long long n, int K, int mode) {
  if (mode == 0) return gemv_workspace_bytes(MPDOK_F64, n, n, K, false);
  if (mode == 1) return align_up(gemv_workspace_bytes(MPDOK_F64, n, n, K, false), 256) + split_gemv_work_bytes(n, n, K);
  return matfree_work_bytes(n, n, K, MPDOK_F64);
}

// Column dot products a . b -> host (K doubles).
static int cdots(const CholPcgWs& w, const double* a, const double* b, long long n, int K, double* host,
                 cudaStream_t s) {
  launch(k_cdot_part, dim3(w.nb, K), 256, 0, s, a, b, n, K, w.parts);
  launch(k_cdot_final, 1, 32, 0, s, (const double*)w.parts, w.nb, K, w.dots);
  MPDOK_LAUNCH_CHECK("chol pcg dots");
  MPDOK_CUDA_TRY(cudaMemcpyAsync(host, w.dots, sizeof(double) * K, cudaMemcpyDeviceToHost, s));
  MPDOK_CUDA_TRY(cudaStreamSynchronize(s));
  return MPDOK_OK;
}

static int set_coef(const CholPcgWs& w, const double* host, int K, cudaStream_t s) {
  MPDOK_CUDA_TRY(cudaMemcpyAsync(w.coef, host, sizeof(double) * K, cudaMemcpyHostToDevice, s));
  MPDOK_CUDA_TRY(cudaStreamSynchronize(s));
  return MPDOK_OK;
}

static int chol_pcg_ir_core(void* plan, const Residual64& R, const Residual64& Ain, long long n, int K,
                            const double* B, long long ldb,
                            double* Xout, long long ldx, double tol, int maxiter_outer, double inner_tol,
                            int inner_maxiter, const CholPcgWs& w, mpdok_solve_info* info, cudaStream_t s) {
  const unsigned g = (unsigned)std::max(1LL, std::min<long long>((n * K + 255) / 256, (long long)num_sms() * 8));
  launch(k_ccopy_in, g, 256, 0, s, B, ldb, w.B, n, K);
  MPDOK_CUDA_TRY(cudaMemsetAsync(w.X, 0, sizeof(double) * n * K, s));
  MPDOK_CUDA_TRY(cudaMemsetAsync(w.zero, 0, sizeof(double) * n * K, s));
  std::vector<double> bn(K), rn(K), rz(K), rz1(K), pq(K), cf(K);
  MPDOK_TRY(cdots(w, w.B, w.B, n, K, bn.data(), s));
  for (int c = 0; c < K; ++c) {
    bn[c] = std::sqrt(bn[c]);
    if (!std::isfinite(bn[c])) {
      set_error("Cholesky-preconditioned CG-IR: right-hand side %d has non-finite entries", c);
      return MPDOK_ERR_NONFINITE;
    }
  }
  if (info) info->bnorm = *std::max_element(bn.begin(), bn.end());
  bool converged = false;
  int inner_total = 0;
  for (int outer = 0; outer <= maxiter_outer; ++outer) {
    // R = B - A X (FP64 products through the operator), ||R_c||
    MPDOK_TRY(R.apply(R.ctx, w.B, w.X, w.R, w.parts, K, n, s));
    MPDOK_TRY(cdots(w, w.R, w.R, n, K, rn.data(), s));
    double worst = 0.0;
    for (int c = 0; c < K; ++c) worst = std::max(worst, bn[c] > 0 ? std::sqrt(rn[c]) / bn[c] : std::sqrt(rn[c]));
    hist_push_info(info, outer, worst);
    if (!std::isfinite(worst)) { set_error("Cholesky-preconditioned CG-IR: non-finite residual"); return MPDOK_ERR_NONFINITE; }
    if (worst < tol) { converged = true; break; }
    if (outer == maxiter_outer) break;
    // inner PCG on A E = R in FP64, every column on its own
    MPDOK_CUDA_TRY(cudaMemsetAsync(w.E, 0, sizeof(double) * n * K, s));
    MPDOK_CUDA_TRY(cudaMemcpyAsync(w.r, w.R, sizeof(double) * n * K, cudaMemcpyDeviceToDevice, s));
    MPDOK_CUDA_TRY(cudaMemcpyAsync(w.z, w.r, sizeof(double) * n * K, cudaMemcpyDeviceToDevice, s));
    MPDOK_TRY(batch_apply_f64(plan, n, K, w.z, s));
    MPDOK_CUDA_TRY(cudaMemcpyAsync(w.p, w.z, sizeof(double) * n * K, cudaMemcpyDeviceToDevice, s));
    MPDOK_TRY(cdots(w, w.r, w.z, n, K, rz.data(), s));
    std::vector<double> r0(rn);
    std::vector<char> live(K, 1);
    for (int it = 0; it < inner_maxiter; ++it) {
      // q = -(A p): the inner operator with a zero right-hand side
      MPDOK_TRY(Ain.apply(Ain.ctx, w.zero, w.p, w.q, w.parts, K, n, s));
      MPDOK_TRY(cdots(w, w.p, w.q, n, K, pq.data(), s));
      for (int c = 0; c < K; ++c) cf[c] = (live[c] && pq[c] != 0.0) ? -rz[c] / pq[c] : 0.0;  // alpha = rz / (p.Ap)
      MPDOK_TRY(set_coef(w, cf.data(), K, s));
      launch(k_caxpy, g, 256, 0, s, w.E, (const double*)w.p, (const double*)w.coef, n, K);  // E += alpha p
      launch(k_caxpy, g, 256, 0, s, w.r, (const double*)w.q, (const double*)w.coef, n, K);  // r -= alpha A p
      MPDOK_LAUNCH_CHECK("chol pcg update");
      ++inner_total;
      MPDOK_TRY(cdots(w, w.r, w.r, n, K, rn.data(), s));
      bool any = false;
      for (int c = 0; c < K; ++c) {
        if (live[c] && std::sqrt(rn[c]) <= inner_tol * std::sqrt(r0[c])) live[c] = 0;
        any = any || live[c];
      }
      if (!any) break;
      MPDOK_CUDA_TRY(cudaMemcpyAsync(w.z, w.r, sizeof(double) * n * K, cudaMemcpyDeviceToDevice, s));
      MPDOK_TRY(batch_apply_f64(plan, n, K, w.z, s));
      MPDOK_TRY(cdots(w, w.r, w.z, n, K, rz1.data(), s));
      for (int c = 0; c < K; ++c) {
        cf[c] = (live[c] && rz[c] != 0.0) ? rz1[c] / rz[c] : 0.0;
        rz[c] = rz1[c];
      }
      MPDOK_TRY(set_coef(w, cf.data(), K, s));
      launch(k_cxpby, g, 256, 0, s, w.p, (const double*)w.z, (const double*)w.coef, n, K);  // p = z + beta p
      MPDOK_LAUNCH_CHECK("chol pcg direction");
    }
    for (int c = 0; c < K; ++c) cf[c] = 1.0;
    MPDOK_TRY(set_coef(w, cf.data(), K, s));
    launch(k_caxpy, g, 256, 0, s, w.X, (const double*)w.E, (const double*)w.coef, n, K);  // X += E
    MPDOK_LAUNCH_CHECK("chol pcg-ir update");
    if (info) info->outer_iters = outer + 1;
  }
  launch(k_ccopy_out, g, 256, 0, s, (const double*)w.X, Xout, ldx, n, K);
  MPDOK_LAUNCH_CHECK("chol pcg-ir out");
  if (info) {
    info->converged = converged ? 1 : 0;
    info->inner_iters = inner_total;
  }
  return MPDOK_OK;
}

}  // namespace mpdok

extern "C" size_t mpdok_chol_cg_ir_workspace_size(long long n, int nrhs, int mode) {
  if (n < 0 || nrhs < 1 || nrhs > 8 || mode < 0 || mode > 2) return 0;
  return chol_layout(n, nrhs, nullptr).total + align_up(chol_op_bytes(n, nrhs, mode), 256) + 256;
}

extern "C" int mpdok_chol_cg_ir(void* plan, const double* A64, long long lda, const double* coords, int dim,
                                int kernel, double gamma, double reg, long long n, int mode, void* opbuf,
                                int op_ready, int nrhs, const double* B, long long ldb, double* X, long long ldx,
                                double tol, int maxiter_outer, double inner_tol, int inner_maxiter, void* work,
                                size_t work_bytes, mpdok_solve_info* info, cudaStream_t s) {
  if (info) std::memset(info, 0, sizeof(*info));
  MPDOK_ARG_CHECK(n >= 0, "negative n");
  MPDOK_ARG_CHECK(mode >= 0 && mode <= 2, "mode must be 0 (stored FP64), 1 (split) or 2 (matrix-free)");
  MPDOK_ARG_CHECK(nrhs >= 1 && nrhs <= 8, "nrhs must be in 1..8");
  if (n == 0) { if (info) info->converged = 1; return MPDOK_OK; }
  MPDOK_ARG_CHECK(plan && B && X && work, "null pointer");
  MPDOK_ARG_CHECK(mode == 2 ? coords != nullptr : A64 != nullptr, "operator inputs missing");
  MPDOK_ARG_CHECK(mode != 1 || opbuf != nullptr, "the split operator needs opbuf");
  MPDOK_ARG_CHECK(ldb >= n && ldx >= n && (mode == 2 || lda >= n), "leading dimension too small");
  MPDOK_ARG_CHECK(work_bytes >= mpdok_chol_cg_ir_workspace_size(n, nrhs, mode), "workspace too small");
  CholPcgWs w = chol_layout(n, nrhs, work);
  char* gw = (char*)work + align_up(w.total, 256);
  const size_t gbytes = work_bytes - align_up(w.total, 256);
  if (mode == 0) {
    StoredCtx c;
    c.A64 = A64;
    c.lda64 = lda;
    c.n = n;
    c.gw = gw;
    c.gbytes = gbytes;
    const Residual64 R = stored_res64(&c);
    return chol_pcg_ir_core(plan, R, R, n, nrhs, B, ldb, X, ldx, tol, maxiter_outer, inner_tol, inner_maxiter, w,
                            info, s);
  }
  if (mode == 1) {
    const long long ld = (long long)align_up((size_t)n, 4);
    float* hi = (float*)opbuf;
    float* lo = (float*)((char*)opbuf + align_up((size_t)ld * n * sizeof(float), 256));
    if (!op_ready) MPDOK_TRY(split_matrix(A64, lda, n, n, hi, lo, ld, s));
    // the inner products come from the split slices (FP32 pipe, 2^-48 products), the outer
    // residual from the FP64 matrix: the split form represents A to about 2^-48, which would
    // hold the attainable relres some 30x above the FP64 floor
    const size_t gb = gemv_workspace_bytes(MPDOK_F64, n, n, nrhs, false);
    StoredCtx r;
    r.A64 = A64;
    r.lda64 = lda;
    r.n = n;
    r.gw = gw;
    r.gbytes = gb;
    SplitCtx c;
    c.hi = hi;
    c.lo = lo;
    c.ld = ld;
    c.n = n;
    c.work = gw + align_up(gb, 256);
    c.work_bytes = gbytes - align_up(gb, 256);
    return chol_pcg_ir_core(plan, stored_res64(&r), split_res64(&c), n, nrhs, B, ldb, X, ldx, tol, maxiter_outer,
                            inner_tol, inner_maxiter, w, info, s);
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
  c.w64 = gw;
  c.w64_bytes = gbytes;
  const Residual64 R = mf_res64(&c);
  return chol_pcg_ir_core(plan, R, R, n, nrhs, B, ldb, X, ldx, tol, maxiter_outer, inner_tol, inner_maxiter, w, info,
                          s);
}
