// Device-resident Krylov machinery shared by the GMRES / CG / LU-IR drivers.
#pragma once
#include "gemv.cuh"

namespace mpdok {

// Device scalars of one solve (one cache line each group).
struct KScal {
  double nrm2;      // target of the last ordered reduction
  double beta;      // ||rhs|| of the current Arnoldi cycle
  double rs;        // CG: r.r
  double alpha;     // CG step
  double betacg;    // CG direction update
  double aux;       // spare reduction target
  int done;         // cycle finished: early stop, breakdown or stop request
  int m_used;       // Arnoldi steps completed in the current cycle
  int breakdown;    // |w| <= 1e-12 met
  int nonfinite;    // NaN / Inf seen in a device scalar
};

// Workspace carve-up for a Krylov solve of size n with restart m.
struct KWs {
  long long n = 0, ldv = 0;
  int m = 0;
  float *V = nullptr, *w = nullptr, *x32 = nullptr, *b32 = nullptr, *p32 = nullptr, *q32 = nullptr;
  double *r64 = nullptr, *x64t = nullptr, *e64 = nullptr;
  double *H = nullptr, *cs = nullptr, *sn = nullptr, *g = nullptr, *y = nullptr, *h2 = nullptr;
  double* parts = nullptr;
  unsigned* tickets = nullptr;  // 8 independent tickets
  KScal* sc = nullptr;
  void* gw = nullptr;
  size_t gbytes = 0;
  int nblk = 1;       // blocks of the row-chunked vector kernels
  long long ch = 256; // rows per block of those kernels
  size_t total = 0;
};

KWs krylov_layout(long long n, int m, void* base);

// Workspace of a multi-RHS CG-IR solve (n x K blocks, leading dimension ld).
struct CgIrWs {
  long long n = 0, ld = 0;
  int K = 1;
  unsigned nblk = 1;
  double *R64 = nullptr, *B64 = nullptr, *X64 = nullptr, *parts = nullptr, *nrm2 = nullptr;
  float *E = nullptr, *r = nullptr, *p = nullptr, *q = nullptr, *z = nullptr;
  void *cols = nullptr, *g = nullptr;
  unsigned* ticket = nullptr;
  size_t total = 0;
};
CgIrWs cgir_layout(long long n, int K, void* base);

// FP32 operator y = A x (nrhs columns, leading dimension ld for x and y, ld a
// multiple of 4) used by the Krylov bodies; `skip` predicates the launches on
// a device flag.
struct Operator32 {
  int (*apply)(const void* ctx, const float* x, float* y, int nrhs, long long ld, cudaStream_t s,
               const int* skip) = nullptr;
  const void* ctx = nullptr;
};

// FP64 residual r = b - A x (nrhs columns, leading dimension ld) with
// per-column ||r||^2 into nrm2[0..nrhs).
struct Residual64 {
  int (*apply)(const void* ctx, const double* b, const double* x, double* r, double* nrm2, int nrhs, long long ld,
               cudaStream_t s) = nullptr;
  const void* ctx = nullptr;
};

// Stored-matrix implementations (FP32 A32 / FP64 A64, column-major).
struct StoredCtx {
  const float* A32 = nullptr;
  long long lda32 = 0;
  const double* A64 = nullptr;
  long long lda64 = 0;
  long long n = 0;
  void* gw = nullptr;
  size_t gbytes = 0;
};
Operator32 stored_op32(const StoredCtx* c);
Residual64 stored_res64(const StoredCtx* c);

// Preconditioner hook for right-preconditioned cycles: z = M^{-1} v.
struct Precond {
  int (*apply)(void* ctx, const float* v, float* z, cudaStream_t s, const int* skip) = nullptr;
  void* ctx = nullptr;
  float* z = nullptr;  // n floats of scratch for M^{-1} v
  // optional: m columns (leading dimension ldz) that keep z_k = M^{-1} v_k of
  // every Arnoldi step, so that the cycle's update x += M^{-1} V y is Z y and
  // needs no further application of M^{-1}
  float* Z = nullptr;
  long long ldz = 0;
  // optional: all K columns (leading dimension ld) in one call; CG-IR uses it
  // when set (a factorization applied to K right-hand sides at once)
  int (*apply_cols)(void* ctx, const float* v, float* z, int K, long long ld, cudaStream_t s) = nullptr;
};

// Preconditioner z = A^-1 v from the Cholesky factor held in a batch plan of
// one system of size n with nrhs == K (double-float trailing update, FP64
// diagonal blocks and solves); tmp holds n * K doubles.  Defined in batch.cu.
struct BatchPcCtx {
  void* plan = nullptr;
  double* tmp = nullptr;
  long long n = 0;
};
int batch_precond(void* plan, long long n, int K, double* tmp, BatchPcCtx* ctx, Precond* pc);
// V := A^-1 V in FP64 with the Cholesky factor of a batch plan of one system
// (V: n x K column-major, ld n, K = the plan's nrhs).  Defined in batch.cu.
int batch_apply_f64(void* plan, long long n, int K, double* V, cudaStream_t s);

// One Arnoldi cycle (up to m steps) on the FP32 operator A32 with the
// unnormalised start vector already in V[:,0] and ws.sc->nrm2 = ||V[:,0]||^2
// set by cycle_setup.  reorth = 1 or 2 Gram-Schmidt passes.  Early stop when
// |g_{k+1}| / beta < tol_rel (tol_rel <= 0 disables it).  The correction
// V y (or M^{-1} V y when preconditioned) is added to x32 or x64.
int arnoldi_cycle(const KWs& ws, const Operator32& A, int m, int reorth, double tol_rel, const Precond* pc,
                  float* x32, double* x64, cudaStream_t s);

// V[:,0] = (float) src64 and sc->nrm2, beta, flags for a new cycle.
int cycle_start_from_f64(const KWs& ws, const double* src64, cudaStream_t s);

int read_scal(const KWs& ws, KScal* host, cudaStream_t s);
int norm2_f64(const KWs& ws, const double* x, long long n, double* out_dev, cudaStream_t s);
int colnorms_f64(const double* r, long long n, int nrhs, long long ld, double* nrm2, cudaStream_t s);
// FP64 residual r64 = b - A x through R, ||r||^2 into sc->nrm2, then the
// scalar block is read back to the host.
int fp64_residual(const KWs& ws, const Residual64& R, const double* b, const double* x, KScal* hs, cudaStream_t s);
// Restarted FP32 GMRES(m) (single Gram-Schmidt pass, FP64 check per restart).
int gmres_core(const KWs& ws, const Operator32& A, const Residual64& R, const double* rhs64, double* x64, double tol,
               int maxiter, int restart, mpdok_solve_info* info, cudaStream_t s);
// GMRES-IR outer loop (mpdok_ooc.py:315-373) over any operator pair.  With
// xbest (n doubles of scratch) the loop is guarded: the best iterate is kept,
// and a non-finite residual or one 1e3 x above the best restores it and stops
// (info->stagnated = 2); without it a non-finite residual is an error.
int gmres_ir_core(const KWs& ws, const Operator32& A, const Residual64& R, const double* b, double* x, double tol,
                  int maxiter_outer, int restart, double inner_tol, const Precond* pc, mpdok_solve_info* info,
                  cudaStream_t s, double* xbest = nullptr);
int ws_prepare(const KWs& ws, size_t work_bytes, cudaStream_t s);
// CG-IR: FP64 residual R = B - A X through R, inner FP32 CG on A E = R for all
// columns in lockstep (relative inner tolerance, inner_maxiter), X += E in FP64.
// pc (optional): inner PCG with z = M^-1 r applied per column.
int cg_ir_core(const CgIrWs& w, const Operator32& A, const Residual64& R, const double* B, long long ldb, double* X,
               long long ldx, double tol, int maxiter_outer, double inner_tol, int inner_maxiter, const Precond* pc,
               mpdok_solve_info* info, cudaStream_t s);
int dense_gmres_ir_core(const KWs& ws, const Operator32& A, const Residual64& R, const double* b, double* x,
                        double tol, int maxiter_outer, int restart, int maxiter_inner, mpdok_solve_info* info,
                        cudaStream_t s);
int cg_core(const KWs& ws, const Operator32& A, const Residual64& R, const double* b, double* x, double tol,
            int maxiter, int check_every, mpdok_solve_info* info, cudaStream_t s);

}  // namespace mpdok
