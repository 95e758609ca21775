// Matrix-free RBF operator (evaluate-and-multiply) shared with the Krylov drivers.
#pragma once
#include "krylov.cuh"

namespace mpdok {

struct MfOperand {
  const double* rows = nullptr;   // (nrows, dim) FP64 centres of the rows
  const double* cols = nullptr;   // (ncols, dim) FP64 centres of the columns
  long long nrows = 0, ncols = 0;
  int dim = 2;
  int kernel = MPDOK_KERNEL_GAUSSIAN;
  double gamma = 1.0;
  double reg = 0.0;               // nugget where row i meets column i + diag_offset
  long long diag_offset = 0;
  const float4* rows_packed = nullptr;  // optional prepacked FP32 centres
  const float4* cols_packed = nullptr;
};

struct MfCtx {
  MfOperand op;
  void* w32 = nullptr;
  size_t w32_bytes = 0;
  void* w64 = nullptr;
  size_t w64_bytes = 0;
};

size_t matfree_work_bytes(long long nrows, long long ncols, int nrhs, int precision);
// Y = alpha * (K X + reg X_shift) + beta * Bsrc in FP32 (float X/Y) or FP64 (double X/Y).
int matfree_apply(const MfOperand& op, int precision, const void* X, long long ldx, int K, void* Y, long long ldy,
                  double alpha, double beta, const void* Bsrc, long long ldb, void* work, size_t work_bytes,
                  cudaStream_t s, const int* skip);
// The FP32 evaluation's bounded TMA waits report through a status word in
// the FP32 workspace: a solve clears it at its start (mf_timeout_clear) and,
// when it ends, turns a set word into MPDOK_ERR_TIMEOUT (mf_timeout_finish).
int mf_timeout_clear(const MfCtx* c, cudaStream_t s);
int mf_timeout_finish(const MfCtx* c, int status, cudaStream_t s);
Operator32 mf_op32(const MfCtx* c);
Residual64 mf_res64(const MfCtx* c);

}  // namespace mpdok
