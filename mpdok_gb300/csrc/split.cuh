// Two-slice FP32 split of an FP64 matrix and its double-float GEMV.
#pragma once
#include "krylov.cuh"

namespace mpdok {

struct SplitCtx {
  const float* hi = nullptr;
  const float* lo = nullptr;
  long long ld = 0;
  long long n = 0;
  void* work = nullptr;
  size_t work_bytes = 0;
};

int split_matrix(const double* A, long long lda, long long m, long long n, float* hi, float* lo, long long ld,
                 cudaStream_t s);
size_t split_gemv_work_bytes(long long m, long long n, int nrhs);
Operator32 split_op32(const SplitCtx* c);
Residual64 split_res64(const SplitCtx* c);

}  // namespace mpdok
