// Trailing-update GEMM of the blocked LU (tensor cores or CUDA cores).
#pragma once
#include "common.cuh"

namespace mpdok {

// C (FP32, column-major, ldc) -= A * B^T with A (M x K) and B (N x K)
// K-major 16-bit operands (fdtype BF16 / FP16).  engine: MPDOK_ENGINE_TENSOR
// (tcgen05) or MPDOK_ENGINE_SIMT (CUDA cores; also the only engine for FP32).
// Operand rows have pitch ldk elements (>= K).
int gemm_update(float* C, long long ldc, const void* A, const void* B, long long ldk, int M, int N, int K, int fdtype,
                int engine, int* err, cudaStream_t s);

}  // namespace mpdok
