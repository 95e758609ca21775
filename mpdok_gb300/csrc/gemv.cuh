// Stored-matrix GEMV building blocks shared by the Krylov drivers.
#pragma once
#include "common.cuh"

namespace mpdok {

template <typename TA> struct GemvTraits;
template <> struct GemvTraits<float> { static constexpr int VEC = 4; static constexpr int UNR = 8; using Acc = float; };
template <> struct GemvTraits<double> { static constexpr int VEC = 2; static constexpr int UNR = 8; using Acc = double; };
template <> struct GemvTraits<__nv_bfloat16> { static constexpr int VEC = 8; static constexpr int UNR = 4; using Acc = float; };
template <> struct GemvTraits<__half> { static constexpr int VEC = 8; static constexpr int UNR = 4; using Acc = float; };

// Load VEC consecutive elements (16 bytes) and widen to the accumulator type.
template <typename TA, typename ACC, int VEC>
__device__ __forceinline__ void load16(const TA* p, ACC (&o)[VEC]);

template <>
__device__ __forceinline__ void load16<float, float, 4>(const float* p, float (&o)[4]) {
  float4 v = __ldg(reinterpret_cast<const float4*>(p));
  o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
}
template <>
__device__ __forceinline__ void load16<double, double, 2>(const double* p, double (&o)[2]) {
  double2 v = __ldg(reinterpret_cast<const double2*>(p));
  o[0] = v.x; o[1] = v.y;
}
template <>
__device__ __forceinline__ void load16<__nv_bfloat16, float, 8>(const __nv_bfloat16* p, float (&o)[8]) {
  uint4 v = __ldg(reinterpret_cast<const uint4*>(p));
  const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&v);
#pragma unroll
  for (int i = 0; i < 4; ++i) { float2 f = __bfloat1622float2(h[i]); o[2 * i] = f.x; o[2 * i + 1] = f.y; }
}
template <>
__device__ __forceinline__ void load16<__half, float, 8>(const __half* p, float (&o)[8]) {
  uint4 v = __ldg(reinterpret_cast<const uint4*>(p));
  const __half2* h = reinterpret_cast<const __half2*>(&v);
#pragma unroll
  for (int i = 0; i < 4; ++i) { float2 f = __half22float2(h[i]); o[2 * i] = f.x; o[2 * i + 1] = f.y; }
}

template <typename TA, typename ACC>
__device__ __forceinline__ ACC widen(TA v);
template <> __device__ __forceinline__ float widen<float, float>(float v) { return v; }
template <> __device__ __forceinline__ double widen<double, double>(double v) { return v; }
template <> __device__ __forceinline__ float widen<__nv_bfloat16, float>(__nv_bfloat16 v) { return __bfloat162float(v); }
template <> __device__ __forceinline__ float widen<__half, float>(__half v) { return __half2float(v); }

// Host-side plan of a split GEMV.
struct GemvPlan {
  int S = 1;                  // number of splits of the reduced dimension
  long long chunk = 0;        // reduced-dimension length per split
  unsigned grid_x = 0;        // blocks along the output dimension
  size_t part_bytes = 0;      // partial-sum buffer
  size_t fin_parts_bytes = 0; // per-block norm parts of the finalize pass
  size_t total_bytes = 0;     // partials + norm parts + ticket
};

GemvPlan plan_gemv(int a_dtype, long long m, long long n, int nrhs, bool trans);

// y = alpha * op(A) x + beta * bsrc  (bsrc may alias y; ignored when beta == 0).
// x / y / bsrc are FP64 when A is FP64, FP32 otherwise.  When nrm2 is not
// null (nrhs == 1), the sum of squares of y lands in *nrm2 (device scalar).
int gemv_launch(int a_dtype, bool trans, const void* A, long long lda, long long m, long long n,
                const void* X, long long ldx, int nrhs, void* Y, long long ldy, double alpha, double beta,
                const void* Bsrc, long long ldb, double* nrm2, void* work, size_t work_bytes,
                cudaStream_t s, bool zero_ticket, const int* skip = nullptr);

size_t gemv_workspace_bytes(int a_dtype, long long m, long long n, int nrhs, bool trans);

}  // namespace mpdok
