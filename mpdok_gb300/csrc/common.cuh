// Shared helpers for the sm_103a kernels and the C-ABI layer.
//
// Error model: every exported entry point returns an int status
// (0 ok, <0 error, >0 numerical information such as a zero pivot index).
// The last error message is kept per host thread and returned by
// mpdok_last_error().  No device code traps or asserts; device-side
// waits carry iteration limits and report through status words.
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>
#include <stddef.h>

#include <algorithm>
#include <type_traits>

#include "mpdok_gb300.h"

namespace mpdok {

void set_error(const char* fmt, ...);
int cuda_status(cudaError_t e, const char* where);

#define MPDOK_CUDA_TRY(expr)                                   \
  do {                                                         \
    cudaError_t _e = (expr);                                   \
    if (_e != cudaSuccess) return ::mpdok::cuda_status(_e, #expr); \
  } while (0)

#define MPDOK_LAUNCH_CHECK(where)                              \
  do {                                                         \
    cudaError_t _e = cudaGetLastError();                       \
    if (_e != cudaSuccess) return ::mpdok::cuda_status(_e, where); \
  } while (0)

#define MPDOK_ARG_CHECK(cond, msg)                             \
  do {                                                         \
    if (!(cond)) {                                             \
      ::mpdok::set_error("invalid argument: %s", msg);         \
      return MPDOK_ERR_INVALID_ARG;                            \
    }                                                          \
  } while (0)

#define MPDOK_TRY(expr)                                        \
  do {                                                         \
    int _s = (expr);                                           \
    if (_s < 0) return _s;                                     \
  } while (0)

int num_sms();             // SM count of the current device (cached per device)
// Raise a kernel's dynamic shared-memory limit to `bytes` on the current
// device.  The attribute is per device, so the set is remembered per (kernel,
// device) under a lock: a second GPU in the same process, or two host threads
// making their first calls together, each get it set before their launch.
int smem_attr(const void* func, size_t bytes);
template <typename K>
inline int set_smem(K* kern, size_t bytes) { return smem_attr(reinterpret_cast<const void*>(kern), bytes); }
int convert_any(const void* src, int sdt, void* dst, int ddt, long long n, cudaStream_t s);
int convert_matrix_f64_f32(const double* src, long long lds, float* dst, long long ldd, long long m, long long n,
                           cudaStream_t s);
inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }
inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// ---------------------------------------------------------------- device helpers

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum; result valid in every thread.  `red` holds >= 32 T.
template <typename T>
__device__ __forceinline__ T block_sum(T v, T* red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  T t = (threadIdx.x < nw) ? red[threadIdx.x] : T(0);
  if (wid == 0) t = warp_sum(t);
  if (threadIdx.x == 0) red[0] = t;
  __syncthreads();
  T r = red[0];
  __syncthreads();
  return r;
}

template <typename T> __device__ __forceinline__ float to_f32(T v);
template <> __device__ __forceinline__ float to_f32<float>(float v) { return v; }
template <> __device__ __forceinline__ float to_f32<double>(double v) { return (float)v; }
template <> __device__ __forceinline__ float to_f32<__nv_bfloat16>(__nv_bfloat16 v) { return __bfloat162float(v); }
template <> __device__ __forceinline__ float to_f32<__half>(__half v) { return __half2float(v); }

template <typename T> __device__ __forceinline__ T from_f32(float v);
template <> __device__ __forceinline__ float from_f32<float>(float v) { return v; }
template <> __device__ __forceinline__ double from_f32<double>(float v) { return (double)v; }
template <> __device__ __forceinline__ __nv_bfloat16 from_f32<__nv_bfloat16>(float v) { return __float2bfloat16_rn(v); }
template <> __device__ __forceinline__ __half from_f32<__half>(float v) { return __float2half_rn(v); }

template <typename T> __device__ __forceinline__ T from_f64(double v);
template <> __device__ __forceinline__ double from_f64<double>(double v) { return v; }
template <> __device__ __forceinline__ float from_f64<float>(double v) { return (float)v; }
template <> __device__ __forceinline__ __nv_bfloat16 from_f64<__nv_bfloat16>(double v) { return __double2bfloat16(v); }
template <> __device__ __forceinline__ __half from_f64<__half>(double v) { return __double2half(v); }

// Deterministic grid-wide sum.  Every block passes its block total (valid in
// thread 0); the last block to arrive sums the per-block parts in index order
// and writes *result, then re-arms *ticket to 0 for the next launch.  The
// summation order never depends on block scheduling.
__device__ __forceinline__ void ordered_grid_sum(double v_block, double* parts, unsigned* ticket,
                                                 double* result) {
  __shared__ bool s_last;
  const unsigned nb = gridDim.x * gridDim.y;
  const unsigned bid = blockIdx.y * gridDim.x + blockIdx.x;
  if (threadIdx.x == 0) {
    parts[bid] = v_block;
    __threadfence();
    unsigned t = atomicAdd(ticket, 1u);
    s_last = (t == nb - 1);
  }
  __syncthreads();
  if (s_last && threadIdx.x < 32) {
    __threadfence();
    double s = 0.0;
    for (unsigned i = threadIdx.x; i < nb; i += 32) s += ((volatile double*)parts)[i];
    s = warp_sum(s);
    if (threadIdx.x == 0) {
      *result = s;
      *ticket = 0u;
    }
  }
}

}  // namespace mpdok

namespace mpdok {

// Every kernel launch of the library goes through launch(), which counts it.
void count_launch();
long long launch_count();

template <typename... P, typename... A>
inline void launch(void (*kern)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, A&&... args) {
  kern<<<grid, block, smem, s>>>(std::forward<A>(args)...);
  count_launch();
}

// Opt-in per-kernel-class timing with CUDA events on the launching stream.
// prof_start returns a slot (or -1 when profiling is off); prof_stop records
// the closing event and the algorithmic bytes / flops of the launch, and for a
// launch predicated on a device skip flag, that flag's value.
int prof_start(int cls, cudaStream_t s);
void prof_stop(int slot, cudaStream_t s, double work, const int* skip = nullptr);
// Algorithmic bytes of the same launch, for classes whose `work` counts flops.
void prof_stop_bytes(int slot, double bytes);

// Row-major FP32 RBF tile computed in FP64 and rounded once, nugget added in
// FP32 after the rounding (the reference's out-of-core tile).
int rbf_tile_f32_from_f64(const double* rows, long long n_rows, const double* cols, long long n_cols, int dim,
                          int kernel, double gamma, double reg, long long diag_offset, float* out, long long ld,
                          cudaStream_t s);

}  // namespace mpdok
