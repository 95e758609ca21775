// Error reporting, device queries and elementwise conversions.
#include "common.cuh"

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <utility>

namespace mpdok {

static thread_local char g_last_error[1024] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
}

int cuda_status(cudaError_t e, const char* where) {
  set_error("CUDA error in %s: %s (%s)", where, cudaGetErrorName(e), cudaGetErrorString(e));
  if (e == cudaErrorMemoryAllocation) return MPDOK_ERR_ALLOC;
  return MPDOK_ERR_CUDA;
}

int num_sms() {
  static std::mutex mu;
  static int cache[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 148;
  std::lock_guard<std::mutex> lk(mu);
  if (cache[dev] == 0) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 148;
    cache[dev] = v;
  }
  return cache[dev];
}

int smem_attr(const void* func, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, size_t> done;
  int dev = 0;
  MPDOK_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  size_t& have = done[{func, dev}];
  if (have >= bytes) return MPDOK_OK;
  MPDOK_CUDA_TRY(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  have = bytes;
  return MPDOK_OK;
}

template <typename S, typename D>
__global__ void convert_kernel(const S* __restrict__ src, D* __restrict__ dst, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    if constexpr (std::is_same<S, double>::value) dst[i] = from_f64<D>(src[i]);
    else dst[i] = from_f32<D>(to_f32<S>(src[i]));
  }
}

// FP64 -> FP32 with 16-byte vector loads (the dominant use: A64 -> A32).
__global__ void convert_f64_f32_vec(const double2* __restrict__ src, float2* __restrict__ dst, long long n2) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += (long long)gridDim.x * blockDim.x) {
    double2 v = src[i];
    dst[i] = make_float2((float)v.x, (float)v.y);
  }
}

template <typename S, typename D>
static void launch_convert(const void* src, void* dst, long long n, cudaStream_t s) {
  long long blocks = (n + 255) / 256;
  long long cap = (long long)num_sms() * 16;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  launch(convert_kernel<S, D>, (unsigned)blocks, 256, 0, s, (const S*)src, (D*)dst, n);
}

template <typename S>
static int convert_from(const void* src, void* dst, int dt, long long n, cudaStream_t s) {
  switch (dt) {
    case MPDOK_F64: launch_convert<S, double>(src, dst, n, s); break;
    case MPDOK_F32: launch_convert<S, float>(src, dst, n, s); break;
    case MPDOK_BF16: launch_convert<S, __nv_bfloat16>(src, dst, n, s); break;
    case MPDOK_F16: launch_convert<S, __half>(src, dst, n, s); break;
    default: set_error("convert: unknown dst dtype %d", dt); return MPDOK_ERR_INVALID_ARG;
  }
  return MPDOK_OK;
}

int convert_any(const void* src, int sdt, void* dst, int ddt, long long n, cudaStream_t s) {
  if (n == 0) return MPDOK_OK;
  MPDOK_ARG_CHECK(src && dst, "null pointer");
  if (sdt == MPDOK_F64 && ddt == MPDOK_F32 && aligned16(src) && (((uintptr_t)dst & 7u) == 0) && n % 2 == 0) {
    long long n2 = n / 2;
    long long blocks = std::min<long long>((n2 + 255) / 256, (long long)num_sms() * 16);
    launch(convert_f64_f32_vec, (unsigned)std::max(1LL, blocks), 256, 0, s, (const double2*)src, (float2*)dst, n2);
    MPDOK_LAUNCH_CHECK("convert");
    return MPDOK_OK;
  }
  int st;
  switch (sdt) {
    case MPDOK_F64: st = convert_from<double>(src, dst, ddt, n, s); break;
    case MPDOK_F32: st = convert_from<float>(src, dst, ddt, n, s); break;
    case MPDOK_BF16: st = convert_from<__nv_bfloat16>(src, dst, ddt, n, s); break;
    case MPDOK_F16: st = convert_from<__half>(src, dst, ddt, n, s); break;
    default: set_error("convert: unknown src dtype %d", sdt); return MPDOK_ERR_INVALID_ARG;
  }
  if (st) return st;
  MPDOK_LAUNCH_CHECK("convert");
  return MPDOK_OK;
}

// Strided matrix conversion (column-major m x n, lds / ldd).
__global__ void convert2d_f64_f32(const double* __restrict__ src, long long lds, float* __restrict__ dst,
                                  long long ldd, long long m, long long n) {
  for (long long j = blockIdx.y; j < n; j += gridDim.y)
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (long long)gridDim.x * blockDim.x)
      dst[i + j * ldd] = (float)src[i + j * lds];
}

int convert_matrix_f64_f32(const double* src, long long lds, float* dst, long long ldd, long long m, long long n,
                           cudaStream_t s) {
  if (m == 0 || n == 0) return MPDOK_OK;
  if (lds == m && ldd == m) return convert_any(src, MPDOK_F64, dst, MPDOK_F32, m * n, s);
  dim3 grid((unsigned)std::min<long long>((m + 255) / 256, 64), (unsigned)std::min<long long>(n, 65535));
  launch(convert2d_f64_f32, grid, 256, 0, s, src, lds, dst, ldd, m, n);
  MPDOK_LAUNCH_CHECK("convert2d");
  return MPDOK_OK;
}

}  // namespace mpdok

using namespace mpdok;

extern "C" int mpdok_version(void) { return 10000; }

extern "C" const char* mpdok_last_error(void) { return g_last_error; }

extern "C" void mpdok_clear_error(void) { g_last_error[0] = '\0'; }

extern "C" const char* mpdok_status_string(int s) {
  switch (s) {
    case MPDOK_OK: return "ok";
    case MPDOK_ERR_INVALID_ARG: return "invalid argument";
    case MPDOK_ERR_CUDA: return "CUDA error";
    case MPDOK_ERR_ALLOC: return "device allocation failed";
    case MPDOK_ERR_NOT_FACTORED: return "no factorization available";
    case MPDOK_ERR_TIMEOUT: return "device-side wait timed out";
    case MPDOK_ERR_UNSUPPORTED: return "unsupported configuration";
    case MPDOK_ERR_IO: return "I/O error";
    case MPDOK_ERR_NONFINITE: return "non-finite value encountered";
    default: return s > 0 ? "numerical information (see solver docs)" : "unknown error";
  }
}

extern "C" int mpdok_convert(const void* src, int src_dtype, void* dst, int dst_dtype, long long n,
                             cudaStream_t stream) {
  MPDOK_ARG_CHECK(n >= 0, "negative n");
  return convert_any(src, src_dtype, dst, dst_dtype, n, stream);
}
