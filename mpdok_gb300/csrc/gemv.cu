// Stored-matrix GEMV / multi-RHS GEMV for sm_103a.
//
// Replaces cp.matmul(A_fp32, x) (dense_krylov.py:61-63), the FP64 residual
// b - A_fp64 @ x (dense_krylov.py:78, :391, :416) and the tiled SGEMV of
// mpdok_ooc.py:158-167.  A is column-major (the reference ABI's Fortran
// order, mpdok_ops.py:363-366).
//
// y = A x streams A once: every thread owns VEC consecutive rows (one 16-byte
// load per column), UNR columns are in flight per thread, x is staged in shared
// memory, and the column range is split S ways so that the grid fills every SM.
// Split partial sums are combined in a fixed order by a finalize pass, so the
// result is bitwise reproducible run to run.
// y = A^T x gives each warp one column (a contiguous stream) and reduces with
// warp shuffles.
#include "gemv.cuh"

#include <algorithm>
#include <mutex>
#include <type_traits>

namespace mpdok {

constexpr int GEMV_THREADS = 256;
constexpr int GEMV_TB = 256;  // columns of x staged per batch (y = A x)

template <typename TA, int K>
__global__ void __launch_bounds__(GEMV_THREADS)
gemv_n_stage1(const TA* __restrict__ A, long long lda, long long m, long long n,
              const typename GemvTraits<TA>::Acc* __restrict__ X, long long ldx, long long chunk,
              typename GemvTraits<TA>::Acc* __restrict__ P, bool vec_ok, const int* skip) {
  using ACC = typename GemvTraits<TA>::Acc;
  constexpr int VEC = GemvTraits<TA>::VEC;
  constexpr int UNR = GemvTraits<TA>::UNR;
  if (skip != nullptr && *skip) return;
  __shared__ ACC sx[K * GEMV_TB];
  const long long row0 = ((long long)blockIdx.x * GEMV_THREADS + threadIdx.x) * VEC;
  const int s = blockIdx.y;
  const long long cb0 = (long long)s * chunk;
  const long long ce = min(n, cb0 + chunk);
  ACC acc[VEC][K];
#pragma unroll
  for (int v = 0; v < VEC; ++v)
#pragma unroll
    for (int k = 0; k < K; ++k) acc[v][k] = ACC(0);
  const bool full = vec_ok && (row0 + VEC <= m);

  for (long long cb = cb0; cb < ce; cb += GEMV_TB) {
    const int nb = (int)min((long long)GEMV_TB, ce - cb);
    __syncthreads();
    for (int t = threadIdx.x; t < K * GEMV_TB; t += GEMV_THREADS) {
      const int k = t / GEMV_TB, j = t % GEMV_TB;
      sx[t] = (j < nb) ? X[(cb + j) + k * ldx] : ACC(0);
    }
    __syncthreads();
    if (row0 >= m) continue;
    const TA* a = A + row0 + cb * lda;
    int j = 0;
    if (full) {
      for (; j + UNR <= nb; j += UNR) {
        ACC av[UNR][VEC];
#pragma unroll
        for (int u = 0; u < UNR; ++u) load16<TA, ACC, VEC>(a + (long long)(j + u) * lda, av[u]);
#pragma unroll
        for (int u = 0; u < UNR; ++u)
#pragma unroll
          for (int k = 0; k < K; ++k) {
            const ACC xv = sx[k * GEMV_TB + j + u];
#pragma unroll
            for (int v = 0; v < VEC; ++v) acc[v][k] = fma(av[u][v], xv, acc[v][k]);
          }
      }
      for (; j < nb; ++j) {
        ACC av[VEC];
        load16<TA, ACC, VEC>(a + (long long)j * lda, av);
#pragma unroll
        for (int k = 0; k < K; ++k) {
          const ACC xv = sx[k * GEMV_TB + j];
#pragma unroll
          for (int v = 0; v < VEC; ++v) acc[v][k] = fma(av[v], xv, acc[v][k]);
        }
      }
    } else {
      for (; j < nb; ++j) {
#pragma unroll
        for (int v = 0; v < VEC; ++v) {
          if (row0 + v >= m) break;
          const ACC av = widen<TA, ACC>(a[(long long)j * lda + v]);
#pragma unroll
          for (int k = 0; k < K; ++k) acc[v][k] = fma(av, sx[k * GEMV_TB + j], acc[v][k]);
        }
      }
    }
  }
  if (row0 < m) {
#pragma unroll
    for (int k = 0; k < K; ++k)
#pragma unroll
      for (int v = 0; v < VEC; ++v)
        if (row0 + v < m) P[((long long)s * K + k) * m + row0 + v] = acc[v][k];
  }
}

// y = A^T x: one warp per column of A, rows split S ways (blockIdx.y).
template <typename TA, int K>
__global__ void __launch_bounds__(GEMV_THREADS)
gemv_t_stage1(const TA* __restrict__ A, long long lda, long long m, long long n,
              const typename GemvTraits<TA>::Acc* __restrict__ X, long long ldx, long long chunk,
              typename GemvTraits<TA>::Acc* __restrict__ P, bool vec_ok, const int* skip) {
  using ACC = typename GemvTraits<TA>::Acc;
  constexpr int VEC = GemvTraits<TA>::VEC;
  constexpr int UNR = 4;
  if (skip != nullptr && *skip) return;
  constexpr int RB = 32 * VEC * UNR;  // rows per staged batch
  __shared__ ACC sx[K * RB];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long long col = (long long)blockIdx.x * (GEMV_THREADS / 32) + warp;
  const int s = blockIdx.y;
  const long long rb0 = (long long)s * chunk;
  const long long re = min(m, rb0 + chunk);
  ACC acc[K];
#pragma unroll
  for (int k = 0; k < K; ++k) acc[k] = ACC(0);
  const TA* a = A + col * lda;
  for (long long rb = rb0; rb < re; rb += RB) {
    const int nb = (int)min((long long)RB, re - rb);
    __syncthreads();
    for (int t = threadIdx.x; t < K * RB; t += GEMV_THREADS) {
      const int k = t / RB, r = t % RB;
      sx[t] = (r < nb) ? X[(rb + r) + k * ldx] : ACC(0);
    }
    __syncthreads();
    if (col >= n) continue;
    if (vec_ok && nb == RB) {
      ACC av[UNR][VEC];
#pragma unroll
      for (int u = 0; u < UNR; ++u) load16<TA, ACC, VEC>(a + rb + (u * 32 + lane) * VEC, av[u]);
#pragma unroll
      for (int u = 0; u < UNR; ++u)
#pragma unroll
        for (int v = 0; v < VEC; ++v)
#pragma unroll
          for (int k = 0; k < K; ++k) acc[k] = fma(av[u][v], sx[k * RB + (u * 32 + lane) * VEC + v], acc[k]);
    } else {
      for (int r = lane; r < nb; r += 32) {
        const ACC av = widen<TA, ACC>(a[rb + r]);
#pragma unroll
        for (int k = 0; k < K; ++k) acc[k] = fma(av, sx[k * RB + r], acc[k]);
      }
    }
  }
  if (col < n) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      ACC t = warp_sum(acc[k]);
      if (lane == 0) P[((long long)s * K + k) * n + col] = t;
    }
  }
}

// y[i,k] = alpha * sum_s P[s,k,i] + beta * bsrc[i,k]; optional sum of y^2.
template <typename ACC>
__global__ void __launch_bounds__(GEMV_THREADS)
gemv_finalize(const ACC* __restrict__ P, int S, int K, long long m, ACC alpha, ACC beta,
              const ACC* bsrc, long long ldb, ACC* y, long long ldy,
              double* nrm_parts, unsigned* ticket, double* nrm2, const int* skip) {
  __shared__ double red[32];
  if (skip != nullptr && *skip) return;
  const long long total = m * K;
  double sq = 0.0;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long i = idx % m;
    const int k = (int)(idx / m);
    ACC sum = ACC(0);
    for (int s = 0; s < S; ++s) sum += P[((long long)s * K + k) * m + i];
    ACC v = alpha * sum;
    if (beta != ACC(0)) v = fma(beta, bsrc[i + k * ldb], v);
    y[i + k * ldy] = v;
    sq += (double)v * (double)v;
  }
  if (nrm2 != nullptr) {
    double b = block_sum(sq, red);
    ordered_grid_sum(b, nrm_parts, ticket, nrm2);
  }
}

static unsigned finalize_blocks(long long total) {
  long long b = (total + GEMV_THREADS - 1) / GEMV_THREADS;
  long long cap = (long long)num_sms() * 4;
  return (unsigned)std::max(1LL, std::min(b, cap));
}

static int elem_bytes(int dt) {
  switch (dt) {
    case MPDOK_F64: return 8;
    case MPDOK_F32: return 4;
    case MPDOK_BF16: case MPDOK_F16: return 2;
    default: return 0;
  }
}

static int vec_of(int dt) { return 16 / std::max(1, elem_bytes(dt)); }

GemvPlan plan_gemv(int a_dtype, long long m, long long n, int nrhs, bool trans) {
  GemvPlan p;
  const int acc_bytes = (a_dtype == MPDOK_F64) ? 8 : 4;
  const long long nsm = num_sms();
  const long long target = nsm * 8;  // one wave at 8 resident 256-thread blocks per SM
  const long long out = trans ? n : m;
  const long long red = trans ? m : n;
  if (!trans) {
    const long long rows_per_block = (long long)GEMV_THREADS * vec_of(a_dtype);
    p.grid_x = (unsigned)((m + rows_per_block - 1) / rows_per_block);
  } else {
    p.grid_x = (unsigned)((n + 7) / 8);
  }
  long long S = (target + p.grid_x - 1) / std::max<long long>(1, p.grid_x);
  const long long min_chunk = trans ? 32LL * vec_of(a_dtype) * 4 : 64;
  S = std::max(1LL, std::min(S, (red + min_chunk - 1) / min_chunk));
  S = std::min(S, 65535LL);
  p.chunk = (red + S - 1) / S;
  if (!trans) p.chunk = (p.chunk + 7) / 8 * 8;
  else p.chunk = (p.chunk + 32LL * vec_of(a_dtype) * 4 - 1) / (32LL * vec_of(a_dtype) * 4) * (32LL * vec_of(a_dtype) * 4);
  p.S = (int)((red + p.chunk - 1) / std::max(1LL, p.chunk));
  if (p.S < 1) p.S = 1;
  p.part_bytes = align_up((size_t)p.S * nrhs * out * acc_bytes, 256);
  p.fin_parts_bytes = align_up((size_t)finalize_blocks(out * nrhs) * sizeof(double), 256);
  p.total_bytes = p.part_bytes + p.fin_parts_bytes + 256;
  return p;
}

template <typename TA, int K>
static void launch_stage1(bool trans, const GemvPlan& p, const void* A, long long lda, long long m, long long n,
                          const void* X, long long ldx, void* P, bool vec_ok, const int* skip, cudaStream_t s) {
  using ACC = typename GemvTraits<TA>::Acc;
  dim3 grid(p.grid_x, p.S);
  if (!trans)
    launch(gemv_n_stage1<TA, K>, grid, GEMV_THREADS, 0, s, (const TA*)A, lda, m, n, (const ACC*)X, ldx, p.chunk,
                                                        (ACC*)P, vec_ok, skip);
  else
    launch(gemv_t_stage1<TA, K>, grid, GEMV_THREADS, 0, s, (const TA*)A, lda, m, n, (const ACC*)X, ldx, p.chunk,
                                                        (ACC*)P, vec_ok, skip);
}

template <typename TA>
static void launch_stage1_k(int K, bool trans, const GemvPlan& p, const void* A, long long lda, long long m,
                            long long n, const void* X, long long ldx, void* P, bool vec_ok, const int* skip,
                            cudaStream_t s) {
  switch (K) {
    case 1: launch_stage1<TA, 1>(trans, p, A, lda, m, n, X, ldx, P, vec_ok, skip, s); break;
    case 2: launch_stage1<TA, 2>(trans, p, A, lda, m, n, X, ldx, P, vec_ok, skip, s); break;
    case 4: launch_stage1<TA, 4>(trans, p, A, lda, m, n, X, ldx, P, vec_ok, skip, s); break;
    default: launch_stage1<TA, 8>(trans, p, A, lda, m, n, X, ldx, P, vec_ok, skip, s); break;
  }
}

int gemv_launch(int a_dtype, bool trans, const void* A, long long lda, long long m, long long n,
                const void* X, long long ldx, int nrhs, void* Y, long long ldy, double alpha, double beta,
                const void* Bsrc, long long ldb, double* nrm2, void* work, size_t work_bytes,
                cudaStream_t s, bool zero_ticket, const int* skip) {
  const int eb = elem_bytes(a_dtype);
  MPDOK_ARG_CHECK(eb > 0, "unknown A dtype");
  MPDOK_ARG_CHECK(m >= 0 && n >= 0 && lda >= std::max(1LL, m), "bad GEMV shape / lda");
  MPDOK_ARG_CHECK(nrhs >= 1, "nrhs must be >= 1");
  MPDOK_ARG_CHECK(nrm2 == nullptr || nrhs == 1, "norm output needs nrhs == 1");
  const long long out = trans ? n : m;
  const long long red = trans ? m : n;
  if (out == 0) return MPDOK_OK;
  const int acc_bytes = (a_dtype == MPDOK_F64) ? 8 : 4;
  const bool vec_ok = aligned16(A) && ((lda * eb) % 16 == 0);
  // Process right-hand sides in groups of 8 / 4 / 2 / 1.
  int done = 0;
  while (done < nrhs) {
    const int left = nrhs - done;
    const int K = left >= 8 ? 8 : left >= 4 ? 4 : left >= 2 ? 2 : 1;
    GemvPlan p = plan_gemv(a_dtype, m, n, K, trans);
    MPDOK_ARG_CHECK(work != nullptr && work_bytes >= p.total_bytes, "GEMV workspace too small");
    char* w = (char*)work;
    void* P = w;
    double* fin_parts = (double*)(w + p.part_bytes);
    unsigned* ticket = (unsigned*)(w + p.part_bytes + p.fin_parts_bytes);
    const char* Xk = (const char*)X + (size_t)done * ldx * acc_bytes;
    char* Yk = (char*)Y + (size_t)done * ldy * acc_bytes;
    const char* Bk = Bsrc ? (const char*)Bsrc + (size_t)done * ldb * acc_bytes : nullptr;
    if (red == 0) {
      // Empty reduction: y = beta * bsrc.  Use one zero split.
      MPDOK_CUDA_TRY(cudaMemsetAsync(P, 0, (size_t)K * out * acc_bytes, s));
      p.S = 1;
    } else {
      const int pslot = prof_start(a_dtype == MPDOK_F64 ? MPDOK_PROF_GEMV_F64 : MPDOK_PROF_GEMV_F32, s);
      switch (a_dtype) {
        case MPDOK_F64: launch_stage1_k<double>(K, trans, p, A, lda, m, n, Xk, ldx, P, vec_ok, skip, s); break;
        case MPDOK_F32: launch_stage1_k<float>(K, trans, p, A, lda, m, n, Xk, ldx, P, vec_ok, skip, s); break;
        case MPDOK_BF16: launch_stage1_k<__nv_bfloat16>(K, trans, p, A, lda, m, n, Xk, ldx, P, vec_ok, skip, s); break;
        case MPDOK_F16: launch_stage1_k<__half>(K, trans, p, A, lda, m, n, Xk, ldx, P, vec_ok, skip, s); break;
      }
      prof_stop(pslot, s, (double)m * (double)n * eb + (double)K * (double)(m + n) * acc_bytes, skip);
      MPDOK_LAUNCH_CHECK("gemv stage1");
    }
    if (nrm2 && zero_ticket) MPDOK_CUDA_TRY(cudaMemsetAsync(ticket, 0, sizeof(unsigned), s));
    const unsigned fb = finalize_blocks(out * K);
    if (a_dtype == MPDOK_F64)
      launch(gemv_finalize<double>, fb, GEMV_THREADS, 0, s, (const double*)P, p.S, K, out, alpha, beta,
                                                       (const double*)Bk, ldb, (double*)Yk, ldy, fin_parts,
                                                       ticket, nrm2, skip);
    else
      launch(gemv_finalize<float>, fb, GEMV_THREADS, 0, s, (const float*)P, p.S, K, out, (float)alpha, (float)beta,
                                                      (const float*)Bk, ldb, (float*)Yk, ldy, fin_parts, ticket,
                                                      nrm2, skip);
    MPDOK_LAUNCH_CHECK("gemv finalize");
    done += K;
  }
  return MPDOK_OK;
}

size_t gemv_workspace_bytes(int a_dtype, long long m, long long n, int nrhs, bool trans) {
  size_t best = 0;
  for (int K : {1, 2, 4, 8}) {
    if (K > std::max(1, nrhs) && K != 1) break;
    GemvPlan p = plan_gemv(a_dtype, m, n, K, trans);
    best = std::max(best, p.total_bytes);
  }
  return best;
}

}  // namespace mpdok

using namespace mpdok;

extern "C" size_t mpdok_gemv_workspace_size(int a_dtype, long long m, long long n, int nrhs, int trans) {
  return gemv_workspace_bytes(a_dtype, m, n, nrhs, trans != 0);
}

extern "C" int mpdok_gemv(int a_dtype, int trans, const void* A, long long lda, long long m, long long n,
                          const void* X, long long ldx, int nrhs, void* Y, long long ldy, double alpha,
                          double beta, void* work, size_t work_bytes, cudaStream_t stream) {
  MPDOK_ARG_CHECK(A != nullptr || m == 0 || n == 0, "null A");
  return gemv_launch(a_dtype, trans != 0, A, lda, m, n, X, ldx, nrhs, Y, ldy, alpha, beta, Y, ldy, nullptr, work,
                     work_bytes, stream, true, nullptr);
}

extern "C" int mpdok_residual(const double* A, long long lda, long long n, const double* b, const double* x,
                              double* r, double* rnorm2, void* work, size_t work_bytes, cudaStream_t stream) {
  MPDOK_ARG_CHECK(n >= 0, "negative n");
  if (n == 0) return MPDOK_OK;
  MPDOK_ARG_CHECK(A && b && x && r, "null pointer");
  return gemv_launch(MPDOK_F64, false, A, lda, n, n, x, n, 1, r, n, -1.0, 1.0, b, n, rnorm2, work, work_bytes,
                     stream, true, nullptr);
}

// ------------------------------------------------------------------------
// GEMV that allocates nothing.
//
// Some callers cannot allocate device memory at the point where they need a
// matrix-vector product: a host application that has already handed every
// byte of the GPU to its own memory pool, or a caller that must not trigger
// the device-wide synchronisation a cudaMalloc / cudaFree can cause while
// other work is in flight.  mpdok_gemv_noalloc serves them with the same
// kernels as mpdok_gemv, using as scratch a file-scope device array of
// MPDOK_NOALLOC_SCRATCH_BYTES that every GPU loading this library holds until
// the process exits.

namespace mpdok {

static __device__ __align__(256) unsigned char g_noalloc_scratch[MPDOK_NOALLOC_SCRATCH_BYTES];

// Device address of g_noalloc_scratch on the current device, looked up once
// per device with that device current (the host-side name is only a stand-in
// for the device array and must never be passed to a kernel).
static int noalloc_scratch(void** out) {
  static std::mutex mu;
  static void* addr[64] = {};
  int dev = 0;
  MPDOK_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) {
    set_error("invalid argument: device ordinal %d out of range", dev);
    return MPDOK_ERR_INVALID_ARG;
  }
  std::lock_guard<std::mutex> lk(mu);
  if (addr[dev] == nullptr) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    addr[dev] = p;
  }
  *out = addr[dev];
  return MPDOK_OK;
}

}  // namespace mpdok

extern "C" int mpdok_gemv_noalloc(int a_dtype, int trans, const void* A, long long lda, long long m, long long n,
                                  const void* X, long long ldx, int nrhs, void* Y, long long ldy, double alpha,
                                  double beta, cudaStream_t stream) {
  MPDOK_ARG_CHECK(A != nullptr || m == 0 || n == 0, "null A");
  MPDOK_ARG_CHECK(m >= 0 && n >= 0 && nrhs >= 1, "bad GEMV shape");
  const size_t need = gemv_workspace_bytes(a_dtype, m, n, nrhs, trans != 0);
  if (need > (size_t)MPDOK_NOALLOC_SCRATCH_BYTES) {
    set_error("invalid argument: this GEMV needs %zu bytes of scratch, more than the %u-byte built-in scratch of "
              "mpdok_gemv_noalloc; use mpdok_gemv with a caller-owned workspace",
              need, (unsigned)MPDOK_NOALLOC_SCRATCH_BYTES);
    return MPDOK_ERR_INVALID_ARG;
  }
  void* scratch = nullptr;
  MPDOK_TRY(noalloc_scratch(&scratch));
  // The partial sums are written in full before they are read and no norm is
  // requested (so the reduction ticket is unused): nothing needs clearing.
  return gemv_launch(a_dtype, trans != 0, A, lda, m, n, X, ldx, nrhs, Y, ldy, alpha, beta, Y, ldy, nullptr, scratch,
                     (size_t)MPDOK_NOALLOC_SCRATCH_BYTES, stream, false, nullptr);
}
