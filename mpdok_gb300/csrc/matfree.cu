// Matrix-free fused evaluate-and-multiply for RBF operators.
//
//   Y = K(rows, cols) X (+ reg X on the matrix diagonal),
//   K(i, j) = phi(||r_i - c_j||): Gaussian exp(-gamma d^2) or multiquadric sqrt(1 + gamma d^2).
//
// Replaces the per-tile DGEMM + exp + GEMV of mpdok_ooc.py:205-227
// (_tiled_dgemv_fp64, matrix-free FP64 residual) and the stored FP32 operator
// of the inner Krylov solves (mpdok_ooc.py:158-195): A never touches HBM.
//
// FP32 kernel: column centres (packed FP32 float4) and the matching X values
// are staged into shared memory by TMA (cp.async.bulk.tensor, two-stage ring on
// mbarriers); every thread owns two rows, keeps their centres in registers and
// recomputes each entry (d^2 from coordinate differences, then ex2.approx or
// rsqrt.approx), accumulating k right-hand sides.  The column range is split
// S ways for occupancy; splits are combined in a fixed order (bitwise
// reproducible).  Bound: the special-function pipe (one MUFU op per entry).
//
// FP64 kernel (residuals): the same loop in FP64 arithmetic with CUDA's exp /
// sqrt, for r = b - K x accurate to FP64 rounding.
#include "krylov.cuh"
#include "matfree.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstring>
#include <mutex>

namespace mpdok {

constexpr int MF_THREADS = 256;
constexpr int MF_RPT = 2;
constexpr int MF_ROWS = MF_THREADS * MF_RPT;  // 512 rows per block
constexpr int MF_BC = 128;                     // columns per staged tile
constexpr long long MF_WAIT = 1LL << 26;

__global__ void k_pack_coords(const double* __restrict__ c, long long n, int dim, float4* __restrict__ out) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float v[3] = {0.f, 0.f, 0.f};
    for (int d = 0; d < dim; ++d) v[d] = (float)c[i * dim + d];
    out[i] = make_float4(v[0], v[1], v[2], 0.f);
  }
}

__device__ __forceinline__ uint32_t s_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool mf_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ float rsqrt_approx(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

template <int KIND, int K>
__global__ void __launch_bounds__(MF_THREADS)
k_matfree_f32(const __grid_constant__ CUtensorMap tmC, const __grid_constant__ CUtensorMap tmX,
              const float4* __restrict__ rowpack, long long nrows, long long ncols, long long chunk, float g,
              float* __restrict__ P, int* err, const int* skip) {
  __shared__ __align__(128) float4 sC[2][MF_BC];
  __shared__ __align__(128) float sX[2][K][MF_BC];
  __shared__ __align__(8) unsigned long long bars[2];
  __shared__ int s_fail;
  if (skip != nullptr && *skip) return;
  const int tid = threadIdx.x;
  const long long r0 = (long long)blockIdx.x * MF_ROWS;
  const int sidx = blockIdx.y;
  const long long cb = (long long)sidx * chunk;
  const long long ce = min(ncols, cb + chunk);
  const int ntiles = (int)((ce - cb + MF_BC - 1) / MF_BC);
  const uint32_t bar0 = s_u32(&bars[0]);
  constexpr uint32_t TILE_BYTES = MF_BC * 16 + K * MF_BC * 4;
  if (tid == 0) {
    s_fail = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar0));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar0 + 8));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  auto issue = [&](int t) {
    const int st = t & 1;
    const uint32_t bar = bar0 + 8 * st;
    const int j0 = (int)(cb + (long long)t * MF_BC);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(TILE_BYTES) : "memory");
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::
            "r"(s_u32(&sC[st][0])), "l"(reinterpret_cast<uint64_t>(&tmC)), "r"(bar), "r"(0), "r"(j0)
        : "memory");
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::
            "r"(s_u32(&sX[st][0][0])), "l"(reinterpret_cast<uint64_t>(&tmX)), "r"(bar), "r"(j0), "r"(0)
        : "memory");
  };
  if (tid == 0) {
    if (ntiles > 0) issue(0);
    if (ntiles > 1) issue(1);
  }
  static_assert(MF_RPT == 2, "a thread's rows are one packed pair");
  float4 rc[MF_RPT];
  float2 accp[K];  // (row 0, row 1) per right-hand side
#pragma unroll
  for (int t = 0; t < MF_RPT; ++t) {
    const long long r = r0 + tid + (long long)t * MF_THREADS;
    rc[t] = (r < nrows) ? rowpack[r] : make_float4(0.f, 0.f, 0.f, 0.f);
  }
#pragma unroll
  for (int kk = 0; kk < K; ++kk) accp[kk] = make_float2(0.f, 0.f);
  const float2 rx = make_float2(rc[0].x, rc[1].x), ry = make_float2(rc[0].y, rc[1].y),
               rz = make_float2(rc[0].z, rc[1].z);
  for (int t = 0; t < ntiles; ++t) {
    const int st = t & 1;
    // every thread observes the completed phase (acquire of the TMA writes)
    bool ok = false;
    for (long long it = 0; it < MF_WAIT; ++it) {
      if (mf_try_wait(bar0 + 8 * st, (uint32_t)((t >> 1) & 1))) { ok = true; break; }
    }
    if (!ok) atomicExch(&s_fail, 1);
    __syncthreads();
    if (s_fail) break;
    const int nb = (int)min((long long)MF_BC, ce - (cb + (long long)t * MF_BC));
#pragma unroll 4
    for (int j = 0; j < nb; ++j) {
      const float4 c = sC[st][j];
      // the thread's two rows as packed pairs (FP32x2 pipe): per lane the
      // same IEEE operations, in the same order, as
      //   d2 = fma(dx, dx, fma(dy, dy, dz * dz)),  acc = fma(v, x_j, acc)
      const float2 dx = __fadd2_rn(rx, make_float2(-c.x, -c.x));
      const float2 dy = __fadd2_rn(ry, make_float2(-c.y, -c.y));
      const float2 dz = __fadd2_rn(rz, make_float2(-c.z, -c.z));
      const float2 d2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __fmul2_rn(dz, dz)));
      float2 v;
      if (KIND == MPDOK_KERNEL_GAUSSIAN) {
        const float2 e = __fmul2_rn(make_float2(g, g), d2);  // g = -gamma * log2(e)
        v = make_float2(ex2_approx(e.x), ex2_approx(e.y));
      } else {
        const float2 a = __ffma2_rn(make_float2(g, g), d2, make_float2(1.f, 1.f));  // g = gamma
        v = __fmul2_rn(a, make_float2(rsqrt_approx(a.x), rsqrt_approx(a.y)));
      }
#pragma unroll
      for (int kk = 0; kk < K; ++kk) {
        const float xj = sX[st][kk][j];
        accp[kk] = __ffma2_rn(v, make_float2(xj, xj), accp[kk]);
      }
    }
    __syncthreads();
    if (tid == 0 && t + 2 < ntiles) issue(t + 2);
  }
  if (s_fail) {
    if (tid == 0 && err) atomicExch(err, 1);
    return;
  }
#pragma unroll
  for (int u = 0; u < MF_RPT; ++u) {
    const long long r = r0 + tid + (long long)u * MF_THREADS;
    if (r < nrows) {
#pragma unroll
      for (int kk = 0; kk < K; ++kk) P[((long long)sidx * K + kk) * nrows + r] = u == 0 ? accp[kk].x : accp[kk].y;
    }
  }
}

// FP64 evaluate-and-multiply (residual accuracy).  Column centres staged in
// shared memory by plain loads; one row per thread.
template <int KIND>
__global__ void __launch_bounds__(MF_THREADS)
k_matfree_f64(const double* __restrict__ rows, const double* __restrict__ cols, int dim, long long nrows,
              long long ncols, long long chunk, double gamma, const double* __restrict__ X, long long ldx, int K,
              double* __restrict__ P) {
  __shared__ double sc[MF_BC][3];
  __shared__ double sx[8][MF_BC];
  const int tid = threadIdx.x;
  const long long r = (long long)blockIdx.x * MF_THREADS + tid;
  const int sidx = blockIdx.y;
  const long long cb = (long long)sidx * chunk;
  const long long ce = min(ncols, cb + chunk);
  double rr[3] = {0.0, 0.0, 0.0};
  if (r < nrows)
    for (int d = 0; d < dim; ++d) rr[d] = rows[r * dim + d];
  double acc[8];
#pragma unroll
  for (int kk = 0; kk < 8; ++kk) acc[kk] = 0.0;
  for (long long j0 = cb; j0 < ce; j0 += MF_BC) {
    const int nb = (int)min((long long)MF_BC, ce - j0);
    __syncthreads();
    for (int t = tid; t < MF_BC * 3; t += MF_THREADS) {
      const int j = t / 3, d = t % 3;
      sc[j][d] = (j < nb && d < dim) ? cols[(j0 + j) * dim + d] : 0.0;
    }
    for (int t = tid; t < K * MF_BC; t += MF_THREADS) {
      const int kk = t / MF_BC, j = t % MF_BC;
      sx[kk][j] = (j < nb) ? X[(j0 + j) + kk * ldx] : 0.0;
    }
    __syncthreads();
    if (r < nrows) {
      for (int j = 0; j < nb; ++j) {
        const double dx = rr[0] - sc[j][0], dy = rr[1] - sc[j][1], dz = rr[2] - sc[j][2];
        const double d2 = fma(dx, dx, fma(dy, dy, dz * dz));
        const double v = (KIND == MPDOK_KERNEL_GAUSSIAN) ? exp(-gamma * d2) : sqrt(fma(gamma, d2, 1.0));
        for (int kk = 0; kk < K; ++kk) acc[kk] = fma(v, sx[kk][j], acc[kk]);
      }
    }
  }
  if (r < nrows)
    for (int kk = 0; kk < K; ++kk) P[((long long)sidx * K + kk) * nrows + r] = acc[kk];
}

// y = alpha * sum_s P + beta * y + reg * x_shift ; FP32 or FP64; optional
// per-column sum of squares (residual mode: alpha = -1, y preloaded with b).
// A timed-out evaluation (err[0] set by k_matfree_f32) leaves its partial
// sums unwritten: the product is then NaN, not a silently wrong number, and
// the sticky word err[1] tells the solve that owns this workspace why.
template <typename T>
__global__ void __launch_bounds__(MF_THREADS)
k_mf_finalize(const T* __restrict__ P, int S, int K, long long nrows, T alpha, T beta, const T* bsrc, long long ldb,
              T reg, const T* xs, long long ldx, T* y, long long ldy, const int* skip, int* err) {
  if (skip != nullptr && *skip) return;
  const long long total = nrows * K;
  if (err != nullptr && *(volatile int*)err != 0) {
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicExch(err + 1, 1);
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x)
      y[idx % nrows + (idx / nrows) * ldy] = T(NAN);
    return;
  }
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long i = idx % nrows;
    const int kk = (int)(idx / nrows);
    T sum = T(0);
    for (int s = 0; s < S; ++s) sum += P[((long long)s * K + kk) * nrows + i];
    T v = alpha * sum;
    if (reg != T(0) && xs) v = fma(alpha * reg, xs[i + kk * ldx], v);
    if (beta != T(0)) v = fma(beta, bsrc[i + kk * ldb], v);
    y[i + kk * ldy] = v;
  }
}

// ------------------------------------------------------------------ host

static PFN_cuTensorMapEncodeTiled_v12000 mf_encode() {
  static std::once_flag once;
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

static int map2d_f32(CUtensorMap* m, const void* ptr, long long inner, long long outer, long long pitch_bytes,
                     int box_inner, int box_outer) {
  auto enc = mf_encode();
  if (!enc) {
    set_error("cuTensorMapEncodeTiled unavailable from the driver");
    return MPDOK_ERR_UNSUPPORTED;
  }
  cuuint64_t gdim[2] = {(cuuint64_t)inner, (cuuint64_t)outer};
  cuuint64_t gstr[1] = {(cuuint64_t)pitch_bytes};
  cuuint32_t box[2] = {(cuuint32_t)box_inner, (cuuint32_t)box_outer};
  cuuint32_t es[2] = {1, 1};
  CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(ptr), gdim, gstr, box, es,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
    return MPDOK_ERR_CUDA;
  }
  return MPDOK_OK;
}

struct MfPlan {
  int S = 1;
  long long chunk = 0;
  unsigned gx = 1;
  size_t part_bytes = 0;
};

static MfPlan mf_plan(long long nrows, long long ncols, int K, bool f64) {
  MfPlan p;
  const long long rows_per_block = f64 ? MF_THREADS : MF_ROWS;
  p.gx = (unsigned)std::max(1LL, (nrows + rows_per_block - 1) / rows_per_block);
  const long long target = (long long)num_sms() * (f64 ? 8 : 4);
  long long S = (target + p.gx - 1) / p.gx;
  S = std::max(1LL, std::min(S, (ncols + MF_BC - 1) / MF_BC));
  S = std::min(S, 65535LL);
  p.chunk = (ncols + S - 1) / S;
  p.chunk = (p.chunk + MF_BC - 1) / MF_BC * MF_BC;
  p.S = (int)std::max(1LL, (ncols + p.chunk - 1) / p.chunk);
  p.part_bytes = align_up((size_t)p.S * K * std::max(1LL, nrows) * (f64 ? 8 : 4), 256);
  return p;
}

// Workspace: [0, 256) status words (err[0] of the last FP32 evaluation, err[1]
// sticky for the solve), then the split partial sums, then (FP32) the packed
// row and column centres.
constexpr size_t MF_STATUS = 256;

size_t matfree_work_bytes(long long nrows, long long ncols, int nrhs, int precision) {
  const bool f64 = precision == MPDOK_F64;
  const MfPlan p = mf_plan(nrows, ncols, nrhs, f64);
  size_t b = p.part_bytes + MF_STATUS;
  if (!f64) b += align_up((size_t)std::max(1LL, nrows) * 16, 256) + align_up((size_t)std::max(1LL, ncols) * 16, 256);
  return b;
}

template <int KIND, int K>
static void launch_mf32(const CUtensorMap& mc, const CUtensorMap& mx, const float4* rp, long long nr, long long nc,
                        const MfPlan& p, float g, float* P, int* err, const int* skip, cudaStream_t s) {
  dim3 grid(p.gx, p.S);
  k_matfree_f32<KIND, K><<<grid, MF_THREADS, 0, s>>>(mc, mx, rp, nr, nc, p.chunk, g, P, err, skip);
  count_launch();
}

int matfree_apply(const MfOperand& op, int precision, const void* X, long long ldx, int K, void* Y, long long ldy,
                  double alpha, double beta, const void* Bsrc, long long ldb, void* work, size_t work_bytes,
                  cudaStream_t s, const int* skip) {
  const bool f64 = precision == MPDOK_F64;
  MPDOK_ARG_CHECK(K >= 1 && K <= 8, "matrix-free apply supports 1..8 right-hand sides");
  MPDOK_ARG_CHECK(op.dim >= 1 && op.dim <= 3, "dim must be 1, 2 or 3");
  const long long nr = op.nrows, nc = op.ncols;
  if (nr == 0) return MPDOK_OK;
  const MfPlan p = mf_plan(nr, nc, K, f64);
  MPDOK_ARG_CHECK(work_bytes >= matfree_work_bytes(nr, nc, K, precision), "matrix-free workspace too small");
  // the nugget applies where row i meets column i + diag_offset, for a row range inside the columns
  const bool has_reg = op.reg != 0.0;
  MPDOK_ARG_CHECK(!has_reg || (op.diag_offset >= 0 && op.diag_offset + nr <= nc),
                  "nugget needs rows [0, n_rows) to map inside the columns");
  char* w = (char*)work;
  int* err = (int*)w;
  void* P = w + MF_STATUS;
  MPDOK_ARG_CHECK(!f64 || skip == nullptr, "FP64 evaluation is not predicated");
  const int slot = prof_start(MPDOK_PROF_MATFREE, s);
  if (nc == 0) {
    MPDOK_CUDA_TRY(cudaMemsetAsync(P, 0, p.part_bytes, s));
  } else if (f64) {
    dim3 grid(p.gx, p.S);
    if (op.kernel == MPDOK_KERNEL_GAUSSIAN)
      launch(k_matfree_f64<MPDOK_KERNEL_GAUSSIAN>, grid, MF_THREADS, 0, s, op.rows, op.cols, op.dim, nr, nc,
             p.chunk, op.gamma, (const double*)X, ldx, K, (double*)P);
    else
      launch(k_matfree_f64<MPDOK_KERNEL_MQ>, grid, MF_THREADS, 0, s, op.rows, op.cols, op.dim, nr, nc, p.chunk,
             op.gamma, (const double*)X, ldx, K, (double*)P);
  } else {
    MPDOK_ARG_CHECK(aligned16(X) && (ldx * 4) % 16 == 0, "FP32 X must be 16-byte aligned with ldx % 4 == 0");
    float4* rp = (float4*)(w + MF_STATUS + p.part_bytes);
    float4* cp = (float4*)((char*)rp + align_up((size_t)nr * 16, 256));
    const float4* rows_p = op.rows_packed;
    const float4* cols_p = op.cols_packed;
    if (!rows_p) {
      launch(k_pack_coords, (unsigned)std::min<long long>((nr + 255) / 256, 1024), 256, 0, s, op.rows, nr, op.dim, rp);
      rows_p = rp;
    }
    if (!cols_p) {
      launch(k_pack_coords, (unsigned)std::min<long long>((nc + 255) / 256, 1024), 256, 0, s, op.cols, nc, op.dim, cp);
      cols_p = cp;
    }
    CUtensorMap mc, mx;
    MPDOK_TRY(map2d_f32(&mc, cols_p, 4, nc, 16, 4, MF_BC));
    MPDOK_TRY(map2d_f32(&mx, X, nc, K, ldx * 4, MF_BC, K));
    const float g = (op.kernel == MPDOK_KERNEL_GAUSSIAN) ? (float)(-op.gamma * 1.4426950408889634) : (float)op.gamma;
    MPDOK_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), s));
#define MF_CASE(KK)                                                                                           \
  case KK:                                                                                                    \
    if (op.kernel == MPDOK_KERNEL_GAUSSIAN)                                                                   \
      launch_mf32<MPDOK_KERNEL_GAUSSIAN, KK>(mc, mx, rows_p, nr, nc, p, g, (float*)P, err, skip, s);                \
    else                                                                                                      \
      launch_mf32<MPDOK_KERNEL_MQ, KK>(mc, mx, rows_p, nr, nc, p, g, (float*)P, err, skip, s);                      \
    break;
    switch (K) {
      MF_CASE(1) MF_CASE(2) MF_CASE(3) MF_CASE(4) MF_CASE(5) MF_CASE(6) MF_CASE(7) MF_CASE(8)
    }
#undef MF_CASE
  }
  MPDOK_LAUNCH_CHECK("matfree");
  prof_stop(slot, s, (double)nr * (double)nc * K, skip);
  const unsigned fb = (unsigned)std::max(1LL, std::min<long long>((nr * K + 255) / 256, (long long)num_sms() * 4));
  if (f64)
    launch(k_mf_finalize<double>, fb, MF_THREADS, 0, s, (const double*)P, p.S, K, nr, alpha, beta,
           (const double*)Bsrc, ldb, op.reg, has_reg ? (const double*)X + op.diag_offset : (const double*)nullptr, ldx,
           (double*)Y, ldy, (const int*)nullptr, (int*)nullptr);
  else
    launch(k_mf_finalize<float>, fb, MF_THREADS, 0, s, (const float*)P, p.S, K, nr, (float)alpha, (float)beta,
           (const float*)Bsrc, ldb, (float)op.reg, has_reg ? (const float*)X + op.diag_offset : (const float*)nullptr,
           ldx, (float*)Y, ldy, skip, nc == 0 ? (int*)nullptr : err);
  MPDOK_LAUNCH_CHECK("matfree finalize");
  return MPDOK_OK;
}

// Krylov operator adapters -------------------------------------------------

static int mf_apply32(const void* ctx, const float* x, float* y, int nrhs, long long ld, cudaStream_t s,
                      const int* skip) {
  const MfCtx* c = (const MfCtx*)ctx;
  return matfree_apply(c->op, MPDOK_F32, x, ld, nrhs, y, ld, 1.0, 0.0, nullptr, 0, c->w32, c->w32_bytes, s, skip);
}

static int mf_residual64(const void* ctx, const double* b, const double* x, double* r, double* nrm2, int nrhs,
                         long long ld, cudaStream_t s) {
  const MfCtx* c = (const MfCtx*)ctx;
  MPDOK_TRY(matfree_apply(c->op, MPDOK_F64, x, ld, nrhs, r, ld, -1.0, 1.0, b, ld, c->w64, c->w64_bytes, s, nullptr));
  return colnorms_f64(r, c->op.nrows, nrhs, ld, nrm2, s);
}

int mf_timeout_clear(const MfCtx* c, cudaStream_t s) {
  MPDOK_CUDA_TRY(cudaMemsetAsync(c->w32, 0, 2 * sizeof(int), s));
  return MPDOK_OK;
}

int mf_timeout_finish(const MfCtx* c, int status, cudaStream_t s) {
  if (status == MPDOK_ERR_CUDA || status == MPDOK_ERR_ALLOC) return status;
  int h = 0;
  MPDOK_CUDA_TRY(cudaMemcpyAsync(&h, (const int*)c->w32 + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
  MPDOK_CUDA_TRY(cudaStreamSynchronize(s));
  if (h != 0) {
    set_error("matrix-free product: a wait on a staged centre tile ran out (device wait limit)");
    return MPDOK_ERR_TIMEOUT;
  }
  return status;
}

Operator32 mf_op32(const MfCtx* c) {
  Operator32 o;
  o.apply = mf_apply32;
  o.ctx = c;
  return o;
}

Residual64 mf_res64(const MfCtx* c) {
  Residual64 o;
  o.apply = mf_residual64;
  o.ctx = c;
  return o;
}

}  // namespace mpdok

using namespace mpdok;

extern "C" size_t mpdok_matfree_workspace_size(long long n_rows, long long n_cols, int nrhs, int precision) {
  if (n_rows < 0 || n_cols < 0 || nrhs < 1) return 0;
  return matfree_work_bytes(n_rows, n_cols, nrhs, precision);
}

extern "C" int mpdok_matfree_apply(const double* rows, long long n_rows, const double* cols, long long n_cols,
                                   int dim, int kernel, double gamma, double reg, long long diag_offset,
                                   int precision, const void* X, long long ldx, int nrhs, void* Y, long long ldy,
                                   void* work, size_t work_bytes, cudaStream_t stream) {
  MPDOK_ARG_CHECK(n_rows >= 0 && n_cols >= 0, "negative size");
  MPDOK_ARG_CHECK(precision == MPDOK_F32 || precision == MPDOK_F64, "precision must be FP32 or FP64");
  MPDOK_ARG_CHECK(kernel == MPDOK_KERNEL_GAUSSIAN || kernel == MPDOK_KERNEL_MQ, "unknown kernel");
  if (n_rows == 0) return MPDOK_OK;
  MPDOK_ARG_CHECK(rows && cols && X && Y && work, "null pointer");
  MPDOK_ARG_CHECK(ldx >= n_cols && ldy >= n_rows, "leading dimension too small");
  MfOperand op;
  op.rows = rows;
  op.cols = cols;
  op.nrows = n_rows;
  op.ncols = n_cols;
  op.dim = dim;
  op.kernel = kernel;
  op.gamma = gamma;
  op.reg = reg;
  op.diag_offset = diag_offset;
  return matfree_apply(op, precision, X, ldx, nrhs, Y, ldy, 1.0, 0.0, nullptr, 0, work, work_bytes, stream, nullptr);
}

extern "C" size_t mpdok_mf_krylov_workspace_size(long long n, int restart) {
  if (n < 0 || restart < 1) return 0;
  return krylov_layout(n, restart, nullptr).total + matfree_work_bytes(n, n, 8, MPDOK_F32) +
         matfree_work_bytes(n, n, 8, MPDOK_F64) + 512;
}

static int mf_setup(const double* coords, long long n, int dim, int kernel, double gamma, double reg, int restart,
                    void* work, size_t work_bytes, KWs* ws, MfCtx* c, cudaStream_t s) {
  MPDOK_ARG_CHECK(work_bytes >= mpdok_mf_krylov_workspace_size(n, restart), "matrix-free Krylov workspace too small");
  *ws = krylov_layout(n, restart, work);
  MPDOK_TRY(ws_prepare(*ws, work_bytes, s));
  char* w = (char*)work + align_up(ws->total, 256);
  c->op.rows = coords;
  c->op.cols = coords;
  c->op.nrows = n;
  c->op.ncols = n;
  c->op.dim = dim;
  c->op.kernel = kernel;
  c->op.gamma = gamma;
  c->op.reg = reg;
  c->op.diag_offset = 0;
  c->w32 = w;
  c->w32_bytes = matfree_work_bytes(n, n, 8, MPDOK_F32);
  c->w64 = w + align_up(c->w32_bytes, 256);
  c->w64_bytes = matfree_work_bytes(n, n, 8, MPDOK_F64);
  // pack the centres once for every FP32 apply of the solve
  const MfPlan p = mf_plan(n, n, 8, false);
  float4* rp = (float4*)(w + MF_STATUS + p.part_bytes);
  launch(k_pack_coords, (unsigned)std::min<long long>((n + 255) / 256, 1024), 256, 0, s, coords, n, dim, rp);
  MPDOK_LAUNCH_CHECK("pack");
  c->op.rows_packed = rp;
  c->op.cols_packed = rp;
  return MPDOK_OK;
}

extern "C" int mpdok_mf_gmres_ir(const double* coords, long long n, int dim, int kernel, double gamma, double reg,
                                 const double* b, double* x, double tol, int maxiter_outer, int restart,
                                 double inner_tol, void* work, size_t work_bytes, mpdok_solve_info* info,
                                 cudaStream_t s) {
  if (info) std::memset(info, 0, sizeof(*info));
  MPDOK_ARG_CHECK(n >= 0, "negative n");
  MPDOK_ARG_CHECK(restart >= 1 && restart <= 1024, "restart must be in [1, 1024]");
  if (n == 0) { if (info) info->converged = 1; return MPDOK_OK; }
  MPDOK_ARG_CHECK(coords && b && x && work, "null pointer");
  KWs ws;
  MfCtx c;
  MPDOK_TRY(mf_setup(coords, n, dim, kernel, gamma, reg, restart, work, work_bytes, &ws, &c, s));
  MPDOK_TRY(mf_timeout_clear(&c, s));
  return mf_timeout_finish(&c, gmres_ir_core(ws, mf_op32(&c), mf_res64(&c), b, x, tol, maxiter_outer, restart,
                                             inner_tol, nullptr, info, s), s);
}

extern "C" int mpdok_mf_cg(const double* coords, long long n, int dim, int kernel, double gamma, double reg,
                           const double* b, double* x, double tol, int maxiter, int check_every, void* work,
                           size_t work_bytes, mpdok_solve_info* info, cudaStream_t s) {
  if (info) std::memset(info, 0, sizeof(*info));
  MPDOK_ARG_CHECK(n >= 0, "negative n");
  MPDOK_ARG_CHECK(check_every >= 1, "check_every must be >= 1");
  if (n == 0) { if (info) info->converged = 1; return MPDOK_OK; }
  MPDOK_ARG_CHECK(coords && b && x && work, "null pointer");
  KWs ws;
  MfCtx c;
  MPDOK_TRY(mf_setup(coords, n, dim, kernel, gamma, reg, 1, work, work_bytes, &ws, &c, s));
  MPDOK_TRY(mf_timeout_clear(&c, s));
  return mf_timeout_finish(&c, cg_core(ws, mf_op32(&c), mf_res64(&c), b, x, tol, maxiter, check_every, info, s), s);
}
