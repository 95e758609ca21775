// Split-precision stored operator ("Ozaki-style" two-slice products).
//
// A (FP64) is stored as two FP32 slices, A = A_hi + A_lo with
// A_hi = fl32(a) and A_lo = fl32(a - A_hi) (48 significant bits, 8 bytes per
// entry: the same HBM traffic as FP64).  The GEMV forms every product with an
// error-free transformation on the FP32 pipe,
//     p = a_hi x_hi,  e = fma(a_hi, x_hi, -p) + a_hi x_lo + a_lo x_hi,
// and sums the p in double-float (two-sum) and the e in FP32, so y = A x is
// accurate to ~2^-44 relative to |A||x| without touching GB300's narrow FP64
// pipe (cuBLAS DGEMM measures 1.1 TFLOP/s there).  It serves
//   * the FP64 residual r = b - A x of the refinement loops (x in FP64, split
//     into x_hi + x_lo when staged), fastest against native FP64 for several
//     right-hand sides;
//   * an FP32-output inner operator whose products are as accurate as the
//     FP64 matrix, for systems too ill-conditioned for an FP32 A (kappa * 6e-8
//     >= 1, the C2 family).
#include "krylov.cuh"
#include "split.cuh"

namespace mpdok {

constexpr int SP_THREADS = 256;
constexpr int SP_VEC = 4;
constexpr int SP_TB = 256;  // columns of x staged per batch
constexpr int SP_UNR = 4;

__global__ void k_split(const double* __restrict__ A, long long lda, float* __restrict__ hi, float* __restrict__ lo,
                        long long ld, long long m, long long n) {
  for (long long j = blockIdx.y; j < n; j += gridDim.y)
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < m;
         i += (long long)gridDim.x * blockDim.x) {
      const double a = A[i + j * lda];
      const float h = (float)a;
      hi[i + j * ld] = h;
      lo[i + j * ld] = (float)(a - (double)h);
    }
}

__device__ __forceinline__ void two_sum(float& s, float& c, float p) {
  const float t = s + p;
  const float z = t - s;
  c += (s - (t - z)) + (p - z);
  s = t;
}

// Partial sums P[s][k][row] (FP64) of (A_hi + A_lo)(x_hi + x_lo) over column split s.
template <int K, typename TX>
__global__ void __launch_bounds__(SP_THREADS)
k_split_gemv(const float* __restrict__ Ahi, const float* __restrict__ Alo, long long lda, long long m, long long n,
             const TX* __restrict__ X, long long ldx, long long chunk, double* __restrict__ P, const int* skip) {
  __shared__ float sxh[K][SP_TB];
  __shared__ float sxl[K][SP_TB];
  if (skip != nullptr && *skip) return;
  const long long row0 = ((long long)blockIdx.x * SP_THREADS + threadIdx.x) * SP_VEC;
  const int sidx = blockIdx.y;
  const long long cb0 = (long long)sidx * chunk;
  const long long ce = min(n, cb0 + chunk);
  float sh[SP_VEC][K], sl[SP_VEC][K];
#pragma unroll
  for (int v = 0; v < SP_VEC; ++v)
#pragma unroll
    for (int k = 0; k < K; ++k) { sh[v][k] = 0.f; sl[v][k] = 0.f; }
  const bool full = row0 + SP_VEC <= m;
  for (long long cb = cb0; cb < ce; cb += SP_TB) {
    const int nb = (int)min((long long)SP_TB, ce - cb);
    __syncthreads();
    for (int t = threadIdx.x; t < K * SP_TB; t += SP_THREADS) {
      const int k = t / SP_TB, j = t % SP_TB;
      if (j < nb) {
        const TX xv = X[(cb + j) + k * ldx];
        const float h = (float)xv;
        sxh[k][j] = h;
        sxl[k][j] = (float)((double)xv - (double)h);
      } else {
        sxh[k][j] = 0.f;
        sxl[k][j] = 0.f;
      }
    }
    __syncthreads();
    if (row0 >= m) continue;
    const float* ah = Ahi + row0 + cb * lda;
    const float* al = Alo + row0 + cb * lda;
    int j = 0;
    for (; j < nb; j += SP_UNR) {
      const int ju = min(SP_UNR, nb - j);
      float4 vh[SP_UNR], vl[SP_UNR];
#pragma unroll
      for (int u = 0; u < SP_UNR; ++u) {
        if (u < ju && full) {
          vh[u] = __ldg(reinterpret_cast<const float4*>(ah + (long long)(j + u) * lda));
          vl[u] = __ldg(reinterpret_cast<const float4*>(al + (long long)(j + u) * lda));
        } else if (u < ju) {
          float th[4] = {0.f, 0.f, 0.f, 0.f}, tl[4] = {0.f, 0.f, 0.f, 0.f};
          for (int v = 0; v < SP_VEC; ++v)
            if (row0 + v < m) { th[v] = ah[(long long)(j + u) * lda + v]; tl[v] = al[(long long)(j + u) * lda + v]; }
          vh[u] = make_float4(th[0], th[1], th[2], th[3]);
          vl[u] = make_float4(tl[0], tl[1], tl[2], tl[3]);
        } else {
          vh[u] = make_float4(0.f, 0.f, 0.f, 0.f);
          vl[u] = vh[u];
        }
      }
#pragma unroll
      for (int u = 0; u < SP_UNR; ++u) {
        if (u >= ju) break;
        const float ahv[4] = {vh[u].x, vh[u].y, vh[u].z, vh[u].w};
        const float alv[4] = {vl[u].x, vl[u].y, vl[u].z, vl[u].w};
#pragma unroll
        for (int k = 0; k < K; ++k) {
          const float xh = sxh[k][j + u], xl = sxl[k][j + u];
#pragma unroll
          for (int v = 0; v < SP_VEC; ++v) {
            const float p = ahv[v] * xh;
            float e = fmaf(ahv[v], xh, -p);
            e = fmaf(ahv[v], xl, e);
            e = fmaf(alv[v], xh, e);
            two_sum(sh[v][k], sl[v][k], p);
            sl[v][k] += e;
          }
        }
      }
    }
  }
  if (row0 < m) {
#pragma unroll
    for (int k = 0; k < K; ++k)
#pragma unroll
      for (int v = 0; v < SP_VEC; ++v)
        if (row0 + v < m) P[((long long)sidx * K + k) * m + row0 + v] = (double)sh[v][k] + (double)sl[v][k];
  }
}

// y = alpha * sum_s P + beta * bsrc, output FP64 or FP32.
template <typename TY>
__global__ void __launch_bounds__(SP_THREADS)
k_split_finalize(const double* __restrict__ P, int S, int K, long long m, double alpha, double beta,
                 const TY* bsrc, long long ldb, TY* y, long long ldy, const int* skip) {
  if (skip != nullptr && *skip) return;
  const long long total = m * K;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long i = idx % m;
    const int k = (int)(idx / m);
    double sum = 0.0;
    for (int s = 0; s < S; ++s) sum += P[((long long)s * K + k) * m + i];
    double v = alpha * sum;
    if (beta != 0.0) v = fma(beta, (double)bsrc[i + k * ldb], v);
    y[i + k * ldy] = (TY)v;
  }
}

struct SpPlan {
  int S = 1;
  long long chunk = 0;
  unsigned gx = 1;
  size_t part_bytes = 0;
};

static SpPlan sp_plan(long long m, long long n, int K) {
  SpPlan p;
  const long long rpb = (long long)SP_THREADS * SP_VEC;
  p.gx = (unsigned)std::max(1LL, (m + rpb - 1) / rpb);
  const long long target = (long long)num_sms() * 6;
  long long S = (target + p.gx - 1) / p.gx;
  S = std::max(1LL, std::min(S, (n + 63) / 64));
  S = std::min(S, 65535LL);
  p.chunk = (n + S - 1) / S;
  p.chunk = (p.chunk + 7) / 8 * 8;
  p.S = (int)std::max(1LL, (n + p.chunk - 1) / p.chunk);
  p.part_bytes = align_up((size_t)p.S * K * std::max(1LL, m) * sizeof(double), 256);
  return p;
}

size_t split_gemv_work_bytes(long long m, long long n, int nrhs) {
  size_t b = 0;
  for (int K = 1; K <= 4; K *= 2) b = std::max(b, sp_plan(m, n, K).part_bytes);
  (void)nrhs;
  return b + 256;
}

template <int K, typename TX>
static void launch_split(const SpPlan& p, const float* hi, const float* lo, long long lda, long long m, long long n,
                         const TX* X, long long ldx, double* P, const int* skip, cudaStream_t s) {
  dim3 grid(p.gx, p.S);
  launch(k_split_gemv<K, TX>, grid, SP_THREADS, 0, s, hi, lo, lda, m, n, X, ldx, p.chunk, P, skip);
}

// y = alpha * A x + beta * bsrc with A = hi + lo (column-major, lda); x FP64 or FP32.
template <typename TX, typename TY>
int split_gemv(const float* hi, const float* lo, long long lda, long long m, long long n, const TX* X, long long ldx,
               int nrhs, TY* Y, long long ldy, double alpha, double beta, const TY* bsrc, long long ldb, void* work,
               size_t work_bytes, cudaStream_t s, const int* skip) {
  MPDOK_ARG_CHECK(aligned16(hi) && aligned16(lo) && lda % 4 == 0, "split slices must be 16-byte aligned, lda % 4 == 0");
  int done = 0;
  while (done < nrhs) {
    const int left = nrhs - done;
    const int K = left >= 4 ? 4 : left >= 2 ? 2 : 1;
    const SpPlan p = sp_plan(m, n, K);
    MPDOK_ARG_CHECK(work_bytes >= p.part_bytes, "split GEMV workspace too small");
    double* P = (double*)work;
    const int slot = prof_start(MPDOK_PROF_GEMV_F64, s);
    const TX* Xk = X + (long long)done * ldx;
    switch (K) {
      case 4: launch_split<4, TX>(p, hi, lo, lda, m, n, Xk, ldx, P, skip, s); break;
      case 2: launch_split<2, TX>(p, hi, lo, lda, m, n, Xk, ldx, P, skip, s); break;
      default: launch_split<1, TX>(p, hi, lo, lda, m, n, Xk, ldx, P, skip, s); break;
    }
    prof_stop(slot, s, 8.0 * (double)m * (double)n + (double)K * (double)(m + n) * sizeof(TX), skip);
    const unsigned fb = (unsigned)std::max(1LL, std::min<long long>((m * K + 255) / 256, (long long)num_sms() * 4));
    launch(k_split_finalize<TY>, fb, SP_THREADS, 0, s, (const double*)P, p.S, K, m, alpha, beta,
           bsrc ? bsrc + (long long)done * ldb : (const TY*)nullptr, ldb, Y + (long long)done * ldy, ldy, skip);
    MPDOK_LAUNCH_CHECK("split gemv");
    done += K;
  }
  return MPDOK_OK;
}

int split_matrix(const double* A, long long lda, long long m, long long n, float* hi, float* lo, long long ld,
                 cudaStream_t s) {
  if (m == 0 || n == 0) return MPDOK_OK;
  dim3 grid((unsigned)std::min<long long>((m + 255) / 256, 16), (unsigned)std::min<long long>(n, 65535));
  launch(k_split, grid, 256, 0, s, A, lda, hi, lo, ld, m, n);
  MPDOK_LAUNCH_CHECK("split");
  return MPDOK_OK;
}

static int split_apply32(const void* ctx, const float* x, float* y, int nrhs, long long ld, cudaStream_t s,
                         const int* skip) {
  const SplitCtx* c = (const SplitCtx*)ctx;
  return split_gemv<float, float>(c->hi, c->lo, c->ld, c->n, c->n, x, ld, nrhs, y, ld, 1.0, 0.0, nullptr, 0, c->work,
                                  c->work_bytes, s, skip);
}

static int split_residual64(const void* ctx, const double* b, const double* x, double* r, double* nrm2, int nrhs,
                            long long ld, cudaStream_t s) {
  const SplitCtx* c = (const SplitCtx*)ctx;
  MPDOK_TRY((split_gemv<double, double>(c->hi, c->lo, c->ld, c->n, c->n, x, ld, nrhs, r, ld, -1.0, 1.0, b, ld,
                                        c->work, c->work_bytes, s, nullptr)));
  return colnorms_f64(r, c->n, nrhs, ld, nrm2, s);
}

Operator32 split_op32(const SplitCtx* c) {
  Operator32 o;
  o.apply = split_apply32;
  o.ctx = c;
  return o;
}

Residual64 split_res64(const SplitCtx* c) {
  Residual64 o;
  o.apply = split_residual64;
  o.ctx = c;
  return o;
}

}  // namespace mpdok

using namespace mpdok;

extern "C" int mpdok_split_matrix(const double* A, long long lda, long long m, long long n, float* hi, float* lo,
                                  long long ld, cudaStream_t stream) {
  MPDOK_ARG_CHECK(m >= 0 && n >= 0 && lda >= m && ld >= m, "bad shape");
  if (m == 0 || n == 0) return MPDOK_OK;
  MPDOK_ARG_CHECK(A && hi && lo, "null pointer");
  return split_matrix(A, lda, m, n, hi, lo, ld, stream);
}

extern "C" size_t mpdok_split_gemv_workspace_size(long long m, long long n, int nrhs) {
  if (m < 0 || n < 0 || nrhs < 1) return 0;
  return split_gemv_work_bytes(m, n, nrhs);
}

extern "C" int mpdok_split_gemv(const float* hi, const float* lo, long long ld, long long m, long long n,
                                const double* X, long long ldx, int nrhs, double* Y, long long ldy, double alpha,
                                double beta, const double* B, long long ldb, void* work, size_t work_bytes,
                                cudaStream_t stream) {
  MPDOK_ARG_CHECK(m >= 0 && n >= 0 && nrhs >= 1, "bad shape");
  if (m == 0) return MPDOK_OK;
  MPDOK_ARG_CHECK(hi && lo && X && Y && work, "null pointer");
  MPDOK_ARG_CHECK(ldx >= n && ldy >= m && (beta == 0.0 || (B && ldb >= m)), "leading dimension too small");
  return split_gemv<double, double>(hi, lo, ld, m, n, X, ldx, nrhs, Y, ldy, alpha, beta, B, ldb, work, work_bytes,
                                    stream, nullptr);
}
