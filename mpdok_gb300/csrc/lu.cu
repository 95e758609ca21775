// Blocked LU (BF16 / FP16 tensor-core trailing update, FP32 panels), its
// triangular-solve application, LU-IR and LU-preconditioned GMRES-IR.
//
// Replaces lu_ir.so of the reference (cusolverDnSgetrf / Sgetrs + cublasDgemv,
// benchmark_mpdok.ipynb:982-993; ABI at mpdok_ops.py:101-141).
//
// Factorization of W = D A D, D = diag(1/sqrt|a_ii|), panel width 128, per panel:
//   1. lu_diag:    LU of the 128 x 128 diagonal block in shared memory (FP32),
//                  plus the inverses of its unit-lower and upper triangles;
//   2. trsm_right: L21 = W21 U11^-1   (FP32 register-tiled, writes 16-bit L21)
//   3. trsm_left:  U12 = L11^-1 W12   (FP32 register-tiled, writes 16-bit U12)
//   4. W22 -= L21 U12 on tcgen05 (tc_gemm.cu), FP32 accumulation.
// Pivots smaller than tau are perturbed to +-tau (counted and returned): the
// factorization is used as a preconditioner / refinement solver, so an
// approximate factor of a nearby matrix is still useful.
//
// Application z = D U^-1 L^-1 D v: two persistent kernels, one per triangle.
// Row block t (128 rows) is claimed in order through an atomic ticket; it
// accumulates L[t, j] y_j as soon as block j publishes y_j (flag + fence),
// then multiplies by the precomputed inverse of its diagonal block.  Tickets
// are handed out in order, so a block only ever waits on blocks that are
// already running; every wait is bounded and reports a timeout.
#include "krylov.cuh"
#include "matfree.cuh"
#include "split.cuh"
#include "tc_gemm.cuh"

#include <cmath>
#include <cstring>
#include <vector>

namespace mpdok {

constexpr int LNB = 128;          // panel width / TRSV block
// Super-panel width: K of the far trailing update.  For 16-bit factors the
// tensor-core update is HBM-bound on its FP32 C tile, and K = 1024 halves that
// read-modify-write against K = 512 (at K = 2048 the longer inner strips cost
// more than that saves).  The FP32 factors' CUDA-core update is compute-bound,
// so there the narrower width, with twice the super-panels to overlap, is
// faster.
inline long long super_panel_width(int fdtype) { return fdtype == MPDOK_F32 ? 512 : 2048; }
constexpr long long SPIN_LIMIT = 1LL << 24;

static int fsize(int fdtype) { return fdtype == MPDOK_F32 ? 4 : 2; }

struct LULayout {
  long long n = 0, ldf = 0;
  int nblk = 0, fdtype = MPDOK_BF16;
  size_t off_lu = 0, off_linv = 0, off_uinv = 0, off_ml = 0, off_mu = 0, off_d = 0, off_dr = 0, off_perm = 0,
         off_ipiv = 0, off_meta = 0, total = 0;
};

struct LUMeta {
  int n_lo, n_hi;
  int fdtype;
  int pivoting;
  int nperturbed;
  int valid;
};

static LULayout lu_layout(long long n, int fdtype) {
  LULayout L;
  L.n = n;
  L.fdtype = fdtype;
  L.ldf = (long long)align_up((size_t)std::max(1LL, n), 8);
  L.nblk = (int)((n + LNB - 1) / LNB);
  size_t off = 0;
  auto take = [&](size_t b) { size_t o = off; off = align_up(off + b, 256); return o; };
  L.off_lu = take((size_t)L.ldf * n * fsize(fdtype));
  L.off_linv = take((size_t)L.nblk * LNB * LNB * sizeof(float));
  L.off_uinv = take((size_t)L.nblk * LNB * LNB * sizeof(float));
  // chain tiles of the triangular solves: Ml_t = Linv_t L(t, t-1), Mu_t = Uinv_t U(t, t+1)
  L.off_ml = take((size_t)L.nblk * LNB * LNB * sizeof(float));
  L.off_mu = take((size_t)L.nblk * LNB * LNB * sizeof(float));
  // W = Dr A Dc with P W = L U, so A^-1 = Dc U^-1 L^-1 P Dr: d holds Dc, dr
  // holds Dr, perm the row permutation ((P x)_i = x_perm[i]) and ipiv the
  // LAPACK-style pivot rows.  Unpivoted factors have Dr = Dc and perm = 1.
  L.off_d = take((size_t)std::max(1LL, n) * sizeof(float));
  L.off_dr = take((size_t)std::max(1LL, n) * sizeof(float));
  L.off_perm = take((size_t)std::max(1LL, n) * sizeof(int));
  L.off_ipiv = take((size_t)std::max(1LL, n) * sizeof(int));
  L.off_meta = take(sizeof(LUMeta));
  L.total = off;
  return L;
}

// Partial pivoting: the panel factorization runs on up to PIV_MAX_CTAS
// co-resident CTAs that meet at one grid barrier per column.
constexpr int PIV_MAX_CTAS = 256;

struct LUWork {
  long long ldw = 0;
  size_t off_W = 0, off_Lp = 0, off_Up = 0, off_err = 0, off_cand = 0, off_crow = 0, off_top = 0, off_bar = 0,
         off_plan = 0, off_scale = 0, total = 0;
};

static LUWork lu_work_layout(long long n, int fdtype) {
  LUWork w;
  w.ldw = (long long)align_up((size_t)std::max(1LL, n), 4);
  size_t off = 0;
  auto take = [&](size_t b) { size_t o = off; off = align_up(off + b, 256); return o; };
  w.off_W = take((size_t)w.ldw * n * sizeof(float));
  // two operand buffers each: super-panel J + 1 is factored while the far
  // update of super-panel J still reads its own operands (look-ahead)
  w.off_Lp = take(2 * (size_t)std::max(1LL, n) * super_panel_width(fdtype) * fsize(fdtype));
  w.off_Up = take(2 * (size_t)std::max(1LL, n) * super_panel_width(fdtype) * fsize(fdtype));
  w.off_err = take(64);
  // pivoting: candidate (|value|, row) per CTA and the candidate rows, double
  // buffered by column parity; the row at the panel's current position; the
  // barrier counter; the panel's row moves (dst, src pairs); row / column
  // maxima of the equilibration
  w.off_cand = take(2 * PIV_MAX_CTAS * 8);
  w.off_crow = take(2 * (size_t)PIV_MAX_CTAS * LNB * sizeof(float));
  w.off_top = take(2 * LNB * sizeof(float));
  w.off_bar = take(64);
  w.off_plan = take((1 + 4 * LNB) * sizeof(int));
  w.off_scale = take(2 * (size_t)std::max(1LL, n) * sizeof(double));
  w.total = off;
  return w;
}

// ----------------------------------------------------------------- scaling
__global__ void k_diag_scale(const double* __restrict__ A, long long lda, long long n, float* __restrict__ d,
                             float* __restrict__ dr, int* __restrict__ perm) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double a = fabs(A[i + i * lda]);
    const float v = (a > 0.0 && isfinite(a)) ? (float)(1.0 / sqrt(a)) : 1.f;
    d[i] = v;
    dr[i] = v;
    perm[i] = (int)i;
  }
}

__global__ void k_scaled_copy(const double* __restrict__ A, long long lda, long long n, const float* __restrict__ d,
                              float* __restrict__ W, long long ldw) {
  for (long long j = blockIdx.y; j < n; j += gridDim.y) {
    const float dj = d[j];
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
      W[i + j * ldw] = (float)A[i + j * lda] * d[i] * dj;
  }
}

// ------------------------------------------------------- diagonal block LU
// Shared memory: T (the block, then its L\U factors), XL / XU (inverses of
// the unit-lower and upper triangles), Tmp (products of the doubling steps).
constexpr int DP = LNB + 1;
constexpr size_t DIAG_SMEM = (size_t)(3 * LNB * DP + 64 * 65) * sizeof(float);
constexpr int DIAG_THREADS = 1024;
constexpr int TRSM_THREADS = 256;

// Copy TOTAL elements, element e = tid + u * THREADS, from global memory into
// shared memory: ld(e) reads one, st(e, v) stores it.  The strides are
// compile-time, so BATCH loads per thread are in flight before their shared
// stores and a tile costs TOTAL / (THREADS * BATCH) memory round trips.
template <int TOTAL, int THREADS, int BATCH, typename Ld, typename St>
__device__ __forceinline__ void stage_tile(int tid, Ld ld, St st) {
  static_assert(TOTAL % (THREADS * BATCH) == 0, "tile must split into whole batches");
#pragma unroll
  for (int u0 = 0; u0 < TOTAL / THREADS; u0 += BATCH) {
    float v[BATCH];
#pragma unroll
    for (int u = 0; u < BATCH; ++u) v[u] = ld(tid + (u0 + u) * THREADS);
#pragma unroll
    for (int u = 0; u < BATCH; ++u) st(tid + (u0 + u) * THREADS, v[u]);
  }
}

// One doubling step of the triangular inverses for diagonal blocks of size
// SZ (a compile-time power of two):
//   lower  X21 = -X22 (L21 X11),   upper  X12 = -X11 (U12 X22).
// Each of the 1024 threads forms U = PER / 1024 outputs at once with
// independent accumulators.  For SZ = 64 the four outputs of a thread share
// their column c, so the column operand is loaded once for four FMAs; the
// triangular operands are zero outside their triangle, so the k ranges run to
// the widest of the four rows.
template <int SZ>
__device__ __forceinline__ void inverse_doubling(const float* T, float* XL, float* XU, float* Tmp) {
  constexpr int NP = LNB / (2 * SZ);
  constexpr int PER = NP * SZ * SZ;
  constexpr int U = PER / DIAG_THREADS;  // outputs per thread: 2 (SZ 32) or 4 (SZ 64)
  static_assert(PER % DIAG_THREADS == 0, "doubling step must split evenly");
  const int tid = threadIdx.x;
  int pr[U], r[U];
  const int c = tid % SZ;
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int idx = tid + u * DIAG_THREADS;
    pr[u] = idx / (SZ * SZ);
    r[u] = (idx % (SZ * SZ)) / SZ;
  }
  float a[U];
  // lower: Tmp = L21 X11, k in [c, SZ)
#pragma unroll
  for (int u = 0; u < U; ++u) a[u] = 0.f;
  for (int k = c; k < SZ; ++k) {
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int R = (2 * pr[u] + 1) * SZ, C = 2 * pr[u] * SZ;
      a[u] = fmaf(T[(R + r[u]) * DP + C + k], XL[(C + k) * DP + C + c], a[u]);
    }
  }
#pragma unroll
  for (int u = 0; u < U; ++u) Tmp[(pr[u] * SZ + r[u]) * 65 + c] = a[u];
  __syncthreads();
  // lower: X21 = -X22 Tmp, k in [0, r] (X22 lower triangular)
  int rmax = 0, rmin = SZ;
#pragma unroll
  for (int u = 0; u < U; ++u) {
    rmax = max(rmax, r[u]);
    rmin = min(rmin, r[u]);
    a[u] = 0.f;
  }
  for (int k = 0; k <= rmax; ++k) {
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int R = (2 * pr[u] + 1) * SZ;
      a[u] = fmaf(XL[(R + r[u]) * DP + R + k], Tmp[(pr[u] * SZ + k) * 65 + c], a[u]);
    }
  }
  __syncthreads();
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int R = (2 * pr[u] + 1) * SZ, C = 2 * pr[u] * SZ;
    XL[(R + r[u]) * DP + C + c] = -a[u];
  }
  // upper: Tmp = U12 X22, k in [0, c]
#pragma unroll
  for (int u = 0; u < U; ++u) a[u] = 0.f;
  for (int k = 0; k <= c; ++k) {
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int R = 2 * pr[u] * SZ, C = (2 * pr[u] + 1) * SZ;
      a[u] = fmaf(T[(R + r[u]) * DP + C + k], XU[(C + k) * DP + C + c], a[u]);
    }
  }
#pragma unroll
  for (int u = 0; u < U; ++u) Tmp[(pr[u] * SZ + r[u]) * 65 + c] = a[u];
  __syncthreads();
  // upper: X12 = -X11 Tmp, k in [r, SZ) (X11 upper triangular)
#pragma unroll
  for (int u = 0; u < U; ++u) a[u] = 0.f;
  for (int k = rmin; k < SZ; ++k) {
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int R = 2 * pr[u] * SZ;
      a[u] = fmaf(XU[(R + r[u]) * DP + R + k], Tmp[(pr[u] * SZ + k) * 65 + c], a[u]);
    }
  }
  __syncthreads();
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int R = 2 * pr[u] * SZ, C = (2 * pr[u] + 1) * SZ;
    XU[(R + r[u]) * DP + C + c] = -a[u];
  }
  __syncthreads();
}

// The 32 x 32 diagonal blocks of L^-1 (unit lower) and U^-1 from the factored
// block T (shared memory, pitch DP): warps 0-3 invert L's four blocks, warps
// 4-7 U's, lane j computing column j of its inverse into a shared-memory
// column w (entry i at w[i * ws]).  Rows are taken in chunks of eight (top
// down for L, bottom up for U): a rolled loop adds the terms of the finished
// chunks, a row's accumulators in registers, then an unrolled 8 x 8 step
// finishes the chunk.  Each entry receives its terms in the order of a
// right-looking substitution: increasing column for L, decreasing for U; terms
// outside a column's triangle are exact zeros and are left out.  The loops stay
// rolled because this runs once per diagonal block, usually on an SM whose
// instruction cache holds other kernels' code: an unrolled substitution took
// 5.4 us alone but 15 us inside the factorization, fetching its code from a
// busy L2.
template <bool LOWER>
__device__ __forceinline__ void diag32_column(const float* __restrict__ Tb, float* __restrict__ w, int ws, int lane) {
  if (LOWER) {
    for (int c = 0; c < 32; c += 8) {
      float acc[8];
#pragma unroll
      for (int r = 0; r < 8; ++r) acc[r] = (c + r == lane) ? 1.f : 0.f;
#pragma unroll 2
      for (int k = lane; k < c; ++k) {  // x_k = 0 above the diagonal (k < lane)
        const float xk = w[k * ws];
#pragma unroll
        for (int r = 0; r < 8; ++r) acc[r] = fmaf(-Tb[(c + r) * DP + k], xk, acc[r]);
      }
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        const float xr = (c + r < lane) ? 0.f : acc[r];
        acc[r] = xr;
        if (c + r >= lane) {
#pragma unroll
          for (int q = r + 1; q < 8; ++q) acc[q] = fmaf(-Tb[(c + q) * DP + c + r], xr, acc[q]);
        }
      }
#pragma unroll
      for (int r = 0; r < 8; ++r) w[(c + r) * ws] = acc[r];
    }
  } else {
    for (int c = 24; c >= 0; c -= 8) {
      float acc[8];
#pragma unroll
      for (int r = 0; r < 8; ++r) acc[r] = 0.f;
#pragma unroll 2
      for (int k = lane; k >= c + 8; --k) {  // x_k = 0 below the diagonal (k > lane)
        const float xk = w[k * ws];
#pragma unroll
        for (int r = 0; r < 8; ++r) acc[r] = fmaf(Tb[(c + r) * DP + k], xk, acc[r]);
      }
#pragma unroll
      for (int r = 7; r >= 0; --r) {
        const int i = c + r;
        const float num = (i == lane) ? 1.f : -acc[r];
        const float xr = (i > lane) ? 0.f : num / Tb[i * DP + i];
        acc[r] = xr;
        if (i <= lane) {
#pragma unroll
          for (int q = 0; q < r; ++q) acc[q] = fmaf(Tb[(c + q) * DP + i], xr, acc[q]);
        }
      }
#pragma unroll
      for (int r = 0; r < 8; ++r) w[(c + r) * ws] = acc[r];
    }
  }
}

// Into shared memory: entry (r, c) of the inverses at XL / XU[r * DP + c].
__device__ __forceinline__ void diag32_inverses_smem(const float* T, float* XL, float* XU) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp >= 8) return;  // idle during the 32 x 32 substitutions
  const int o = (warp & 3) * 32;
  if (warp < 4)
    diag32_column<true>(T + o * DP + o, XL + o * DP + o + lane, DP, lane);
  else
    diag32_column<false>(T + o * DP + o, XU + o * DP + o + lane, DP, lane);
}

// Into global memory, column-major with pitch ld, through a staging area of
// 32 x 33 floats per warp: each warp writes its block column by column in
// 128-byte runs.
__device__ __forceinline__ void diag32_inverses_global(const float* T, float* Linv, float* Uinv, int ld,
                                                       float* stage) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp >= 8) return;
  const int o = (warp & 3) * 32;
  float* st = stage + warp * 32 * 33;
  if (warp < 4)
    diag32_column<true>(T + o * DP + o, st + lane, 33, lane);
  else
    diag32_column<false>(T + o * DP + o, st + lane, 33, lane);
  __syncwarp();
  float* X = warp < 4 ? Linv : Uinv;
#pragma unroll 4
  for (int c = 0; c < 32; ++c) X[(o + lane) + (long long)(o + c) * ld] = st[lane * 33 + c];
}

// Inverses by recursive doubling: the 32 x 32 diagonal blocks by substitution,
// then
//   [X11 0; L21 X22]^-1 off-diagonal block = -X22 L21 X11,
//   [X11 U12; 0 X22]^-1 off-diagonal block = -X11 U12 X22,
// for block sizes 32 and 64, each product spread over all 1024 threads.
__device__ void tri_inverses(const float* T, float* XL, float* XU, float* Tmp) {
  const int tid = threadIdx.x;
  for (int idx = tid; idx < LNB * DP; idx += blockDim.x) { XL[idx] = 0.f; XU[idx] = 0.f; }
  __syncthreads();
  diag32_inverses_smem(T, XL, XU);
  __syncthreads();
  inverse_doubling<32>(T, XL, XU, Tmp);
  inverse_doubling<64>(T, XL, XU, Tmp);
}


// Unpivoted LU of the 128 x 128 diagonal block, blocked in four 32-column
// sub-panels with the block in shared memory (T, pitch DP).  For sub-panel p:
//  (a) one warp per 32-row block of the sub-panel's rows: lane i holds its
//      row's 32 sub-panel columns, and every warp also holds the sub-panel's
//      32 x 32 diagonal block, whose elimination it repeats with shuffles, so
//      the 32 steps need no barrier.  The pivot u_kk is replaced by +-tau
//      when |u_kk| < tau (counted once) and every multiplier is
//        l_r = a_rk * rcp(u_kk),   a_rj <- fma(-l_r, u_kj, a_rj)
//      (rcp: the hardware reciprocal, within 1 ulp, for 16-bit factors; the
//      correctly rounded one for FP32 factors);
//  (b) one thread per column right of the sub-panel: its 32 rows of U by the
//      same FMAs, the multipliers read from shared memory;
//  (c) the trailing block: a_rj <- fma(-l_rk, u_kj, a_rj) for the sub-panel's
//      32 k in increasing order, a register tile per thread.
// Every entry therefore receives the operations of a step-by-step
// elimination in the same order, with three barriers per sub-panel instead
// of one per step.  The kernel then writes L\U into the factor and back into
// W's diagonal block (FP32, for the panel solves and the inverses), and the
// inverses of its 32 x 32 diagonal blocks of L and U into the diagonal
// positions of Linv / Uinv; the panel solves need only those, and
// k_tri_inv_complete fills in the rest of the 128 x 128 inverses once the
// factorization is done.
constexpr int DIAG_LU_THREADS = 256;
constexpr size_t DIAG_RR_SMEM = (size_t)(LNB * DP + 8 * 32 * 33) * sizeof(float);
// The launch asks for most of an SM's shared memory, so the block runs on an
// SM of its own rather than beside the updates' CTAs on the other streams.
constexpr size_t DIAG_RR_ALLOC = 200 * 1024;
static_assert(DIAG_RR_SMEM <= DIAG_RR_ALLOC, "the diagonal LU's shared memory");

// Four consecutive entries of a factor column (16-byte aligned for FP32,
// 8-byte for 16-bit factors).
template <typename F>
__device__ __forceinline__ void store4(F* p, const float (&v)[4]) {
  if constexpr (sizeof(F) == 4) {
    *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
  } else {
    union {
      F h[4];
      uint2 u;
    } pk;
#pragma unroll
    for (int e = 0; e < 4; ++e) pk.h[e] = from_f32<F>(v[e]);
    *reinterpret_cast<uint2*>(p) = pk.u;
  }
}
static_assert(LNB == 128 && DIAG_LU_THREADS == 256, "the diagonal LU's map: 4 sub-panels, 8 warps, 16 x 16 tiles");

// The hardware reciprocal (rcp.approx.ftz.f32: at most 1 ulp from 1 / x).  It
// sits on the diagonal LU's step-to-step critical path, where the correctly
// rounded reciprocal costs about 1 us per 32 steps.  16-bit factors use it (its
// error is far below their rounding); FP32 factors keep the correctly rounded
// reciprocal, which near-FP64 refinement tolerances can tell apart.  A pivot
// is at least tau in magnitude, and the scaled matrix's entries are of order
// one, so neither the pivot nor its reciprocal is subnormal.
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// Step K of a sub-panel's elimination, then the steps after it, for the
// sub-panel's diagonal block (d: lane i's row) and, with X, one more row
// block (x: lane i's row).  Recursion over K keeps every register index a
// constant.
template <int K, bool X, bool EXACT>
__device__ __forceinline__ void subpanel_steps(float (&d)[32], float (&x)[32], int lane, bool counts, int kmax,
                                               float tau, int* nperturb) {
  if constexpr (K < 32) {
    constexpr unsigned FULL = 0xffffffffu;
    float piv = __shfl_sync(FULL, d[K], K);
    const bool fix = K < kmax && !(fabsf(piv) >= tau);
    if (fix) piv = (piv < 0.f) ? -tau : tau;
    if (fix && counts && lane == K) atomicAdd(nperturb, 1);
    if (lane == K) d[K] = piv;
    const float pinv = EXACT ? __frcp_rn(piv) : rcp_approx(piv);
    const float ld = d[K] * pinv;
    const float lx = X ? x[K] * pinv : 0.f;
#pragma unroll
    for (int j = K + 1; j < 32; ++j) {
      const float u = __shfl_sync(FULL, d[j], K);
      if (lane > K) d[j] = fmaf(-ld, u, d[j]);
      if (X) x[j] = fmaf(-lx, u, x[j]);
    }
    if (lane > K) d[K] = ld;
    if (X) x[K] = lx;
    subpanel_steps<K + 1, X, EXACT>(d, x, lane, counts, kmax, tau, nperturb);
  }
}

// The trailing block of sub-panel p (m = 96 - 32 p rows and columns from
// q = 32 p + 32): thread (ty, tx) of 16 x 16 owns rows q + ty + 16 i and
// columns q + tx + 16 j, i, j < TS.
template <int TS>
__device__ __forceinline__ void subpanel_trailing(float* T, int P0, int tid) {
  const int q = P0 + 32, ty = tid >> 4, tx = tid & 15;
  float acc[TS][TS];
#pragma unroll
  for (int i = 0; i < TS; ++i)
#pragma unroll
    for (int j = 0; j < TS; ++j) acc[i][j] = T[(q + ty + 16 * i) * DP + q + tx + 16 * j];
#pragma unroll 4
  for (int k = 0; k < 32; ++k) {
    float l[TS], u[TS];
#pragma unroll
    for (int i = 0; i < TS; ++i) l[i] = T[(q + ty + 16 * i) * DP + P0 + k];
#pragma unroll
    for (int j = 0; j < TS; ++j) u[j] = T[(P0 + k) * DP + q + tx + 16 * j];
#pragma unroll
    for (int i = 0; i < TS; ++i)
#pragma unroll
      for (int j = 0; j < TS; ++j) acc[i][j] = fmaf(-l[i], u[j], acc[i][j]);
  }
#pragma unroll
  for (int i = 0; i < TS; ++i)
#pragma unroll
    for (int j = 0; j < TS; ++j) T[(q + ty + 16 * i) * DP + q + tx + 16 * j] = acc[i][j];
}

template <typename F>
__global__ void __launch_bounds__(DIAG_LU_THREADS, 1)
k_lu_diag(float* __restrict__ W, long long ldw, long long j0, int nbk, F* __restrict__ LU, long long ldf,
          float* __restrict__ Linv, float* __restrict__ Uinv, int* nperturb, float tau) {
  extern __shared__ float sm[];
  float* T = sm;                  // [128][DP]: the block
  float* stage = sm + LNB * DP;   // [8][32][33]: the inverses on their way out
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // 32 threads per column, four rows each (16-byte accesses; W's pitch is a
  // multiple of 4 and j0 of 128), 8 columns per pass
  const int r4 = 4 * lane;
#pragma unroll 4
  for (int c = warp; c < LNB; c += DIAG_LU_THREADS / 32) {
    float v[4];
    if (c < nbk && r4 + 3 < nbk) {
      const float4 q = *reinterpret_cast<const float4*>(W + (j0 + r4) + (j0 + c) * ldw);
      v[0] = q.x, v[1] = q.y, v[2] = q.z, v[3] = q.w;
    } else {
#pragma unroll
      for (int e = 0; e < 4; ++e)
        v[e] = (r4 + e < nbk && c < nbk) ? W[(j0 + r4 + e) + (j0 + c) * ldw] : (r4 + e == c ? 1.f : 0.f);
    }
#pragma unroll
    for (int e = 0; e < 4; ++e) T[(r4 + e) * DP + c] = v[e];
  }
  __syncthreads();
  for (int p = 0; p < 4 && 32 * p < nbk; ++p) {
    const int P0 = 32 * p;
    // (a) the sub-panel: warp w < 4 - p takes rows P0 + 32 w + lane
    // (warp 0 keeps the diagonal block and carries zero rows, so that every
    // warp runs the same code: the kernel's instructions are fetched per
    // launch, often from a busy L2)
    const int kmax = nbk - P0;  // pivots past the block's edge are the padding's ones
    if (warp < 4 - p) {
      float d[32], x[32];
      const int R = P0 + 32 * warp + lane;
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        d[j] = T[(P0 + lane) * DP + P0 + j];
        x[j] = warp == 0 ? 0.f : T[R * DP + P0 + j];
      }
      subpanel_steps<0, true, sizeof(F) == 4>(d, x, lane, warp == 0, kmax, tau, nperturb);
      if (warp == 0) {
#pragma unroll
        for (int j = 0; j < 32; ++j) T[(P0 + lane) * DP + P0 + j] = d[j];
      } else {
#pragma unroll
        for (int j = 0; j < 32; ++j) T[R * DP + P0 + j] = x[j];
      }
    }
    __syncthreads();
    if (p == 3) break;
    // (b) U's rows P0 .. P0 + 31 right of the sub-panel, a column per thread
    const int c = P0 + 32 + tid;
    if (c < LNB) {
      float u[32];
#pragma unroll
      for (int i = 0; i < 32; ++i) u[i] = T[(P0 + i) * DP + c];
#pragma unroll
      for (int k = 0; k < 32; ++k)
#pragma unroll
        for (int i = k + 1; i < 32; ++i) u[i] = fmaf(-T[(P0 + i) * DP + P0 + k], u[k], u[i]);
#pragma unroll
      for (int i = 1; i < 32; ++i) T[(P0 + i) * DP + c] = u[i];
    }
    __syncthreads();
    // (c) the trailing block
    if (p == 0) subpanel_trailing<6>(T, P0, tid);
    else if (p == 1) subpanel_trailing<4>(T, P0, tid);
    else subpanel_trailing<2>(T, P0, tid);
    __syncthreads();
  }
  // L\U out: the factor (F) and W's diagonal block (FP32), in the load's map
  // (the factor's pitch is a multiple of 8)
  for (int c = warp; c < nbk; c += DIAG_LU_THREADS / 32) {
    float v[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) v[e] = T[(r4 + e) * DP + c];
    if (r4 + 3 < nbk) {
      *reinterpret_cast<float4*>(W + (j0 + r4) + (j0 + c) * ldw) = make_float4(v[0], v[1], v[2], v[3]);
      store4(LU + (j0 + r4) + (j0 + c) * ldf, v);
    } else {
      for (int e = 0; e < 4 && r4 + e < nbk; ++e) {
        W[(j0 + r4 + e) + (j0 + c) * ldw] = v[e];
        LU[(j0 + r4 + e) + (j0 + c) * ldf] = from_f32<F>(v[e]);
      }
    }
  }
  diag32_inverses_global(T, Linv, Uinv, LNB, stage);
}

// The full 128 x 128 inverses of every diagonal block (for the triangular
// solves of the preconditioner) from W's factored diagonal blocks and the
// 32 x 32 diagonal-block inverses that k_lu_diag left in Linv / Uinv: the
// doubling steps of tri_inverses, one CTA per block.
__global__ void __launch_bounds__(DIAG_THREADS, 1)
k_tri_inv_complete(const float* __restrict__ W, long long ldw, long long n, float* __restrict__ Linv,
                   float* __restrict__ Uinv) {
  extern __shared__ float sm[];
  float* T = sm;
  float* XL = sm + LNB * DP;
  float* XU = sm + 2 * LNB * DP;
  float* Tmp = sm + 3 * LNB * DP;
  const int tid = threadIdx.x;
  const long long j0 = (long long)blockIdx.x * LNB;
  const int nbk = (int)min((long long)LNB, n - j0);
  float* Li = Linv + (long long)blockIdx.x * LNB * LNB;
  float* Ui = Uinv + (long long)blockIdx.x * LNB * LNB;
  for (int idx = tid; idx < LNB * LNB; idx += DIAG_THREADS) {
    const int r = idx % LNB, c = idx / LNB;
    T[r * DP + c] = (r < nbk && c < nbk) ? W[(j0 + r) + (j0 + c) * ldw] : (r == c ? 1.f : 0.f);
    const bool diag = (r >> 5) == (c >> 5);
    XL[r * DP + c] = diag ? Li[c * LNB + r] : 0.f;
    XU[r * DP + c] = diag ? Ui[c * LNB + r] : 0.f;
  }
  __syncthreads();
  inverse_doubling<32>(T, XL, XU, Tmp);
  inverse_doubling<64>(T, XL, XU, Tmp);
  for (int idx = tid; idx < LNB * LNB; idx += DIAG_THREADS) {
    const int r = idx % LNB, c = idx / LNB;
    Li[c * LNB + r] = XL[r * DP + c];
    Ui[c * LNB + r] = XU[r * DP + c];
  }
}

// --------------------------------------------------------------- TRSMs
// Both panel solves work block column by block column (block row by block
// row) with the 32 x 32 diagonal-block inverses that k_lu_diag leaves in
// Linv / Uinv and the off-diagonal blocks of the factored diagonal block in W:
//   L21 = W21 U^-1:  X_b = (W_b - sum_{a<b} X_a U_ab) Uinv_bb,
//   U12 = L^-1 W12:  Z_b = Linv_bb (W_b - sum_{a<b} L_ba Z_a),  b = 0..3.

// L21 = W21 U^-1 for RB rows x 128 columns; thread: column j of the current
// block column, rows tid / 32 + 8 u.
template <typename F, int RB>
__device__ __forceinline__ void trsm_right_body(const float* __restrict__ W, long long ldw, long long j0,
                                                long long r_begin, long long n, const float* __restrict__ Uinv,
                                                F* __restrict__ Lp, long long lp_pitch, long long lp_row0, int koff,
                                                F* __restrict__ LU, long long ldf, int bid) {
  static_assert(RB % 16 == 0 && RB <= 64, "rows per block: a multiple of 16, at most 64");
  constexpr int RU = RB / 8;      // rows per thread
  extern __shared__ float sm[];
  constexpr int XP = LNB + 4;     // rows read as float4 runs along k
  constexpr int TSP = LNB + 4;
  float* Xs = sm;                 // [RB][XP]   rows of W21, solved in place
  float* Ts = sm + RB * XP;       // [128][TSP] U row-major [k][c], diagonal 32 x 32 blocks = their inverses
  const int tid = threadIdx.x;
  const long long r0 = r_begin + (long long)bid * RB;
  const int rows = (int)min((long long)RB, n - r0);
  stage_tile<RB * LNB, TRSM_THREADS, (RB * LNB / TRSM_THREADS < 32 ? RB * LNB / TRSM_THREADS : 32)>(
      tid,
      [&](int idx) {
        const int r = idx % RB, c = idx / RB;
        return (r < rows) ? W[(r0 + r) + (j0 + c) * ldw] : 0.f;
      },
      [&](int idx, float v) { Xs[(idx % RB) * XP + idx / RB] = v; });
  stage_tile<LNB * LNB, TRSM_THREADS, 32>(
      tid,
      [&](int idx) {
        const int k = idx % LNB, c = idx / LNB;
        if ((k >> 5) == (c >> 5)) return Uinv[idx];
        return k < c ? W[(j0 + k) + (j0 + c) * ldw] : 0.f;
      },
      [&](int idx, float v) { Ts[(idx % LNB) * TSP + idx / LNB] = v; });
  __syncthreads();
  const int j = tid & 31, i0 = tid >> 5;
  for (int cb = 0; cb < 4; ++cb) {
    const int c = 32 * cb + j;
    float y[RU];
#pragma unroll
    for (int u = 0; u < RU; ++u) y[u] = Xs[(i0 + 8 * u) * XP + c];
    for (int k = 0; k < 32 * cb; k += 4) {
      float t[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) t[q] = Ts[(k + q) * TSP + c];
#pragma unroll
      for (int u = 0; u < RU; ++u) {
        const float4 xv = *reinterpret_cast<const float4*>(&Xs[(i0 + 8 * u) * XP + k]);
        y[u] = fmaf(-xv.x, t[0], y[u]);
        y[u] = fmaf(-xv.y, t[1], y[u]);
        y[u] = fmaf(-xv.z, t[2], y[u]);
        y[u] = fmaf(-xv.w, t[3], y[u]);
      }
    }
#pragma unroll
    for (int u = 0; u < RU; ++u) Xs[(i0 + 8 * u) * XP + c] = y[u];
    __syncthreads();
    float x[RU];
#pragma unroll
    for (int u = 0; u < RU; ++u) x[u] = 0.f;
#pragma unroll 2
    for (int m = 0; m < 32; m += 4) {
      float t[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) t[q] = Ts[(32 * cb + m + q) * TSP + c];
#pragma unroll
      for (int u = 0; u < RU; ++u) {
        const float4 xv = *reinterpret_cast<const float4*>(&Xs[(i0 + 8 * u) * XP + 32 * cb + m]);
        x[u] = fmaf(xv.x, t[0], x[u]);
        x[u] = fmaf(xv.y, t[1], x[u]);
        x[u] = fmaf(xv.z, t[2], x[u]);
        x[u] = fmaf(xv.w, t[3], x[u]);
      }
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < RU; ++u) Xs[(i0 + 8 * u) * XP + c] = x[u];
    __syncthreads();
  }
  // K-major operand for the trailing GEMM: Lp[row][k]
  for (int idx = tid; idx < RB * LNB; idx += TRSM_THREADS) {
    const int r = idx / LNB, c = idx % LNB;
    if (r < rows) Lp[(r0 - lp_row0 + r) * lp_pitch + koff + c] = from_f32<F>(Xs[r * XP + c]);
  }
  // column-major factor
  for (int idx = tid; idx < RB * LNB; idx += TRSM_THREADS) {
    const int r = idx % RB, c = idx / RB;
    if (r < rows) LU[(r0 + r) + (j0 + c) * ldf] = from_f32<F>(Xs[r * XP + c]);
  }
}

// U12 = L^-1 W12 for 128 rows x RB columns; thread: column tid % RB, rows
// tid / RB + (256 / RB) u of the current block row.
template <typename F, int RB>
__device__ __forceinline__ void trsm_left_body(const float* __restrict__ W, long long ldw, long long j0,
                                               long long c_begin, long long n, const float* __restrict__ Linv,
                                               F* __restrict__ Up, long long up_pitch, long long up_col0, int koff,
                                               F* __restrict__ LU, long long ldf, int bid) {
  static_assert(RB % 16 == 0 && RB <= 64, "columns per block: a multiple of 16, at most 64");
  constexpr int RS = TRSM_THREADS / RB;  // row stride between a thread's rows
  constexpr int RU = 32 / RS;            // rows per thread in a block row
  extern __shared__ float sm[];
  constexpr int XP = RB + 4;
  float* Xs = sm;                   // [128][XP]  W12 tile [k][c], solved in place
  float* Ts = sm + LNB * XP;        // [128][TP] L row-major [r][k], diagonal 32 x 32 blocks = their inverses
  constexpr int TP = LNB + 4;       // rows read as float4 runs along k
  const int tid = threadIdx.x;
  const long long c0 = c_begin + (long long)bid * RB;
  const int cols = (int)min((long long)RB, n - c0);
  stage_tile<LNB * RB, TRSM_THREADS, (LNB * RB / TRSM_THREADS < 32 ? LNB * RB / TRSM_THREADS : 32)>(
      tid,
      [&](int idx) {
        const int k = idx % LNB, c = idx / LNB;
        return (c < cols) ? W[(j0 + k) + (c0 + c) * ldw] : 0.f;
      },
      [&](int idx, float v) { Xs[(idx % LNB) * XP + idx / LNB] = v; });
  stage_tile<LNB * LNB, TRSM_THREADS, 32>(
      tid,
      [&](int idx) {
        const int r = idx % LNB, k = idx / LNB;
        if ((r >> 5) == (k >> 5)) return Linv[idx];
        return r > k ? W[(j0 + r) + (j0 + k) * ldw] : 0.f;
      },
      [&](int idx, float v) { Ts[(idx % LNB) * TP + idx / LNB] = v; });
  __syncthreads();
  const int cc = tid % RB, i0 = tid / RB;
  for (int rb = 0; rb < 4; ++rb) {
    float y[RU];
#pragma unroll
    for (int u = 0; u < RU; ++u) y[u] = Xs[(32 * rb + i0 + RS * u) * XP + cc];
    for (int k = 0; k < 32 * rb; k += 4) {
      float z[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) z[q] = Xs[(k + q) * XP + cc];
#pragma unroll
      for (int u = 0; u < RU; ++u) {
        const float4 lv = *reinterpret_cast<const float4*>(&Ts[(32 * rb + i0 + RS * u) * TP + k]);
        y[u] = fmaf(-lv.x, z[0], y[u]);
        y[u] = fmaf(-lv.y, z[1], y[u]);
        y[u] = fmaf(-lv.z, z[2], y[u]);
        y[u] = fmaf(-lv.w, z[3], y[u]);
      }
    }
#pragma unroll
    for (int u = 0; u < RU; ++u) Xs[(32 * rb + i0 + RS * u) * XP + cc] = y[u];
    __syncthreads();
    float x[RU];
#pragma unroll
    for (int u = 0; u < RU; ++u) x[u] = 0.f;
#pragma unroll 2
    for (int m = 0; m < 32; m += 4) {
      float z[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) z[q] = Xs[(32 * rb + m + q) * XP + cc];
#pragma unroll
      for (int u = 0; u < RU; ++u) {
        const float4 lv = *reinterpret_cast<const float4*>(&Ts[(32 * rb + i0 + RS * u) * TP + 32 * rb + m]);
        x[u] = fmaf(lv.x, z[0], x[u]);
        x[u] = fmaf(lv.y, z[1], x[u]);
        x[u] = fmaf(lv.z, z[2], x[u]);
        x[u] = fmaf(lv.w, z[3], x[u]);
      }
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < RU; ++u) Xs[(32 * rb + i0 + RS * u) * XP + cc] = x[u];
    __syncthreads();
  }
  for (int idx = tid; idx < LNB * RB; idx += TRSM_THREADS) {
    const int r = idx % LNB, c = idx / LNB;
    if (c < cols) {
      const F v = from_f32<F>(Xs[r * XP + c]);
      Up[(c0 - up_col0 + c) * up_pitch + koff + r] = v;
      LU[(j0 + r) + (c0 + c) * ldf] = v;
    }
  }
}

// Shared memory of k_trsm_pair<F, RB>: the larger of its two bodies.
constexpr size_t trsm_pair_smem(int rb) {
  const size_t right = (size_t)(rb * (LNB + 4) + LNB * (LNB + 4)) * sizeof(float);
  const size_t left = (size_t)(LNB * (rb + 4) + LNB * (LNB + 4)) * sizeof(float);
  return right > left ? right : left;
}

// Both panel solves of one inner panel in one launch: blocks [0, nb) form
// L21 = W21 U^-1 (RB rows each), the rest U12 = L^-1 W12 (RB columns each);
// they write disjoint outputs, so they run side by side.  RB = 64 for the
// strips; RB = 16 for the 128 rows and columns of the next panel, which sit
// on the chain: four times the CTAs, a quarter of the work each.
template <typename F, int RB>
__global__ void __launch_bounds__(TRSM_THREADS)
k_trsm_pair(const float* __restrict__ W, long long ldw, long long j0, long long begin, long long n,
            const float* __restrict__ Uinv, const float* __restrict__ Linv, F* __restrict__ Lp, F* __restrict__ Up,
            long long pitch, long long base0, int koff, F* __restrict__ LU, long long ldf, int nb) {
  if ((int)blockIdx.x < nb)
    trsm_right_body<F, RB>(W, ldw, j0, begin, n, Uinv, Lp, pitch, base0, koff, LU, ldf, (int)blockIdx.x);
  else
    trsm_left_body<F, RB>(W, ldw, j0, begin, n, Linv, Up, pitch, base0, koff, LU, ldf, (int)blockIdx.x - nb);
}

// CUDA-core trailing update for FP32 factors: C -= A B^T, A (M x K) and B
// (N x K) K-major FP32 with row pitch ldk.  CTA tile 128 x 128; K in slabs
// of 16 staged transposed in shared memory, double-buffered (the next slab's
// global loads sit in registers while the current slab is used, one barrier
// per slab); thread tile 8 x 8 = rows {4 ty .. +3, 64 + 4 ty .. +3} x columns
// {4 tx .. +3, 64 + 4 tx .. +3}, read as float4 (conflict-free).  Every
// output accumulates its products in ascending k, one FMA each.
constexpr int SG_BK = 16;
constexpr int SG_P = 128 + 4;

// Eight consecutive K-values of one operand row (zero past M or K).
__device__ __forceinline__ void sg_load8(const float* __restrict__ X, int row, int rows, int k, int K, long long ldk,
                                         float (&r)[8]) {
  const float* p = X + (long long)row * ldk + k;
  if (row < rows && k + 8 <= K && (reinterpret_cast<uintptr_t>(p) & 15) == 0) {
    const float4 u = __ldg(reinterpret_cast<const float4*>(p));
    const float4 v = __ldg(reinterpret_cast<const float4*>(p) + 1);
    r[0] = u.x; r[1] = u.y; r[2] = u.z; r[3] = u.w; r[4] = v.x; r[5] = v.y; r[6] = v.z; r[7] = v.w;
  } else {
#pragma unroll
    for (int i = 0; i < 8; ++i) r[i] = (row < rows && k + i < K) ? __ldg(p + i) : 0.f;
  }
}

__global__ void __launch_bounds__(256)
k_gemm_update_f32(float* __restrict__ C, long long ldc, const float* __restrict__ A, const float* __restrict__ B,
                  long long ldk, int M, int N, int K) {
  __shared__ __align__(16) float As[2][SG_BK][SG_P];
  __shared__ __align__(16) float Bs[2][SG_BK][SG_P];
  const int tid = threadIdx.x;
  const int m0 = blockIdx.x * 128, n0 = blockIdx.y * 128;
  const int ty = tid / 16, tx = tid % 16;
  const int lr = tid >> 1, lk = (tid & 1) * 8;  // staging: row lr, K-values lk .. lk + 7 of the slab
  float ra[8], rb[8];
  auto stage = [&](int buf) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      As[buf][lk + i][lr] = ra[i];
      Bs[buf][lk + i][lr] = rb[i];
    }
  };
  float acc[8][8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;
  sg_load8(A, m0 + lr, M, lk, K, ldk, ra);
  sg_load8(B, n0 + lr, N, lk, K, ldk, rb);
  stage(0);
  __syncthreads();
  for (int kb = 0; kb < K; kb += SG_BK) {
    const int cur = (kb / SG_BK) & 1;
    const bool more = kb + SG_BK < K;
    if (more) {
      sg_load8(A, m0 + lr, M, kb + SG_BK + lk, K, ldk, ra);
      sg_load8(B, n0 + lr, N, kb + SG_BK + lk, K, ldk, rb);
    }
#pragma unroll
    for (int k = 0; k < SG_BK; ++k) {
      const float4 a0 = *reinterpret_cast<const float4*>(&As[cur][k][4 * ty]);
      const float4 a1 = *reinterpret_cast<const float4*>(&As[cur][k][64 + 4 * ty]);
      const float4 b0 = *reinterpret_cast<const float4*>(&Bs[cur][k][4 * tx]);
      const float4 b1 = *reinterpret_cast<const float4*>(&Bs[cur][k][64 + 4 * tx]);
      const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
      const float b[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    if (more) stage(cur ^ 1);  // the other buffer was last read before the previous barrier
    __syncthreads();
  }
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const int col = n0 + (j < 4 ? 4 * tx + j : 64 + 4 * tx + j - 4);
    if (col >= N) continue;
    float* c = C + (long long)col * ldc;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int row = m0 + h * 64 + 4 * ty;
      float* cp = c + row;
      if (row + 4 <= M && (reinterpret_cast<uintptr_t>(cp) & 15) == 0) {
        float4 v = *reinterpret_cast<float4*>(cp);
        v.x -= acc[4 * h + 0][j];
        v.y -= acc[4 * h + 1][j];
        v.z -= acc[4 * h + 2][j];
        v.w -= acc[4 * h + 3][j];
        *reinterpret_cast<float4*>(cp) = v;
      } else {
#pragma unroll
        for (int i = 0; i < 4; ++i)
          if (row + i < M) cp[i] -= acc[4 * h + i][j];
      }
    }
  }
}

// ------------------------------------------------------------ TRSV (apply)
// Lower: y = L^-1 (d .* v), L unit lower (off-diagonal blocks from LU, diagonal
// blocks through Linv).  Upper: z = U^-1 y (scaled by d afterwards).
// Block t walks the column blocks it depends on in the order they are
// published (ascending for L, descending for U); the 128 x 8 slice of each
// tile that a thread multiplies is loaded before waiting on that tile's flag,
// so HBM latency overlaps the dependency chain.  The diagonal-block inverse
// sits in shared memory from the start.
template <typename F>
struct TileRegs;
template <>
struct TileRegs<__nv_bfloat16> { uint4 r[8]; };
template <>
struct TileRegs<__half> { uint4 r[8]; };
template <>
struct TileRegs<float> { float4 r[16]; };

template <typename F>
__device__ __forceinline__ void tile_load(TileRegs<F>& T, const F* LU, long long ldf, long long c0, int cols,
                                          long long rbase, long long n, int cg) {
  const bool full_rows = rbase + 8 <= n;
#pragma unroll
  for (int cc = 0; cc < 8; ++cc) {
    const int c = cg + 16 * cc;
    const F* col = LU + (c0 + c) * ldf + rbase;
    if constexpr (sizeof(F) == 2) {
      if (c < cols && full_rows) {
        T.r[cc] = __ldg(reinterpret_cast<const uint4*>(col));
      } else {
        F tmp[8];
#pragma unroll
        for (int v = 0; v < 8; ++v) tmp[v] = (c < cols && rbase + v < n) ? col[v] : from_f32<F>(0.f);
        T.r[cc] = *reinterpret_cast<uint4*>(tmp);
      }
    } else {
      if (c < cols && full_rows) {
        T.r[2 * cc] = __ldg(reinterpret_cast<const float4*>(col));
        T.r[2 * cc + 1] = __ldg(reinterpret_cast<const float4*>(col) + 1);
      } else {
        float tmp[8];
#pragma unroll
        for (int v = 0; v < 8; ++v) tmp[v] = (c < cols && rbase + v < n) ? (float)col[v] : 0.f;
        T.r[2 * cc] = make_float4(tmp[0], tmp[1], tmp[2], tmp[3]);
        T.r[2 * cc + 1] = make_float4(tmp[4], tmp[5], tmp[6], tmp[7]);
      }
    }
  }
}

template <typename F>
__device__ __forceinline__ void tile_fma(const TileRegs<F>& T, const float* sx, int cg, float (&acc)[8]) {
#pragma unroll
  for (int cc = 0; cc < 8; ++cc) {
    const float xv = sx[cg + 16 * cc];
    if constexpr (sizeof(F) == 2) {
      const F* h = reinterpret_cast<const F*>(&T.r[cc]);
#pragma unroll
      for (int v = 0; v < 8; ++v) acc[v] = fmaf(to_f32<F>(h[v]), xv, acc[v]);
    } else {
      const float* f = reinterpret_cast<const float*>(&T.r[2 * cc]);
#pragma unroll
      for (int v = 0; v < 8; ++v) acc[v] = fmaf(f[v], xv, acc[v]);
    }
  }
}

// Outputs of the triangular solves start as this bit pattern (a NaN that
// GPU arithmetic never produces: generated NaNs are 0x7fffffff); a consumer
// polls the values themselves instead of a separate ready flag.
constexpr unsigned TRSV_EMPTY = 0xffffffffu;

__device__ __forceinline__ float ld_relaxed_f(const float* p) {
  unsigned v;
  asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return __uint_as_float(v);
}
__device__ __forceinline__ void st_relaxed_f(float* p, float x) {
  asm volatile("st.relaxed.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(__float_as_uint(x)) : "memory");
}
// Iteration limit of the triangular solves' waits on a predecessor block.  A
// device variable so that a test can shorten it (mpdok_debug_set).
__device__ long long g_spin_limit = SPIN_LIMIT;

// Spin until out[i] holds a value; false when the limit ran out.
__device__ __forceinline__ bool wait_value(const float* p, float& v) {
  const long long limit = g_spin_limit;
  for (long long it = 0; it < limit; ++it) {
    v = ld_relaxed_f(p);
    if (__float_as_uint(v) != TRSV_EMPTY) return true;
    if (it > 256) __nanosleep(32);
  }
  return false;
}

// Blocked triangular solve, one CTA per 128-row block, blocks taken in
// dependency order through a ticket.  Block t needs x_j for all j before it
// (after it, for the upper solve).  The last of them, x_{t-1}, is the chain:
//   x_t = Dinv_t (b_t - sum_{j<t-1} L_tj x_j) - M_t x_{t-1},  M_t = Dinv_t L_{t,t-1}
// The first part (every earlier tile, the reduction and the 128-long
// diagonal-block product) is formed while block t-1 is still being solved;
// once x_{t-1} arrives, one 128 x 128 product with M_t (held in registers,
// two threads per row) finishes the block.  Values are published by relaxed
// stores and consumed by polling them (TRSV_EMPTY marks "not yet").
template <typename F, bool LOWER>
__global__ void __launch_bounds__(256)
k_trsv(const F* __restrict__ LU, long long ldf, const float* __restrict__ Dinv, const float* __restrict__ Mt,
       long long n, int nblk, const float* __restrict__ rhs, const float* __restrict__ dsc,
       const int* __restrict__ perm, float* out, int* ticket, int* err, const int* skip) {
  extern __shared__ float sDi[];      // 128 x 128 diagonal-block inverse (column-major)
  __shared__ int s_t;
  __shared__ int s_abort;
  __shared__ float s_x[2][LNB];
  __shared__ float s_part[16][LNB + 1];
  __shared__ float s_y[LNB];
  __shared__ float s_rhs[LNB];
  if (skip != nullptr && *skip) return;
  const int tid = threadIdx.x;
  if (tid == 0) {
    s_t = atomicAdd(ticket, 1);
    s_abort = 0;
  }
  __syncthreads();
  const int tk = s_t;
  if (tk >= nblk) return;
  const int t = LOWER ? tk : (nblk - 1 - tk);
  const long long r0 = (long long)t * LNB;
  const int rows = (int)min((long long)LNB, n - r0);
  const int cnt = LOWER ? t : (nblk - 1 - t);
  // chain tile M_t: thread (row = tid / 2, half = tid % 2) holds M_t(row, 64 half .. 64 half + 63)
  const int mrow = tid >> 1, mhalf = tid & 1;
  float m[64];
  if (cnt > 0) {
    const float* M = Mt + (long long)t * LNB * LNB;
#pragma unroll
    for (int c = 0; c < 64; ++c) m[c] = __ldg(M + (long long)(mhalf * 64 + c) * LNB + mrow);
  }
  const float* Di = Dinv + (long long)t * LNB * LNB;
  for (int idx = tid; idx < LNB * LNB; idx += blockDim.x) sDi[idx] = __ldg(Di + idx);
  // the block's right-hand side, staged now so that its latency stays off the
  // path from x_{t-2} to y_t
  // (the lower solve takes P Dr v: row i of its right-hand side is row perm[i] of v)
  if (tid < LNB) {
    float r = 0.f;
    if (tid < rows) {
      if (LOWER) {
        const int pi = __ldg(perm + r0 + tid);
        r = rhs[pi] * __ldg(dsc + pi);
      } else {
        r = rhs[r0 + tid];
      }
    }
    s_rhs[tid] = r;
  }
  const int rg = tid % 16, cg = tid / 16;
  const long long rbase = r0 + rg * 8;
  float acc[8];
#pragma unroll
  for (int v = 0; v < 8; ++v) acc[v] = 0.f;
  // every tile except the chain tile
  for (int q = 0; q + 1 < cnt; ++q) {
    const int j = LOWER ? q : (nblk - 1 - q);
    const long long c0 = (long long)j * LNB;
    const int cols = (int)min((long long)LNB, n - c0);
    TileRegs<F> T;
    tile_load<F>(T, LU, ldf, c0, cols, rbase, n, cg);
    if (tid < LNB) {
      float v = 0.f;
      if (tid < cols && !wait_value(out + c0 + tid, v)) {
        s_abort = 1;
        atomicExch(err, 2);
      }
      s_x[q & 1][tid] = v;
    }
    __syncthreads();
    if (s_abort) return;
    tile_fma<F>(T, s_x[q & 1], cg, acc);
  }
#pragma unroll
  for (int v = 0; v < 8; ++v) s_part[cg][rg * 8 + v] = acc[v];
  __syncthreads();
  if (tid < LNB) {
    float sum = 0.f;
#pragma unroll
    for (int g = 0; g < 16; ++g) sum += s_part[g][tid];
    s_x[0][tid] = s_rhs[tid] - sum;  // a_t
  }
  __syncthreads();
  // the chain input x_prev = x_{t-1} (x_{t+1} for the upper solve), read
  // speculatively now: it is usually published by the time y_t is formed, and
  // the read then overlaps the product below
  const int jp = LOWER ? t - 1 : t + 1;
  const long long cp = (long long)jp * LNB;
  const int colsp = cnt > 0 ? (int)min((long long)LNB, n - cp) : 0;
  float xs = 0.f;
  if (tid < colsp) xs = ld_relaxed_f(out + cp + tid);
  if (tid < LNB) {
    // y_t = Dinv_t a_t, four independent partial sums over the full tile
    // (Dinv_t holds exact zeros outside its triangle, which add nothing)
    float y[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 8
    for (int c0 = 0; c0 < LNB; c0 += 4) {
#pragma unroll
      for (int u = 0; u < 4; ++u) y[u] = fmaf(sDi[(c0 + u) * LNB + tid], s_x[0][c0 + u], y[u]);
    }
    s_y[tid] = (y[0] + y[1]) + (y[2] + y[3]);
  }
  if (cnt == 0) {
    if (tid < rows) st_relaxed_f(out + r0 + tid, s_y[tid]);
    return;
  }
  // the chain: x_t = y_t - M_t x_prev
  if (tid < LNB) {
    float v = xs;
    if (tid < colsp && __float_as_uint(v) == TRSV_EMPTY && !wait_value(out + cp + tid, v)) {
      s_abort = 1;
      atomicExch(err, 2);
    }
    s_x[1][tid] = v;
  }
  __syncthreads();
  if (s_abort) return;
  float z = 0.f;
#pragma unroll
  for (int c = 0; c < 64; ++c) z = fmaf(m[c], s_x[1][mhalf * 64 + c], z);
  z += __shfl_xor_sync(0xffffffffu, z, 1);
  if (mhalf == 0 && mrow < rows) st_relaxed_f(out + r0 + mrow, s_y[mrow] - z);
}

// Chain tiles of the triangular solves (one CTA per (block, triangle)):
//   Ml_t = Linv_t L(t, t-1)   (t >= 1),   Mu_t = Uinv_t U(t, t+1)   (t < nblk - 1),
// from the stored factors, so the solves multiply by exactly these values.
template <typename F>
__global__ void __launch_bounds__(256)
k_trsv_chain_tiles(const F* __restrict__ LU, long long ldf, const float* __restrict__ Linv,
                   const float* __restrict__ Uinv, float* __restrict__ Ml, float* __restrict__ Mu, long long n,
                   int nblk) {
  extern __shared__ float sm[];
  float* sI = sm;                   // inverse, column-major [c * 128 + r]
  float* sT = sm + LNB * LNB;       // factor tile, column-major
  const int t = blockIdx.x, upper = blockIdx.y;
  if (upper ? t >= nblk - 1 : t == 0) return;
  const int tt = upper ? t + 1 : t - 1;  // column block of the off-diagonal tile
  const long long r0 = (long long)t * LNB, c0 = (long long)tt * LNB;
  const float* I = (upper ? Uinv : Linv) + (long long)t * LNB * LNB;
  for (int e = threadIdx.x; e < LNB * LNB; e += blockDim.x) {
    sI[e] = I[e];
    const int r = e % LNB, c = e / LNB;
    sT[e] = (r0 + r < n && c0 + c < n) ? to_f32<F>(LU[(r0 + r) + (c0 + c) * ldf]) : 0.f;
  }
  __syncthreads();
  // out(r, c) = sum_k I(r, k) T(k, c); thread: 8 rows x 8 columns
  const int tr = threadIdx.x % 16, tc = threadIdx.x / 16;
  float acc[8][8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;
  for (int k = 0; k < LNB; ++k) {
    float a[8], b[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = sI[k * LNB + tr * 8 + i];
#pragma unroll
    for (int j = 0; j < 8; ++j) b[j] = sT[(tc * 8 + j) * LNB + k];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
  }
  float* M = (upper ? Mu : Ml) + (long long)t * LNB * LNB;
#pragma unroll
  for (int j = 0; j < 8; ++j)
#pragma unroll
    for (int i = 0; i < 8; ++i) M[(tc * 8 + j) * LNB + tr * 8 + i] = acc[i][j];
}

__global__ void k_scale_out(const float* __restrict__ z, const float* __restrict__ d, float* __restrict__ out,
                            long long n, const int* skip) {
  if (skip != nullptr && *skip) return;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = z[i] * d[i];
}

// Triangular solve with K right-hand sides (columns of rhs / out, leading
// dimension ld), the chained block sweep of k_trsv: each factor tile is
// loaded once into registers and applied to all K columns, so the factor
// bytes per right-hand side drop by K; the chain tile M_t (registers) and the
// value polling are those of k_trsv.
template <typename F, bool LOWER, int K>
__global__ void __launch_bounds__(256)
k_trsv_multi(const F* __restrict__ LU, long long ldf, const float* __restrict__ Dinv, const float* __restrict__ Mt,
             long long n, int nblk, const float* __restrict__ rhs, long long ld, const float* __restrict__ dsc,
             const int* __restrict__ perm, float* out, int* ticket, int* err) {
  extern __shared__ float sDi[];      // 128 x 128 diagonal-block inverse (column-major)
  __shared__ int s_t;
  __shared__ int s_abort;
  __shared__ float s_x[2][K][LNB];
  __shared__ float s_part[16][LNB + 1];
  __shared__ float s_a[K][LNB];
  __shared__ float s_y[K][LNB];
  const int tid = threadIdx.x;
  if (tid == 0) {
    s_t = atomicAdd(ticket, 1);
    s_abort = 0;
  }
  __syncthreads();
  const int tk = s_t;
  if (tk >= nblk) return;
  const int t = LOWER ? tk : (nblk - 1 - tk);
  const long long r0 = (long long)t * LNB;
  const int rows = (int)min((long long)LNB, n - r0);
  const int cnt = LOWER ? t : (nblk - 1 - t);
  const float* Di = Dinv + (long long)t * LNB * LNB;
  for (int idx = tid; idx < LNB * LNB; idx += blockDim.x) sDi[idx] = __ldg(Di + idx);
  // the block's right-hand sides, staged now so that their latency stays off
  // the path from x_{t-2} to y_t
  for (int e = tid; e < LNB * K; e += blockDim.x) {
    const int row = e % LNB, k = e / LNB;
    float r = 0.f;
    if (row < rows) {
      if (LOWER) {
        const int pi = __ldg(perm + r0 + row);
        r = rhs[(long long)k * ld + pi] * __ldg(dsc + pi);
      } else {
        r = rhs[(long long)k * ld + r0 + row];
      }
    }
    s_a[k][row] = r;
  }
  const int rg = tid % 16, cg = tid / 16;
  const long long rbase = r0 + rg * 8;
  float acc[K][8];
#pragma unroll
  for (int k = 0; k < K; ++k)
#pragma unroll
    for (int v = 0; v < 8; ++v) acc[k][v] = 0.f;
  for (int q = 0; q + 1 < cnt; ++q) {
    const int j = LOWER ? q : (nblk - 1 - q);
    const long long c0 = (long long)j * LNB;
    const int cols = (int)min((long long)LNB, n - c0);
    TileRegs<F> T;
    tile_load<F>(T, LU, ldf, c0, cols, rbase, n, cg);
    if (tid < LNB) {
#pragma unroll
      for (int k = 0; k < K; ++k) {
        float v = 0.f;
        if (tid < cols && !wait_value(out + (long long)k * ld + c0 + tid, v)) {
          s_abort = 1;
          atomicExch(err, 2);
        }
        s_x[q & 1][k][tid] = v;
      }
    }
    __syncthreads();
    if (s_abort) return;
#pragma unroll
    for (int k = 0; k < K; ++k) tile_fma<F>(T, s_x[q & 1][k], cg, acc[k]);
  }
#pragma unroll
  for (int k = 0; k < K; ++k) {
    __syncthreads();
#pragma unroll
    for (int v = 0; v < 8; ++v) s_part[cg][rg * 8 + v] = acc[k][v];
    __syncthreads();
    if (tid < LNB) {
      float sum = 0.f;
#pragma unroll
      for (int g = 0; g < 16; ++g) sum += s_part[g][tid];
      s_a[k][tid] -= sum;
    }
  }
  __syncthreads();
  for (int e = tid; e < LNB * K; e += blockDim.x) {
    const int row = e % LNB, k = e / LNB;
    // Dinv_t holds exact zeros outside its triangle, which add nothing
    float y[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 8
    for (int c0 = 0; c0 < LNB; c0 += 4) {
#pragma unroll
      for (int u = 0; u < 4; ++u) y[u] = fmaf(sDi[(c0 + u) * LNB + row], s_a[k][c0 + u], y[u]);
    }
    s_y[k][row] = (y[0] + y[1]) + (y[2] + y[3]);
  }
  __syncthreads();
  if (cnt == 0) {
    for (int e = tid; e < LNB * K; e += blockDim.x) {
      const int row = e % LNB, k = e / LNB;
      if (row < rows) st_relaxed_f(out + (long long)k * ld + r0 + row, s_y[k][row]);
    }
    return;
  }
  // chain tile into registers now that the tile registers and accumulators are
  // dead (still before the predecessor's values can arrive)
  const int mrow = tid >> 1, mhalf = tid & 1;
  float m[64];
  {
    const float* M = Mt + (long long)t * LNB * LNB;
#pragma unroll
    for (int c = 0; c < 64; ++c) m[c] = __ldg(M + (long long)(mhalf * 64 + c) * LNB + mrow);
  }
  const int jp = LOWER ? t - 1 : t + 1;
  const long long cp = (long long)jp * LNB;
  const int colsp = (int)min((long long)LNB, n - cp);
  if (tid < LNB) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      float v = 0.f;
      if (tid < colsp && !wait_value(out + (long long)k * ld + cp + tid, v)) {
        s_abort = 1;
        atomicExch(err, 2);
      }
      s_x[1][k][tid] = v;
    }
  }
  __syncthreads();
  if (s_abort) return;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    float z = 0.f;
#pragma unroll
    for (int c = 0; c < 64; ++c) z = fmaf(m[c], s_x[1][k][mhalf * 64 + c], z);
    z += __shfl_xor_sync(0xffffffffu, z, 1);
    if (mhalf == 0 && mrow < rows) st_relaxed_f(out + (long long)k * ld + r0 + mrow, s_y[k][mrow] - z);
  }
}

// out[:, k] = z[:, k] * d for K columns (leading dimension ld).
__global__ void k_scale_out_multi(const float* __restrict__ z, const float* __restrict__ d, float* __restrict__ out,
                                  long long n, long long ld, int K) {
  const long long total = n * K;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
    const long long i = e % n, k = e / n;
    out[k * ld + i] = z[k * ld + i] * d[i];
  }
}

// ------------------------------------------------------- partial pivoting
// The LU with row pivoting behind the reference's lu_ir.so (cusolverDnSgetrf +
// Sgetrs with L, U, P: benchmark_mpdok.ipynb:989-990; py_lu_factor's info is
// LAPACK's, mpdok_ops.py:195-202).  The matrix is first equilibrated with
// power-of-two row and column scales (W = Dr A Dc, exact, |W| <= 1 in every
// row and column, which keeps 16-bit operands in range), then factored
// right-looking in 128-column panels:
//   1. k_getf2: the tall panel W[jp:n, jp:jp+128] with partial pivoting on G
//      co-resident CTAs, each holding a slice of its rows in shared memory;
//      one grid barrier per column (pivot search, row exchange, rank-1 update);
//   2. k_laswp: the panel's row exchanges applied to every other column of W;
//   3. k_piv_diag: the 128 x 128 diagonal block's unit-lower / upper inverses;
//   4. U12 = L11^-1 W12 (the panel solve of the unpivoted path), L21 to the
//      K-major operand, and W22 -= L21 U12 (tensor cores or CUDA cores);
// and at the end the strictly lower part of W is rounded into the factor.

// |a_ij| maxima per row over a column chunk (non-negative doubles compare as
// their bit patterns).
__global__ void k_row_absmax(const double* __restrict__ A, long long lda, long long n, long long cchunk,
                             unsigned long long* __restrict__ rmax) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const long long c0 = (long long)blockIdx.y * cchunk, c1 = min(n, c0 + cchunk);
  double m = 0.0;
  for (long long c = c0; c < c1; ++c) m = fmax(m, fabs(A[i + c * lda]));
  atomicMax(rmax + i, (unsigned long long)__double_as_longlong(m));
}

// 2^-e with max * 2^-e in [0.5, 1): an exact scale; 1 for a zero or non-finite max.
__device__ __forceinline__ float pow2_inv_scale(double m) {
  if (!(m > 0.0) || !isfinite(m)) return 1.f;
  int e = 0;
  frexp(m, &e);
  e = max(-120, min(120, e));
  return ldexpf(1.f, -e);
}

__global__ void k_row_scale(const unsigned long long* __restrict__ rmax, long long n, float* __restrict__ dr,
                            int* __restrict__ perm) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    dr[i] = pow2_inv_scale(__longlong_as_double((long long)rmax[i]));
    perm[i] = (int)i;
  }
}

// Column scales of the row-scaled matrix (one CTA per column) and W = Dr A Dc
// rounded once to FP32.
__global__ void __launch_bounds__(256)
k_col_scale_copy(const double* __restrict__ A, long long lda, long long n, const float* __restrict__ dr,
                 float* __restrict__ dc, float* __restrict__ W, long long ldw) {
  __shared__ double red[32];
  const long long j = blockIdx.x;
  double m = 0.0;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) m = fmax(m, fabs(A[i + j * lda]) * (double)dr[i]);
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    double t = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) t = fmax(t, __shfl_xor_sync(0xffffffffu, t, o));
    if (threadIdx.x == 0) red[0] = t;
  }
  __syncthreads();
  const float c = pow2_inv_scale(red[0]);
  if (threadIdx.x == 0) dc[j] = c;
  for (long long i = threadIdx.x; i < n; i += blockDim.x)
    W[i + j * ldw] = (float)(A[i + j * lda] * (double)dr[i] * (double)c);
}

struct PivCand {
  float val;  // |candidate|, -1 when the CTA has no eligible row
  int row;    // global row, -1 when none
};

// (v2, i2) beats (v1, i1): larger magnitude, ties to the smaller row (LAPACK's
// isamax takes the first maximum).
__device__ __forceinline__ bool piv_better(float v2, int i2, float v1, int i1) {
  return v2 > v1 || (v2 == v1 && i2 >= 0 && (i1 < 0 || i2 < i1));
}

__device__ __forceinline__ void warp_argmax(float& v, int& i) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float v2 = __shfl_xor_sync(0xffffffffu, v, o);
    const int i2 = __shfl_xor_sync(0xffffffffu, i, o);
    if (piv_better(v2, i2, v, i)) { v = v2; i = i2; }
  }
}

// Block-wide argmax; the result is valid in every thread.
__device__ __forceinline__ void block_argmax(float& v, int& i, float* sv, int* si) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  warp_argmax(v, i);
  if (lane == 0) { sv[wid] = v; si[wid] = i; }
  __syncthreads();
  if (wid == 0) {
    float a = lane < nw ? sv[lane] : -1.f;
    int b = lane < nw ? si[lane] : -1;
    warp_argmax(a, b);
    if (lane == 0) { sv[0] = a; si[0] = b; }
  }
  __syncthreads();
  v = sv[0];
  i = si[0];
  __syncthreads();
}

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

constexpr int GETF2_THREADS = 512;
constexpr long long GRID_WAIT_LIMIT = 1LL << 22;

// Partial-pivoting LU of the panel W[jp:n, jp:jp+nb] (nb <= 128) on G CTAs
// (gridDim.x, all co-resident: cooperative launch).  CTA g holds rows
// [jp + g R, jp + (g + 1) R) column-major in shared memory.  Per column j:
//   a. each CTA finds its largest |w| among rows >= jp + j and publishes the
//      value, the row and that row's nb values (buffer j & 1); the owner of
//      row jp + j publishes that row too;
//   b. grid barrier (counter reaches (j + 1) G; bounded wait);
//   c. every CTA picks the same winner from the G candidates (largest, ties
//      to the smaller row), exchanges rows jp + j and the winner's from the
//      published copies, scales the column below the pivot by the pivot's
//      reciprocal and applies the rank-1 update to the rest of its rows.
// A zero pivot (LAPACK's info > 0) leaves the column as it is and records the
// first such column in *info (1-based).  The winner rows go to ipiv; CTA 0
// finally turns the panel's exchanges into a list of row moves (dst <- src)
// that k_laswp applies to the other columns.
__global__ void __launch_bounds__(GETF2_THREADS, 1)
k_getf2(float* __restrict__ W, long long ldw, long long n, long long jp, int nb, int R, int* __restrict__ ipiv,
        int* info, PivCand* cand, float* crow, float* top, unsigned* bar, int* plan, int* err) {
  extern __shared__ float P[];  // [nb][R]
  __shared__ float s_u[LNB];
  __shared__ float s_rv[32];
  __shared__ int s_ri[32];
  __shared__ int s_abort;
  __shared__ int s_piv[LNB];
  const int tid = threadIdx.x, G = gridDim.x, g = blockIdx.x;
  const long long rbeg = jp + (long long)g * R;
  const int rows = (int)max(0LL, min((long long)R, n - rbeg));
  for (int e = tid; e < nb * R; e += blockDim.x) {
    const int c = e / R, r = e % R;
    P[e] = r < rows ? W[(rbeg + r) + (jp + c) * ldw] : 0.f;
  }
  if (tid == 0) s_abort = 0;
  __syncthreads();
  for (int j = 0; j < nb; ++j) {
    const int q = j & 1;
    const long long trow = jp + j;  // the position this column's pivot moves to
    float best = -1.f;
    int bi = -1;
    for (int r = tid; r < rows; r += blockDim.x) {
      if (rbeg + r < trow) continue;
      const float v = fabsf(P[j * R + r]);
      if (piv_better(v, (int)(rbeg + r), best, bi)) { best = v; bi = (int)(rbeg + r); }
    }
    block_argmax(best, bi, s_rv, s_ri);
    if (tid == 0) {
      const long long raw = ((long long)bi << 32) | (long long)(unsigned)__float_as_int(best);
      reinterpret_cast<long long*>(cand)[q * G + g] = raw;
    }
    if (bi >= 0 && tid < nb) crow[((size_t)q * G + g) * LNB + tid] = P[tid * R + (int)(bi - rbeg)];
    if (trow >= rbeg && trow < rbeg + rows && tid < nb) top[q * LNB + tid] = P[tid * R + (int)(trow - rbeg)];
    __syncthreads();
    if (tid == 0) {
      __threadfence();
      atomicAdd(bar, 1u);
      const unsigned target = (unsigned)(j + 1) * (unsigned)G;
      bool ok = false;
      for (long long it = 0; it < GRID_WAIT_LIMIT; ++it) {
        if (ld_acquire_u32(bar) >= target) { ok = true; break; }
        if (it > 64) __nanosleep(64);
      }
      if (!ok) {
        s_abort = 1;
        atomicExch(err, 3);
      }
      __threadfence();
    }
    __syncthreads();
    if (s_abort) return;
    // the winner among the G candidates
    float v = -1.f;
    int wr = -1, wc = -1;
    if (tid < G) {
      // one 8-byte load of (|value|, row), past L1 (written by other CTAs)
      const long long raw = __ldcg(reinterpret_cast<const long long*>(cand) + q * G + tid);
      v = __int_as_float((int)(raw & 0xffffffffLL));
      wr = (int)(raw >> 32);
    }
    // the winner's CTA follows from its row
    block_argmax(v, wr, s_rv, s_ri);
    if (wr >= 0) wc = (int)((wr - jp) / R);
    if (tid < nb) s_u[tid] = wr >= 0 ? __ldcg(crow + ((size_t)q * G + wc) * LNB + tid) : 0.f;
    __syncthreads();
    const float pv = wr >= 0 ? s_u[j] : 0.f;
    if (wr < 0 || pv == 0.f) {
      // zero pivot: LAPACK records the first one and leaves the column
      if (g == 0 && tid == 0) {
        ipiv[trow] = (int)trow;
        s_piv[j] = (int)trow;
        atomicCAS(info, 0, (int)(trow + 1));
      }
      __syncthreads();
      continue;
    }
    if (g == 0 && tid == 0) {
      ipiv[trow] = wr;
      s_piv[j] = wr;
    }
    if ((long long)wr != trow) {
      if (trow >= rbeg && trow < rbeg + rows && tid < nb) P[tid * R + (int)(trow - rbeg)] = s_u[tid];
      if (wr >= rbeg && wr < rbeg + rows && tid < nb) P[tid * R + (int)(wr - rbeg)] = __ldcg(top + q * LNB + tid);
    }
    __syncthreads();
    const float pinv = __frcp_rn(pv);
    for (int r = tid; r < rows; r += blockDim.x)
      if (rbeg + r > trow) P[j * R + r] *= pinv;
    __syncthreads();
    const int ncol = nb - 1 - j;
    for (int e = tid; e < ncol * rows; e += blockDim.x) {
      const int c = j + 1 + e / rows, r = e % rows;
      if (rbeg + r > trow) P[c * R + r] = fmaf(-P[j * R + r], s_u[c], P[c * R + r]);
    }
    __syncthreads();
  }
  for (int e = tid; e < nb * R; e += blockDim.x) {
    const int c = e / R, r = e % R;
    if (r < rows) W[(rbeg + r) + (jp + c) * ldw] = P[e];
  }
  // the panel's exchanges as row moves: position jp + k receives the content
  // that the exchanges leave there (warp 0 of CTA 0 replays them)
  if (g == 0 && tid < 32) {
    int* cnt = plan;
    int* dst = plan + 1;
    int* src = plan + 1 + 2 * LNB;
    __shared__ int s_in[LNB];        // content of positions jp .. jp + nb - 1
    __shared__ int s_key[LNB], s_val[LNB];
    __shared__ int s_nout;
    for (int k = tid; k < nb; k += 32) s_in[k] = (int)(jp + k);
    if (tid == 0) s_nout = 0;
    __syncwarp();
    for (int k = 0; k < nb; ++k) {
      const int p = s_piv[k];
      if (p == (int)(jp + k)) continue;
      if (p < jp + nb) {
        if (tid == 0) {
          const int t = s_in[k];
          s_in[k] = s_in[p - jp];
          s_in[p - jp] = t;
        }
      } else {
        // find p among the rows outside the panel moved so far
        int found = -1;
        const int nout = s_nout;
        for (int b = 0; b < nout; b += 32) {
          const unsigned m = __ballot_sync(0xffffffffu, b + tid < nout && s_key[b + tid] == p);
          if (m) { found = b + __ffs(m) - 1; break; }
        }
        if (tid == 0) {
          if (found >= 0) {
            const int t = s_in[k];
            s_in[k] = s_val[found];
            s_val[found] = t;
          } else {
            s_key[nout] = p;
            s_val[nout] = s_in[k];
            s_in[k] = p;
            s_nout = nout + 1;
          }
        }
      }
      __syncwarp();
    }
    if (tid == 0) {
      int c = 0;
      for (int k = 0; k < nb; ++k)
        if (s_in[k] != (int)(jp + k)) { dst[c] = (int)(jp + k); src[c] = s_in[k]; ++c; }
      for (int t = 0; t < s_nout; ++t)
        if (s_val[t] != s_key[t]) { dst[c] = s_key[t]; src[c] = s_val[t]; ++c; }
      *cnt = c;
    }
  }
}

// The panel's row moves (dst <- src, all reads before all writes) applied to
// columns [c0, c0 + ncols) and [c1, c1 + ncols1) of W, 32 columns per CTA.
constexpr int LASWP_COLS = 32;
__global__ void __launch_bounds__(256)
k_laswp(float* __restrict__ W, long long ldw, const int* __restrict__ plan, long long c0, long long ncols0,
        long long c1, long long ncols1) {
  __shared__ float tile[2 * LNB * LASWP_COLS];
  __shared__ int s_dst[2 * LNB], s_src[2 * LNB];
  const int cnt = plan[0];
  if (cnt == 0) return;
  for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
    s_dst[t] = plan[1 + t];
    s_src[t] = plan[1 + 2 * LNB + t];
  }
  const long long t0 = (long long)blockIdx.x * LASWP_COLS;
  __syncthreads();
  const int total = cnt * LASWP_COLS;
  auto col_of = [&](int cc) -> long long {
    const long long t = t0 + cc;
    if (t < ncols0) return c0 + t;
    if (t - ncols0 < ncols1) return c1 + (t - ncols0);
    return -1;
  };
  for (int e = threadIdx.x; e < total; e += blockDim.x) {
    const int i = e % cnt, cc = e / cnt;
    const long long c = col_of(cc);
    tile[e] = c >= 0 ? W[(long long)s_src[i] + c * ldw] : 0.f;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < total; e += blockDim.x) {
    const int i = e % cnt, cc = e / cnt;
    const long long c = col_of(cc);
    if (c >= 0) W[(long long)s_dst[i] + c * ldw] = tile[e];
  }
}

// Inverses of the factored diagonal block (unit-lower and upper triangles)
// and the block itself rounded into the factor.
template <typename F>
__global__ void __launch_bounds__(DIAG_THREADS, 1)
k_piv_diag(const float* __restrict__ W, long long ldw, long long j0, int nbk, F* __restrict__ LU, long long ldf,
           float* __restrict__ Linv, float* __restrict__ Uinv) {
  extern __shared__ float sm[];
  float* T = sm;
  float* XL = sm + LNB * DP;
  float* XU = sm + 2 * LNB * DP;
  float* Tmp = sm + 3 * LNB * DP;
  const int tid = threadIdx.x;
  for (int idx = tid; idx < LNB * LNB; idx += DIAG_THREADS) {
    const int r = idx % LNB, c = idx / LNB;
    T[r * DP + c] = (r < nbk && c < nbk) ? W[(j0 + r) + (j0 + c) * ldw] : (r == c ? 1.f : 0.f);
  }
  __syncthreads();
  for (int idx = tid; idx < nbk * nbk; idx += blockDim.x) {
    const int r = idx % nbk, c = idx / nbk;
    LU[(j0 + r) + (j0 + c) * ldf] = from_f32<F>(T[r * DP + c]);
  }
  tri_inverses(T, XL, XU, Tmp);
  for (int idx = tid; idx < LNB * LNB; idx += blockDim.x) {
    const int r = idx % LNB, c = idx / LNB;
    Linv[c * LNB + r] = XL[r * DP + c];
    Uinv[c * LNB + r] = XU[r * DP + c];
  }
}

// L21 (rows [r0, n) of the panel's columns in W) into the K-major operand
// Lp[(r - r0) * pitch + k], rounded to the factor type; 32 rows per CTA.
template <typename F>
__global__ void __launch_bounds__(256)
k_make_lop(const float* __restrict__ W, long long ldw, long long jp, int nb, long long r0, long long n,
           F* __restrict__ Lp, long long pitch) {
  __shared__ float t[LNB][33];
  const long long rb = r0 + (long long)blockIdx.x * 32;
  for (int e = threadIdx.x; e < 32 * LNB; e += blockDim.x) {
    const int i = e % 32, k = e / 32;
    t[k][i] = (k < nb && rb + i < n) ? W[(rb + i) + (jp + k) * ldw] : 0.f;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < 32 * LNB; e += blockDim.x) {
    const int k = e % LNB, i = e / LNB;
    if (rb + i < n && k < nb) Lp[(rb + i - r0) * pitch + k] = from_f32<F>(t[k][i]);
  }
}

// The strictly lower part below the diagonal blocks, W -> factor (rounded).
template <typename F>
__global__ void k_store_lower(const float* __restrict__ W, long long ldw, long long n, F* __restrict__ LU,
                              long long ldf) {
  for (long long c = blockIdx.y; c < n; c += gridDim.y) {
    const long long rs = (c / LNB + 1) * LNB;
    for (long long r = rs + (long long)blockIdx.x * blockDim.x + threadIdx.x; r < n;
         r += (long long)gridDim.x * blockDim.x)
      LU[r + c * ldf] = from_f32<F>(W[r + c * ldw]);
  }
}

// ---------------------------------------------------------------- host side

// First ticket of the next triangular solves; 0 except under a test hook
// (mpdok_debug_set), which raises it so that no block ever solves block 0.
static int g_first_ticket = 0;

static int reset_tickets(int* tk, cudaStream_t s) {
  MPDOK_CUDA_TRY(cudaMemsetAsync(tk, 0, sizeof(int) * 2, s));
  if (g_first_ticket != 0) {
    const int t0 = g_first_ticket;
    MPDOK_CUDA_TRY(cudaMemcpyAsync(tk, &t0, sizeof(int), cudaMemcpyHostToDevice, s));
    MPDOK_CUDA_TRY(cudaStreamSynchronize(s));
  }
  return MPDOK_OK;
}

// The triangular solves report a wait that ran out through an error word in
// their workspace.  A solve clears it once at its start and reads it when it
// ends: a timed-out block leaves its outputs unset (NaN), which the solve
// would otherwise report as a non-finite residual or a stalled iteration.
static int err_clear(int* err, cudaStream_t s) {
  MPDOK_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int) * 4, s));
  return MPDOK_OK;
}

static int err_finish(const int* err, int status, cudaStream_t s) {
  if (status == MPDOK_ERR_CUDA || status == MPDOK_ERR_ALLOC) return status;
  int h = 0;
  MPDOK_CUDA_TRY(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  MPDOK_CUDA_TRY(cudaStreamSynchronize(s));
  if (h != 0) {
    set_error("triangular solve: a block's wait on its predecessor ran out (device wait limit)");
    return MPDOK_ERR_TIMEOUT;
  }
  return status;
}

static unsigned grid_for(long long n, int per = 256) {
  long long b = (n + per - 1) / per;
  return (unsigned)std::max(1LL, std::min(b, (long long)num_sms() * 8));
}

struct ApplyWork {
  size_t off_y = 0, off_z = 0, off_tk = 0, off_err = 0, total = 0;
};

static ApplyWork apply_layout(long long n) {
  ApplyWork a;
  size_t off = 0;
  auto take = [&](size_t b) { size_t o = off; off = align_up(off + b, 256); return o; };
  a.off_y = take((size_t)std::max(1LL, n) * sizeof(float));
  a.off_z = take((size_t)std::max(1LL, n) * sizeof(float));
  a.off_tk = take(4 * sizeof(int));
  a.off_err = take(16);
  a.total = off;
  return a;
}

template <typename F>
static int lu_apply_t(const void* fbuf, long long n, int fdtype, const float* v, float* z, void* work,
                      cudaStream_t s, const int* skip) {
  const LULayout L = lu_layout(n, fdtype);
  const ApplyWork aw = apply_layout(n);
  const char* fb = (const char*)fbuf;
  char* wb = (char*)work;
  const F* LU = (const F*)(fb + L.off_lu);
  const float* Linv = (const float*)(fb + L.off_linv);
  const float* Uinv = (const float*)(fb + L.off_uinv);
  const float* d = (const float*)(fb + L.off_d);
  const float* Ml = (const float*)(fb + L.off_ml);
  const float* Mu = (const float*)(fb + L.off_mu);
  float* y = (float*)(wb + aw.off_y);
  float* zz = (float*)(wb + aw.off_z);
  int* tk = (int*)(wb + aw.off_tk);
  int* err = (int*)(wb + aw.off_err);
  // outputs start empty (TRSV_EMPTY in every word): the solves poll them
  MPDOK_CUDA_TRY(cudaMemsetAsync(y, 0xff, sizeof(float) * n, s));
  MPDOK_CUDA_TRY(cudaMemsetAsync(zz, 0xff, sizeof(float) * n, s));
  MPDOK_TRY(reset_tickets(tk, s));
  const int slot = prof_start(MPDOK_PROF_TRSV, s);
  const size_t smem = (size_t)LNB * LNB * sizeof(float);
  const float* dr = (const float*)(fb + L.off_dr);
  const int* perm = (const int*)(fb + L.off_perm);
  MPDOK_TRY(set_smem(k_trsv<F, true>, smem));
  MPDOK_TRY(set_smem(k_trsv<F, false>, smem));
  launch(k_trsv<F, true>, L.nblk, 256, smem, s, LU, L.ldf, Linv, Ml, n, L.nblk, v, dr, perm, y, tk, err, skip);
  launch(k_trsv<F, false>, L.nblk, 256, smem, s, LU, L.ldf, Uinv, Mu, n, L.nblk, (const float*)y, d, perm, zz,
         tk + 1, err, skip);
  launch(k_scale_out, grid_for(n), 256, 0, s, (const float*)zz, d, z, n, skip);
  prof_stop(slot, s, (double)n * (double)n * sizeof(F), skip);
  MPDOK_LAUNCH_CHECK("lu apply");
  return MPDOK_OK;
}

int lu_apply_any(const void* fbuf, long long n, int fdtype, const float* v, float* z, void* work, cudaStream_t s,
                 const int* skip) {
  switch (fdtype) {
    case MPDOK_BF16: return lu_apply_t<__nv_bfloat16>(fbuf, n, fdtype, v, z, work, s, skip);
    case MPDOK_F16: return lu_apply_t<__half>(fbuf, n, fdtype, v, z, work, s, skip);
    case MPDOK_F32: return lu_apply_t<float>(fbuf, n, fdtype, v, z, work, s, skip);
    default: set_error("invalid argument: factor dtype"); return MPDOK_ERR_INVALID_ARG;
  }
}

// ------------------------------------------------------ factorization schedule
// Two-level right-looking LU.  Super-panel [J, Jend) of <= spw columns is
// factored with 128-wide panels whose updates are confined to the
// super-panel's row strip (rows < Jend, all columns right of the panel) and
// column strip (rows >= Jend, columns < Jend); the far trailing matrix
// (rows, columns >= Jend) then receives all of them at once, K = spw.
//
// Look-ahead: super-panels are factored on a high-priority chain stream.  The
// far update of super-panel J has two parts: (a) the rows and columns of
// super-panel J + 1 (rows [Jend, Jn) x columns >= Jend, and rows >= Jn x
// columns [Jend, Jn)), which the chain stream applies itself once the work
// below J and part (b) of J - 1 are done, and then factors J + 1; (b) the
// rest, rows and columns >= Jn, on the caller's stream, concurrently with
// J + 1.  The two touch disjoint parts of W: the inner loop of J + 1 writes
// rows < Jn or columns < Jn only.  Operands alternate between two buffers, so
// (b) of J still reads its own while J + 1 writes the other.
//
// Inside a super-panel the chain stream (sa) runs, per panel p with columns
// [jp, r1 = jp + 128): the diagonal-block LU; the panel solve for the rest of
// the super-panel (rows and columns [r1, Jend), 16-row blocks, one launch);
// the update of the rest of the super-panel, rows and columns [r1, Jend) (one
// launch); then the next diagonal LU.  A panel therefore costs three dependent
// launches on one stream and no cross-stream hand-off.  Two below streams (sc,
// sd, lower priority) handle the rows and columns past the super-panel
// left-looking: for panel p they apply every earlier panel of the super-panel
// to p's own column block rows >= Jend (sc) and row block columns >= Jend
// (sd, concurrently), one update each with K = jp - J instead of a K = 128
// update of the whole row and column strips per panel (1/4.5 of the FP32
// traffic); then sc solves p's panel there.  Only later panels' below work and
// the far update read what they write, so the chain never waits for them
// until the end of the super-panel.
//
// The schedule is data: lu_schedule lists every launch, event record and
// event wait of one factorization in issue order, lu_factor_t executes the
// list, and mpdok_lu_schedule exports it, so that a host-only check can verify
// that every pair of launches touching the same data is ordered by the
// streams and events.
enum LuStream : int { LU_MAIN = 0, LU_CHAIN = 1, LU_BELOW = 2, LU_BELOW2 = 3 };
constexpr int LU_NSTREAMS = 4;
enum LuKind : int { LU_DIAG = 0, LU_SOLVE = 1, LU_UPDATE = 2, LU_RECORD = 3, LU_WAIT = 4, LU_PROF_START = 5,
                    LU_PROF_STOP = 6 };
enum LuEvent : int { LU_EV_READY = 0, LU_EV_PANEL = 1, LU_EV_A = 2, LU_EV_C = 3, LU_EV_B = 4, LU_EV_D = 5,
                     LU_EV_E = 6 };
constexpr int LU_NEVENTS = 7;
struct LuStep {
  int kind = 0, stream = 0;
  long long J = 0;           // super-panel start (operand buffer (J / spw) & 1)
  long long jp = 0;          // DIAG, SOLVE: panel start
  long long a = 0, b = 0;    // SOLVE: rows and columns [a, b); UPDATE: first C row and column
  long long m = 0, nn = 0;   // UPDATE: C rows x columns (operand rows a.., b.. of L21, U12)
  long long K = 0, koff = 0; // UPDATE: depth and first operand column (K-slot)
  int rb = 0;                // SOLVE: rows per block
  int event = 0;             // RECORD, WAIT: event; PROF_START, PROF_STOP: window
  double work = 0.0;         // PROF_STOP: flops of the window
};

static std::vector<LuStep> lu_schedule(long long n, long long spw) {
  std::vector<LuStep> v;
  const bool lookahead = n > spw;
  auto add = [&](int kind, int stream) {
    LuStep st;
    st.kind = kind;
    st.stream = stream;
    v.push_back(st);
    return v.size() - 1;
  };
  auto record = [&](int stream, int ev) { v[add(LU_RECORD, stream)].event = ev; };
  auto wait = [&](int stream, int ev) { v[add(LU_WAIT, stream)].event = ev; };
  auto update = [&](int stream, long long J, long long koff, long long K, long long crow, long long ccol, long long m,
                    long long nn) {
    if (m <= 0 || nn <= 0) return;
    LuStep& st = v[add(LU_UPDATE, stream)];
    st.J = J;
    st.koff = koff;
    st.K = K;
    st.a = crow;
    st.b = ccol;
    st.m = m;
    st.nn = nn;
  };
  auto solve = [&](int stream, long long J, long long jp, long long begin, long long end, int rb) {
    LuStep& st = v[add(LU_SOLVE, stream)];
    st.J = J;
    st.jp = jp;
    st.a = begin;
    st.b = end;
    st.rb = rb;
  };
  auto prof = [&](int stream, int window, bool start, double work) {
    LuStep& st = v[add(start ? LU_PROF_START : LU_PROF_STOP, stream)];
    st.event = window;
    st.work = work;
  };
  if (lookahead) {  // the chain stream starts after the scaling and the working copy
    record(LU_MAIN, LU_EV_READY);
    wait(LU_CHAIN, LU_EV_READY);
  }
  for (long long J = 0; J < n; J += spw) {
    const long long Jend = std::min<long long>(n, J + spw);
    const int sa = lookahead ? LU_CHAIN : LU_MAIN;
    const int sc = LU_BELOW, sd = LU_BELOW2;
    const bool below = lookahead && Jend < n;  // rows and columns past the super-panel
    for (long long jp = J; jp < Jend; jp += LNB) {
      const long long r1 = jp + LNB;  // first row / column after the panel
      const bool has_next = r1 < Jend;
      const long long koff = jp - J;  // the panel's K-slot in the operands
      // chain: the diagonal LU, the panel's solve for the rest of the
      // super-panel (16-row blocks, one launch), then its update of the rest
      // of the super-panel (one launch); every update a later panel of J needs
      // is issued on this stream before it
      prof(sa, 0, true, 0.0);
      {
        LuStep& st = v[add(LU_DIAG, sa)];
        st.J = J;
        st.jp = jp;
      }
      if (has_next) solve(sa, J, jp, r1, Jend, 16);
      prof(sa, 0, false, 2.0 * 2.0 * (double)(Jend - std::min(r1, Jend)) * LNB * LNB + (2.0 / 3.0) * LNB * LNB * LNB);
      if (below) record(sa, LU_EV_A);
      if (has_next) update(sa, J, koff, LNB, r1, r1, Jend - r1, Jend - r1);
      // below, left-looking: panel p's own column and row blocks past the
      // super-panel receive the updates of every earlier panel of J at once
      // (K = jp - J), then the panel solve there; off the chain's path
      if (below) {
        wait(sc, LU_EV_A);  // the chain's solves of panels J .. p, and p's diagonal LU
        if (jp > J) {
          // the column block here, the row block concurrently on the second
          // below stream; the row block reads U12 of the earlier panels past
          // the super-panel, so it waits for the previous panel solve below
          // (which itself followed the chain's solve of that panel)
          wait(sd, LU_EV_E);
          update(sc, J, 0, jp - J, Jend, jp, n - Jend, std::min<long long>(LNB, Jend - jp));
          update(sd, J, 0, jp - J, jp, Jend, std::min<long long>(LNB, Jend - jp), n - Jend);
          record(sd, LU_EV_D);
          wait(sc, LU_EV_D);
        }
        prof(sc, 2, true, 0.0);
        solve(sc, J, jp, Jend, n, 64);
        prof(sc, 2, false, 2.0 * 2.0 * (double)(n - Jend) * LNB * LNB);
        record(sc, LU_EV_E);
      }
    }
    if (below) {  // join the below stream
      record(sc, LU_EV_C);
      wait(sa, LU_EV_C);
    }
    if (lookahead) {
      record(LU_CHAIN, LU_EV_PANEL);
      wait(LU_MAIN, LU_EV_PANEL);
    }
    if (Jend < n) {
      const long long K = Jend - J;
      if (!lookahead) {
        update(LU_MAIN, J, 0, K, Jend, Jend, n - Jend, n - Jend);
      } else {
        const long long Jn = std::min<long long>(n, Jend + spw);
        // (a) what super-panel J + 1 reads and writes first, on the chain
        // stream at its priority, once part (b) of J - 1 (which covers J + 1's
        // rows and columns too) is done
        if (J > 0) wait(LU_CHAIN, LU_EV_B);
        update(LU_CHAIN, J, 0, K, Jend, Jend, Jn - Jend, n - Jend);
        update(LU_CHAIN, J, 0, K, Jn, Jend, n - Jn, Jn - Jend);
        // (b) the rest of the trailing matrix on the caller's stream,
        // concurrent with J + 1, in up to four column chunks: a kernel
        // boundary on this stream drains the SMs, which lets the panel kernels
        // (one of them needs a whole SM) in without waiting for the whole update
        const long long rest = n - Jn;
        const long long chunk = std::max<long long>(2048, (rest / 4 + 255) / 256 * 256);
        for (long long c = Jn; c < n; c += chunk) update(LU_MAIN, J, 0, K, Jn, c, n - Jn, std::min(chunk, n - c));
        if (Jn < n) record(LU_MAIN, LU_EV_B);
      }
    }
  }
  if (lookahead) {  // the caller's stream owns the result
    record(LU_CHAIN, LU_EV_PANEL);
    wait(LU_MAIN, LU_EV_PANEL);
  }
  return v;
}

// The look-ahead streams (chain at the highest priority, the two below-panel
// streams one step lower) and the schedule's events, made once per host thread and device
// and kept for the life of the process, so a factorization creates none.
// Every event is recorded before it is waited on in issue order within one
// factorization, and a factorization ends with the caller's stream joined to
// both streams and synchronised, so reusing them across calls orders nothing
// that the schedule did not.
struct LuStreams {
  cudaStream_t chain = nullptr, below = nullptr, below2 = nullptr;
  cudaEvent_t ev[LU_NEVENTS] = {};
  cudaError_t err = cudaSuccess;
  LuStreams() {
    int lo = 0, hi = 0;
    err = cudaDeviceGetStreamPriorityRange(&lo, &hi);
    const int mid = hi < lo ? hi + 1 : hi;
    if (err == cudaSuccess) err = cudaStreamCreateWithPriority(&chain, cudaStreamNonBlocking, hi);
    if (err == cudaSuccess) err = cudaStreamCreateWithPriority(&below, cudaStreamNonBlocking, mid);
    if (err == cudaSuccess) err = cudaStreamCreateWithPriority(&below2, cudaStreamNonBlocking, mid);
    for (cudaEvent_t& e : ev)
      if (err == cudaSuccess) err = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    if (err != cudaSuccess) cudaGetLastError();
  }
};

static int lu_streams(LuStreams** out) {
  constexpr int MAX_DEV = 64;
  thread_local LuStreams* sets[MAX_DEV] = {};
  int dev = 0;
  MPDOK_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= MAX_DEV) {
    set_error("lu look-ahead streams: device ordinal out of range");
    return MPDOK_ERR_INVALID_ARG;
  }
  if (sets[dev] == nullptr) sets[dev] = new LuStreams();
  if (sets[dev]->err != cudaSuccess) {
    const cudaError_t e = sets[dev]->err;
    delete sets[dev];  // a later call tries again
    sets[dev] = nullptr;
    return cuda_status(e, "lu look-ahead streams / events");
  }
  *out = sets[dev];
  return MPDOK_OK;
}

template <typename F>
static int lu_factor_t(const double* A, long long lda, long long n, int fdtype, int pivoting, void* fbuf,
                       void* work, cudaStream_t s, int* nperturb_host) {
  const LULayout L = lu_layout(n, fdtype);
  const LUWork w = lu_work_layout(n, fdtype);
  char* fb = (char*)fbuf;
  char* wb = (char*)work;
  F* LU = (F*)(fb + L.off_lu);
  float* Linv = (float*)(fb + L.off_linv);
  float* Uinv = (float*)(fb + L.off_uinv);
  float* d = (float*)(fb + L.off_d);
  LUMeta* meta = (LUMeta*)(fb + L.off_meta);
  float* W = (float*)(wb + w.off_W);
  F* Lp2 = (F*)(wb + w.off_Lp);
  F* Up2 = (F*)(wb + w.off_Up);
  const long long spw = super_panel_width(fdtype);
  const size_t opsz = (size_t)std::max(1LL, n) * spw;  // elements of one operand buffer
  int* errw = (int*)(wb + w.off_err);
  MPDOK_CUDA_TRY(cudaMemsetAsync(errw, 0, 64, s));
  MPDOK_CUDA_TRY(cudaMemsetAsync(meta, 0, sizeof(LUMeta), s));
  launch(k_diag_scale, grid_for(n), 256, 0, s, A, lda, n, d, (float*)(fb + L.off_dr), (int*)(fb + L.off_perm));
  dim3 g2((unsigned)std::min<long long>((n + 255) / 256, 16), (unsigned)std::min<long long>(n, 65535));
  launch(k_scaled_copy, g2, 256, 0, s, A, lda, n, (const float*)d, W, w.ldw);
  MPDOK_LAUNCH_CHECK("lu scale");

  const size_t smem_diag = DIAG_RR_ALLOC;
  constexpr size_t smem_tp = trsm_pair_smem(64), smem_tp16 = trsm_pair_smem(16);
  MPDOK_TRY(set_smem(k_lu_diag<F>, smem_diag));
  MPDOK_TRY(set_smem(k_trsm_pair<F, 64>, smem_tp));
  MPDOK_TRY(set_smem(k_trsm_pair<F, 16>, smem_tp16));
  const float tau = 1e-6f;
  // C -= A B^T on one strip: A rows / B rows at the given Lp / Up offsets.
  auto update = [&](long long crow, long long ccol, long long m, long long nn, const F* Ab, const F* Bb, int K,
                    cudaStream_t st) -> int {
    if (m <= 0 || nn <= 0) return MPDOK_OK;
    float* C = W + crow + ccol * w.ldw;
    if (fdtype == MPDOK_F32) {
      const int gs = prof_start(MPDOK_PROF_LU_GEMM, st);
      dim3 gg((unsigned)((m + 127) / 128), (unsigned)((nn + 127) / 128));
      launch(k_gemm_update_f32, gg, 256, 0, st, C, w.ldw, (const float*)Ab, (const float*)Bb, spw,
             (int)m, (int)nn, K);
      prof_stop(gs, st, 2.0 * (double)m * (double)nn * K);
      prof_stop_bytes(gs, 8.0 * (double)m * (double)nn + 4.0 * (double)K * ((double)m + (double)nn));
      MPDOK_LAUNCH_CHECK("lu gemm f32");
      return MPDOK_OK;
    }
    return gemm_update(C, w.ldw, Ab, Bb, spw, (int)m, (int)nn, K, fdtype, MPDOK_ENGINE_TENSOR, errw, st);
  };
  const bool lookahead = n > spw;
  // the chain first; the panel work below the super-panel next; the far update last
  cudaStream_t side = nullptr, below = nullptr, below2 = nullptr;
  const cudaEvent_t* evs = nullptr;
  if (lookahead) {
    LuStreams* ls = nullptr;
    MPDOK_TRY(lu_streams(&ls));
    side = ls->chain;
    below = ls->below;
    below2 = ls->below2;
    evs = ls->ev;
  }
  const std::vector<LuStep> sched = lu_schedule(n, spw);
  const cudaStream_t streams[LU_NSTREAMS] = {s, side, below, below2};  // LU_MAIN, LU_CHAIN, LU_BELOW, LU_BELOW2
  int prof_window[3] = {-1, -1, -1};
  auto body = [&]() -> int {
    for (const LuStep& st : sched) {
      if (st.stream != LU_MAIN && streams[st.stream] == nullptr) {
        set_error("lu schedule: step on a stream that was not created");
        return MPDOK_ERR_INVALID_ARG;
      }
      const cudaStream_t cs = streams[st.stream];
      const int buf = (int)((st.J / spw) & 1);
      F* Lp = Lp2 + (size_t)buf * opsz;
      F* Up = Up2 + (size_t)buf * opsz;
      switch (st.kind) {
        case LU_DIAG: {
          const int k = (int)(st.jp / LNB);
          const int nbk = (int)std::min<long long>(LNB, n - st.jp);
          launch(k_lu_diag<F>, 1, DIAG_LU_THREADS, smem_diag, cs, W, w.ldw, st.jp, nbk, LU, L.ldf,
                 Linv + (size_t)k * LNB * LNB, Uinv + (size_t)k * LNB * LNB, errw + 1, tau);
          MPDOK_LAUNCH_CHECK("lu diagonal block");
          break;
        }
        case LU_SOLVE: {
          const int k = (int)(st.jp / LNB);
          const int koff = (int)(st.jp - st.J);
          const float* ui = Uinv + (size_t)k * LNB * LNB;
          const float* li = Linv + (size_t)k * LNB * LNB;
          if (st.rb == 16) {
            const int nb = (int)((st.b - st.a + 15) / 16);
            launch(k_trsm_pair<F, 16>, (unsigned)(2 * nb), TRSM_THREADS, smem_tp16, cs, (const float*)W, w.ldw, st.jp,
                   st.a, st.b, ui, li, Lp, Up, spw, st.J, koff, LU, L.ldf, nb);
          } else {
            const int nb = (int)((st.b - st.a + 63) / 64);
            launch(k_trsm_pair<F, 64>, (unsigned)(2 * nb), TRSM_THREADS, smem_tp, cs, (const float*)W, w.ldw, st.jp,
                   st.a, st.b, ui, li, Lp, Up, spw, st.J, koff, LU, L.ldf, nb);
          }
          MPDOK_LAUNCH_CHECK("lu panel solve");
          break;
        }
        case LU_UPDATE:
          MPDOK_TRY(update(st.a, st.b, st.m, st.nn, Lp + (st.a - st.J) * spw + st.koff,
                           Up + (st.b - st.J) * spw + st.koff, (int)st.K, cs));
          break;
        case LU_RECORD:
          MPDOK_CUDA_TRY(cudaEventRecord(evs[st.event], cs));
          break;
        case LU_WAIT:
          MPDOK_CUDA_TRY(cudaStreamWaitEvent(cs, evs[st.event], 0));
          break;
        case LU_PROF_START:
          prof_window[st.event] = prof_start(MPDOK_PROF_LU_PANEL, cs);
          break;
        case LU_PROF_STOP:
          prof_stop(prof_window[st.event], cs, st.work);
          break;
        default:
          set_error("lu schedule: unknown step");
          return MPDOK_ERR_INVALID_ARG;
      }
    }
    return MPDOK_OK;
  };
  const int bst = body();
  if (lookahead && bst != MPDOK_OK) {
    // on an error the side streams may still hold work: let it finish first
    cudaStreamSynchronize(side);
    cudaStreamSynchronize(below);
    cudaStreamSynchronize(below2);
  }
  if (bst < 0) return bst;
  {
    // the full diagonal-block inverses of the triangular solves, then their chain tiles
    MPDOK_TRY(set_smem(k_tri_inv_complete, DIAG_SMEM));
    launch(k_tri_inv_complete, L.nblk, DIAG_THREADS, DIAG_SMEM, s, (const float*)W, w.ldw, n, Linv, Uinv);
    MPDOK_LAUNCH_CHECK("lu diagonal-block inverses");
    const size_t smem_ct = 2 * (size_t)LNB * LNB * sizeof(float);
    MPDOK_TRY(set_smem(k_trsv_chain_tiles<F>, smem_ct));
    launch(k_trsv_chain_tiles<F>, dim3(L.nblk, 2), 256, smem_ct, s, (const F*)LU, L.ldf, (const float*)Linv,
           (const float*)Uinv, (float*)(fb + L.off_ml), (float*)(fb + L.off_mu), n, L.nblk);
    MPDOK_LAUNCH_CHECK("lu chain tiles");
  }
  int herr[2] = {0, 0};
  MPDOK_CUDA_TRY(cudaMemcpyAsync(herr, errw, sizeof(herr), cudaMemcpyDeviceToHost, s));
  MPDOK_CUDA_TRY(cudaStreamSynchronize(s));
  if (herr[0] != 0) {
    set_error("tensor-core update timed out waiting on an mbarrier");
    return MPDOK_ERR_TIMEOUT;
  }
  LUMeta hm;
  hm.n_lo = (int)(n & 0x7fffffff);
  hm.n_hi = (int)(n >> 31);
  hm.fdtype = fdtype;
  hm.pivoting = pivoting;
  hm.nperturbed = herr[1];
  hm.valid = 1;
  MPDOK_CUDA_TRY(cudaMemcpyAsync(meta, &hm, sizeof(hm), cudaMemcpyHostToDevice, s));
  MPDOK_CUDA_TRY(cudaStreamSynchronize(s));
  if (nperturb_host) *nperturb_host = herr[1];
  return MPDOK_OK;
}

// Rows per CTA of the pivoted panel factorization for m panel rows, or -1
// when the slices would not fit in shared memory.
static int piv_rows_per_cta(long long m, int nb, int* grid) {
  int dev = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
    return -1;
  const int g0 = std::min(PIV_MAX_CTAS, num_sms());
  long long R = (m + g0 - 1) / g0;
  R = std::max(32LL, (R + 31) / 32 * 32);
  const long long budget = (long long)optin - 8 * 1024;  // the kernel's static shared memory and slack
  if (R * nb * (long long)sizeof(float) > budget) return -1;
  *grid = (int)((m + R - 1) / R);
  return (int)R;
}

template <typename F>
static int lu_factor_piv(const double* A, long long lda, long long n, int fdtype, void* fbuf, void* work,
                         cudaStream_t s, int* info_host) {
  const LULayout L = lu_layout(n, fdtype);
  const LUWork w = lu_work_layout(n, fdtype);
  char* fb = (char*)fbuf;
  char* wb = (char*)work;
  F* LU = (F*)(fb + L.off_lu);
  float* Linv = (float*)(fb + L.off_linv);
  float* Uinv = (float*)(fb + L.off_uinv);
  float* dc = (float*)(fb + L.off_d);
  float* dr = (float*)(fb + L.off_dr);
  int* perm = (int*)(fb + L.off_perm);
  int* ipiv = (int*)(fb + L.off_ipiv);
  LUMeta* meta = (LUMeta*)(fb + L.off_meta);
  float* W = (float*)(wb + w.off_W);
  F* Lp = (F*)(wb + w.off_Lp);
  F* Up = (F*)(wb + w.off_Up);
  const long long pitch = super_panel_width(fdtype);
  int* errw = (int*)(wb + w.off_err);  // [0] tensor-core wait, [2] first zero pivot, [3] panel barrier wait
  PivCand* cand = (PivCand*)(wb + w.off_cand);
  float* crow = (float*)(wb + w.off_crow);
  float* top = (float*)(wb + w.off_top);
  unsigned* bar = (unsigned*)(wb + w.off_bar);
  int* plan = (int*)(wb + w.off_plan);
  unsigned long long* rmax = (unsigned long long*)(wb + w.off_scale);
  MPDOK_CUDA_TRY(cudaMemsetAsync(errw, 0, 64, s));
  MPDOK_CUDA_TRY(cudaMemsetAsync(meta, 0, sizeof(LUMeta), s));
  // equilibration W = Dr A Dc (powers of two)
  MPDOK_CUDA_TRY(cudaMemsetAsync(rmax, 0, sizeof(unsigned long long) * n, s));
  const long long cchunk = 256;
  dim3 gr((unsigned)((n + 255) / 256), (unsigned)std::min<long long>((n + cchunk - 1) / cchunk, 65535));
  launch(k_row_absmax, gr, 256, 0, s, A, lda, n, (n + gr.y - 1) / gr.y, rmax);
  launch(k_row_scale, grid_for(n), 256, 0, s, (const unsigned long long*)rmax, n, dr, perm);
  launch(k_col_scale_copy, (unsigned)n, 256, 0, s, A, lda, n, (const float*)dr, dc, W, w.ldw);
  MPDOK_LAUNCH_CHECK("lu equilibration");
  constexpr size_t smem_tp = trsm_pair_smem(64);
  MPDOK_TRY(set_smem(k_piv_diag<F>, DIAG_SMEM));
  MPDOK_TRY(set_smem(k_trsm_pair<F, 64>, smem_tp));
  for (long long jp = 0; jp < n; jp += LNB) {
    const int nb = (int)std::min<long long>(LNB, n - jp);
    const long long m = n - jp;
    int G = 0;
    const int R = piv_rows_per_cta(m, nb, &G);
    if (R < 0) {
      set_error("pivoted LU: a %lld-row panel does not fit the co-resident CTAs' shared memory (n too large for "
                "pivoting = 1 on this device)", m);
      return MPDOK_ERR_UNSUPPORTED;
    }
    const size_t smem = (size_t)nb * R * sizeof(float);
    MPDOK_TRY(set_smem(k_getf2, smem));
    MPDOK_CUDA_TRY(cudaMemsetAsync(bar, 0, sizeof(unsigned), s));
    {
      float* aW = W;
      long long aldw = w.ldw, an = n, ajp = jp;
      int anb = nb, aR = R;
      int* aipiv = ipiv;
      int* ainfo = errw + 2;
      int* aerr = errw + 3;
      void* args[] = {&aW, &aldw, &an, &ajp, &anb, &aR, &aipiv, &ainfo, &cand, &crow, &top, &bar, &plan, &aerr};
      MPDOK_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)k_getf2, dim3(G), dim3(GETF2_THREADS), args, smem, s));
      count_launch();
    }
    const long long rest = n - jp - nb;
    if (jp + rest > 0) {
      const unsigned gl = (unsigned)((jp + rest + LASWP_COLS - 1) / LASWP_COLS);
      launch(k_laswp, gl, 256, 0, s, W, w.ldw, (const int*)plan, 0LL, jp, jp + nb, rest);
    }
    const int k = (int)(jp / LNB);
    launch(k_piv_diag<F>, 1, DIAG_THREADS, DIAG_SMEM, s, (const float*)W, w.ldw, jp, nb, LU, L.ldf,
           Linv + (size_t)k * LNB * LNB, Uinv + (size_t)k * LNB * LNB);
    MPDOK_LAUNCH_CHECK("pivoted panel");
    if (rest <= 0) continue;
    const long long r1 = jp + nb;
    // U12 = L11^-1 W12 (rows jp .. jp + 128, every column to the right)
    launch(k_trsm_pair<F, 64>, (unsigned)((rest + 63) / 64), TRSM_THREADS, smem_tp, s, (const float*)W, w.ldw, jp,
           r1, n, (const float*)(Uinv + (size_t)k * LNB * LNB), (const float*)(Linv + (size_t)k * LNB * LNB), Lp, Up,
           pitch, r1, 0, LU, L.ldf, 0);
    launch(k_make_lop<F>, (unsigned)((rest + 31) / 32), 256, 0, s, (const float*)W, w.ldw, jp, nb, r1, n, Lp, pitch);
    MPDOK_LAUNCH_CHECK("pivoted panel solve");
    float* C = W + r1 + r1 * w.ldw;
    if (fdtype == MPDOK_F32) {
      const int gs = prof_start(MPDOK_PROF_LU_GEMM, s);
      dim3 gg((unsigned)((rest + 127) / 128), (unsigned)((rest + 127) / 128));
      launch(k_gemm_update_f32, gg, 256, 0, s, C, w.ldw, (const float*)Lp, (const float*)Up, pitch, (int)rest,
             (int)rest, nb);
      prof_stop(gs, s, 2.0 * (double)rest * (double)rest * nb);
      prof_stop_bytes(gs, 8.0 * (double)rest * (double)rest + 4.0 * nb * 2.0 * (double)rest);
      MPDOK_LAUNCH_CHECK("pivoted update f32");
    } else {
      MPDOK_TRY(gemm_update(C, w.ldw, Lp, Up, pitch, (int)rest, (int)rest, nb, fdtype, MPDOK_ENGINE_TENSOR, errw, s));
    }
  }
  {
    dim3 g2((unsigned)std::min<long long>((n + 255) / 256, 16), (unsigned)std::min<long long>(n, 65535));
    launch(k_store_lower<F>, g2, 256, 0, s, (const float*)W, w.ldw, n, LU, L.ldf);
    const size_t smem_ct = 2 * (size_t)LNB * LNB * sizeof(float);
    MPDOK_TRY(set_smem(k_trsv_chain_tiles<F>, smem_ct));
    launch(k_trsv_chain_tiles<F>, dim3(L.nblk, 2), 256, smem_ct, s, (const F*)LU, L.ldf, (const float*)Linv,
           (const float*)Uinv, (float*)(fb + L.off_ml), (float*)(fb + L.off_mu), n, L.nblk);
    MPDOK_LAUNCH_CHECK("pivoted factor store");
  }
  int herr[4] = {0, 0, 0, 0};
  MPDOK_CUDA_TRY(cudaMemcpyAsync(herr, errw, sizeof(herr), cudaMemcpyDeviceToHost, s));
  std::vector<int> hp((size_t)n), hperm((size_t)n);
  MPDOK_CUDA_TRY(cudaMemcpyAsync(hp.data(), ipiv, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
  MPDOK_CUDA_TRY(cudaStreamSynchronize(s));
  if (herr[0] != 0) {
    set_error("tensor-core update timed out waiting on an mbarrier");
    return MPDOK_ERR_TIMEOUT;
  }
  if (herr[3] != 0) {
    set_error("pivoted panel factorization: the grid barrier wait ran out");
    return MPDOK_ERR_TIMEOUT;
  }
  // P as a gather: (P x)_i = x_perm[i], the row exchanges of ipiv applied in order
  for (long long i = 0; i < n; ++i) hperm[(size_t)i] = (int)i;
  for (long long i = 0; i < n; ++i) {
    const int p = hp[(size_t)i];
    if (p < 0 || p >= n) {
      set_error("pivoted LU: invalid pivot row %d at step %lld", p, i);
      return MPDOK_ERR_CUDA;
    }
    std::swap(hperm[(size_t)i], hperm[(size_t)p]);
  }
  MPDOK_CUDA_TRY(cudaMemcpyAsync(perm, hperm.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
  LUMeta hm;
  hm.n_lo = (int)(n & 0x7fffffff);
  hm.n_hi = (int)(n >> 31);
  hm.fdtype = fdtype;
  hm.pivoting = 1;
  hm.nperturbed = 0;
  hm.valid = 1;
  MPDOK_CUDA_TRY(cudaMemcpyAsync(meta, &hm, sizeof(hm), cudaMemcpyHostToDevice, s));
  MPDOK_CUDA_TRY(cudaStreamSynchronize(s));
  if (info_host) *info_host = herr[2];
  return MPDOK_OK;
}

static int read_meta(const void* fbuf, long long n, int fdtype, LUMeta* hm, cudaStream_t s) {
  const LULayout L = lu_layout(n, fdtype);
  MPDOK_CUDA_TRY(cudaMemcpyAsync(hm, (const char*)fbuf + L.off_meta, sizeof(LUMeta), cudaMemcpyDeviceToHost, s));
  MPDOK_CUDA_TRY(cudaStreamSynchronize(s));
  return MPDOK_OK;
}

struct PcCtx {
  const void* fbuf;
  long long n;
  int fdtype;
  void* work;
};

static int pc_apply(void* ctx, const float* v, float* z, cudaStream_t s, const int* skip) {
  PcCtx* c = (PcCtx*)ctx;
  return lu_apply_any(c->fbuf, c->n, c->fdtype, v, z, c->work, s, skip);
}

__global__ void k_f64_to_f32(const double* __restrict__ a, float* __restrict__ b, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

__global__ void k_add_f32_to_f64(const float* __restrict__ e, double* __restrict__ x, long long n, int assign) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    x[i] = assign ? (double)e[i] : x[i] + (double)e[i];
}

}  // namespace mpdok

using namespace mpdok;

extern "C" int mpdok_debug_set(int key, long long value) {
  switch (key) {
    case MPDOK_DEBUG_WAIT_LIMIT: {
      const long long v = value > 0 ? value : SPIN_LIMIT;
      MPDOK_CUDA_TRY(cudaMemcpyToSymbol(g_spin_limit, &v, sizeof(v)));
      return MPDOK_OK;
    }
    case MPDOK_DEBUG_TRSV_FIRST_TICKET:
      MPDOK_ARG_CHECK(value >= 0 && value < (1LL << 30), "first ticket out of range");
      g_first_ticket = (int)value;
      return MPDOK_OK;
    default:
      set_error("invalid argument: unknown debug key %d", key);
      return MPDOK_ERR_INVALID_ARG;
  }
}

extern "C" size_t mpdok_lu_factor_size(long long n, int fdtype) {
  if (n < 0) return 0;
  return lu_layout(n, fdtype).total;
}

extern "C" size_t mpdok_lu_work_size(long long n, int fdtype) {
  if (n < 0) return 0;
  return lu_work_layout(n, fdtype).total;
}

extern "C" size_t mpdok_lu_apply_work_size(long long n) {
  if (n < 0) return 0;
  return apply_layout(n).total;
}

extern "C" long long mpdok_lu_schedule(long long n, int fdtype, long long* out, long long max_steps) {
  if (n < 0 || (fdtype != MPDOK_F32 && fdtype != MPDOK_BF16 && fdtype != MPDOK_F16)) {
    set_error("invalid argument: mpdok_lu_schedule needs n >= 0 and an FP32 / BF16 / FP16 factor type");
    return MPDOK_ERR_INVALID_ARG;
  }
  const std::vector<LuStep> v = lu_schedule(n, super_panel_width(fdtype));
  if (out != nullptr) {
    const long long cnt = std::min<long long>((long long)v.size(), std::max(0LL, max_steps));
    for (long long i = 0; i < cnt; ++i) {
      const LuStep& st = v[(size_t)i];
      const long long row[12] = {st.kind, st.stream, st.J, st.jp, st.a, st.b, st.m, st.nn, st.K, st.koff, st.rb,
                                 st.event};
      for (int f = 0; f < 12; ++f) out[12 * i + f] = row[f];
    }
  }
  return (long long)v.size();
}

extern "C" int mpdok_lu_factor(const double* A, long long lda, long long n, int fdtype, int pivoting, void* factors,
                               size_t factor_bytes, void* work, size_t work_bytes, cudaStream_t s) {
  MPDOK_ARG_CHECK(n >= 0, "negative n");
  MPDOK_ARG_CHECK(fdtype == MPDOK_BF16 || fdtype == MPDOK_F16 || fdtype == MPDOK_F32, "factor dtype");
  MPDOK_ARG_CHECK(pivoting == 0 || pivoting == 1, "pivoting must be 0 (none) or 1 (partial, by rows)");
  if (n == 0) return MPDOK_OK;
  MPDOK_ARG_CHECK(A && factors && work, "null pointer");
  MPDOK_ARG_CHECK(lda >= n, "lda < n");
  MPDOK_ARG_CHECK(factor_bytes >= lu_layout(n, fdtype).total, "factor buffer too small");
  MPDOK_ARG_CHECK(work_bytes >= lu_work_layout(n, fdtype).total, "work buffer too small");
  MPDOK_ARG_CHECK(n < (1LL << 31), "n too large");
  int np = 0;
  int st;
  if (pivoting == 1) {
    switch (fdtype) {
      case MPDOK_BF16: st = lu_factor_piv<__nv_bfloat16>(A, lda, n, fdtype, factors, work, s, &np); break;
      case MPDOK_F16: st = lu_factor_piv<__half>(A, lda, n, fdtype, factors, work, s, &np); break;
      default: st = lu_factor_piv<float>(A, lda, n, fdtype, factors, work, s, &np); break;
    }
    if (st < 0) return st;
    return np;  // LAPACK's info: 0, or the first column whose pivot is exactly zero (1-based)
  }
  switch (fdtype) {
    case MPDOK_BF16: st = lu_factor_t<__nv_bfloat16>(A, lda, n, fdtype, pivoting, factors, work, s, &np); break;
    case MPDOK_F16: st = lu_factor_t<__half>(A, lda, n, fdtype, pivoting, factors, work, s, &np); break;
    default: st = lu_factor_t<float>(A, lda, n, fdtype, pivoting, factors, work, s, &np); break;
  }
  if (st < 0) return st;
  return np;
}

template <typename F>
__global__ void k_export_lu(const F* __restrict__ LU, long long ldf, long long n, float* __restrict__ out,
                            long long ldo) {
  for (long long c = blockIdx.y; c < n; c += gridDim.y)
    for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (long long)gridDim.x * blockDim.x)
      out[r + c * ldo] = to_f32<F>(LU[r + c * ldf]);
}

// The factors in plain form: L\U (unit L below the diagonal, U on and above)
// as an n x n column-major FP32 matrix, LAPACK's 0-based pivot rows, the row
// permutation as a gather ((P x)_i = x_perm[i]) and the two scalings, so that
// P (Dr A Dc) = L U.  Any output may be NULL.
extern "C" int mpdok_lu_export(const void* factors, long long n, int fdtype, float* lu, long long ldo, int* ipiv,
                               int* perm, float* dr, float* dc, cudaStream_t s) {
  MPDOK_ARG_CHECK(n >= 0 && factors, "n >= 0 and a factor buffer");
  MPDOK_ARG_CHECK(fdtype == MPDOK_BF16 || fdtype == MPDOK_F16 || fdtype == MPDOK_F32, "factor dtype");
  if (n == 0) return MPDOK_OK;
  LUMeta hm;
  MPDOK_TRY(read_meta(factors, n, fdtype, &hm, s));
  if (!hm.valid || hm.fdtype != fdtype || hm.n_lo != (int)(n & 0x7fffffff)) {
    set_error("no factorization of this size / type in the factor buffer");
    return MPDOK_ERR_NOT_FACTORED;
  }
  const LULayout L = lu_layout(n, fdtype);
  const char* fb = (const char*)factors;
  if (lu) {
    MPDOK_ARG_CHECK(ldo >= n, "ldo < n");
    dim3 g((unsigned)std::min<long long>((n + 255) / 256, 16), (unsigned)std::min<long long>(n, 65535));
    switch (fdtype) {
      case MPDOK_BF16: launch(k_export_lu<__nv_bfloat16>, g, 256, 0, s, (const __nv_bfloat16*)(fb + L.off_lu), L.ldf, n, lu, ldo); break;
      case MPDOK_F16: launch(k_export_lu<__half>, g, 256, 0, s, (const __half*)(fb + L.off_lu), L.ldf, n, lu, ldo); break;
      default: launch(k_export_lu<float>, g, 256, 0, s, (const float*)(fb + L.off_lu), L.ldf, n, lu, ldo); break;
    }
    MPDOK_LAUNCH_CHECK("lu export");
  }
  if (ipiv) {
    if (hm.pivoting) {
      MPDOK_CUDA_TRY(cudaMemcpyAsync(ipiv, fb + L.off_ipiv, sizeof(int) * n, cudaMemcpyDeviceToDevice, s));
    } else {
      MPDOK_CUDA_TRY(cudaMemcpyAsync(ipiv, fb + L.off_perm, sizeof(int) * n, cudaMemcpyDeviceToDevice, s));
    }
  }
  if (perm) MPDOK_CUDA_TRY(cudaMemcpyAsync(perm, fb + L.off_perm, sizeof(int) * n, cudaMemcpyDeviceToDevice, s));
  if (dr) MPDOK_CUDA_TRY(cudaMemcpyAsync(dr, fb + L.off_dr, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
  if (dc) MPDOK_CUDA_TRY(cudaMemcpyAsync(dc, fb + L.off_d, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
  return MPDOK_OK;
}

extern "C" int mpdok_lu_apply(const void* factors, long long n, int fdtype, const float* v, float* z, void* work,
                              size_t work_bytes, cudaStream_t s) {
  MPDOK_ARG_CHECK(n >= 0, "negative n");
  if (n == 0) return MPDOK_OK;
  MPDOK_ARG_CHECK(factors && v && z && work, "null pointer");
  MPDOK_ARG_CHECK(work_bytes >= apply_layout(n).total, "apply work buffer too small");
  int* err = (int*)((char*)work + apply_layout(n).off_err);
  MPDOK_TRY(err_clear(err, s));
  return err_finish(err, lu_apply_any(factors, n, fdtype, v, z, work, s, nullptr), s);
}

extern "C" size_t mpdok_lu_ir_work_size(long long n) {
  if (n < 0) return 0;
  return apply_layout(n).total + krylov_layout(n, 1, nullptr).total + 256;
}

static int lu_ir_body(const double* A, long long lda, long long n, const void* factors, int fdtype, const double* b,
                      double* x, double tol, int maxiter_outer, char* wb, mpdok_solve_info* info, cudaStream_t s);

extern "C" int mpdok_lu_ir_solve(const double* A, long long lda, long long n, const void* factors, int fdtype,
                                 const double* b, double* x, double tol, int maxiter_outer, void* work,
                                 size_t work_bytes, mpdok_solve_info* info, cudaStream_t s) {
  if (info) std::memset(info, 0, sizeof(*info));
  MPDOK_ARG_CHECK(n >= 0, "negative n");
  if (n == 0) { if (info) info->converged = 1; return MPDOK_OK; }
  MPDOK_ARG_CHECK(A && factors && b && x && work, "null pointer");
  MPDOK_ARG_CHECK(work_bytes >= mpdok_lu_ir_work_size(n), "LU-IR work buffer too small");
  LUMeta hm;
  MPDOK_TRY(read_meta(factors, n, fdtype, &hm, s));
  if (!hm.valid || hm.fdtype != fdtype || hm.n_lo != (int)(n & 0x7fffffff)) {
    set_error("no factorization of this size / type in the factor buffer");
    return MPDOK_ERR_NOT_FACTORED;
  }
  char* wb = (char*)work;
  int* aerr = (int*)(wb + apply_layout(n).off_err);
  MPDOK_TRY(err_clear(aerr, s));
  return err_finish(aerr, lu_ir_body(A, lda, n, factors, fdtype, b, x, tol, maxiter_outer, wb, info, s), s);
}

static int lu_ir_body(const double* A, long long lda, long long n, const void* factors, int fdtype, const double* b,
                      double* x, double tol, int maxiter_outer, char* wb, mpdok_solve_info* info, cudaStream_t s) {
  const ApplyWork aw = apply_layout(n);
  void* awork = wb;
  KWs ws = krylov_layout(n, 1, wb + align_up(aw.total, 256));
  MPDOK_CUDA_TRY(cudaMemsetAsync(ws.tickets, 0, sizeof(unsigned) * 8, s));
  MPDOK_CUDA_TRY(cudaMemsetAsync(ws.sc, 0, sizeof(KScal), s));
  float* v32 = ws.w;
  float* z32 = ws.x32;
  // bnorm
  MPDOK_TRY(norm2_f64(ws, b, n, &ws.sc->aux, s));
  KScal hs;
  MPDOK_TRY(read_scal(ws, &hs, s));
  const double bnorm = std::sqrt(hs.aux);
  if (info) info->bnorm = bnorm;
  if (!std::isfinite(bnorm)) {
    set_error("LU-IR: the right-hand side has non-finite entries");
    return MPDOK_ERR_NONFINITE;
  }
  if (bnorm == 0.0) {
    MPDOK_CUDA_TRY(cudaMemsetAsync(x, 0, sizeof(double) * n, s));
    if (info) { info->converged = 1; info->n_history = 1; info->history[0] = 0.0; }
    return MPDOK_OK;
  }
  // initial solve x = LU^-1 b
  launch(k_f64_to_f32, grid_for(n), 256, 0, s, b, v32, n);
  MPDOK_TRY(lu_apply_any(factors, n, fdtype, v32, z32, awork, s, nullptr));
  launch(k_add_f32_to_f64, grid_for(n), 256, 0, s, (const float*)z32, x, n, 1);
  bool conv = false;
  int it = 0;
  for (it = 0; it < maxiter_outer; ++it) {
    MPDOK_TRY(gemv_launch(MPDOK_F64, false, A, lda, n, n, x, n, 1, ws.r64, n, -1.0, 1.0, b, n, &ws.sc->nrm2, ws.gw,
                          ws.gbytes, s, true, nullptr));
    MPDOK_TRY(read_scal(ws, &hs, s));
    const double rel = std::sqrt(hs.nrm2) / bnorm;
    if (info && info->n_history < MPDOK_HISTORY_MAX) {
      info->hist_iter[info->n_history] = it;
      info->history[info->n_history++] = rel;
      info->relres = rel;
    }
    if (!std::isfinite(rel)) { set_error("LU-IR: non-finite residual"); return MPDOK_ERR_NONFINITE; }
    if (rel < tol) { conv = true; break; }
    launch(k_f64_to_f32, grid_for(n), 256, 0, s, (const double*)ws.r64, v32, n);
    MPDOK_TRY(lu_apply_any(factors, n, fdtype, v32, z32, awork, s, nullptr));
    launch(k_add_f32_to_f64, grid_for(n), 256, 0, s, (const float*)z32, x, n, 0);
    if (info) info->outer_iters = it + 1;
  }
  if (!conv) {
    MPDOK_TRY(gemv_launch(MPDOK_F64, false, A, lda, n, n, x, n, 1, ws.r64, n, -1.0, 1.0, b, n, &ws.sc->nrm2, ws.gw,
                          ws.gbytes, s, true, nullptr));
    MPDOK_TRY(read_scal(ws, &hs, s));
    const double rel = std::sqrt(hs.nrm2) / bnorm;
    if (info && info->n_history < MPDOK_HISTORY_MAX) {
      info->hist_iter[info->n_history] = maxiter_outer;
      info->history[info->n_history++] = rel;
    }
    if (info) info->relres = rel;
    conv = rel < tol;
  }
  if (info) { info->converged = conv ? 1 : 0; info->inner_iters = it + 1; }
  MPDOK_LAUNCH_CHECK("lu_ir");
  return MPDOK_OK;
}

// ---------------------------------------------------- multi-RHS LU-IR
struct MultiWork {
  size_t off_y = 0, off_z = 0, off_v = 0, off_tk = 0, off_err = 0, off_r = 0, off_nrm = 0,
         off_g = 0, total = 0;
};

static MultiWork multi_layout(long long n, int K) {
  MultiWork m;
  size_t off = 0;
  auto take = [&](size_t b) { size_t o = off; off = align_up(off + b, 256); return o; };
  const size_t nv = (size_t)std::max(1LL, n) * K;
  m.off_y = take(nv * sizeof(float));
  m.off_z = take(nv * sizeof(float));
  m.off_v = take(nv * sizeof(float));
  m.off_tk = take(4 * sizeof(int));
  m.off_err = take(16);
  m.off_r = take(nv * sizeof(double));
  m.off_nrm = take((size_t)K * sizeof(double));
  m.off_g = take(gemv_workspace_bytes(MPDOK_F64, n, n, K, false));
  m.total = off;
  return m;
}

template <typename F, int K>
static int lu_apply_multi_t(const void* fbuf, long long n, int fdtype, const float* v, float* z, void* work,
                            cudaStream_t s) {
  const LULayout L = lu_layout(n, fdtype);
  const MultiWork mw = multi_layout(n, K);
  const char* fb = (const char*)fbuf;
  char* wb = (char*)work;
  const F* LU = (const F*)(fb + L.off_lu);
  const float* Linv = (const float*)(fb + L.off_linv);
  const float* Uinv = (const float*)(fb + L.off_uinv);
  const float* d = (const float*)(fb + L.off_d);
  const float* Ml = (const float*)(fb + L.off_ml);
  const float* Mu = (const float*)(fb + L.off_mu);
  float* y = (float*)(wb + mw.off_y);
  float* zz = (float*)(wb + mw.off_z);
  int* tk = (int*)(wb + mw.off_tk);
  int* err = (int*)(wb + mw.off_err);
  MPDOK_CUDA_TRY(cudaMemsetAsync(y, 0xff, sizeof(float) * n * K, s));
  MPDOK_CUDA_TRY(cudaMemsetAsync(zz, 0xff, sizeof(float) * n * K, s));
  MPDOK_TRY(reset_tickets(tk, s));
  const size_t smem = (size_t)LNB * LNB * sizeof(float);
  MPDOK_TRY(set_smem(k_trsv_multi<F, true, K>, smem));
  MPDOK_TRY(set_smem(k_trsv_multi<F, false, K>, smem));
  const int slot = prof_start(MPDOK_PROF_TRSV, s);
  const float* dr = (const float*)(fb + L.off_dr);
  const int* perm = (const int*)(fb + L.off_perm);
  launch(k_trsv_multi<F, true, K>, L.nblk, 256, smem, s, LU, L.ldf, Linv, Ml, n, L.nblk, v, n, dr, perm, y, tk, err);
  launch(k_trsv_multi<F, false, K>, L.nblk, 256, smem, s, LU, L.ldf, Uinv, Mu, n, L.nblk, (const float*)y, n, d,
         perm, zz, tk + 1, err);
  launch(k_scale_out_multi, grid_for(n * K), 256, 0, s, (const float*)zz, d, z, n, n, K);
  prof_stop(slot, s, (double)n * (double)n * sizeof(F));
  MPDOK_LAUNCH_CHECK("lu apply multi");
  return MPDOK_OK;
}

template <typename F>
static int lu_apply_multi_f(const void* fbuf, long long n, int fdtype, int K, const float* v, float* z, void* work,
                            cudaStream_t s) {
  switch (K) {
    case 1: return lu_apply_multi_t<F, 1>(fbuf, n, fdtype, v, z, work, s);
    case 2: return lu_apply_multi_t<F, 2>(fbuf, n, fdtype, v, z, work, s);
    case 3: return lu_apply_multi_t<F, 3>(fbuf, n, fdtype, v, z, work, s);
    case 4: return lu_apply_multi_t<F, 4>(fbuf, n, fdtype, v, z, work, s);
    case 5: return lu_apply_multi_t<F, 5>(fbuf, n, fdtype, v, z, work, s);
    case 6: return lu_apply_multi_t<F, 6>(fbuf, n, fdtype, v, z, work, s);
    case 7: return lu_apply_multi_t<F, 7>(fbuf, n, fdtype, v, z, work, s);
    default: return lu_apply_multi_t<F, 8>(fbuf, n, fdtype, v, z, work, s);
  }
}

static int lu_apply_multi(const void* fbuf, long long n, int fdtype, int K, const float* v, float* z, void* work,
                          cudaStream_t s) {
  switch (fdtype) {
    case MPDOK_BF16: return lu_apply_multi_f<__nv_bfloat16>(fbuf, n, fdtype, K, v, z, work, s);
    case MPDOK_F16: return lu_apply_multi_f<__half>(fbuf, n, fdtype, K, v, z, work, s);
    default: return lu_apply_multi_f<float>(fbuf, n, fdtype, K, v, z, work, s);
  }
}

__global__ void k_f64_to_f32_cols(const double* __restrict__ a, long long lda, float* __restrict__ b, long long n,
                                  int K) {
  const long long total = n * K;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
    const long long i = e % n, k = e / n;
    b[e] = (float)a[k * lda + i];
  }
}

__global__ void k_add_f32_cols(const float* __restrict__ e32, double* __restrict__ x, long long ldx, long long n, int K,
                               int assign) {
  const long long total = n * K;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
    const long long i = e % n, k = e / n;
    x[k * ldx + i] = assign ? (double)e32[e] : x[k * ldx + i] + (double)e32[e];
  }
}

extern "C" size_t mpdok_lu_ir_multi_work_size(long long n, int nrhs) {
  if (n < 0 || nrhs < 1 || nrhs > 8) return 0;
  return multi_layout(n, nrhs).total + 256;
}

// LU-IR on nrhs <= 8 right-hand sides together: X = LU^-1 B, then until every
// column meets tol: R = B - A X (one FP64 multi-RHS GEMV), X += LU^-1 R (one
// multi-RHS triangular sweep pair).  The per-solve form of the reference's
// LUIRSolver.solve_factored (mpdok_ops.py:280-320), batched over right-hand
// sides the way its time-series use (factor once, many fields) calls it.
extern "C" int mpdok_lu_ir_solve_multi(const double* A, long long lda, long long n, const void* factors, int fdtype,
                                       int nrhs, const double* B, long long ldb, double* X, long long ldx, double tol,
                                       int maxiter_outer, void* work, size_t work_bytes, mpdok_solve_info* info,
                                       cudaStream_t s) {
  if (info) std::memset(info, 0, sizeof(*info));
  MPDOK_ARG_CHECK(n >= 0 && nrhs >= 1 && nrhs <= 8, "n >= 0 and nrhs in [1, 8]");
  if (n == 0) { if (info) info->converged = 1; return MPDOK_OK; }
  MPDOK_ARG_CHECK(A && factors && B && X && work, "null pointer");
  MPDOK_ARG_CHECK(lda >= n && ldb >= n && ldx >= n, "leading dimensions must be >= n");
  MPDOK_ARG_CHECK(work_bytes >= mpdok_lu_ir_multi_work_size(n, nrhs), "multi-RHS LU-IR work buffer too small");
  LUMeta hm;
  MPDOK_TRY(read_meta(factors, n, fdtype, &hm, s));
  if (!hm.valid || hm.fdtype != fdtype || hm.n_lo != (int)(n & 0x7fffffff)) {
    set_error("no factorization of this size / type in the factor buffer");
    return MPDOK_ERR_NOT_FACTORED;
  }
  const MultiWork mw = multi_layout(n, nrhs);
  char* wb = (char*)work;
  int* merr = (int*)(wb + mw.off_err);
  MPDOK_TRY(err_clear(merr, s));
  auto body = [&]() -> int {
  float* v32 = (float*)(wb + mw.off_v);  // FP32 right-hand sides in, corrections out (in place)
  double* R = (double*)(wb + mw.off_r);
  double* nrm = (double*)(wb + mw.off_nrm);
  void* gw = wb + mw.off_g;
  const size_t gbytes = gemv_workspace_bytes(MPDOK_F64, n, n, nrhs, false);
  float* zout = v32;  // the sweeps run through the y / z buffers of the workspace; the scaled result lands in v32
  std::vector<double> bn(nrhs), rn(nrhs);
  MPDOK_TRY(colnorms_f64(B, n, nrhs, ldb, nrm, s));
  MPDOK_CUDA_TRY(cudaMemcpyAsync(bn.data(), nrm, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, s));
  MPDOK_CUDA_TRY(cudaStreamSynchronize(s));
  for (int k = 0; k < nrhs; ++k) {
    bn[k] = std::sqrt(bn[k]);
    if (!std::isfinite(bn[k])) {
      set_error("multi-RHS LU-IR: right-hand side %d has non-finite entries", k);
      return MPDOK_ERR_NONFINITE;
    }
  }
  if (info) info->bnorm = *std::max_element(bn.begin(), bn.end());
  const unsigned g = grid_for(n * nrhs);
  launch(k_f64_to_f32_cols, g, 256, 0, s, B, ldb, v32, n, nrhs);
  MPDOK_TRY(lu_apply_multi(factors, n, fdtype, nrhs, v32, zout, wb, s));
  launch(k_add_f32_cols, g, 256, 0, s, (const float*)zout, X, ldx, n, nrhs, 1);
  bool conv = false;
  int it = 0;
  double worst = 0.0;
  for (it = 0; it <= maxiter_outer; ++it) {
    MPDOK_TRY(gemv_launch(MPDOK_F64, false, A, lda, n, n, X, ldx, nrhs, R, n, -1.0, 1.0, B, ldb, nullptr, gw, gbytes,
                          s, true, nullptr));
    MPDOK_TRY(colnorms_f64(R, n, nrhs, n, nrm, s));
    MPDOK_CUDA_TRY(cudaMemcpyAsync(rn.data(), nrm, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, s));
    MPDOK_CUDA_TRY(cudaStreamSynchronize(s));
    worst = 0.0;
    for (int k = 0; k < nrhs; ++k) {
      const double rel = bn[k] > 0.0 ? std::sqrt(rn[k]) / bn[k] : std::sqrt(rn[k]);
      if (!std::isfinite(rel)) { set_error("multi-RHS LU-IR: non-finite residual"); return MPDOK_ERR_NONFINITE; }
      worst = std::max(worst, rel);
    }
    if (info && info->n_history < MPDOK_HISTORY_MAX) {
      info->hist_iter[info->n_history] = it;
      info->history[info->n_history++] = worst;
    }
    if (worst < tol) { conv = true; break; }
    if (it == maxiter_outer) break;
    launch(k_f64_to_f32_cols, g, 256, 0, s, (const double*)R, n, v32, n, nrhs);
    MPDOK_TRY(lu_apply_multi(factors, n, fdtype, nrhs, v32, zout, wb, s));
    launch(k_add_f32_cols, g, 256, 0, s, (const float*)zout, X, ldx, n, nrhs, 0);
    if (info) info->outer_iters = it + 1;
  }
  if (info) {
    info->relres = worst;
    info->converged = conv ? 1 : 0;
    info->inner_iters = it + 1;
  }
  MPDOK_LAUNCH_CHECK("lu_ir multi");
  return MPDOK_OK;
  };
  return err_finish(merr, body(), s);
}

// Leading dimension of the preconditioned directions Z kept by the LU-GMRES-IR.
static long long zcols_ld(long long n) { return (std::max(1LL, n) + 63) / 64 * 64; }

extern "C" size_t mpdok_lu_gmres_ir_work_size(long long n, int restart) {
  if (n < 0 || restart < 1) return 0;
  return align_up(apply_layout(n).total, 256) + align_up((size_t)std::max(1LL, n) * sizeof(float), 256) +
         align_up(krylov_layout(n, restart, nullptr).total, 256) + align_up((size_t)std::max(1LL, n) * 8, 256) +
         align_up((size_t)restart * zcols_ld(n) * sizeof(float), 256) + 256;
}

extern "C" int mpdok_lu_gmres_ir(const double* A64, long long lda, const float* A32, long long lda32, long long n,
                                 const void* factors, int fdtype, const double* b, double* x, double tol,
                                 int maxiter_outer, int restart, double inner_tol, void* work, size_t work_bytes,
                                 mpdok_solve_info* info, cudaStream_t s) {
  if (info) std::memset(info, 0, sizeof(*info));
  MPDOK_ARG_CHECK(n >= 0, "negative n");
  MPDOK_ARG_CHECK(restart >= 1 && restart <= 1024, "restart must be in [1, 1024]");
  if (n == 0) { if (info) info->converged = 1; return MPDOK_OK; }
  MPDOK_ARG_CHECK(A64 && A32 && factors && b && x && work, "null pointer");
  MPDOK_ARG_CHECK(work_bytes >= mpdok_lu_gmres_ir_work_size(n, restart), "work buffer too small");
  LUMeta hm;
  MPDOK_TRY(read_meta(factors, n, fdtype, &hm, s));
  if (!hm.valid || hm.fdtype != fdtype || hm.n_lo != (int)(n & 0x7fffffff)) {
    set_error("no factorization of this size / type in the factor buffer");
    return MPDOK_ERR_NOT_FACTORED;
  }
  char* wb = (char*)work;
  const size_t a_bytes = align_up(apply_layout(n).total, 256);
  int* aerr = (int*)(wb + apply_layout(n).off_err);
  MPDOK_TRY(err_clear(aerr, s));
  PcCtx ctx{factors, n, fdtype, wb};
  Precond pc;
  pc.apply = pc_apply;
  pc.ctx = &ctx;
  pc.z = (float*)(wb + a_bytes);
  KWs ws = krylov_layout(n, restart, wb + a_bytes + align_up((size_t)n * sizeof(float), 256));
  MPDOK_CUDA_TRY(cudaMemsetAsync(ws.tickets, 0, sizeof(unsigned) * 8, s));
  MPDOK_CUDA_TRY(cudaMemsetAsync(ws.sc, 0, sizeof(KScal), s));
  StoredCtx c;
  c.A32 = A32;
  c.lda32 = lda32;
  c.A64 = A64;
  c.lda64 = lda;
  c.n = n;
  c.gw = ws.gw;
  c.gbytes = ws.gbytes;
  // the mixed solve is guarded: on a singular or badly scaled system it returns
  // the best iterate with info->stagnated = 2 instead of diverging
  double* xbest = (double*)(wb + a_bytes + align_up((size_t)n * sizeof(float), 256) + align_up(ws.total, 256));
  // z_k = M^-1 v_k of every Arnoldi step: the cycle's update needs no extra
  // application of the triangular solves
  pc.Z = (float*)((char*)xbest + align_up((size_t)n * 8, 256));
  pc.ldz = zcols_ld(n);
  return err_finish(aerr, gmres_ir_core(ws, stored_op32(&c), stored_res64(&c), b, x, tol, maxiter_outer, restart,
                                        inner_tol, &pc, info, s, xbest), s);
}

// --------------------------------------------------- LU-preconditioned CG-IR
// CG-IR whose inner CG is preconditioned by the BF16/FP16 factors (PCG, z =
// (LU)^-1 r per column): the FP32 CG body then works on a well-conditioned
// operator, which it needs once kappa(A) * 6e-8 >= 1 (the C2 family).
// op_mode 0: FP32 copy of A + native FP64 residual; 1: split A for both;
// 2: matrix-free (coords) FP32 inside, FP64 matrix-free residual.
extern "C" size_t mpdok_lu_cg_ir_workspace_size(long long n, int nrhs, int op_mode) {
  if (n < 0 || nrhs < 1 || nrhs > 8 || op_mode < 0 || op_mode > 2) return 0;
  size_t g;
  if (op_mode == 0)
    g = std::max(gemv_workspace_bytes(MPDOK_F32, n, n, nrhs, false), gemv_workspace_bytes(MPDOK_F64, n, n, nrhs, false));
  else if (op_mode == 1)
    g = split_gemv_work_bytes(n, n, nrhs);
  else
    g = align_up(matfree_work_bytes(n, n, nrhs, MPDOK_F32), 256) + matfree_work_bytes(n, n, nrhs, MPDOK_F64);
  return align_up(apply_layout(n).total, 256) + align_up(cgir_layout(n, nrhs, nullptr).total, 256) + align_up(g, 256) +
         256;
}

static int lu_cg_ir_run(const Operator32& A, const Residual64& R, long long n, const void* factors, int fdtype, int nrhs,
                        const double* B, long long ldb, double* X, long long ldx, double tol, int maxiter_outer,
                        double inner_tol, int inner_maxiter, char* awork, const CgIrWs& w, mpdok_solve_info* info,
                        cudaStream_t s) {
  LUMeta hm;
  MPDOK_TRY(read_meta(factors, n, fdtype, &hm, s));
  if (!hm.valid || hm.fdtype != fdtype || hm.n_lo != (int)(n & 0x7fffffff)) {
    set_error("no factorization of this size / type in the factor buffer");
    return MPDOK_ERR_NOT_FACTORED;
  }
  PcCtx ctx{factors, n, fdtype, awork};
  Precond pc;
  pc.apply = pc_apply;
  pc.ctx = &ctx;
  int* aerr = (int*)(awork + apply_layout(n).off_err);
  MPDOK_TRY(err_clear(aerr, s));
  return err_finish(aerr, cg_ir_core(w, A, R, B, ldb, X, ldx, tol, maxiter_outer, inner_tol, inner_maxiter, &pc, info, s),
                    s);
}

extern "C" int mpdok_lu_cg_ir(const double* A64, long long lda, long long n, int op_mode, void* opbuf, int op_ready,
                              const void* factors, int fdtype, int nrhs, const double* B, long long ldb, double* X,
                              long long ldx, double tol, int maxiter_outer, double inner_tol, int inner_maxiter,
                              void* work, size_t work_bytes, mpdok_solve_info* info, cudaStream_t s) {
  if (info) std::memset(info, 0, sizeof(*info));
  MPDOK_ARG_CHECK(n >= 0, "negative n");
  MPDOK_ARG_CHECK(op_mode == 0 || op_mode == 1, "op_mode must be 0 (FP32 copy) or 1 (split)");
  MPDOK_ARG_CHECK(nrhs >= 1 && nrhs <= 8, "nrhs must be in 1..8");
  if (n == 0) { if (info) info->converged = 1; return MPDOK_OK; }
  MPDOK_ARG_CHECK(A64 && opbuf && factors && B && X && work, "null pointer");
  MPDOK_ARG_CHECK(work_bytes >= mpdok_lu_cg_ir_workspace_size(n, nrhs, op_mode), "workspace too small");
  char* wb = (char*)work;
  char* awork = wb;
  const size_t a_bytes = align_up(apply_layout(n).total, 256);
  CgIrWs w = cgir_layout(n, nrhs, wb + a_bytes);
  char* gw = wb + a_bytes + align_up(w.total, 256);
  const size_t gbytes = work_bytes - a_bytes - align_up(w.total, 256);
  const long long ld = (long long)align_up((size_t)n, 4);
  if (op_mode == 0) {
    float* A32 = (float*)opbuf;
    if (!op_ready) MPDOK_TRY(convert_matrix_f64_f32(A64, lda, A32, ld, n, n, s));
    StoredCtx c;
    c.A32 = A32;
    c.lda32 = ld;
    c.A64 = A64;
    c.lda64 = lda;
    c.n = n;
    c.gw = gw;
    c.gbytes = gbytes;
    return lu_cg_ir_run(stored_op32(&c), stored_res64(&c), n, factors, fdtype, nrhs, B, ldb, X, ldx, tol,
                        maxiter_outer, inner_tol, inner_maxiter, awork, w, info, s);
  }
  float* hi = (float*)opbuf;
  float* lo = (float*)((char*)opbuf + align_up((size_t)ld * n * sizeof(float), 256));
  if (!op_ready) MPDOK_TRY(split_matrix(A64, lda, n, n, hi, lo, ld, s));
  SplitCtx c;
  c.hi = hi;
  c.lo = lo;
  c.ld = ld;
  c.n = n;
  c.work = gw;
  c.work_bytes = gbytes;
  return lu_cg_ir_run(split_op32(&c), split_res64(&c), n, factors, fdtype, nrhs, B, ldb, X, ldx, tol, maxiter_outer,
                      inner_tol, inner_maxiter, awork, w, info, s);
}

extern "C" int mpdok_mf_lu_cg_ir(const double* coords, long long n, int dim, int kernel, double gamma, double reg,
                                 const void* factors, int fdtype, int nrhs, const double* B, long long ldb, double* X,
                                 long long ldx, double tol, int maxiter_outer, double inner_tol, int inner_maxiter,
                                 void* work, size_t work_bytes, mpdok_solve_info* info, cudaStream_t s) {
  if (info) std::memset(info, 0, sizeof(*info));
  MPDOK_ARG_CHECK(n >= 0, "negative n");
  MPDOK_ARG_CHECK(nrhs >= 1 && nrhs <= 8, "nrhs must be in 1..8");
  if (n == 0) { if (info) info->converged = 1; return MPDOK_OK; }
  MPDOK_ARG_CHECK(coords && factors && B && X && work, "null pointer");
  MPDOK_ARG_CHECK(work_bytes >= mpdok_lu_cg_ir_workspace_size(n, nrhs, 2), "workspace too small");
  char* wb = (char*)work;
  const size_t a_bytes = align_up(apply_layout(n).total, 256);
  CgIrWs w = cgir_layout(n, nrhs, wb + a_bytes);
  char* base = wb + a_bytes + align_up(w.total, 256);
  MfCtx c;
  c.op.rows = coords;
  c.op.cols = coords;
  c.op.nrows = n;
  c.op.ncols = n;
  c.op.dim = dim;
  c.op.kernel = kernel;
  c.op.gamma = gamma;
  c.op.reg = reg;
  c.w32 = base;
  c.w32_bytes = matfree_work_bytes(n, n, nrhs, MPDOK_F32);
  c.w64 = base + align_up(c.w32_bytes, 256);
  c.w64_bytes = matfree_work_bytes(n, n, nrhs, MPDOK_F64);
  MPDOK_TRY(mf_timeout_clear(&c, s));
  return mf_timeout_finish(&c, lu_cg_ir_run(mf_op32(&c), mf_res64(&c), n, factors, fdtype, nrhs, B, ldb, X, ldx, tol,
                                            maxiter_outer, inner_tol, inner_maxiter, wb, w, info, s), s);
}
