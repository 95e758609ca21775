// Batched solver for many RBF systems of uneven size, each with several
// right-hand sides, plus the adjoint contraction for gradients.
//
// Not in the reference (its solvers take one system per call); this serves
// the batched-and-differentiated workload: S Gaussian or multiquadric systems
// A_s = phi_eps(||c_i - c_j||) + reg_s I, N_s from hundreds to thousands,
// k <= 8 right-hand sides each.
//
// Design:
//  * The systems are SPD with kappa up to ~1e11, far beyond what a 16- or
//    32-bit factorization can precondition, so the factorization is a
//    Cholesky with FP64-accurate updates.  GB300 runs FP64 at 2 DFMA per
//    clock per SM (1/64 of FP32), so the O(N^3) trailing update can run in
//    double-float arithmetic on the FP32 pipe (hi/lo FP32 pairs, error-free
//    products by FMA, two-sum accumulation, about 2^-48 relative) or in
//    native FP64; the diagonal blocks, the panel solves, the triangular solves
//    and the refinement residual stay in FP64.
//  * Systems are sorted by N, largest first, so the systems still active at
//    block level k are a prefix of the sorted order.  Each level is three
//    launches over ALL active systems: the 64x64 diagonal-block factor
//    (one CTA per system), the panel solve (one task per (system, row tile))
//    and the trailing update (one task per (system, lower tile), run by a
//    persistent grid that strides over the task list).  Task lists are
//    prefix sums per level, decoded on the device.
//  * Nothing in factor / solve / refine synchronises with the host, so the
//    whole sequence is captured once into a CUDA graph and replayed with a
//    single graph launch.
//  * Storage of A_s: the lower triangle with the diagonal, which becomes the
//    factor, holds double-float pairs (hi, lo FP32 in the 8-byte slot), so the
//    trailing update reads and writes it on the FP32 pipe without a single
//    FP64 conversion; the strict upper triangle keeps A in FP64, and the FP64
//    refinement residual is a symmetric product from it and the known
//    diagonal phi(0) + reg.
//  * The adjoint contraction recomputes phi and its derivatives from the
//    coordinates (nothing of size N^2 is stored for the gradient).
#include "krylov.cuh"

#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

namespace mpdok {

constexpr int BNB = 64;          // block size of the level schedule
constexpr int BT = 256;          // threads of the tile kernels
constexpr int BPAD = BNB + 1;    // padded smem row
constexpr int BMAX_RHS = 8;

struct BSys {
  long long offA;   // A_s in the plan's arena, column-major, lda = n
  long long offX;   // B / X in the caller's packing: n x nrhs column-major, ld = n
  long long offC;   // coordinates in the caller's packing: n x dim row-major
  long long offL;   // diagonal-block inverses: nblk x 64 x 64 column-major
  long long offR;   // per-row scratch (n doubles)
  int n, nblk, user, pad;
  double eps, gamma, reg;
};

struct BatchPlan {
  int nsys = 0, dim = 2, nrhs = 1, kernel = 0, arith = 1, grid_mult = 2, maxblk = 0;
  std::vector<BSys> sys;              // sorted by n, descending
  std::vector<int> act;               // systems with nblk > k, per level
  std::vector<long long> preT, preS;  // per level: prefix sums (act[k] + 1 entries each)
  std::vector<long long> preT_off, preS_off;
  std::vector<long long> preRow;      // prefix of nblk over all systems (row-tile tasks)
  long long total_x = 0, total_c = 0;
  BSys* d_sys = nullptr;
  long long* d_pre = nullptr;         // preT | preS | preRow
  long long d_preS_base = 0, d_preRow_base = 0;
  double* arena = nullptr;            // A | Linv | V | R | rowscratch
  double *A = nullptr, *Linv = nullptr, *V = nullptr, *R = nullptr, *rows = nullptr, *coords = nullptr;
  int* d_pert = nullptr;
  size_t bytes = 0;
  int syrk_grid = 0;
  cudaStream_t cap = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  size_t graph_nodes = 0;
  // schedule of the captured step: 0 level-synchronous launches, 1 one
  // persistent task-graph launch (dag_ctas_per_sm CTAs per SM)
  int schedule = 0, dag_ctas_per_sm = 3;
  int dag_refine = -1, dag_nsec = 0;
  long long dag_total = 0, dag_st_off = 0, dag_v_off = 0, dag_v_total = 0;
  size_t dag_n_neg = 0, dag_n_zero = 0, dag_head_idx = 0;
  long long* d_dagpre = nullptr;
  void* d_secs = nullptr;
  int* d_dagstate = nullptr;
};

// ------------------------------------------------------------------ helpers

// Locate the system of flat task t in a prefix array pre[0..cnt] (pre[0] = 0).
__device__ __forceinline__ int task_system(const long long* pre, int cnt, long long t) {
  int lo = 0, hi = cnt - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (pre[mid] <= t) lo = mid; else hi = mid - 1;
  }
  return lo;
}

struct DF {  // double-float: value = h + l
  float h, l;
};

__device__ __forceinline__ DF to_df(double v) {
  DF r;
  r.h = __double2float_rn(v);
  r.l = __double2float_rn(v - (double)r.h);
  return r;
}

// Lower-triangle slots hold double-float pairs.
__device__ __forceinline__ DF ld_df(const double* p) {
  const float2 f = *reinterpret_cast<const float2*>(p);
  DF r;
  r.h = f.x;
  r.l = f.y;
  return r;
}
__device__ __forceinline__ void st_df(double* p, DF v) {
  *reinterpret_cast<float2*>(p) = make_float2(v.h, v.l);
}
__device__ __forceinline__ double df_to_f64(DF v) { return (double)v.h + (double)v.l; }
// (a - b) in double-float with renormalisation (two-sum based).
__device__ __forceinline__ DF df_sub(DF a, float bh, float bl) {
  const float s = a.h - bh;
  const float bb = s - a.h;
  float e = (a.h - (s - bb)) + (-bh - bb);
  e += a.l - bl;
  DF r;
  r.h = s + e;
  r.l = e - (r.h - s);
  return r;
}

// phi(r2) and its partial derivatives: g = dphi/d(r2), h = dphi/dgamma.
template <int KIND>
__device__ __forceinline__ void phi_derivs(double r2, double gamma, double& phi, double& g, double& h) {
  if (KIND == MPDOK_KERNEL_GAUSSIAN) {
    phi = exp(-gamma * r2);
    g = -gamma * phi;
    h = -r2 * phi;
  } else {
    phi = sqrt(fma(gamma, r2, 1.0));
    const double ip = 0.5 / phi;
    g = gamma * ip;
    h = r2 * ip;
  }
}

template <int KIND>
__device__ __forceinline__ double phi_only(double r2, double gamma) {
  return KIND == MPDOK_KERNEL_GAUSSIAN ? exp(-gamma * r2) : sqrt(fma(gamma, r2, 1.0));
}

// ------------------------------------------------------------------ assembly
// One task per (system, 64x64 tile) of the full matrix (both triangles).
template <int KIND, int D>
__global__ void __launch_bounds__(BT) k_bassemble(const BSys* __restrict__ sys, const long long* __restrict__ pre,
                                                  int nsys, const double* __restrict__ coords,
                                                  double* __restrict__ A) {
  __shared__ double sR[BNB * D], sC[BNB * D];
  const long long t = blockIdx.x;
  const int s = task_system(pre, nsys + 1, t);
  const BSys q = sys[s];
  const long long u = t - pre[s];
  const int ti = (int)(u % q.nblk), tj = (int)(u / q.nblk);
  const int r0 = ti * BNB, c0 = tj * BNB;
  const double* X = coords + q.offC;
  for (int e = threadIdx.x; e < BNB * D; e += BT) {
    const int i = e / D, d = e % D;
    sR[e] = (r0 + i < q.n) ? X[(long long)(r0 + i) * D + d] : 0.0;
    sC[e] = (c0 + i < q.n) ? X[(long long)(c0 + i) * D + d] : 0.0;
  }
  __syncthreads();
  double* Ab = A + q.offA;
  const int row = threadIdx.x & 63;
  for (int col = threadIdx.x >> 6; col < BNB; col += BT / BNB) {
    const int i = r0 + row, j = c0 + col;
    if (i >= q.n || j >= q.n) continue;
    double r2 = 0.0;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const double df = sR[row * D + d] - sC[col * D + d];
      r2 = fma(df, df, r2);
    }
    double v = phi_only<KIND>(r2, q.gamma);
    if (i == j) v += q.reg;
    double* slot = Ab + (long long)i + (long long)j * q.n;
    if (i >= j) st_df(slot, to_df(v));
    else *slot = v;
  }
}

// ------------------------------------------------------------------ level k: diagonal block
// Cholesky of the 64x64 diagonal block (FP64, in shared memory), its inverse,
// L11 written over the lower triangle, Linv kept for the panel and the solves.
__global__ void __launch_bounds__(BT) k_bpotrf(const BSys* __restrict__ sys, int k, double* __restrict__ A,
                                                double* __restrict__ Linv, int* __restrict__ pert) {
  extern __shared__ double smem[];
  double* sL = smem;                 // BNB x BPAD, sL[i * BPAD + j] = L(i, j)
  double* sI = smem + BNB * BPAD;    // inverse, same layout
  __shared__ double s_inv;
  const BSys q = sys[blockIdx.x];
  const int kb = k * BNB;
  const int nb = min(BNB, q.n - kb);
  double* Ab = A + q.offA;
  const long long lda = q.n;
  for (int e = threadIdx.x; e < BNB * BNB; e += BT) {
    const int i = e & 63, j = e >> 6;
    double v = 0.0;
    if (i < nb && j < nb && i >= j) v = df_to_f64(ld_df(Ab + (long long)(kb + i) + (long long)(kb + j) * lda));
    sL[i * BPAD + j] = v;
    sI[i * BPAD + j] = 0.0;
  }
  __syncthreads();
  const double dref = 1.0 + q.reg;  // phi(0) + reg: the diagonal of A
  for (int j = 0; j < nb; ++j) {
    if (threadIdx.x == 0) {
      double d = sL[j * BPAD + j];
      if (!(d > 1e-15 * dref)) {  // not positive in FP64: perturb and count
        d = 1e-15 * dref;
        atomicAdd(pert, 1);
      }
      const double p = sqrt(d);
      sL[j * BPAD + j] = p;
      s_inv = 1.0 / p;
    }
    __syncthreads();
    const double ip = s_inv;
    for (int i = j + 1 + threadIdx.x; i < nb; i += BT) sL[i * BPAD + j] *= ip;
    __syncthreads();
    const int m = nb - j - 1;
    for (int e = threadIdx.x; e < m * m; e += BT) {
      const int i = j + 1 + e / m, l = j + 1 + e % m;
      if (l <= i) sL[i * BPAD + l] -= sL[i * BPAD + j] * sL[l * BPAD + j];
    }
    __syncthreads();
  }
  // inverse of the lower-triangular L11, row by row: Linv(i, c) for c <= i
  for (int i = 0; i < nb; ++i) {
    const int c = threadIdx.x;
    if (c <= i && c < BNB) {
      double acc = (c == i) ? 1.0 : 0.0;
      for (int l = c; l < i; ++l) acc -= sL[i * BPAD + l] * sI[l * BPAD + c];
      sI[i * BPAD + c] = acc / sL[i * BPAD + i];
    }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < BNB * BNB; e += BT) {
    const int i = e & 63, j = e >> 6;
    if (i < nb && j < nb && i >= j) st_df(Ab + (long long)(kb + i) + (long long)(kb + j) * lda, to_df(sL[i * BPAD + j]));
    Linv[q.offL + (long long)k * BNB * BNB + i + (long long)j * BNB] = sI[i * BPAD + j];
  }
}

// ------------------------------------------------------------------ tile GEMM core
// acc(4x4 per thread) = sum_kk sA[kk][row] * sB[kk][col], 64x64 tile, FP64.
__device__ __forceinline__ void tile_fma_f64(const double* sA, const double* sB, double (&acc)[4][4], int ty,
                                             int tx) {
#pragma unroll 4
  for (int kk = 0; kk < BNB; ++kk) {
    double a[4], b[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) a[i] = sA[kk * BPAD + ty * 4 + i];
#pragma unroll
    for (int j = 0; j < 4; ++j) b[j] = sB[kk * BPAD + tx * 4 + j];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
  }
}

// Double-float version: products error-free by FMA, sums by two-sum into (s, c).
__device__ __forceinline__ void tile_fma_df(const DF* sA, const DF* sB, float (&s)[4][4], float (&c)[4][4], int ty,
                                            int tx) {
#pragma unroll 2
  for (int kk = 0; kk < BNB; ++kk) {
    DF a[4], b[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) a[i] = sA[kk * BPAD + ty * 4 + i];
#pragma unroll
    for (int j = 0; j < 4; ++j) b[j] = sB[kk * BPAD + tx * 4 + j];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const float ph = a[i].h * b[j].h;
        float pl = fmaf(a[i].h, b[j].h, -ph);
        pl = fmaf(a[i].h, b[j].l, pl);
        pl = fmaf(a[i].l, b[j].h, pl);
        const float t = s[i][j] + ph;
        const float bp = t - s[i][j];
        const float err = (s[i][j] - (t - bp)) + (ph - bp);
        s[i][j] = t;
        c[i][j] += err + pl;
      }
  }
}

// Stage a (rows x 64) block of the lower triangle (double-float slots) into
// sT[kk][row], as FP64 or as double-float (rows beyond `nr` and columns
// beyond `nc` are zero).
template <typename T>
__device__ __forceinline__ void stage_block(T* sT, const double* __restrict__ src, long long ld, int nr, int nc) {
  for (int e = threadIdx.x; e < BNB * BNB; e += BT) {
    const int r = e & 63, kk = e >> 6;
    DF v;
    v.h = 0.f;
    v.l = 0.f;
    if (r < nr && kk < nc) v = ld_df(src + (long long)r + (long long)kk * ld);
    if constexpr (std::is_same<T, double>::value) sT[kk * BPAD + r] = df_to_f64(v);
    else sT[kk * BPAD + r] = v;
  }
}

// ------------------------------------------------------------------ level k: panel solve
// L21 = A21 * Linv11^T for every row tile below the diagonal block (FP64).
__global__ void __launch_bounds__(BT) k_btrsm(const BSys* __restrict__ sys, const long long* __restrict__ pre,
                                               int cnt, int k, double* __restrict__ A,
                                               const double* __restrict__ Linv) {
  extern __shared__ double smem[];
  double* sA = smem;
  double* sB = smem + BNB * BPAD;
  const long long t = blockIdx.x;
  const int s = task_system(pre, cnt + 1, t);
  const BSys q = sys[s];
  const int r = k + 1 + (int)(t - pre[s]);
  const int kb = k * BNB, r0 = r * BNB;
  const int nb = min(BNB, q.n - kb), nr = min(BNB, q.n - r0);
  double* Ab = A + q.offA;
  const long long lda = q.n;
  stage_block(sA, Ab + r0 + (long long)kb * lda, lda, nr, nb);
  // sB[kk][col] = Linv(col, kk)
  const double* Li = Linv + q.offL + (long long)k * BNB * BNB;
  for (int e = threadIdx.x; e < BNB * BNB; e += BT) {
    const int col = e & 63, kk = e >> 6;
    sB[kk * BPAD + col] = Li[col + kk * BNB];
  }
  __syncthreads();
  double acc[4][4] = {};
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  tile_fma_f64(sA, sB, acc, ty, tx);
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int row = ty * 4 + i, col = tx * 4 + j;
      if (row < nr && col < nb) st_df(Ab + (long long)(r0 + row) + (long long)(kb + col) * lda, to_df(acc[i][j]));
    }
}

// ------------------------------------------------------------------ level k: trailing update
// A[ti, tj] -= L[ti, k] L[tj, k]^T over the lower tiles of the trailing matrix
// (diagonal tiles: lower triangle only, so A's upper triangle stays intact).
// Persistent grid striding over the level's task list.
template <int ARITH>  // 0 = FP64, 1 = double-float on the FP32 pipe
__global__ void __launch_bounds__(BT) k_bsyrk(const BSys* __restrict__ sys, const long long* __restrict__ pre,
                                               int cnt, int k, double* __restrict__ A) {
  extern __shared__ double smem[];
  using ST = typename std::conditional<ARITH == 0, double, DF>::type;
  ST* sA = reinterpret_cast<ST*>(smem);
  ST* sB = sA + BNB * BPAD;
  const long long total = pre[cnt];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  for (long long t = blockIdx.x; t < total; t += gridDim.x) {
    const int s = task_system(pre, cnt + 1, t);
    const BSys q = sys[s];
    const long long u = t - pre[s];
    // triangular index -> (a, b) with b <= a
    int a = (int)((sqrt(8.0 * (double)u + 1.0) - 1.0) * 0.5);
    while ((long long)(a + 1) * (a + 2) / 2 <= u) ++a;
    while ((long long)a * (a + 1) / 2 > u) --a;
    const int b = (int)(u - (long long)a * (a + 1) / 2);
    const int ti = k + 1 + a, tj = k + 1 + b;
    const int kb = k * BNB, r0 = ti * BNB, c0 = tj * BNB;
    const int nb = min(BNB, q.n - kb), nr = min(BNB, q.n - r0), nc = min(BNB, q.n - c0);
    double* Ab = A + q.offA;
    const long long lda = q.n;
    __syncthreads();  // previous task's smem reads are done
    stage_block(sA, Ab + r0 + (long long)kb * lda, lda, nr, nb);
    stage_block(sB, Ab + c0 + (long long)kb * lda, lda, nc, nb);
    __syncthreads();
    if (ARITH == 0) {
      double acc[4][4] = {};
      tile_fma_f64(reinterpret_cast<const double*>(sA), reinterpret_cast<const double*>(sB), acc, ty, tx);
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int row = ty * 4 + i, col = tx * 4 + j;
          if (row < nr && col < nc && (ti != tj || row >= col)) {
            double* p = Ab + (long long)(r0 + row) + (long long)(c0 + col) * lda;
            st_df(p, to_df(df_to_f64(ld_df(p)) - acc[i][j]));
          }
        }
    } else {
      float sh[4][4] = {}, sl[4][4] = {};
      tile_fma_df(reinterpret_cast<const DF*>(sA), reinterpret_cast<const DF*>(sB), sh, sl, ty, tx);
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int row = ty * 4 + i, col = tx * 4 + j;
          if (row < nr && col < nc && (ti != tj || row >= col)) {
            double* p = Ab + (long long)(r0 + row) + (long long)(c0 + col) * lda;
            // renormalise the accumulator, then C - acc in double-float
            const float h = sh[i][j] + sl[i][j];
            const float l = sl[i][j] - (h - sh[i][j]);
            st_df(p, df_sub(ld_df(p), h, l));
          }
        }
    }
  }
}

// ------------------------------------------------------------------ triangular solves (FP64, nrhs <= 8)
// V_k := Linv_k V_k (forward) or Linv_k^T V_k (backward) for each active system.
template <bool TRANS>
__global__ void __launch_bounds__(BT) k_bsolve_diag(const BSys* __restrict__ sys, int k, int nrhs,
                                                    const double* __restrict__ Linv, double* __restrict__ V) {
  __shared__ double sX[BNB * BMAX_RHS];
  __shared__ double sLi[BNB * BPAD];
  const BSys q = sys[blockIdx.x];
  const int kb = k * BNB, nb = min(BNB, q.n - kb);
  double* Vb = V + q.offX;
  const double* Li = Linv + q.offL + (long long)k * BNB * BNB;
  for (int e = threadIdx.x; e < BNB * nrhs; e += BT) {
    const int i = e % BNB, r = e / BNB;
    sX[e] = (i < nb) ? Vb[(long long)(kb + i) + (long long)r * q.n] : 0.0;
  }
  for (int e = threadIdx.x; e < BNB * BNB; e += BT) {
    const int i = e & 63, j = e >> 6;
    sLi[i * BPAD + j] = Li[i + j * BNB];  // sLi[i][j] = Linv(i, j)
  }
  __syncthreads();
  for (int e = threadIdx.x; e < BNB * nrhs; e += BT) {
    const int i = e % BNB, r = e / BNB;
    if (i >= nb) continue;
    double acc = 0.0;
    if (!TRANS) {
      for (int c = 0; c <= i; ++c) acc = fma(sLi[i * BPAD + c], sX[r * BNB + c], acc);
    } else {
      for (int c = i; c < nb; ++c) acc = fma(sLi[c * BPAD + i], sX[r * BNB + c], acc);
    }
    Vb[(long long)(kb + i) + (long long)r * q.n] = acc;
  }
}

// Forward: V_r -= L(r, k) V_k for r > k.  Backward: V_r -= L(k, r)^T V_k for r < k.
// The products run in double-float on the FP32 pipe (the factor is stored
// that way; V_k is split once per tile), the subtraction from V_r in FP64:
// these are correction solves inside FP64 refinement, where 2^-48 products
// are ample, and FP64 arithmetic here would run at 1/64 of the FP32 rate.
template <bool TRANS>
__global__ void __launch_bounds__(BT) k_bsolve_upd(const BSys* __restrict__ sys, const long long* __restrict__ pre,
                                                   int cnt, int k, int nrhs, const double* __restrict__ A,
                                                   double* __restrict__ V) {
  __shared__ DF sT[BNB * BPAD];   // sT[kk][row] = multiplier (row of the target, kk of V_k)
  __shared__ DF sX[BNB * BMAX_RHS];
  const long long t = blockIdx.x;
  int s, r;
  if (!TRANS) {
    s = task_system(pre, cnt + 1, t);
    r = k + 1 + (int)(t - pre[s]);
  } else {
    s = (int)(t / k);
    r = (int)(t % k);
  }
  const BSys q = sys[s];
  const int kb = k * BNB, r0 = r * BNB;
  const int nb = min(BNB, q.n - kb), nr = min(BNB, q.n - r0);
  const double* Ab = A + q.offA;
  const long long lda = q.n;
  double* Vb = V + q.offX;
  if (!TRANS) {
    stage_block(sT, Ab + r0 + (long long)kb * lda, lda, nr, nb);  // sT[kk][row] = L(r0+row, kb+kk)
  } else {
    // sT[kk][row] = L(kb+kk, r0+row): read the tile (kb rows, r0 cols) coalesced along kk
    for (int e = threadIdx.x; e < BNB * BNB; e += BT) {
      const int kk = e & 63, row = e >> 6;
      DF v;
      v.h = 0.f;
      v.l = 0.f;
      if (kk < nb && row < nr) v = ld_df(Ab + (long long)(kb + kk) + (long long)(r0 + row) * lda);
      sT[kk * BPAD + row] = v;
    }
  }
  for (int e = threadIdx.x; e < BNB * nrhs; e += BT) {
    const int i = e % BNB, rr = e / BNB;
    sX[e] = to_df((i < nb) ? Vb[(long long)(kb + i) + (long long)rr * q.n] : 0.0);
  }
  __syncthreads();
  for (int e = threadIdx.x; e < BNB * nrhs; e += BT) {
    const int row = e % BNB, rr = e / BNB;
    if (row >= nr) continue;
    float sh = 0.f, sl = 0.f;
#pragma unroll 4
    for (int kk = 0; kk < BNB; ++kk) {
      const DF a = sT[kk * BPAD + row], b = sX[rr * BNB + kk];
      const float ph = a.h * b.h;
      float pl = fmaf(a.h, b.h, -ph);
      pl = fmaf(a.h, b.l, pl);
      pl = fmaf(a.l, b.h, pl);
      const float tt = sh + ph;
      const float bp = tt - sh;
      const float er = (sh - (tt - bp)) + (ph - bp);
      sh = tt;
      sl += er + pl;
    }
    Vb[(long long)(r0 + row) + (long long)rr * q.n] -= (double)sh + (double)sl;
  }
}

// ------------------------------------------------------------------ FP64 residual R = B - A X
// One task per (system, row tile); A(i, j) read from the stored upper
// triangle (i < j direct, i > j mirrored) and the diagonal phi(0) + reg.
__global__ void __launch_bounds__(BT) k_bsymv_res(const BSys* __restrict__ sys, const long long* __restrict__ pre,
                                                  int nsys, int nrhs, const double* __restrict__ A,
                                                  const double* __restrict__ B, const double* __restrict__ X,
                                                  double* __restrict__ R) {
  __shared__ double sT[BNB * BPAD];  // sT[col][row] = A(r0+row, c0+col)
  __shared__ double sX[BNB * BMAX_RHS];
  const long long t = blockIdx.x;
  const int s = task_system(pre, nsys + 1, t);
  const BSys q = sys[s];
  const int r = (int)(t - pre[s]);
  const int r0 = r * BNB, nr = min(BNB, q.n - r0);
  const double* Ab = A + q.offA;
  const long long lda = q.n;
  const double dia = 1.0 + q.reg;
  const int row = threadIdx.x & 63, g = threadIdx.x >> 6;  // 4 RHS groups
  double acc[2] = {0.0, 0.0};
  for (int c = 0; c < q.nblk; ++c) {
    const int c0 = c * BNB, nc = min(BNB, q.n - c0);
    __syncthreads();
    for (int e = threadIdx.x; e < BNB * BNB; e += BT) {
      const int i = e & 63, j = e >> 6;  // i fast
      double v = 0.0;
      if (r < c) {
        // A(r0+i, c0+j), upper: coalesced along i
        if (i < nr && j < nc) v = Ab[(long long)(r0 + i) + (long long)(c0 + j) * lda];
        sT[j * BPAD + i] = v;
      } else if (r > c) {
        // A(r0+j, c0+i) = A(c0+i, r0+j), upper: coalesced along i
        if (i < nc && j < nr) v = Ab[(long long)(c0 + i) + (long long)(r0 + j) * lda];
        sT[i * BPAD + j] = v;
      } else {
        // diagonal tile: A(r0+i, r0+j) from the upper part of the tile
        if (i < nr && j < nr) {
          if (i < j) v = Ab[(long long)(r0 + i) + (long long)(r0 + j) * lda];
          else if (i > j) v = Ab[(long long)(r0 + j) + (long long)(r0 + i) * lda];
          else v = dia;
        }
        sT[j * BPAD + i] = v;
      }
    }
    for (int e = threadIdx.x; e < BNB * nrhs; e += BT) {
      const int i = e % BNB, rr = e / BNB;
      sX[e] = (i < nc) ? X[q.offX + (long long)(c0 + i) + (long long)rr * q.n] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int rr = g + 4 * h;
      if (rr < nrhs) {
        double a = acc[h];
#pragma unroll 8
        for (int j = 0; j < BNB; ++j) a = fma(sT[j * BPAD + row], sX[rr * BNB + j], a);
        acc[h] = a;
      }
    }
  }
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int rr = g + 4 * h;
    if (rr < nrhs && row < nr) {
      const long long o = q.offX + (long long)(r0 + row) + (long long)rr * q.n;
      R[o] = B[o] - acc[h];
    }
  }
}

// Per system: max over RHS of ||R_r|| / ||B_r|| (fixed-order reduction).
__global__ void __launch_bounds__(BT) k_brelres(const BSys* __restrict__ sys, int nrhs, const double* __restrict__ B,
                                                const double* __restrict__ R, double* __restrict__ out) {
  __shared__ double red[32];
  const BSys q = sys[blockIdx.x];
  double worst = 0.0;
  for (int rr = 0; rr < nrhs; ++rr) {
    double sb = 0.0, sr = 0.0;
    for (int i = threadIdx.x; i < q.n; i += BT) {
      const long long o = q.offX + i + (long long)rr * q.n;
      sb = fma(B[o], B[o], sb);
      sr = fma(R[o], R[o], sr);
    }
    sb = block_sum(sb, red);
    sr = block_sum(sr, red);
    const double rel = sb > 0.0 ? sqrt(sr / sb) : sqrt(sr);
    worst = fmax(worst, rel);
  }
  if (threadIdx.x == 0) out[q.user] = worst;
}

__global__ void k_badd(double* __restrict__ X, const double* __restrict__ D, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    X[i] += D[i];
}

// ------------------------------------------------------------------ adjoint contraction
// For L(X) with Lam = A^{-T} dL/dX (A symmetric), per row k of each system:
//   dL/dc_k = -sum_j w_kj * 2 (c_k - c_j) * g_kj,   w_kj = sum_r (lam_kr x_jr + x_kr lam_jr)
//   dL/deps partial_k = -2 eps sum_j u_kj * h_kj,   u_kj = sum_r lam_kr x_jr
//   dL/dreg partial_k = -sum_r lam_kr x_kr
// with g = dphi/d(r^2), h = dphi/dgamma, gamma = eps^2, phi recomputed in FP64.
// Four threads per row split the columns; their partial sums combine by
// shuffles in a fixed order.
template <int KIND, int D>
__global__ void __launch_bounds__(BT) k_badjoint(const BSys* __restrict__ sys, const long long* __restrict__ pre,
                                                 int nsys, int nrhs, const double* __restrict__ coords,
                                                 const double* __restrict__ X, const double* __restrict__ Lam,
                                                 double* __restrict__ gC, double* __restrict__ rowscr) {
  __shared__ double sC[BNB * D];
  __shared__ double sXj[BMAX_RHS * BNB], sLj[BMAX_RHS * BNB];
  const long long t = blockIdx.x;
  const int s = task_system(pre, nsys + 1, t);
  const BSys q = sys[s];
  const int r = (int)(t - pre[s]);
  const int r0 = r * BNB;
  const int lr = threadIdx.x >> 2, part = threadIdx.x & 3;
  const int k = r0 + lr;
  const bool live = k < q.n;
  const double* Cb = coords + q.offC;
  double ck[D], xk[BMAX_RHS], lk[BMAX_RHS];
#pragma unroll
  for (int d = 0; d < D; ++d) ck[d] = live ? Cb[(long long)k * D + d] : 0.0;
#pragma unroll
  for (int rr = 0; rr < BMAX_RHS; ++rr) {
    xk[rr] = (live && rr < nrhs) ? X[q.offX + k + (long long)rr * q.n] : 0.0;
    lk[rr] = (live && rr < nrhs) ? Lam[q.offX + k + (long long)rr * q.n] : 0.0;
  }
  double G[D], E = 0.0;
#pragma unroll
  for (int d = 0; d < D; ++d) G[d] = 0.0;
  for (int c = 0; c < q.nblk; ++c) {
    const int c0 = c * BNB, nc = min(BNB, q.n - c0);
    __syncthreads();
    for (int e = threadIdx.x; e < BNB * D; e += BT) sC[e] = (e / D < nc) ? Cb[(long long)c0 * D + e] : 0.0;
    for (int e = threadIdx.x; e < BNB * BMAX_RHS; e += BT) {
      const int j = e % BNB, rr = e / BNB;
      const bool ok = j < nc && rr < nrhs;
      sXj[e] = ok ? X[q.offX + c0 + j + (long long)rr * q.n] : 0.0;
      sLj[e] = ok ? Lam[q.offX + c0 + j + (long long)rr * q.n] : 0.0;
    }
    __syncthreads();
    if (!live) continue;
    for (int j = part; j < nc; j += 4) {
      double df[D], r2 = 0.0;
#pragma unroll
      for (int d = 0; d < D; ++d) {
        df[d] = ck[d] - sC[j * D + d];
        r2 = fma(df[d], df[d], r2);
      }
      double phi, g, h;
      phi_derivs<KIND>(r2, q.gamma, phi, g, h);
      double u = 0.0, v = 0.0;
#pragma unroll
      for (int rr = 0; rr < BMAX_RHS; ++rr) {
        u = fma(lk[rr], sXj[rr * BNB + j], u);
        v = fma(xk[rr], sLj[rr * BNB + j], v);
      }
      const double wg = -2.0 * (u + v) * g;
#pragma unroll
      for (int d = 0; d < D; ++d) G[d] = fma(wg, df[d], G[d]);
      E = fma(-u, h, E);
    }
  }
  // combine the four column parts (lanes 4m .. 4m+3) in a fixed order
#pragma unroll
  for (int o = 1; o < 4; o <<= 1) {
#pragma unroll
    for (int d = 0; d < D; ++d) G[d] += __shfl_xor_sync(0xffffffffu, G[d], o);
    E += __shfl_xor_sync(0xffffffffu, E, o);
  }
  if (live && part == 0) {
#pragma unroll
    for (int d = 0; d < D; ++d) gC[q.offC + (long long)k * D + d] = G[d];
    double lx = 0.0;
#pragma unroll
    for (int rr = 0; rr < BMAX_RHS; ++rr) lx = fma(lk[rr], xk[rr], lx);
    rowscr[q.offR + 2LL * k] = 2.0 * q.eps * E;
    rowscr[q.offR + 2LL * k + 1] = -lx;
  }
}

// Per system: grad_eps = sum_k partial, grad_reg = sum_k partial (fixed order).
__global__ void __launch_bounds__(BT) k_badj_reduce(const BSys* __restrict__ sys, const double* __restrict__ rowscr,
                                                    double* __restrict__ geps, double* __restrict__ greg) {
  __shared__ double red[32];
  const BSys q = sys[blockIdx.x];
  double a = 0.0, b = 0.0;
  for (int i = threadIdx.x; i < q.n; i += BT) {
    a += rowscr[q.offR + 2LL * i];
    b += rowscr[q.offR + 2LL * i + 1];
  }
  a = block_sum(a, red);
  b = block_sum(b, red);
  if (threadIdx.x == 0) {
    geps[q.user] = a;
    greg[q.user] = b;
  }
}

// ------------------------------------------------------------------ persistent task-graph step
// The whole step (assembly, Cholesky, solve and FP64 refinement of every
// system) as ONE persistent launch.  The work is a list of tile tasks in a
// topological order:
//   COPY(s, r)             X_r := B_r
//   ASM(s, i, j)           tile (i, j) of A_s
//   per level k: POTRF(s, k), TRSM(s, k, i), SYRK(s, k, i, j)
//   per phase f = 0 .. refine (f = 0 solves into X, f >= 1 refines):
//     RES(f, s, r)         V_r := B_r - (A X)_r                (f >= 1)
//     forward, level k:    DIAG_F(f, s, k), UPD_F(f, s, k, r)   (r > k)
//     backward, level k:   DIAG_B(f, s, k), UPD_B(f, s, k, r)   (r < k), k descending
//     ADD(f, s, r)         X_r += V_r                            (f >= 1)
// CTAs take tasks in list order from one atomic counter and wait (bounded,
// one thread, acquire loads) until the task's inputs are final; every
// dependency points to an earlier task, so a running CTA only ever waits on
// tasks that running CTAs hold or have finished, and the launch needs no
// co-residency.  Completion is published with a release after a fence:
//   st[s](i, j)     lower tile: -1 unassembled, 0..j updates applied, j + 1 final
//   fw[f][s][r]     block r of the phase's vector: -1 not ready, 0..r updates, r + 1 solved
//   bw[f][s][r]     backward updates applied (from blocks > r), nblk - r once solved
//   done[f][s]      blocks of X final after phase f;  asm_done[s]  tiles assembled
// Reads of data other tasks wrote bypass L1 (ld.global.cg); the arithmetic of
// every task is that of the level-scheduled kernels.
enum BTaskKind : int { BT_COPY = 0, BT_ASM, BT_POTRF, BT_TRSM, BT_SYRK, BT_RES, BT_DIAGF, BT_UPDF, BT_DIAGB, BT_UPDB,
                       BT_ADD, BT_SYRKC, BT_SYRKR };

struct DagSec {         // one contiguous run of tasks of one kind
  long long begin;      // first global task index
  int kind, k, phase, pad;
  long long pre_off;    // offset of its per-system prefix (cnt + 1 entries) in d_pre
  int cnt, pad2;        // systems covered (a prefix of the sorted systems)
};

struct DagState {
  int* st;        // Σ nblk (nblk + 1) / 2
  int* fw;        // (refine + 1) x Σ nblk
  int* bw;        // (refine + 1) x Σ nblk
  int* done;      // (refine + 1) x nsys
  int* asm_done;  // nsys
  unsigned long long* head;
  int* err;
};

__device__ __forceinline__ int ld_acq(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_rel(int* p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

constexpr long long DAG_WAIT = 1LL << 25;

// thread 0: spin until *p == want; false when the limit ran out or another
// CTA has already given up (then every CTA stops within one poll)
__device__ __forceinline__ bool dag_wait(const int* p, int want, const int* err) {
  for (long long it = 0; it < DAG_WAIT; ++it) {
    if (ld_acq(p) == want) return true;
    if (it > 32) {
      if ((it & 255) == 0 && *(volatile const int*)err) return false;
      __nanosleep(it > 4096 ? 256 : 32);
    }
  }
  return false;
}

__device__ __forceinline__ DF ld_df_cg(const double* p) {
  const float2 f = __ldcg(reinterpret_cast<const float2*>(p));
  DF r;
  r.h = f.x;
  r.l = f.y;
  return r;
}

template <typename T>
__device__ __forceinline__ void stage_block_cg(T* sT, const double* __restrict__ src, long long ld, int nr, int nc) {
  for (int e = threadIdx.x; e < BNB * BNB; e += BT) {
    const int r = e & 63, kk = e >> 6;
    DF v;
    v.h = 0.f;
    v.l = 0.f;
    if (r < nr && kk < nc) v = ld_df_cg(src + (long long)r + (long long)kk * ld);
    if constexpr (std::is_same<T, double>::value) sT[kk * BPAD + r] = df_to_f64(v);
    else sT[kk * BPAD + r] = v;
  }
}

__device__ __forceinline__ int tri_idx(int i, int j) { return i * (i + 1) / 2 + j; }

// Tiles (ti, tj), tj <= ti, of a level-k trailing-update task u.  BT_SYRK: all
// lower tiles right of the panel in triangular order; BT_SYRKC: the next
// panel column tj = k + 1 only; BT_SYRKR: the rest (tj >= k + 2).  The split
// lets the queue put the next column's updates, and the next panel's factor
// and solve, ahead of the bulk of the level (a look-ahead of one panel).
__device__ __forceinline__ void syrk_tiles(int kind, int k, long long u, int& ti, int& tj) {
  if (kind == BT_SYRKC) {
    ti = k + 1 + (int)u;
    tj = k + 1;
    return;
  }
  int a = (int)((sqrt(8.0 * (double)u + 1.0) - 1.0) * 0.5);
  while ((long long)(a + 1) * (a + 2) / 2 <= u) ++a;
  while ((long long)a * (a + 1) / 2 > u) --a;
  const int b = (int)(u - (long long)a * (a + 1) / 2);
  const int sh = kind == BT_SYRKR ? 2 : 1;
  ti = k + sh + a;
  tj = k + sh + b;
}

template <int KIND, int D, int ARITH>
__global__ void __launch_bounds__(BT) k_bstep_dag(const BSys* __restrict__ sys, const long long* __restrict__ pre,
                                                  const DagSec* __restrict__ secs, int nsec, long long total,
                                                  const long long* __restrict__ st_off, const long long* __restrict__ v_off,
                                                  long long v_total, int nsys, int nrhs,
                                                  const double* __restrict__ coords, double* __restrict__ A,
                                                  double* __restrict__ Linv, const double* __restrict__ B,
                                                  double* __restrict__ X, double* __restrict__ V, int* pert,
                                                  DagState S) {
  extern __shared__ double smem[];
  __shared__ long long s_t;
  __shared__ int s_ok;
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  for (;;) {
    if (tid == 0) s_t = *(volatile const int*)S.err ? total : (long long)atomicAdd(S.head, 1ULL);
    __syncthreads();
    const long long t = s_t;
    if (t >= total) return;
    // section of t
    int lo = 0, hi = nsec - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (secs[mid].begin <= t) lo = mid; else hi = mid - 1;
    }
    const DagSec sec = secs[lo];
    const long long u0 = t - sec.begin;
    const long long* sp = pre + sec.pre_off;
    const int s = task_system(sp, sec.cnt + 1, u0);
    const BSys q = sys[s];
    const long long u = u0 - sp[s];
    const int k = sec.k, f = sec.phase;
    int* st = S.st + st_off[s];
    int* fw = S.fw + (long long)f * v_total + v_off[s];
    int* bw = S.bw + (long long)f * v_total + v_off[s];
    double* Ab = A + q.offA;
    const long long lda = q.n;
    const int nblk = q.nblk;
    // ---- decode the task's tiles, wait for its inputs
    int ti = 0, tj = 0;
    if (tid == 0) {
      bool ok = true;
      switch (sec.kind) {
        case BT_COPY: case BT_ASM: break;
        case BT_POTRF: ok = dag_wait(st + tri_idx(k, k), k, S.err); break;
        case BT_TRSM:
          ti = k + 1 + (int)u;
          ok = dag_wait(st + tri_idx(k, k), k + 1, S.err) && dag_wait(st + tri_idx(ti, k), k, S.err);
          break;
        case BT_SYRK:
        case BT_SYRKC:
        case BT_SYRKR:
          syrk_tiles(sec.kind, k, u, ti, tj);
          ok = dag_wait(st + tri_idx(ti, k), k + 1, S.err) && dag_wait(st + tri_idx(tj, k), k + 1, S.err) &&
               dag_wait(st + tri_idx(ti, tj), k, S.err);
          break;
        case BT_RES:
          ok = dag_wait(S.done + (long long)(f - 1) * nsys + s, nblk, S.err) &&
               dag_wait(S.asm_done + s, nblk * nblk, S.err);
          break;
        case BT_DIAGF: ok = dag_wait(st + tri_idx(k, k), k + 1, S.err) && dag_wait(fw + k, k, S.err); break;
        case BT_UPDF:
          ti = k + 1 + (int)u;
          ok = dag_wait(st + tri_idx(ti, k), k + 1, S.err) && dag_wait(fw + k, k + 1, S.err) &&
               dag_wait(fw + ti, k, S.err);
          break;
        case BT_DIAGB: ok = dag_wait(fw + k, k + 1, S.err) && dag_wait(bw + k, nblk - 1 - k, S.err); break;
        case BT_UPDB:
          ti = (int)u;  // r < k
          ok = dag_wait(bw + k, nblk - k, S.err) && dag_wait(bw + ti, nblk - 1 - k, S.err) &&
               dag_wait(fw + ti, ti + 1, S.err);
          break;
        case BT_ADD: ti = (int)u; ok = dag_wait(bw + ti, nblk - ti, S.err); break;
      }
      s_ok = ok ? 1 : 0;
      if (!ok) atomicExch(S.err, 1);
    }
    __syncthreads();
    if (!s_ok) return;
    if (sec.kind == BT_TRSM || sec.kind == BT_UPDF || sec.kind == BT_UPDB || sec.kind == BT_ADD) {
      ti = (sec.kind == BT_TRSM || sec.kind == BT_UPDF) ? k + 1 + (int)u : (int)u;
    } else if (sec.kind == BT_SYRK || sec.kind == BT_SYRKC || sec.kind == BT_SYRKR) {
      syrk_tiles(sec.kind, k, u, ti, tj);
    }
    // ---- the task
    int* pub = nullptr;  // state word set to pub_val when the task is done
    int pub_val = 0;
    int* cnt_add = nullptr;  // counter incremented when the task is done
    switch (sec.kind) {
      case BT_COPY: {
        const int r = (int)u, r0 = r * BNB, nr = min(BNB, q.n - r0);
        for (int e = tid; e < BNB * nrhs; e += BT) {
          const int i = e % BNB, c = e / BNB;
          if (i < nr) {
            const long long o = q.offX + (long long)(r0 + i) + (long long)c * q.n;
            X[o] = B[o];
          }
        }
        pub = S.fw + v_off[s] + r;  // phase 0
        pub_val = 0;
        break;
      }
      case BT_ASM: {
        ti = (int)(u % nblk);
        tj = (int)(u / nblk);
        double* sR = smem;
        double* sC = smem + BNB * D;
        const int r0 = ti * BNB, c0 = tj * BNB;
        const double* Xc = coords + q.offC;
        for (int e = tid; e < BNB * D; e += BT) {
          const int i = e / D, d = e % D;
          sR[e] = (r0 + i < q.n) ? Xc[(long long)(r0 + i) * D + d] : 0.0;
          sC[e] = (c0 + i < q.n) ? Xc[(long long)(c0 + i) * D + d] : 0.0;
        }
        __syncthreads();
        const int row = tid & 63;
        for (int col = tid >> 6; col < BNB; col += BT / BNB) {
          const int i = r0 + row, j = c0 + col;
          if (i >= q.n || j >= q.n) continue;
          double r2 = 0.0;
#pragma unroll
          for (int d = 0; d < D; ++d) {
            const double df = sR[row * D + d] - sC[col * D + d];
            r2 = fma(df, df, r2);
          }
          double v = phi_only<KIND>(r2, q.gamma);
          if (i == j) v += q.reg;
          double* slot = Ab + (long long)i + (long long)j * q.n;
          if (i >= j) st_df(slot, to_df(v));
          else *slot = v;
        }
        if (ti >= tj) {
          pub = st + tri_idx(ti, tj);
          pub_val = 0;
        }
        cnt_add = S.asm_done + s;
        break;
      }
      case BT_POTRF: {
        double* sL = smem;
        double* sI = smem + BNB * BPAD;
        double* s_inv = smem + 2 * BNB * BPAD;
        const int kb = k * BNB;
        const int nb = min(BNB, q.n - kb);
        for (int e = tid; e < BNB * BNB; e += BT) {
          const int i = e & 63, j = e >> 6;
          double v = 0.0;
          if (i < nb && j < nb && i >= j) v = df_to_f64(ld_df_cg(Ab + (long long)(kb + i) + (long long)(kb + j) * lda));
          sL[i * BPAD + j] = v;
          sI[i * BPAD + j] = 0.0;
        }
        __syncthreads();
        const double dref = 1.0 + q.reg;
        for (int j = 0; j < nb; ++j) {
          if (tid == 0) {
            double d = sL[j * BPAD + j];
            if (!(d > 1e-15 * dref)) {
              d = 1e-15 * dref;
              atomicAdd(pert, 1);
            }
            const double p = sqrt(d);
            sL[j * BPAD + j] = p;
            *s_inv = 1.0 / p;
          }
          __syncthreads();
          const double ip = *s_inv;
          for (int i = j + 1 + tid; i < nb; i += BT) sL[i * BPAD + j] *= ip;
          __syncthreads();
          const int m = nb - j - 1;
          for (int e = tid; e < m * m; e += BT) {
            const int i = j + 1 + e / m, l = j + 1 + e % m;
            if (l <= i) sL[i * BPAD + l] -= sL[i * BPAD + j] * sL[l * BPAD + j];
          }
          __syncthreads();
        }
        for (int i = 0; i < nb; ++i) {
          const int c = tid;
          if (c <= i && c < BNB) {
            double acc = (c == i) ? 1.0 : 0.0;
            for (int l = c; l < i; ++l) acc -= sL[i * BPAD + l] * sI[l * BPAD + c];
            sI[i * BPAD + c] = acc / sL[i * BPAD + i];
          }
          __syncthreads();
        }
        for (int e = tid; e < BNB * BNB; e += BT) {
          const int i = e & 63, j = e >> 6;
          if (i < nb && j < nb && i >= j)
            st_df(Ab + (long long)(kb + i) + (long long)(kb + j) * lda, to_df(sL[i * BPAD + j]));
          Linv[q.offL + (long long)k * BNB * BNB + i + (long long)j * BNB] = sI[i * BPAD + j];
        }
        pub = st + tri_idx(k, k);
        pub_val = k + 1;
        break;
      }
      case BT_TRSM: {
        double* sA = smem;
        double* sB = smem + BNB * BPAD;
        const int kb = k * BNB, r0 = ti * BNB;
        const int nb = min(BNB, q.n - kb), nr = min(BNB, q.n - r0);
        stage_block_cg(sA, Ab + r0 + (long long)kb * lda, lda, nr, nb);
        const double* Li = Linv + q.offL + (long long)k * BNB * BNB;
        for (int e = tid; e < BNB * BNB; e += BT) {
          const int col = e & 63, kk = e >> 6;
          sB[kk * BPAD + col] = __ldcg(Li + col + kk * BNB);
        }
        __syncthreads();
        double acc[4][4] = {};
        tile_fma_f64(sA, sB, acc, ty, tx);
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const int row = ty * 4 + i, col = tx * 4 + j;
            if (row < nr && col < nb)
              st_df(Ab + (long long)(r0 + row) + (long long)(kb + col) * lda, to_df(acc[i][j]));
          }
        pub = st + tri_idx(ti, k);
        pub_val = k + 1;
        break;
      }
      case BT_SYRK:
      case BT_SYRKC:
      case BT_SYRKR: {
        using STT = typename std::conditional<ARITH == 0, double, DF>::type;
        STT* sA = reinterpret_cast<STT*>(smem);
        STT* sB = sA + BNB * BPAD;
        const int kb = k * BNB, r0 = ti * BNB, c0 = tj * BNB;
        const int nb = min(BNB, q.n - kb), nr = min(BNB, q.n - r0), nc = min(BNB, q.n - c0);
        stage_block_cg(sA, Ab + r0 + (long long)kb * lda, lda, nr, nb);
        stage_block_cg(sB, Ab + c0 + (long long)kb * lda, lda, nc, nb);
        __syncthreads();
        if (ARITH == 0) {
          double acc[4][4] = {};
          tile_fma_f64(reinterpret_cast<const double*>(sA), reinterpret_cast<const double*>(sB), acc, ty, tx);
#pragma unroll
          for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) {
              const int row = ty * 4 + i, col = tx * 4 + j;
              if (row < nr && col < nc && (ti != tj || row >= col)) {
                double* p = Ab + (long long)(r0 + row) + (long long)(c0 + col) * lda;
                st_df(p, to_df(df_to_f64(ld_df_cg(p)) - acc[i][j]));
              }
            }
        } else {
          float sh[4][4] = {}, sl[4][4] = {};
          tile_fma_df(reinterpret_cast<const DF*>(sA), reinterpret_cast<const DF*>(sB), sh, sl, ty, tx);
#pragma unroll
          for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) {
              const int row = ty * 4 + i, col = tx * 4 + j;
              if (row < nr && col < nc && (ti != tj || row >= col)) {
                double* p = Ab + (long long)(r0 + row) + (long long)(c0 + col) * lda;
                const float h = sh[i][j] + sl[i][j];
                const float l = sl[i][j] - (h - sh[i][j]);
                st_df(p, df_sub(ld_df_cg(p), h, l));
              }
            }
        }
        pub = st + tri_idx(ti, tj);
        pub_val = k + 1;
        break;
      }
      case BT_RES: {
        const int r = (int)u, r0 = r * BNB, nr = min(BNB, q.n - r0);
        double* sT = smem;
        double* sX = smem + BNB * BPAD;
        const double dia = 1.0 + q.reg;
        const int row = tid & 63, g = tid >> 6;
        double acc[2] = {0.0, 0.0};
        for (int c = 0; c < nblk; ++c) {
          const int c0 = c * BNB, nc = min(BNB, q.n - c0);
          __syncthreads();
          for (int e = tid; e < BNB * BNB; e += BT) {
            const int i = e & 63, j = e >> 6;
            double v = 0.0;
            if (r < c) {
              if (i < nr && j < nc) v = __ldcg(Ab + (long long)(r0 + i) + (long long)(c0 + j) * lda);
              sT[j * BPAD + i] = v;
            } else if (r > c) {
              if (i < nc && j < nr) v = __ldcg(Ab + (long long)(c0 + i) + (long long)(r0 + j) * lda);
              sT[i * BPAD + j] = v;
            } else {
              if (i < nr && j < nr) {
                if (i < j) v = __ldcg(Ab + (long long)(r0 + i) + (long long)(r0 + j) * lda);
                else if (i > j) v = __ldcg(Ab + (long long)(r0 + j) + (long long)(r0 + i) * lda);
                else v = dia;
              }
              sT[j * BPAD + i] = v;
            }
          }
          for (int e = tid; e < BNB * nrhs; e += BT) {
            const int i = e % BNB, rr = e / BNB;
            sX[e] = (i < nc) ? __ldcg(X + q.offX + (long long)(c0 + i) + (long long)rr * q.n) : 0.0;
          }
          __syncthreads();
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const int rr = g + 4 * h;
            if (rr < nrhs) {
              double a = acc[h];
#pragma unroll 8
              for (int j = 0; j < BNB; ++j) a = fma(sT[j * BPAD + row], sX[rr * BNB + j], a);
              acc[h] = a;
            }
          }
        }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int rr = g + 4 * h;
          if (rr < nrhs && row < nr) {
            const long long o = q.offX + (long long)(r0 + row) + (long long)rr * q.n;
            V[o] = B[o] - acc[h];
          }
        }
        pub = fw + r;
        pub_val = 0;
        break;
      }
      case BT_DIAGF:
      case BT_DIAGB: {
        const bool trans = sec.kind == BT_DIAGB;
        double* Vec = f == 0 ? X : V;
        double* sX = smem;
        double* sLi = smem + BNB * BMAX_RHS;
        const int kb = k * BNB, nb = min(BNB, q.n - kb);
        double* Vb = Vec + q.offX;
        const double* Li = Linv + q.offL + (long long)k * BNB * BNB;
        for (int e = tid; e < BNB * nrhs; e += BT) {
          const int i = e % BNB, r = e / BNB;
          sX[e] = (i < nb) ? __ldcg(Vb + (long long)(kb + i) + (long long)r * q.n) : 0.0;
        }
        for (int e = tid; e < BNB * BNB; e += BT) {
          const int i = e & 63, j = e >> 6;
          sLi[i * BPAD + j] = __ldcg(Li + i + j * BNB);
        }
        __syncthreads();
        for (int e = tid; e < BNB * nrhs; e += BT) {
          const int i = e % BNB, r = e / BNB;
          if (i >= nb) continue;
          double acc = 0.0;
          if (!trans) {
            for (int c = 0; c <= i; ++c) acc = fma(sLi[i * BPAD + c], sX[r * BNB + c], acc);
          } else {
            for (int c = i; c < nb; ++c) acc = fma(sLi[c * BPAD + i], sX[r * BNB + c], acc);
          }
          Vb[(long long)(kb + i) + (long long)r * q.n] = acc;
        }
        if (!trans) {
          pub = fw + k;
          pub_val = k + 1;
        } else {
          pub = bw + k;
          pub_val = nblk - k;
          if (f == 0) cnt_add = S.done + s;  // phase 0 solves straight into X
        }
        break;
      }
      case BT_UPDF:
      case BT_UPDB: {
        const bool trans = sec.kind == BT_UPDB;
        double* Vec = f == 0 ? X : V;
        DF* sT = reinterpret_cast<DF*>(smem);
        DF* sX = sT + BNB * BPAD;
        const int r = ti;
        const int kb = k * BNB, r0 = r * BNB;
        const int nb = min(BNB, q.n - kb), nr = min(BNB, q.n - r0);
        double* Vb = Vec + q.offX;
        if (!trans) {
          stage_block_cg(sT, Ab + r0 + (long long)kb * lda, lda, nr, nb);
        } else {
          for (int e = tid; e < BNB * BNB; e += BT) {
            const int kk = e & 63, row = e >> 6;
            DF v;
            v.h = 0.f;
            v.l = 0.f;
            if (kk < nb && row < nr) v = ld_df_cg(Ab + (long long)(kb + kk) + (long long)(r0 + row) * lda);
            sT[kk * BPAD + row] = v;
          }
        }
        for (int e = tid; e < BNB * nrhs; e += BT) {
          const int i = e % BNB, rr = e / BNB;
          sX[e] = to_df((i < nb) ? __ldcg(Vb + (long long)(kb + i) + (long long)rr * q.n) : 0.0);
        }
        __syncthreads();
        for (int e = tid; e < BNB * nrhs; e += BT) {
          const int row = e % BNB, rr = e / BNB;
          if (row >= nr) continue;
          float sh = 0.f, sl = 0.f;
#pragma unroll 4
          for (int kk = 0; kk < BNB; ++kk) {
            const DF a = sT[kk * BPAD + row], b = sX[rr * BNB + kk];
            const float ph = a.h * b.h;
            float pl = fmaf(a.h, b.h, -ph);
            pl = fmaf(a.h, b.l, pl);
            pl = fmaf(a.l, b.h, pl);
            const float tt = sh + ph;
            const float bp = tt - sh;
            const float er = (sh - (tt - bp)) + (ph - bp);
            sh = tt;
            sl += er + pl;
          }
          double* pv = Vb + (long long)(r0 + row) + (long long)rr * q.n;
          *pv = __ldcg(pv) - ((double)sh + (double)sl);
        }
        if (!trans) {
          pub = fw + r;
          pub_val = k + 1;
        } else {
          pub = bw + r;
          pub_val = nblk - k;
        }
        break;
      }
      case BT_ADD: {
        const int r = ti, r0 = r * BNB, nr = min(BNB, q.n - r0);
        for (int e = tid; e < BNB * nrhs; e += BT) {
          const int i = e % BNB, c = e / BNB;
          if (i < nr) {
            const long long o = q.offX + (long long)(r0 + i) + (long long)c * q.n;
            X[o] = __ldcg(X + o) + __ldcg(V + o);
          }
        }
        cnt_add = S.done + (long long)f * nsys + s;
        break;
      }
    }
    // ---- publish
    __syncthreads();
    if (tid == 0) {
      __threadfence();
      if (pub) st_rel(pub, pub_val);
      if (cnt_add) atomicAdd(cnt_add, 1);
    }
  }
}

// ------------------------------------------------------------------ host side

static const long long* preT_dev(const BatchPlan* p, int k) { return p->d_pre + p->preT_off[k]; }
static const long long* preS_dev(const BatchPlan* p, int k) { return p->d_pre + p->d_preS_base + p->preS_off[k]; }
static const long long* preRow_dev(const BatchPlan* p) { return p->d_pre + p->d_preRow_base; }

#define BKIND_DIM_SWITCH(KIND, DIM, ...)                                           \
  do {                                                                             \
    if ((KIND) == MPDOK_KERNEL_GAUSSIAN) {                                         \
      constexpr int KK_ = MPDOK_KERNEL_GAUSSIAN;                                   \
      if ((DIM) == 1) { constexpr int DD_ = 1; __VA_ARGS__; }                     \
      else if ((DIM) == 2) { constexpr int DD_ = 2; __VA_ARGS__; }                \
      else { constexpr int DD_ = 3; __VA_ARGS__; }                                 \
    } else {                                                                       \
      constexpr int KK_ = MPDOK_KERNEL_MQ;                                         \
      if ((DIM) == 1) { constexpr int DD_ = 1; __VA_ARGS__; }                     \
      else if ((DIM) == 2) { constexpr int DD_ = 2; __VA_ARGS__; }                \
      else { constexpr int DD_ = 3; __VA_ARGS__; }                                 \
    }                                                                              \
  } while (0)

static int batch_factor(BatchPlan* p, cudaStream_t s) {
  MPDOK_CUDA_TRY(cudaMemsetAsync(p->d_pert, 0, sizeof(int), s));
  // assembly: one task per (system, tile); its prefix follows the row prefix
  const long long* preA = p->d_pre + p->d_preRow_base + (p->nsys + 1);
  long long totalA = 0;
  for (auto& q : p->sys) totalA += (long long)q.nblk * q.nblk;
  if (totalA > 0) {
    BKIND_DIM_SWITCH(p->kernel, p->dim,
                     launch(k_bassemble<KK_, DD_>, dim3((unsigned)totalA), BT, 0, s, (const BSys*)p->d_sys, preA,
                            p->nsys, (const double*)p->coords, p->A));
  }
  const size_t tsm = 2 * (size_t)BNB * BPAD * sizeof(double);
  for (int k = 0; k < p->maxblk; ++k) {
    const int cnt = p->act[k];
    launch(k_bpotrf, dim3(cnt), BT, tsm, s, (const BSys*)p->d_sys, k, p->A, p->Linv, p->d_pert);
    const long long nt = p->preT[p->preT_off[k] + cnt];
    if (nt > 0)
      launch(k_btrsm, dim3((unsigned)nt), BT, tsm, s, (const BSys*)p->d_sys, preT_dev(p, k), cnt, k, p->A,
             (const double*)p->Linv);
    const long long ns = p->preS[p->preS_off[k] + cnt];
    if (ns > 0) {
      const unsigned g = (unsigned)std::min<long long>(ns, p->syrk_grid);
      if (p->arith == 0)
        launch(k_bsyrk<0>, dim3(g), BT, tsm, s, (const BSys*)p->d_sys, preS_dev(p, k), cnt, k, p->A);
      else
        launch(k_bsyrk<1>, dim3(g), BT, tsm, s, (const BSys*)p->d_sys, preS_dev(p, k), cnt, k, p->A);
    }
  }
  MPDOK_LAUNCH_CHECK("batch factor");
  return MPDOK_OK;
}

// V := A^{-1} V in place (V in the caller's packing).
static int batch_solve_inplace(BatchPlan* p, double* V, cudaStream_t s) {
  for (int k = 0; k < p->maxblk; ++k) {
    const int cnt = p->act[k];
    launch(k_bsolve_diag<false>, dim3(cnt), BT, 0, s, (const BSys*)p->d_sys, k, p->nrhs, (const double*)p->Linv, V);
    const long long nt = p->preT[p->preT_off[k] + cnt];
    if (nt > 0)
      launch(k_bsolve_upd<false>, dim3((unsigned)nt), BT, 0, s, (const BSys*)p->d_sys, preT_dev(p, k), cnt, k,
             p->nrhs, (const double*)p->A, V);
  }
  for (int k = p->maxblk - 1; k >= 0; --k) {
    const int cnt = p->act[k];
    launch(k_bsolve_diag<true>, dim3(cnt), BT, 0, s, (const BSys*)p->d_sys, k, p->nrhs, (const double*)p->Linv, V);
    if (k > 0)
      launch(k_bsolve_upd<true>, dim3((unsigned)((long long)cnt * k)), BT, 0, s, (const BSys*)p->d_sys,
             (const long long*)nullptr, cnt, k, p->nrhs, (const double*)p->A, V);
  }
  MPDOK_LAUNCH_CHECK("batch solve");
  return MPDOK_OK;
}

static int batch_residual(BatchPlan* p, const double* B, const double* X, double* R, cudaStream_t s) {
  const long long nt = p->preRow.back();
  if (nt > 0)
    launch(k_bsymv_res, dim3((unsigned)nt), BT, 0, s, (const BSys*)p->d_sys, preRow_dev(p), p->nsys, p->nrhs,
           (const double*)p->A, B, X, R);
  MPDOK_LAUNCH_CHECK("batch residual");
  return MPDOK_OK;
}

static int batch_solve(BatchPlan* p, const double* B, double* X, int refine, cudaStream_t s) {
  const long long nx = p->total_x;
  if (nx == 0) return MPDOK_OK;
  MPDOK_CUDA_TRY(cudaMemcpyAsync(X, B, (size_t)nx * sizeof(double), cudaMemcpyDeviceToDevice, s));
  MPDOK_TRY(batch_solve_inplace(p, X, s));
  const unsigned g = (unsigned)std::min<long long>((nx + 255) / 256, (long long)num_sms() * 8);
  for (int it = 0; it < refine; ++it) {
    MPDOK_TRY(batch_residual(p, B, X, p->V, s));
    MPDOK_TRY(batch_solve_inplace(p, p->V, s));
    launch(k_badd, dim3(g), 256, 0, s, X, (const double*)p->V, nx);
  }
  MPDOK_LAUNCH_CHECK("batch refine");
  return MPDOK_OK;
}

// FP32 columns (leading dimension ld) <-> the plan's FP64 packing (n x K, ld n).
__global__ void k_cols_f32_to_f64(const float* __restrict__ v, long long ld, double* __restrict__ t, long long n,
                                  int K) {
  const long long total = n * K;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x)
    t[e] = (double)v[(e / n) * ld + e % n];
}
__global__ void k_cols_f64_to_f32(const double* __restrict__ t, float* __restrict__ z, long long ld, long long n,
                                  int K) {
  const long long total = n * K;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x)
    z[(e / n) * ld + e % n] = (float)t[e];
}

static int bpc_apply_cols(void* ctx, const float* v, float* z, int K, long long ld, cudaStream_t s) {
  BatchPcCtx* c = (BatchPcCtx*)ctx;
  BatchPlan* p = (BatchPlan*)c->plan;
  const long long total = c->n * K;
  const unsigned g = (unsigned)std::max(1LL, std::min<long long>((total + 255) / 256, (long long)num_sms() * 8));
  launch(k_cols_f32_to_f64, g, 256, 0, s, v, ld, c->tmp, c->n, K);
  MPDOK_TRY(batch_solve_inplace(p, c->tmp, s));
  launch(k_cols_f64_to_f32, g, 256, 0, s, (const double*)c->tmp, z, ld, c->n, K);
  MPDOK_LAUNCH_CHECK("batch preconditioner");
  return MPDOK_OK;
}

int batch_apply_f64(void* plan, long long n, int K, double* V, cudaStream_t s) {
  MPDOK_ARG_CHECK(plan && V, "null pointer");
  BatchPlan* p = (BatchPlan*)plan;
  MPDOK_ARG_CHECK(p->nsys == 1 && p->sys[0].n == n, "the preconditioner plan must hold one system of size n");
  MPDOK_ARG_CHECK(p->nrhs == K, "the preconditioner plan's nrhs must equal the solve's nrhs");
  return batch_solve_inplace(p, V, s);
}

int batch_precond(void* plan, long long n, int K, double* tmp, BatchPcCtx* ctx, Precond* pc) {
  MPDOK_ARG_CHECK(plan && tmp && ctx && pc, "null pointer");
  BatchPlan* p = (BatchPlan*)plan;
  MPDOK_ARG_CHECK(p->nsys == 1 && p->sys[0].n == n, "the preconditioner plan must hold one system of size n");
  MPDOK_ARG_CHECK(p->nrhs == K, "the preconditioner plan's nrhs must equal the solve's nrhs");
  ctx->plan = plan;
  ctx->tmp = tmp;
  ctx->n = n;
  pc->apply = nullptr;
  pc->apply_cols = bpc_apply_cols;
  pc->ctx = ctx;
  return MPDOK_OK;
}

static void dag_release(BatchPlan* p) {
  if (p->d_dagpre) cudaFree(p->d_dagpre);
  if (p->d_secs) cudaFree(p->d_secs);
  if (p->d_dagstate) cudaFree(p->d_dagstate);
  p->d_dagpre = nullptr;
  p->d_secs = nullptr;
  p->d_dagstate = nullptr;
  p->dag_refine = -1;
}

// Host side of the task-graph step: the section table for `refine` refinement
// phases, the prefix tables it needs beyond the level tables, and the state.
static int dag_prepare(BatchPlan* p, int refine) {
  if (p->dag_refine == refine && p->d_secs) return MPDOK_OK;
  std::vector<long long> pre;  // appended prefix arrays; offsets into d_dagpre
  std::vector<DagSec> secs;
  long long begin = 0;
  auto add_prefix = [&](const std::vector<long long>& v) {
    const long long off = (long long)pre.size();
    pre.insert(pre.end(), v.begin(), v.end());
    return off;
  };
  auto prefix_of = [&](int cnt, auto count) {
    std::vector<long long> v(1, 0);
    for (int i = 0; i < cnt; ++i) v.push_back(v.back() + count(i));
    return v;
  };
  auto add_sec = [&](int kind, int k, int phase, int cnt, const std::vector<long long>& v) {
    if (v.back() == 0) return;
    DagSec d{};
    d.begin = begin;
    d.kind = kind;
    d.k = k;
    d.phase = phase;
    d.pre_off = add_prefix(v);
    d.cnt = cnt;
    secs.push_back(d);
    begin += v.back();
  };
  const int ns = p->nsys;
  const auto rows = prefix_of(ns, [&](int i) { return (long long)p->sys[i].nblk; });
  add_sec(BT_COPY, 0, 0, ns, rows);
  add_sec(BT_ASM, 0, 0, ns, prefix_of(ns, [&](int i) { return (long long)p->sys[i].nblk * p->sys[i].nblk; }));
  // factor, with a look-ahead of one panel in the queue order:
  //   POTRF(0) TRSM(0) | per k: SYRK(k, column k+1) POTRF(k+1) TRSM(k+1) SYRK(k, columns >= k+2)
  auto panel = [&](int k) {
    const int cnt = p->act[k];
    add_sec(BT_POTRF, k, 0, cnt, prefix_of(cnt, [](int) { return 1LL; }));
    add_sec(BT_TRSM, k, 0, cnt, prefix_of(cnt, [&](int i) { return (long long)(p->sys[i].nblk - k - 1); }));
  };
  panel(0);
  for (int k = 0; k < p->maxblk; ++k) {
    const int cnt = p->act[k];
    add_sec(BT_SYRKC, k, 0, cnt, prefix_of(cnt, [&](int i) { return (long long)(p->sys[i].nblk - k - 1); }));
    if (k + 1 < p->maxblk) panel(k + 1);
    add_sec(BT_SYRKR, k, 0, cnt, prefix_of(cnt, [&](int i) {
      const long long T = p->sys[i].nblk - k - 2;
      return T > 0 ? T * (T + 1) / 2 : 0LL;
    }));
  }
  for (int f = 0; f <= refine; ++f) {
    if (f > 0) add_sec(BT_RES, 0, f, ns, rows);
    for (int k = 0; k < p->maxblk; ++k) {
      const int cnt = p->act[k];
      add_sec(BT_DIAGF, k, f, cnt, prefix_of(cnt, [](int) { return 1LL; }));
      add_sec(BT_UPDF, k, f, cnt, prefix_of(cnt, [&](int i) { return (long long)(p->sys[i].nblk - k - 1); }));
    }
    for (int k = p->maxblk - 1; k >= 0; --k) {
      const int cnt = p->act[k];
      add_sec(BT_DIAGB, k, f, cnt, prefix_of(cnt, [](int) { return 1LL; }));
      add_sec(BT_UPDB, k, f, cnt, prefix_of(cnt, [&](int) { return (long long)k; }));
    }
    if (f > 0) add_sec(BT_ADD, 0, f, ns, rows);
  }
  // per-system offsets of the tile states and of the vector blocks
  std::vector<long long> st_off(ns), v_off(ns);
  long long ast = 0, av = 0;
  for (int i = 0; i < ns; ++i) {
    st_off[i] = ast;
    v_off[i] = av;
    ast += (long long)p->sys[i].nblk * (p->sys[i].nblk + 1) / 2;
    av += p->sys[i].nblk;
  }
  const long long off_st = add_prefix(st_off), off_v = add_prefix(v_off);
  dag_release(p);
  MPDOK_CUDA_TRY(cudaMalloc(&p->d_dagpre, pre.size() * sizeof(long long)));
  MPDOK_CUDA_TRY(cudaMemcpy(p->d_dagpre, pre.data(), pre.size() * sizeof(long long), cudaMemcpyHostToDevice));
  MPDOK_CUDA_TRY(cudaMalloc(&p->d_secs, secs.size() * sizeof(DagSec)));
  MPDOK_CUDA_TRY(cudaMemcpy(p->d_secs, secs.data(), secs.size() * sizeof(DagSec), cudaMemcpyHostToDevice));
  p->dag_nsec = (int)secs.size();
  p->dag_total = begin;
  p->dag_st_off = off_st;
  p->dag_v_off = off_v;
  p->dag_v_total = av;
  // states: [st | fw] start at -1, [bw | done | asm_done | head | err] at 0
  p->dag_n_neg = (size_t)ast + (size_t)(refine + 1) * av;
  size_t head = p->dag_n_neg + (size_t)(refine + 1) * av + (size_t)(refine + 1) * ns + ns;
  head = (head + 1) & ~(size_t)1;  // the 8-byte queue counter
  p->dag_head_idx = head;
  p->dag_n_zero = head + 4 - p->dag_n_neg;  // head (2 ints), err, spare
  MPDOK_CUDA_TRY(cudaMalloc(&p->d_dagstate, (p->dag_n_neg + p->dag_n_zero) * sizeof(int)));
  p->dag_refine = refine;
  return MPDOK_OK;
}

static int batch_step_dag(BatchPlan* p, const double* B, double* X, int refine, cudaStream_t s) {
  MPDOK_TRY(dag_prepare(p, refine));
  int* base = p->d_dagstate;
  MPDOK_CUDA_TRY(cudaMemsetAsync(base, 0xff, p->dag_n_neg * sizeof(int), s));
  MPDOK_CUDA_TRY(cudaMemsetAsync(base + p->dag_n_neg, 0, p->dag_n_zero * sizeof(int), s));
  MPDOK_CUDA_TRY(cudaMemsetAsync(p->d_pert, 0, sizeof(int), s));
  const long long av = p->dag_v_total;
  const size_t ast = p->dag_n_neg - (size_t)(refine + 1) * av;
  DagState S;
  S.st = base;
  S.fw = base + ast;
  S.bw = base + p->dag_n_neg;
  S.done = S.bw + (refine + 1) * av;
  S.asm_done = S.done + (refine + 1) * p->nsys;
  S.head = reinterpret_cast<unsigned long long*>(base + p->dag_head_idx);
  S.err = base + p->dag_head_idx + 2;
  const size_t smem = (2 * (size_t)BNB * BPAD + 32) * sizeof(double);
  const int grid = std::max(1, p->dag_ctas_per_sm) * num_sms();
  const long long* sto = p->d_dagpre + p->dag_st_off;
  const long long* vo = p->d_dagpre + p->dag_v_off;
#define DAG_LAUNCH(KK, DD, AR)                                                                                   \
  do {                                                                                                           \
    MPDOK_TRY(set_smem(k_bstep_dag<KK, DD, AR>, smem));                                                          \
    launch(k_bstep_dag<KK, DD, AR>, dim3(grid), BT, smem, s, (const BSys*)p->d_sys, (const long long*)p->d_dagpre, \
           (const DagSec*)p->d_secs, p->dag_nsec, p->dag_total, sto, vo, av, p->nsys, p->nrhs,                   \
           (const double*)p->coords, p->A, p->Linv, B, X, p->V, p->d_pert, S);                                   \
  } while (0)
  if (p->arith == 0) {
    BKIND_DIM_SWITCH(p->kernel, p->dim, DAG_LAUNCH(KK_, DD_, 0));
  } else {
    BKIND_DIM_SWITCH(p->kernel, p->dim, DAG_LAUNCH(KK_, DD_, 1));
  }
#undef DAG_LAUNCH
  MPDOK_LAUNCH_CHECK("batch task-graph step");
  return MPDOK_OK;
}

static void plan_free(BatchPlan* p) {
  dag_release(p);
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  if (p->cap) cudaStreamDestroy(p->cap);
  if (p->arena) cudaFree(p->arena);
  if (p->d_sys) cudaFree(p->d_sys);
  if (p->d_pre) cudaFree(p->d_pre);
  if (p->d_pert) cudaFree(p->d_pert);
  delete p;
}

}  // namespace mpdok

using namespace mpdok;

extern "C" int mpdok_batch_create(int nsys, const long long* n, int dim, int nrhs, int kernel, int arith,
                                  int grid_mult, void** plan) {
  MPDOK_ARG_CHECK(plan != nullptr, "null plan pointer");
  *plan = nullptr;
  MPDOK_ARG_CHECK(nsys >= 1 && n != nullptr, "need at least one system");
  MPDOK_ARG_CHECK(dim >= 1 && dim <= 3, "dim must be 1, 2 or 3");
  MPDOK_ARG_CHECK(nrhs >= 1 && nrhs <= BMAX_RHS, "nrhs must be in [1, 8]");
  MPDOK_ARG_CHECK(kernel == MPDOK_KERNEL_GAUSSIAN || kernel == MPDOK_KERNEL_MQ, "unknown kernel");
  MPDOK_ARG_CHECK(arith == 0 || arith == 1, "arith must be 0 (FP64) or 1 (double-float)");
  MPDOK_ARG_CHECK(grid_mult >= 1 && grid_mult <= 16, "grid_mult must be in [1, 16]");
  for (int i = 0; i < nsys; ++i) MPDOK_ARG_CHECK(n[i] >= 1 && n[i] <= (1LL << 20), "system size out of range");
  BatchPlan* p = new BatchPlan();
  p->nsys = nsys;
  p->dim = dim;
  p->nrhs = nrhs;
  p->kernel = kernel;
  p->arith = arith;
  p->grid_mult = grid_mult;
  // caller-order offsets
  std::vector<long long> offX(nsys), offC(nsys);
  long long ax = 0, ac = 0;
  for (int i = 0; i < nsys; ++i) {
    offX[i] = ax;
    offC[i] = ac;
    ax += n[i] * nrhs;
    ac += n[i] * dim;
  }
  p->total_x = ax;
  p->total_c = ac;
  std::vector<int> order(nsys);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return n[a] > n[b]; });
  long long aA = 0, aL = 0, aR = 0;
  for (int idx = 0; idx < nsys; ++idx) {
    const int i = order[idx];
    BSys q{};
    q.n = (int)n[i];
    q.nblk = (q.n + BNB - 1) / BNB;
    q.user = i;
    q.offA = aA;
    q.offX = offX[i];
    q.offC = offC[i];
    q.offL = aL;
    q.offR = aR;
    aA += (long long)q.n * q.n;
    aL += (long long)q.nblk * BNB * BNB;
    aR += 2LL * q.n;
    p->sys.push_back(q);
  }
  p->maxblk = p->sys[0].nblk;
  // level tables
  std::vector<long long> all;
  for (int k = 0; k < p->maxblk; ++k) {
    int cnt = 0;
    while (cnt < nsys && p->sys[cnt].nblk > k) ++cnt;
    p->act.push_back(cnt);
    p->preT_off.push_back((long long)p->preT.size());
    p->preT.push_back(0);
    for (int i = 0; i < cnt; ++i) p->preT.push_back(p->preT.back() + (p->sys[i].nblk - k - 1));
  }
  for (int k = 0; k < p->maxblk; ++k) {
    const int cnt = p->act[k];
    p->preS_off.push_back((long long)p->preS.size());
    p->preS.push_back(0);
    for (int i = 0; i < cnt; ++i) {
      const long long T = p->sys[i].nblk - k - 1;
      p->preS.push_back(p->preS.back() + T * (T + 1) / 2);
    }
  }
  p->preRow.push_back(0);
  for (int i = 0; i < nsys; ++i) p->preRow.push_back(p->preRow.back() + p->sys[i].nblk);
  std::vector<long long> preA(1, 0);
  for (int i = 0; i < nsys; ++i) preA.push_back(preA.back() + (long long)p->sys[i].nblk * p->sys[i].nblk);
  all.insert(all.end(), p->preT.begin(), p->preT.end());
  p->d_preS_base = (long long)all.size();
  all.insert(all.end(), p->preS.begin(), p->preS.end());
  p->d_preRow_base = (long long)all.size();
  all.insert(all.end(), p->preRow.begin(), p->preRow.end());
  all.insert(all.end(), preA.begin(), preA.end());
  auto fail = [&](cudaError_t e, const char* what) {
    cuda_status(e, what);
    plan_free(p);
    return e == cudaErrorMemoryAllocation ? MPDOK_ERR_ALLOC : MPDOK_ERR_CUDA;
  };
  cudaError_t e = cudaMalloc(&p->d_pre, all.size() * sizeof(long long));
  if (e != cudaSuccess) return fail(e, "cudaMalloc (batch tables)");
  e = cudaMemcpy(p->d_pre, all.data(), all.size() * sizeof(long long), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return fail(e, "cudaMemcpy (batch tables)");
  e = cudaMalloc(&p->d_sys, p->sys.size() * sizeof(BSys));
  if (e != cudaSuccess) return fail(e, "cudaMalloc (batch systems)");
  e = cudaMalloc(&p->d_pert, sizeof(int));
  if (e != cudaSuccess) return fail(e, "cudaMalloc (batch counter)");
  const size_t nA = align_up((size_t)aA, 32), nL = align_up((size_t)aL, 32), nV = align_up((size_t)ax, 32),
               nR = align_up((size_t)aR, 32), nCo = align_up((size_t)ac, 32);
  p->bytes = (nA + nL + 2 * nV + nR + nCo) * sizeof(double);
  e = cudaMalloc(&p->arena, p->bytes);
  if (e != cudaSuccess) return fail(e, "cudaMalloc (batch arena)");
  p->A = p->arena;
  p->Linv = p->A + nA;
  p->V = p->Linv + nL;
  p->R = p->V + nV;
  p->rows = p->R + nV;
  p->coords = p->rows + nR;
  e = cudaMemset(p->Linv, 0, nL * sizeof(double));
  if (e != cudaSuccess) return fail(e, "cudaMemset (batch)");
  const int tsm = 2 * BNB * BPAD * (int)sizeof(double);
  cudaFuncSetAttribute(k_bpotrf, cudaFuncAttributeMaxDynamicSharedMemorySize, tsm);
  cudaFuncSetAttribute(k_btrsm, cudaFuncAttributeMaxDynamicSharedMemorySize, tsm);
  cudaFuncSetAttribute(k_bsyrk<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, tsm);
  cudaFuncSetAttribute(k_bsyrk<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, tsm);
  int occ = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, arith == 0 ? k_bsyrk<0> : k_bsyrk<1>, BT, tsm);
  p->syrk_grid = std::max(1, occ) * num_sms() * grid_mult;
  e = cudaStreamCreateWithFlags(&p->cap, cudaStreamNonBlocking);
  if (e != cudaSuccess) return fail(e, "cudaStreamCreate (batch)");
  *plan = p;
  return MPDOK_OK;
}

extern "C" int mpdok_batch_destroy(void* plan) {
  if (!plan) return MPDOK_OK;
  BatchPlan* p = (BatchPlan*)plan;
  cudaDeviceSynchronize();
  plan_free(p);
  return MPDOK_OK;
}

extern "C" size_t mpdok_batch_bytes(void* plan) { return plan ? ((BatchPlan*)plan)->bytes : 0; }

extern "C" int mpdok_batch_load(void* plan, const double* coords, const double* eps, const double* reg,
                                cudaStream_t s) {
  MPDOK_ARG_CHECK(plan && coords && eps && reg, "null pointer");
  BatchPlan* p = (BatchPlan*)plan;
  for (auto& q : p->sys) {
    MPDOK_ARG_CHECK(std::isfinite(eps[q.user]) && std::isfinite(reg[q.user]) && reg[q.user] >= 0.0,
                    "eps must be finite and reg finite and >= 0");
    q.eps = eps[q.user];
    q.gamma = eps[q.user] * eps[q.user];
    q.reg = reg[q.user];
  }
  MPDOK_CUDA_TRY(cudaMemcpyAsync(p->d_sys, p->sys.data(), p->sys.size() * sizeof(BSys), cudaMemcpyHostToDevice, s));
  MPDOK_CUDA_TRY(cudaMemcpyAsync(p->coords, coords, (size_t)p->total_c * sizeof(double), cudaMemcpyDeviceToDevice,
                                 s));
  // the host copy of the table must stay valid until the copy ran
  MPDOK_CUDA_TRY(cudaStreamSynchronize(s));
  return MPDOK_OK;
}

extern "C" int mpdok_batch_factor(void* plan, cudaStream_t s) {
  MPDOK_ARG_CHECK(plan, "null plan");
  return batch_factor((BatchPlan*)plan, s);
}

extern "C" int mpdok_batch_solve(void* plan, const double* B, double* X, int refine, cudaStream_t s) {
  MPDOK_ARG_CHECK(plan && B && X, "null pointer");
  MPDOK_ARG_CHECK(refine >= 0 && refine <= 16, "refine must be in [0, 16]");
  MPDOK_ARG_CHECK(B != X, "B and X must not alias");
  return batch_solve((BatchPlan*)plan, B, X, refine, s);
}

extern "C" int mpdok_batch_relres(void* plan, const double* B, const double* X, double* relres, cudaStream_t s) {
  MPDOK_ARG_CHECK(plan && B && X && relres, "null pointer");
  BatchPlan* p = (BatchPlan*)plan;
  MPDOK_TRY(batch_residual(p, B, X, p->R, s));
  launch(k_brelres, dim3(p->nsys), BT, 0, s, (const BSys*)p->d_sys, p->nrhs, B, (const double*)p->R, relres);
  MPDOK_LAUNCH_CHECK("batch relres");
  return MPDOK_OK;
}

extern "C" int mpdok_batch_adjoint(void* plan, const double* X, const double* Lam, double* grad_coords,
                                   double* grad_eps, double* grad_reg, cudaStream_t s) {
  MPDOK_ARG_CHECK(plan && X && Lam && grad_coords && grad_eps && grad_reg, "null pointer");
  BatchPlan* p = (BatchPlan*)plan;
  const long long nt = p->preRow.back();
  if (nt > 0) {
    BKIND_DIM_SWITCH(p->kernel, p->dim,
                     launch(k_badjoint<KK_, DD_>, dim3((unsigned)nt), BT, 0, s, (const BSys*)p->d_sys,
                            preRow_dev(p), p->nsys, p->nrhs, (const double*)p->coords, X, Lam, grad_coords,
                            p->rows));
  }
  launch(k_badj_reduce, dim3(p->nsys), BT, 0, s, (const BSys*)p->d_sys, (const double*)p->rows, grad_eps, grad_reg);
  MPDOK_LAUNCH_CHECK("batch adjoint");
  return MPDOK_OK;
}

// The adjoint contraction of ONE system (the in-core path's gradients), with
// the batch kernels on a one-system description kept in the workspace:
// [BSys | prefix (2) | per-row partials (2 n)].
extern "C" size_t mpdok_rbf_adjoint_workspace_size(long long n) {
  if (n < 0) return 0;
  return 256 + 256 + align_up((size_t)std::max(1LL, n) * 2 * sizeof(double), 256);
}

extern "C" int mpdok_rbf_adjoint(const double* coords, long long n, int dim, int kernel, double eps, int nrhs,
                                 const double* X, const double* Lam, double* grad_coords, double* grad_eps,
                                 double* grad_reg, void* work, size_t work_bytes, cudaStream_t s) {
  MPDOK_ARG_CHECK(n >= 1 && n <= (1LL << 30), "n out of range");
  MPDOK_ARG_CHECK(dim >= 1 && dim <= 3, "dim must be 1, 2 or 3");
  MPDOK_ARG_CHECK(kernel == MPDOK_KERNEL_GAUSSIAN || kernel == MPDOK_KERNEL_MQ, "unknown kernel");
  MPDOK_ARG_CHECK(nrhs >= 1 && nrhs <= BMAX_RHS, "nrhs must be in [1, 8]");
  MPDOK_ARG_CHECK(coords && X && Lam && grad_coords && grad_eps && grad_reg && work, "null pointer");
  MPDOK_ARG_CHECK(work_bytes >= mpdok_rbf_adjoint_workspace_size(n), "adjoint workspace too small");
  BSys q{};
  q.n = (int)n;
  q.nblk = (int)((n + BNB - 1) / BNB);
  q.eps = eps;
  q.gamma = eps * eps;
  char* w = (char*)work;
  BSys* d_sys = (BSys*)w;
  long long* d_pre = (long long*)(w + 256);
  double* rows = (double*)(w + 512);
  const long long pre[2] = {0, q.nblk};
  MPDOK_CUDA_TRY(cudaMemcpyAsync(d_sys, &q, sizeof(BSys), cudaMemcpyHostToDevice, s));
  MPDOK_CUDA_TRY(cudaMemcpyAsync(d_pre, pre, sizeof(pre), cudaMemcpyHostToDevice, s));
  BKIND_DIM_SWITCH(kernel, dim,
                   launch(k_badjoint<KK_, DD_>, dim3((unsigned)q.nblk), BT, 0, s, (const BSys*)d_sys,
                          (const long long*)d_pre, 1, nrhs, coords, X, Lam, grad_coords, rows));
  launch(k_badj_reduce, dim3(1), BT, 0, s, (const BSys*)d_sys, (const double*)rows, grad_eps, grad_reg);
  MPDOK_LAUNCH_CHECK("rbf adjoint");
  // the host copies above read stack memory: finish them before returning
  MPDOK_CUDA_TRY(cudaStreamSynchronize(s));
  return MPDOK_OK;
}

extern "C" int mpdok_batch_perturbed(void* plan, cudaStream_t s) {
  if (!plan) return MPDOK_ERR_INVALID_ARG;
  BatchPlan* p = (BatchPlan*)plan;
  int h = 0;
  MPDOK_CUDA_TRY(cudaMemcpyAsync(&h, p->d_pert, sizeof(int), cudaMemcpyDeviceToHost, s));
  MPDOK_CUDA_TRY(cudaStreamSynchronize(s));
  return h;
}

// Capture factor + solve (+ refine) on fixed B / X into one CUDA graph.
extern "C" int mpdok_batch_graph_build(void* plan, const double* B, double* X, int refine) {
  MPDOK_ARG_CHECK(plan && B && X, "null pointer");
  MPDOK_ARG_CHECK(refine >= 0 && refine <= 16, "refine must be in [0, 16]");
  BatchPlan* p = (BatchPlan*)plan;
  if (p->exec) {
    cudaGraphExecDestroy(p->exec);
    p->exec = nullptr;
  }
  if (p->graph) {
    cudaGraphDestroy(p->graph);
    p->graph = nullptr;
  }
  if (p->schedule == 1) MPDOK_TRY(dag_prepare(p, refine));  // (allocates: before the capture)
  MPDOK_CUDA_TRY(cudaStreamBeginCapture(p->cap, cudaStreamCaptureModeThreadLocal));
  int st;
  if (p->schedule == 1) {
    st = batch_step_dag(p, B, X, refine, p->cap);
  } else {
    st = batch_factor(p, p->cap);
    if (st == MPDOK_OK) st = batch_solve(p, B, X, refine, p->cap);
  }
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(p->cap, &g);
  if (st != MPDOK_OK) {
    if (g) cudaGraphDestroy(g);
    return st;
  }
  if (e != cudaSuccess) return cuda_status(e, "cudaStreamEndCapture (batch)");
  p->graph = g;
  size_t nn = 0;
  cudaGraphGetNodes(g, nullptr, &nn);
  p->graph_nodes = nn;
  MPDOK_CUDA_TRY(cudaGraphInstantiate(&p->exec, g, 0));
  return MPDOK_OK;
}

extern "C" int mpdok_batch_graph_launch(void* plan, cudaStream_t s) {
  MPDOK_ARG_CHECK(plan, "null plan");
  BatchPlan* p = (BatchPlan*)plan;
  if (!p->exec) {
    set_error("no graph: call mpdok_batch_graph_build first");
    return MPDOK_ERR_NOT_FACTORED;
  }
  MPDOK_CUDA_TRY(cudaGraphLaunch(p->exec, s));
  count_launch();
  return MPDOK_OK;
}

extern "C" int mpdok_batch_schedule(void* plan, int schedule, int ctas_per_sm) {
  MPDOK_ARG_CHECK(plan, "null plan");
  MPDOK_ARG_CHECK(schedule == 0 || schedule == 1, "schedule must be 0 (levels) or 1 (task graph)");
  MPDOK_ARG_CHECK(ctas_per_sm >= 1 && ctas_per_sm <= 3, "ctas_per_sm must be in [1, 3]");
  BatchPlan* p = (BatchPlan*)plan;
  p->schedule = schedule;
  p->dag_ctas_per_sm = ctas_per_sm;
  return MPDOK_OK;
}

extern "C" int mpdok_batch_step(void* plan, const double* B, double* X, int refine, cudaStream_t s) {
  MPDOK_ARG_CHECK(plan && B && X, "null pointer");
  MPDOK_ARG_CHECK(refine >= 0 && refine <= 16, "refine must be in [0, 16]");
  BatchPlan* p = (BatchPlan*)plan;
  if (p->schedule == 1) return batch_step_dag(p, B, X, refine, s);
  MPDOK_TRY(batch_factor(p, s));
  return batch_solve(p, B, X, refine, s);
}

extern "C" int mpdok_batch_dag_status(void* plan, cudaStream_t s) {
  MPDOK_ARG_CHECK(plan, "null plan");
  BatchPlan* p = (BatchPlan*)plan;
  if (!p->d_dagstate) return MPDOK_OK;
  int h = 0;
  const int* err = p->d_dagstate + p->dag_head_idx + 2;
  MPDOK_CUDA_TRY(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  MPDOK_CUDA_TRY(cudaStreamSynchronize(s));
  if (h) {
    set_error("batch task graph: a task's wait on its inputs ran out");
    return MPDOK_ERR_TIMEOUT;
  }
  return MPDOK_OK;
}

extern "C" long long mpdok_batch_graph_nodes(void* plan) {
  return plan ? (long long)((BatchPlan*)plan)->graph_nodes : 0;
}
