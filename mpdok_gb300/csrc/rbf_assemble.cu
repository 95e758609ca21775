// Fused RBF kernel-matrix assembly (Gaussian / multiquadric) for sm_103a.
//
// Replaces the chunked GEMM-identity build of rbf_kernel.py:158-227
// (DGEMM c_chunk @ coords.T, broadcast add, cp.maximum, cp.exp, then the
// A[idx,idx] += reg scatter at :223-224) and the FP32 tile build of
// mpdok_ooc.py:39-46 with ONE pass that writes each output entry once.
//
// Entry (i, j) = phi(||r_i - c_j||) + reg * [i + diag_offset == j], with
//   Gaussian      phi = exp(-gamma d^2)          (rbf_kernel.py:162)
//   multiquadric  phi = sqrt(1 + gamma d^2)      (gamma = eps^2)
// d^2 is summed from coordinate differences (D <= 3 here, so 3 FMAs per
// entry instead of the identity's cancellation-prone |a|^2+|b|^2-2ab).
//
// FP64 output computes in FP64 (the reference's arithmetic).  FP32 / BF16 /
// FP16 outputs compute d^2 and phi in FP32: the stored operator only needs
// FP32 accuracy and GB300's FP64 pipe is narrow.
#include "common.cuh"

namespace mpdok {

constexpr int ASM_ROWS = 128;  // rows per block (4 per thread x 32 lanes)
constexpr int ASM_COLS = 64;   // columns per block (8 warps x 8 columns)

// Diagonal nugget of the FP64-math path: FP64 output adds it in FP64; FP32
// output rounds phi first and adds the nugget in FP32, the order of
// mpdok_ooc.py:45,122 (astype(float32), then tile[k, i+k] += reg).
template <typename OutT>
__device__ __forceinline__ double nugget(double v, double reg) {
  if (std::is_same<OutT, float>::value) return (double)((float)v + (float)reg);
  return v + reg;
}

template <int D, int KIND, typename OutT, bool COLMAJOR, bool F64MATH>
__global__ void __launch_bounds__(256)
rbf_assemble_kernel(const double* __restrict__ R, long long nr,
                    const double* __restrict__ C, long long nc,
                    double gamma, double reg, long long diag_off,
                    OutT* __restrict__ out, long long ld) {
  using CT = typename std::conditional<F64MATH, double, float>::type;  // coordinate type in shared memory
  __shared__ CT sR[ASM_ROWS * D];
  __shared__ CT sC[ASM_COLS * D];
  const long long r0 = (long long)blockIdx.x * ASM_ROWS;
  const long long c0 = (long long)blockIdx.y * ASM_COLS;
  for (int t = threadIdx.x; t < ASM_ROWS * D; t += blockDim.x) {
    long long i = r0 + t / D;
    sR[t] = (CT)((i < nr) ? R[i * D + (t % D)] : 0.0);
  }
  for (int t = threadIdx.x; t < ASM_COLS * D; t += blockDim.x) {
    long long j = c0 + t / D;
    sC[t] = (CT)((j < nc) ? C[j * D + (t % D)] : 0.0);
  }
  __syncthreads();

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (COLMAJOR) {
    // lane -> rows (coalesced down a column), warp -> 8 columns
#pragma unroll 1
    for (int cc = 0; cc < 8; ++cc) {
      const int jl = warp * 8 + cc;
      const long long j = c0 + jl;
      if (j >= nc) break;
#pragma unroll
      for (int rr = 0; rr < 4; ++rr) {
        const int il = rr * 32 + lane;
        const long long i = r0 + il;
        if (i >= nr) continue;
        double v;
        if (F64MATH) {
          double d2 = 0.0;
#pragma unroll
          for (int k = 0; k < D; ++k) { double t = (double)sR[il * D + k] - (double)sC[jl * D + k]; d2 = fma(t, t, d2); }
          v = (KIND == MPDOK_KERNEL_GAUSSIAN) ? exp(-gamma * d2) : sqrt(fma(gamma, d2, 1.0));
          if (i + diag_off == j) v = nugget<OutT>(v, reg);
        } else {
          float d2 = 0.f;
#pragma unroll
          for (int k = 0; k < D; ++k) { float t = (float)sR[il * D + k] - (float)sC[jl * D + k]; d2 = fmaf(t, t, d2); }
          float vf = (KIND == MPDOK_KERNEL_GAUSSIAN) ? expf(-(float)gamma * d2) : sqrtf(fmaf((float)gamma, d2, 1.f));
          if (i + diag_off == j) vf += (float)reg;
          v = vf;
        }
        out[i + j * ld] = F64MATH ? from_f64<OutT>(v) : from_f32<OutT>((float)v);
      }
    }
  } else {
    // row-major: lane -> columns (coalesced along a row), warp -> 16 rows
#pragma unroll 1
    for (int rr = 0; rr < 16; ++rr) {
      const int il = warp * 16 + rr;
      const long long i = r0 + il;
      if (i >= nr) break;
#pragma unroll
      for (int cc = 0; cc < 2; ++cc) {
        const int jl = cc * 32 + lane;
        const long long j = c0 + jl;
        if (j >= nc) continue;
        double v;
        if (F64MATH) {
          double d2 = 0.0;
#pragma unroll
          for (int k = 0; k < D; ++k) { double t = (double)sR[il * D + k] - (double)sC[jl * D + k]; d2 = fma(t, t, d2); }
          v = (KIND == MPDOK_KERNEL_GAUSSIAN) ? exp(-gamma * d2) : sqrt(fma(gamma, d2, 1.0));
          if (i + diag_off == j) v = nugget<OutT>(v, reg);
        } else {
          float d2 = 0.f;
#pragma unroll
          for (int k = 0; k < D; ++k) { float t = (float)sR[il * D + k] - (float)sC[jl * D + k]; d2 = fmaf(t, t, d2); }
          float vf = (KIND == MPDOK_KERNEL_GAUSSIAN) ? expf(-(float)gamma * d2) : sqrtf(fmaf((float)gamma, d2, 1.f));
          if (i + diag_off == j) vf += (float)reg;
          v = vf;
        }
        out[i * ld + j] = F64MATH ? from_f64<OutT>(v) : from_f32<OutT>((float)v);
      }
    }
  }
}

template <int D, int KIND, typename OutT>
static void launch_asm(const double* R, long long nr, const double* C, long long nc, double gamma,
                       double reg, long long diag_off, void* out, long long ld, bool colmajor,
                       cudaStream_t s) {
  dim3 grid((unsigned)((nr + ASM_ROWS - 1) / ASM_ROWS), (unsigned)((nc + ASM_COLS - 1) / ASM_COLS));
  constexpr bool F64 = std::is_same<OutT, double>::value;
  if (colmajor)
    launch(rbf_assemble_kernel<D, KIND, OutT, true, F64>, grid, 256, 0, s, R, nr, C, nc, gamma, reg, diag_off, (OutT*)out, ld);
  else
    launch(rbf_assemble_kernel<D, KIND, OutT, false, F64>, grid, 256, 0, s, R, nr, C, nc, gamma, reg, diag_off, (OutT*)out, ld);
}

// FP32 row-major tile computed in FP64 and rounded once (the reference's
// out-of-core tile, mpdok_ooc.py:39-46).
template <int D, int KIND>
static void launch_f32_exact(const double* R, long long nr, const double* C, long long nc, double gamma, double reg,
                             long long diag_off, float* out, long long ld, cudaStream_t s) {
  dim3 grid((unsigned)((nr + ASM_ROWS - 1) / ASM_ROWS), (unsigned)((nc + ASM_COLS - 1) / ASM_COLS));
  launch(rbf_assemble_kernel<D, KIND, float, false, true>, grid, 256, 0, s, R, nr, C, nc, gamma, reg, diag_off, out, ld);
}

template <int D, int KIND>
static int dispatch_dtype(int dt, const double* R, long long nr, const double* C, long long nc, double gamma,
                          double reg, long long doff, void* out, long long ld, bool cm, cudaStream_t s) {
  switch (dt) {
    case MPDOK_F64: launch_asm<D, KIND, double>(R, nr, C, nc, gamma, reg, doff, out, ld, cm, s); break;
    case MPDOK_F32: launch_asm<D, KIND, float>(R, nr, C, nc, gamma, reg, doff, out, ld, cm, s); break;
    case MPDOK_BF16: launch_asm<D, KIND, __nv_bfloat16>(R, nr, C, nc, gamma, reg, doff, out, ld, cm, s); break;
    case MPDOK_F16: launch_asm<D, KIND, __half>(R, nr, C, nc, gamma, reg, doff, out, ld, cm, s); break;
    default: set_error("rbf_assemble: unknown out dtype %d", dt); return MPDOK_ERR_INVALID_ARG;
  }
  return MPDOK_OK;
}

int rbf_tile_f32_from_f64(const double* rows, long long n_rows, const double* cols, long long n_cols, int dim,
                          int kernel, double gamma, double reg, long long diag_offset, float* out, long long ld,
                          cudaStream_t s) {
  MPDOK_ARG_CHECK(dim >= 1 && dim <= 3, "dim must be 1, 2 or 3");
  MPDOK_ARG_CHECK(kernel == MPDOK_KERNEL_GAUSSIAN || kernel == MPDOK_KERNEL_MQ, "unknown kernel");
  MPDOK_ARG_CHECK(ld >= n_cols && (n_cols + ASM_COLS - 1) / ASM_COLS < 65536, "bad tile shape");
  if (n_rows == 0 || n_cols == 0) return MPDOK_OK;
  const int pslot = prof_start(MPDOK_PROF_ASSEMBLE, s);
  const bool g = kernel == MPDOK_KERNEL_GAUSSIAN;
  if (dim == 1) (g ? launch_f32_exact<1, MPDOK_KERNEL_GAUSSIAN> : launch_f32_exact<1, MPDOK_KERNEL_MQ>)(
      rows, n_rows, cols, n_cols, gamma, reg, diag_offset, out, ld, s);
  else if (dim == 2) (g ? launch_f32_exact<2, MPDOK_KERNEL_GAUSSIAN> : launch_f32_exact<2, MPDOK_KERNEL_MQ>)(
      rows, n_rows, cols, n_cols, gamma, reg, diag_offset, out, ld, s);
  else (g ? launch_f32_exact<3, MPDOK_KERNEL_GAUSSIAN> : launch_f32_exact<3, MPDOK_KERNEL_MQ>)(
      rows, n_rows, cols, n_cols, gamma, reg, diag_offset, out, ld, s);
  prof_stop(pslot, s, (double)n_rows * (double)n_cols * 4.0);
  MPDOK_LAUNCH_CHECK("rbf_tile_f32_from_f64");
  return MPDOK_OK;
}

}  // namespace mpdok

using namespace mpdok;

extern "C" int mpdok_rbf_assemble(const double* rows, long long n_rows, const double* cols, long long n_cols,
                                  int dim, int kernel, double gamma, double reg, long long diag_offset,
                                  int out_dtype, void* out, long long ld, int col_major, cudaStream_t stream) {
  MPDOK_ARG_CHECK(n_rows >= 0 && n_cols >= 0, "negative size");
  if (n_rows == 0 || n_cols == 0) return MPDOK_OK;
  MPDOK_ARG_CHECK(rows && cols && out, "null pointer");
  MPDOK_ARG_CHECK(dim >= 1 && dim <= 3, "dim must be 1, 2 or 3");
  MPDOK_ARG_CHECK(kernel == MPDOK_KERNEL_GAUSSIAN || kernel == MPDOK_KERNEL_MQ, "unknown kernel");
  MPDOK_ARG_CHECK(col_major ? ld >= n_rows : ld >= n_cols, "ld too small");
  MPDOK_ARG_CHECK((n_rows + ASM_ROWS - 1) / ASM_ROWS < (1LL << 31) && (n_cols + ASM_COLS - 1) / ASM_COLS < 65536,
                  "matrix too large for one launch");
  int st;
  const int pslot = prof_start(MPDOK_PROF_ASSEMBLE, stream);
#define ASM_CASE(DD)                                                                                     \
  if (dim == DD) {                                                                                       \
    st = (kernel == MPDOK_KERNEL_GAUSSIAN)                                                               \
             ? dispatch_dtype<DD, MPDOK_KERNEL_GAUSSIAN>(out_dtype, rows, n_rows, cols, n_cols, gamma, reg, \
                                                        diag_offset, out, ld, col_major != 0, stream)   \
             : dispatch_dtype<DD, MPDOK_KERNEL_MQ>(out_dtype, rows, n_rows, cols, n_cols, gamma, reg,      \
                                                  diag_offset, out, ld, col_major != 0, stream);        \
  }
  ASM_CASE(1) else ASM_CASE(2) else ASM_CASE(3) else st = MPDOK_ERR_INVALID_ARG;
#undef ASM_CASE
  const int ob = out_dtype == MPDOK_F64 ? 8 : out_dtype == MPDOK_F32 ? 4 : 2;
  prof_stop(pslot, stream, (double)n_rows * (double)n_cols * ob);
  if (st != MPDOK_OK) return st;
  MPDOK_LAUNCH_CHECK("rbf_assemble");
  return MPDOK_OK;
}
