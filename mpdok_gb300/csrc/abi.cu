// The reference's ctypes ABI (mpdok.so symbols, mpdok_ops.py:361-382).
//
// These entry points keep the reference's calling convention: device or
// managed pointers, column-major A, void return, status via int* out-params,
// the caller synchronises the null stream afterwards.  Like the reference they
// hold process-wide state (one managed matrix, a cached Krylov workspace); the
// handle-free mpdok_* functions underneath hold none.
#include "common.cuh"

#include <mutex>

namespace mpdok {

struct AbiState {
  std::mutex mu;
  void* managed = nullptr;       // py_alloc_managed
  void* work = nullptr;          // cached Krylov workspace for py_gmres_ir
  size_t work_bytes = 0;
};

AbiState& abi_state() {
  static AbiState st;
  return st;
}

int abi_workspace(AbiState& st, size_t need, void** out) {
  if (st.work_bytes < need) {
    if (st.work) cudaFree(st.work);
    st.work = nullptr;
    st.work_bytes = 0;
    MPDOK_CUDA_TRY(cudaMalloc(&st.work, need));
    st.work_bytes = need;
  }
  *out = st.work;
  return MPDOK_OK;
}

}  // namespace mpdok

using namespace mpdok;

extern "C" void py_gmres_ir(double* A, double* b, double* x, float* A_fp32, int N, double tol, int maxiter_outer,
                            int restart, int* converged_out) {
  if (converged_out) *converged_out = 0;
  if (N <= 0) {
    if (converged_out) *converged_out = (N == 0);
    return;
  }
  AbiState& st = abi_state();
  std::lock_guard<std::mutex> lk(st.mu);
  if (restart < 1) restart = 1;
  if (restart > 1024) restart = 1024;
  void* work = nullptr;
  if (abi_workspace(st, mpdok_krylov_workspace_size(N, restart), &work) != MPDOK_OK) return;
  mpdok_solve_info info;
  // mpdok_ooc.py:299 stops each inner cycle at |g_{k+1}| / beta < 1e-6.
  int s = mpdok_gmres_ir(A, N, A_fp32, N, 0, N, b, x, tol, maxiter_outer, restart, 1e-6, work, st.work_bytes,
                         &info, (cudaStream_t)0);
  if (s == MPDOK_OK && converged_out) *converged_out = info.converged;
}

// Storage behind py_alloc_managed / py_lu_alloc_managed (mpdok_ops.py:34-66,
// :147-174, :388-418).  The reference uses managed memory so that an 8 GB card
// can hold A beyond its memory, at the price of page migration (thrashing
// once A exceeds the device).  With 280 GB of HBM, A (N x N FP64) fits up to
// N ~ 180000: the buffer is plain device memory, and only when that
// allocation fails is it managed memory placed on the device (preferred
// location + prefetch), so that it still runs from HBM as far as it fits.
// Returns 0 for device memory, 1 for managed, -1 on failure.
static int alloc_matrix(size_t bytes, void** p) {
  *p = nullptr;
  if (cudaMalloc(p, bytes) == cudaSuccess) return 0;
  cudaGetLastError();  // clear the allocation failure
  cudaError_t e = cudaMallocManaged(p, bytes, cudaMemAttachGlobal);
  if (e != cudaSuccess) {
    cuda_status(e, "managed allocation");
    *p = nullptr;
    return -1;
  }
  int dev = 0;
  cudaGetDevice(&dev);
  cudaMemLocation loc;
  loc.type = cudaMemLocationTypeDevice;
  loc.id = dev;
  cudaMemAdvise(*p, bytes, cudaMemAdviseSetPreferredLocation, loc);
  cudaMemPrefetchAsync(*p, bytes, loc, 0, (cudaStream_t)0);
  cudaGetLastError();  // advice and prefetch are hints
  return 1;
}

static int g_last_alloc_kind = -1;

extern "C" int mpdok_managed_kind(void) { return g_last_alloc_kind; }

extern "C" void py_alloc_managed(int N, void** ptr_out) {
  if (!ptr_out) return;
  *ptr_out = nullptr;
  if (N <= 0) return;
  AbiState& st = abi_state();
  std::lock_guard<std::mutex> lk(st.mu);
  if (st.managed) {
    cudaFree(st.managed);
    st.managed = nullptr;
  }
  void* p = nullptr;
  g_last_alloc_kind = alloc_matrix((size_t)N * (size_t)N * sizeof(double), &p);
  if (!p) return;
  st.managed = p;
  *ptr_out = p;
}

extern "C" void py_free_managed(void) {
  AbiState& st = abi_state();
  std::lock_guard<std::mutex> lk(st.mu);
  if (st.managed) {
    cudaDeviceSynchronize();
    cudaFree(st.managed);
    st.managed = nullptr;
  }
}

// ------------------------------------------------- lu_ir.so symbols
// mpdok_ops.py:101-141.  One process-wide saved factorization, as in the
// reference (py_lu_factor keeps it until py_lu_free_factored).  Factors are
// FP32 with partial pivoting by rows (the reference's Sgetrf: L, U and P,
// benchmark_mpdok.ipynb:989-990), so that two or three refinement steps reach
// FP64 accuracy on general non-singular matrices, and info has LAPACK's
// meaning: > 0 is the first exactly zero pivot (1-based).

namespace mpdok {

struct LuAbiState {
  void* factors = nullptr;
  size_t factor_bytes = 0;
  void* work = nullptr;
  size_t work_bytes = 0;
  long long n = -1;
  void* managed = nullptr;
};

static LuAbiState& lu_state() {
  static LuAbiState st;
  return st;
}

static int ensure(void** p, size_t* have, size_t need) {
  if (*have >= need && *p) return MPDOK_OK;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *have = 0;
  MPDOK_CUDA_TRY(cudaMalloc(p, need));
  *have = need;
  return MPDOK_OK;
}

static void lu_release(LuAbiState& st) {
  if (st.factors) cudaFree(st.factors);
  if (st.work) cudaFree(st.work);
  st.factors = st.work = nullptr;
  st.factor_bytes = st.work_bytes = 0;
  st.n = -1;
}

static int lu_factor_global(double* A, int N) {
  LuAbiState& st = lu_state();
  const size_t fb = mpdok_lu_factor_size(N, MPDOK_F32);
  const size_t wb = std::max({mpdok_lu_work_size(N, MPDOK_F32), mpdok_lu_ir_work_size(N)});
  MPDOK_TRY(ensure(&st.factors, &st.factor_bytes, fb));
  MPDOK_TRY(ensure(&st.work, &st.work_bytes, wb));
  st.n = -1;
  const int s = mpdok_lu_factor(A, N, N, MPDOK_F32, 1, st.factors, st.factor_bytes, st.work, st.work_bytes, 0);
  if (s == 0) st.n = N;  // a singular factorization (info > 0) is not kept for solves, as LAPACK getrs would divide by 0
  return s;
}

}  // namespace mpdok

extern "C" void py_lu_factor(double* A, int N, int* info_out) {
  std::lock_guard<std::mutex> lk(abi_state().mu);
  int s = (N <= 0) ? 0 : lu_factor_global(A, N);
  if (N <= 0) lu_state().n = 0;
  if (info_out) *info_out = s;  // > 0: U(s, s) is exactly zero (LAPACK's info), < 0: error
}

extern "C" void py_lu_solve_factored(double* A, double* b, double* x, int N, double tol, int maxiter,
                                     int* converged_out) {
  std::lock_guard<std::mutex> lk(abi_state().mu);
  LuAbiState& st = lu_state();
  if (converged_out) *converged_out = 0;
  if (st.n < 0 || st.n != N) {
    if (converged_out) *converged_out = -1;
    return;
  }
  if (N == 0) {
    if (converged_out) *converged_out = 1;
    return;
  }
  mpdok_solve_info info;
  int s = mpdok_lu_ir_solve(A, N, N, st.factors, MPDOK_F32, b, x, tol, maxiter, st.work, st.work_bytes, &info, 0);
  if (s == MPDOK_OK && converged_out) *converged_out = info.converged;
}

extern "C" void py_lu_ir(double* A, double* b, double* x, int N, double tol, int maxiter, int* converged_out) {
  int info = 0;
  py_lu_factor(A, N, &info);
  if (info != 0) {
    if (info > 0) set_error("LU-IR: U(%d, %d) is exactly zero; the matrix is singular", info, info);
    if (converged_out) *converged_out = 0;
    return;
  }
  py_lu_solve_factored(A, b, x, N, tol, maxiter, converged_out);
}

extern "C" void py_lu_free_factored(void) {
  std::lock_guard<std::mutex> lk(abi_state().mu);
  lu_release(lu_state());
}

extern "C" void py_lu_alloc_managed(int N, void** ptr_out) {
  if (!ptr_out) return;
  *ptr_out = nullptr;
  if (N <= 0) return;
  std::lock_guard<std::mutex> lk(abi_state().mu);
  LuAbiState& st = lu_state();
  if (st.managed) {
    cudaFree(st.managed);
    st.managed = nullptr;
  }
  void* p = nullptr;
  g_last_alloc_kind = alloc_matrix((size_t)N * (size_t)N * sizeof(double), &p);
  if (!p) return;
  st.managed = p;
  *ptr_out = p;
}

extern "C" void py_lu_free_managed(void) {
  std::lock_guard<std::mutex> lk(abi_state().mu);
  LuAbiState& st = lu_state();
  if (st.managed) {
    cudaDeviceSynchronize();
    cudaFree(st.managed);
    st.managed = nullptr;
  }
}
