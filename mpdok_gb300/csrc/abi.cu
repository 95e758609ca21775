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
  cudaError_t e = cudaMallocManaged(&p, (size_t)N * (size_t)N * sizeof(double), cudaMemAttachGlobal);
  if (e != cudaSuccess) {
    cuda_status(e, "py_alloc_managed");
    return;
  }
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
