"""SciPy-style solver objects over the native library (drop-in for MPDOK's mpdok_ops.py).

``MPDOKSolver`` calls the reference-compatible ``py_gmres_ir`` symbol and
``LUIRSolver`` the ``py_lu_*`` symbols of libmpdok_gb300.so, through ctypes,
exactly as mpdok_ops.py binds mpdok.so / lu_ir.so: device pointers, A in
Fortran order, an int out-parameter for convergence, a null-stream
synchronise after the call, RuntimeWarning on non-convergence and a
ResourceWarning + re-raise on device out-of-memory.

Arrays are PyTorch CUDA tensors (NumPy inputs are uploaded); solutions are
FP64 CUDA tensors.
"""
from __future__ import annotations

import ctypes
import os
import warnings

import torch

from . import _native as N
from ._device import as_fortran, as_vector, fortran_empty, require_cuda


class _CudaArrayView:
    """__cuda_array_interface__ for a raw (N, N) Fortran-order FP64 device pointer."""

    def __init__(self, p: int, n: int):
        self.__cuda_array_interface__ = {
            "shape": (n, n), "typestr": "<f8", "data": (p, False), "version": 3, "strides": (8, 8 * n),
        }


class _ManagedArray:
    """Torch tensor view of a managed (N, N) FP64 allocation owned by the library.

    mpdok_ops.py:34-66: the lifetime is controlled by the owning solver's
    free_managed(), not by the tensor's reference count.
    """

    def __init__(self, tensor, free_fn):
        self._arr = tensor
        self._free_fn = free_fn
        self._freed = False

    def __getattr__(self, name):
        return getattr(self._arr, name)

    def __setitem__(self, key, value):
        self._arr[key] = value

    def __getitem__(self, key):
        return self._arr[key]

    @property
    def array(self):
        return self._arr

    def free(self):
        if not self._freed:
            self._free_fn()
            self._freed = True

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def _wrap_managed(p: int, n: int) -> torch.Tensor:
    return torch.as_tensor(_CudaArrayView(p, n), device=require_cuda())


def _default_lib(lib_path):
    if lib_path is None:
        return N.load()
    if not os.path.exists(lib_path):
        raise FileNotFoundError(f"{lib_path} not found. Build libmpdok_gb300.so first.")
    return N.load(lib_path)


def _clear_error(lib):
    fn = getattr(lib, "mpdok_clear_error", None)
    if fn is not None:
        fn()


def _why(lib) -> str:
    """' (library error: ...)' when the last py_* call failed rather than not converging."""
    msg = N.call_error(lib)
    return f" (library error: {msg})" if msg else ""


def _oom_warning(A, N_):
    needed_gb = N_ * N_ * 12 / 1e9
    warnings.warn(
        f"VRAM insufficient for N={N_} ({needed_gb:.1f} GB needed). "
        "Use solver.alloc_managed(N) to build the matrix in CUDA managed "
        "memory from the start — no host-to-device transfer required.",
        ResourceWarning, stacklevel=3)


class MPDOKSolver:
    """GMRES-IR on sm_103a wrapped as a SciPy-style solver (mpdok_ops.py:323-508).

    ``solve(A, b)`` converts A to FP32 into a caller-owned scratch, runs FP32
    GMRES inner cycles (two-pass Gram-Schmidt, FP64 Givens) with FP64
    residuals and FP64 updates, and returns x as an FP64 CUDA tensor.
    """

    def __init__(self, lib_path=None):
        self._lib = _default_lib(lib_path)
        self._managed = None
        self._fp32_buf = None

    # -- managed memory ---------------------------------------------------
    def alloc_managed(self, N_):
        """(N, N) FP64 matrix for the solver (py_alloc_managed): device memory on
        GB300, managed memory placed on the device only if that does not fit."""
        p = ctypes.c_void_p()
        self._lib.py_alloc_managed(ctypes.c_int(N_), ctypes.byref(p))
        if not p.value:
            raise MemoryError(f"py_alloc_managed failed for N={N_}")
        managed = _ManagedArray(_wrap_managed(p.value, N_), self._lib.py_free_managed)
        self._managed = managed
        return managed

    def free_managed(self):
        if self._managed is not None:
            self._managed.free()
            self._managed = None
        else:
            self._lib.py_free_managed()

    def free_fp32_buf(self):
        """Release the FP32 scratch and return cached blocks to the driver."""
        self._fp32_buf = None
        torch.cuda.empty_cache()

    # -- solve --------------------------------------------------------------
    def solve(self, A, b, tol=1e-11, maxiter_outer=5, restart=50):
        try:
            return self._solve(A, b, tol, maxiter_outer, restart)
        except torch.cuda.OutOfMemoryError:
            A_arr = A.array if isinstance(A, _ManagedArray) else A
            _oom_warning(A, int(A_arr.shape[0]))
            raise

    def _solve(self, A, b, tol, maxiter_outer, restart):
        is_managed = isinstance(A, _ManagedArray)
        A_gpu = A.array if is_managed else as_fortran(A, torch.float64)
        b_gpu = as_vector(b, torch.float64)
        n = int(A_gpu.shape[0])
        if tuple(A_gpu.shape) != (n, n):
            raise ValueError(f"A must be square (N×N), got {tuple(A_gpu.shape)}")
        if tuple(b_gpu.shape) != (n,):
            raise ValueError(f"b must be (N,), got {tuple(b_gpu.shape)}")
        if self._fp32_buf is None or tuple(self._fp32_buf.shape) != (n, n):
            self._fp32_buf = fortran_empty(n, n, torch.float32)
        x_gpu = torch.zeros(n, dtype=torch.float64, device=b_gpu.device)
        converged = ctypes.c_int(0)
        _clear_error(self._lib)
        self._lib.py_gmres_ir(
            ctypes.c_void_p(A_gpu.data_ptr()), ctypes.c_void_p(b_gpu.data_ptr()), ctypes.c_void_p(x_gpu.data_ptr()),
            ctypes.c_void_p(self._fp32_buf.data_ptr()), ctypes.c_int(n), ctypes.c_double(tol),
            ctypes.c_int(maxiter_outer), ctypes.c_int(restart), ctypes.byref(converged))
        torch.cuda.synchronize()
        if not converged.value:
            warnings.warn(
                f"GMRES-IR did not converge to tol={tol:.1e} within {maxiter_outer} outer iterations. "
                f"Try increasing maxiter_outer or restart.{_why(self._lib)}",
                RuntimeWarning, stacklevel=3)
        return x_gpu


class LUIRSolver:
    """LU with FP64 iterative refinement over the lu_ir.so symbols (mpdok_ops.py:69-320).

    ``factor(A)`` keeps one process-wide FP32 factorization in the library
    (blocked LU on sm_103a with partial pivoting by rows, as Sgetrf);
    ``solve_factored(b)`` refines with FP64 residuals; ``solve(A, b)`` does
    both.  ``factor`` raises when LAPACK's info is not 0 (an exactly zero
    pivot).  For BF16 / FP16 tensor-core factors use
    ``mpdok_gb300.lu.LUFactorization`` instead.
    """

    def __init__(self, lib_path=None):
        self._lib = _default_lib(lib_path)
        self._managed = None

    # -- managed memory ---------------------------------------------------
    def alloc_managed(self, N_):
        p = ctypes.c_void_p()
        self._lib.py_lu_alloc_managed(ctypes.c_int(N_), ctypes.byref(p))
        if not p.value:
            raise MemoryError(f"py_lu_alloc_managed failed for N={N_}")
        managed = _ManagedArray(_wrap_managed(p.value, N_), self._lib.py_lu_free_managed)
        self._managed = managed
        return managed

    def free_managed(self):
        if self._managed is not None:
            self._managed.free()
            self._managed = None
        else:
            self._lib.py_lu_free_managed()

    # -- factor once, solve many ---------------------------------------------
    def factor(self, A):
        A_arr = A.array if isinstance(A, _ManagedArray) else A
        A_gpu = as_fortran(A_arr, torch.float64)
        n = int(A_gpu.shape[0])
        self._factored_A = A_gpu
        self._factored_N = n
        info = ctypes.c_int(0)
        self._lib.py_lu_factor(ctypes.c_void_p(A_gpu.data_ptr()), ctypes.c_int(n), ctypes.byref(info))
        torch.cuda.synchronize()
        if info.value != 0:
            raise RuntimeError(f"py_lu_factor failed: info={info.value}")

    def solve_factored(self, b, tol=1e-11, maxiter_outer=3):
        if not hasattr(self, "_factored_A"):
            raise RuntimeError("Call factor(A) before solve_factored(b).")
        A_gpu = self._factored_A
        b_gpu = as_vector(b, torch.float64)
        n = int(A_gpu.shape[0])
        x_gpu = torch.zeros(n, dtype=torch.float64, device=b_gpu.device)
        converged = ctypes.c_int(0)
        _clear_error(self._lib)
        self._lib.py_lu_solve_factored(
            ctypes.c_void_p(A_gpu.data_ptr()), ctypes.c_void_p(b_gpu.data_ptr()), ctypes.c_void_p(x_gpu.data_ptr()),
            ctypes.c_int(n), ctypes.c_double(tol), ctypes.c_int(maxiter_outer), ctypes.byref(converged))
        torch.cuda.synchronize()
        if converged.value == -1:
            raise RuntimeError("solve_factored: no factorization available — call factor(A) first.")
        if not converged.value:
            warnings.warn(f"LU-IR solve_factored did not converge to tol={tol:.1e} within {maxiter_outer} outer "
                          f"iterations.{_why(self._lib)}", RuntimeWarning, stacklevel=2)
        return x_gpu

    def free_factored(self):
        self._lib.py_lu_free_factored()
        if hasattr(self, "_factored_A"):
            del self._factored_A
            del self._factored_N

    # -- solve ----------------------------------------------------------------
    def solve(self, A, b, tol=1e-11, maxiter_outer=3):
        try:
            return self._solve(A, b, tol, maxiter_outer)
        except torch.cuda.OutOfMemoryError:
            A_arr = A.array if isinstance(A, _ManagedArray) else A
            _oom_warning(A, int(A_arr.shape[0]))
            raise

    def _solve(self, A, b, tol, maxiter_outer):
        is_managed = isinstance(A, _ManagedArray)
        A_gpu = A.array if is_managed else as_fortran(A, torch.float64)
        b_gpu = as_vector(b, torch.float64)
        n = int(A_gpu.shape[0])
        if tuple(A_gpu.shape) != (n, n):
            raise ValueError(f"A must be square (N×N), got {tuple(A_gpu.shape)}")
        if tuple(b_gpu.shape) != (n,):
            raise ValueError(f"b must be (N,), got {tuple(b_gpu.shape)}")
        x_gpu = torch.zeros(n, dtype=torch.float64, device=b_gpu.device)
        converged = ctypes.c_int(0)
        _clear_error(self._lib)
        self._lib.py_lu_ir(ctypes.c_void_p(A_gpu.data_ptr()), ctypes.c_void_p(b_gpu.data_ptr()),
                           ctypes.c_void_p(x_gpu.data_ptr()), ctypes.c_int(n), ctypes.c_double(tol),
                           ctypes.c_int(maxiter_outer), ctypes.byref(converged))
        torch.cuda.synchronize()
        if not converged.value:
            warnings.warn(f"LU-IR did not converge to tol={tol:.1e} within {maxiter_outer} outer iterations."
                          f"{_why(self._lib)}", RuntimeWarning, stacklevel=3)
        return x_gpu
