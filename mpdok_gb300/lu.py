"""Blocked LU on sm_103a (BF16 / FP16 tensor-core trailing update, FP32 panels).

``LUFactorization(A, dtype)`` factors W = D A D (D = diag(1/sqrt|a_ii|)) with
128-wide FP32 panels and a tcgen05 trailing update whose operands are rounded
to BF16 or FP16 (FP32 accumulation).  ``dtype='fp32'`` keeps FP32 operands and
runs the update on CUDA cores (the reference's Sgetrf precision).
``pivoting=True`` equilibrates rows and columns by powers of two and pivots by
rows (P Dr A Dc = L U), the reference's cusolverDnSgetrf semantics.

The factorization is then used as
* a direct refinement solver: ``solve_ir`` (LU-IR, benchmark_mpdok.ipynb:982-993),
* a right preconditioner of FP32 GMRES inside FP64 refinement: ``gmres_ir``
  (three-precision GMRES-IR).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _native as N
from ._device import Workspace, as_columns, as_fortran, as_vector, fortran_empty, ptr, stream_handle

DTYPES = {"bf16": N.BF16, "bfloat16": N.BF16, "fp16": N.F16, "float16": N.F16, "half": N.F16,
          "fp32": N.F32, "float32": N.F32}


def _info(info: N.SolveInfo) -> dict:
    return {"converged": bool(info.converged), "outer_iters": int(info.outer_iters),
            "inner_iters": int(info.inner_iters), "relres": float(info.relres), "history": info.history_list(),
            "diverged": int(info.stagnated) == 2}


class LUFactorization:
    """Factors of one dense matrix, owned in a device buffer."""

    def __init__(self, A, dtype: str = "fp16", pivoting: bool = False, work: Workspace | None = None):
        """pivoting=False: W = D A D with D = diag(1/sqrt|a_ii|), no row exchanges
        (SPD / diagonally dominant systems; tiny pivots perturbed, counted in
        ``n_perturbed``).  pivoting=True: power-of-two row / column
        equilibration and partial pivoting by rows, P (Dr A Dc) = L U as
        LAPACK getrf; ``info`` is LAPACK's (first exactly zero pivot, 1-based)."""
        self.fdtype = DTYPES[dtype]
        self.pivoting = bool(pivoting)
        self.dtype = dtype
        A64 = as_fortran(A, torch.float64)
        self.n = n = int(A64.shape[0])
        lib = N.load()
        self.factors = torch.empty(max(256, lib.mpdok_lu_factor_size(n, self.fdtype)), dtype=torch.uint8,
                                   device=A64.device)
        ws = work or Workspace()
        w = ws.get(lib.mpdok_lu_work_size(n, self.fdtype))
        st = lib.mpdok_lu_factor(ptr(A64), n, n, self.fdtype, 1 if self.pivoting else 0, ptr(self.factors),
                                 self.factors.numel(), ptr(w), w.numel(), stream_handle())
        N.check(st, "lu_factor")
        self.n_perturbed = 0 if self.pivoting else int(st)
        self.info = int(st) if self.pivoting else 0
        self._ws = Workspace()

    def export(self):
        """(LU, ipiv, perm, dr, dc) as CUDA tensors: L\\U column-major FP32 (unit L
        below the diagonal), LAPACK's 0-based pivot rows, the gather
        permutation ((P x)_i = x[perm[i]]) and the scalings, P (Dr A Dc) = L U."""
        n = self.n
        dev = self.factors.device
        LU = fortran_empty(n, n, torch.float32, dev)
        ipiv = torch.empty(n, dtype=torch.int32, device=dev)
        perm = torch.empty(n, dtype=torch.int32, device=dev)
        dr = torch.empty(n, dtype=torch.float32, device=dev)
        dc = torch.empty(n, dtype=torch.float32, device=dev)
        N.check(N.load().mpdok_lu_export(ptr(self.factors), n, self.fdtype, ptr(LU), n, ptr(ipiv), ptr(perm),
                                         ptr(dr), ptr(dc), stream_handle()), "lu_export")
        return LU, ipiv, perm, dr, dc

    def apply(self, v) -> torch.Tensor:
        """z = A^-1 v through the factors (FP32 vectors)."""
        v32 = as_vector(v, torch.float32)
        z = torch.empty_like(v32)
        lib = N.load()
        w = self._ws.get(lib.mpdok_lu_apply_work_size(self.n))
        N.check(lib.mpdok_lu_apply(ptr(self.factors), self.n, self.fdtype, ptr(v32), ptr(z), ptr(w), w.numel(),
                                   stream_handle()), "lu_apply")
        return z

    def solve_ir(self, A, b, tol: float = 1e-11, maxiter_outer: int = 3):
        """LU-IR: x = LU^-1 b, then FP64 residual / correction solve / FP64 update."""
        A64 = as_fortran(A, torch.float64)
        b64 = as_vector(b)
        x = torch.zeros(self.n, dtype=torch.float64, device=b64.device)
        lib = N.load()
        w = self._ws.get(lib.mpdok_lu_ir_work_size(self.n))
        info = N.SolveInfo()
        N.check(lib.mpdok_lu_ir_solve(ptr(A64), self.n, self.n, ptr(self.factors), self.fdtype, ptr(b64), ptr(x),
                                      float(tol), int(maxiter_outer), ptr(w), w.numel(), ctypes.byref(info),
                                      stream_handle()), "lu_ir_solve")
        return x, _info(info)

    def solve_ir_many(self, A, B, tol: float = 1e-11, maxiter_outer: int = 3):
        """LU-IR for many right-hand sides at once (columns of B), 8 per sweep.

        Returns (X (n, k) FP64, info) with info["relres"] the worst column and
        info["converged"] true when every column met tol.
        """
        A64 = as_fortran(A, torch.float64)
        Bc = as_columns(B, torch.float64)
        k = Bc.shape[1]
        X = fortran_empty(self.n, k, torch.float64)
        lib = N.load()
        worst, conv, outer = 0.0, True, 0
        hist = []
        for j0 in range(0, k, 8):
            kk = min(8, k - j0)
            Bj = Bc[:, j0:j0 + kk]
            w = self._ws.get(lib.mpdok_lu_ir_multi_work_size(self.n, kk))
            info = N.SolveInfo()
            N.check(lib.mpdok_lu_ir_solve_multi(ptr(A64), self.n, self.n, ptr(self.factors), self.fdtype, kk,
                                                ptr(Bj), Bc.stride(1) if k > 1 else self.n, ptr(X[:, j0:j0 + kk]),
                                                self.n, float(tol), int(maxiter_outer), ptr(w), w.numel(),
                                                ctypes.byref(info), stream_handle()), "lu_ir_solve_multi")
            worst = max(worst, float(info.relres))
            conv = conv and bool(info.converged)
            outer = max(outer, int(info.outer_iters))
            hist.append(info.history_list())
        squeeze = (B.dim() == 1) if isinstance(B, torch.Tensor) else (np.asarray(B).ndim == 1)
        return (X.reshape(-1) if squeeze else X), {"converged": conv, "relres": worst, "outer_iters": outer,
                                                   "history": hist}

    def gmres_ir(self, A, b, A32=None, tol: float = 1e-12, maxiter_outer: int = 10, restart: int = 30,
                 inner_tol: float = 1e-6):
        """Three-precision GMRES-IR preconditioned by these factors."""
        A64 = as_fortran(A, torch.float64)
        if A32 is None:
            A32 = fortran_empty(self.n, self.n, torch.float32)
            N.check(N.load().mpdok_convert(ptr(A64), N.F64, ptr(A32), N.F32, self.n * self.n, stream_handle()),
                    "convert")
        b64 = as_vector(b)
        x = torch.zeros(self.n, dtype=torch.float64, device=b64.device)
        lib = N.load()
        w = self._ws.get(lib.mpdok_lu_gmres_ir_work_size(self.n, restart))
        info = N.SolveInfo()
        N.check(lib.mpdok_lu_gmres_ir(ptr(A64), self.n, ptr(A32), self.n, self.n, ptr(self.factors), self.fdtype,
                                      ptr(b64), ptr(x), float(tol), int(maxiter_outer), int(restart),
                                      float(inner_tol), ptr(w), w.numel(), ctypes.byref(info), stream_handle()),
                "lu_gmres_ir")
        return x, _info(info)


def gemm_update(C: torch.Tensor, A16: torch.Tensor, B16: torch.Tensor, engine: str = "tensor") -> torch.Tensor:
    """C (FP32 column-major) -= A16 @ B16^T with K-major BF16/FP16 operands (the LU trailing update)."""
    M, K = A16.shape
    Nn = B16.shape[0]
    fd = N.BF16 if A16.dtype == torch.bfloat16 else N.F16
    err = torch.zeros(4, dtype=torch.int32, device=C.device)
    N.check(N.load().mpdok_gemm_update(ptr(C), C.stride(1) if Nn > 1 else M, ptr(A16.contiguous()),
                                       ptr(B16.contiguous()), M, Nn, K, fd,
                                       N.ENGINE_TENSOR if engine == "tensor" else N.ENGINE_SIMT, ptr(err),
                                       stream_handle()), "gemm_update")
    if int(err[0].item()) != 0:
        raise N.MPDOKError(N.ERR_TIMEOUT, "tensor-core update reported a timed-out wait")
    return C
