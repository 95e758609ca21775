"""Dense linear operator and Krylov solvers (CG, GMRES, GMRES-IR) on sm_103a.

Drop-in for MPDOK's dense_krylov.py: same names, arguments, defaults and
return conventions ``(x_fp64, history, converged)``.  The loops run natively
(libmpdok_gb300.so) with the Krylov state on the device; the reference's
per-iteration host round trips are gone, the arithmetic precisions are the
reference's (FP32 operator and Krylov vectors, FP64 residual and update,
FP64 Hessenberg / Givens).
"""
from __future__ import annotations

import ctypes

import torch

from . import _native as N
from ._device import Workspace, as_fortran, as_vector, fortran_empty, ptr, require_cuda, stream_handle


class DenseLinearOperator:
    """Dense matrix held on the device in FP32 (Krylov matvecs) and FP64 (residuals).

    dense_krylov.py:18-112.  ``matvec`` runs the streaming sm_103a GEMV on the
    FP32 copy (exact FP32 products, FP32 accumulation), ``residual_norm`` the
    FP64 residual kernel.  ``free_fp64`` releases the FP64 copy, after which
    ``residual_norm`` raises as in the reference.
    """

    def __init__(self, A, verbose: bool = True):
        shape = tuple(A.shape)
        if len(shape) != 2 or shape[0] != shape[1]:
            raise ValueError(f"A must be square 2-D, got shape {shape}")
        self.N = int(shape[0])
        self.A_fp64 = as_fortran(A.array if hasattr(A, "array") else A, torch.float64)
        self.A_fp32 = fortran_empty(self.N, self.N, torch.float32)
        N.check(N.load().mpdok_convert(ptr(self.A_fp64), N.F64, ptr(self.A_fp32), N.F32, self.N * self.N,
                                       stream_handle()), "convert")
        self._ws = Workspace()
        if verbose:
            mb32 = self.A_fp32.numel() * 4 / 1e6
            mb64 = self.A_fp64.numel() * 8 / 1e6
            print(f"DenseLinearOperator: N={self.N:,}  FP32={mb32:.1f} MB  FP64={mb64:.1f} MB  "
                  f"total={mb32 + mb64:.1f} MB")

    # -- core operations -------------------------------------------------
    def matvec(self, x) -> torch.Tensor:
        """A @ x with the FP32 matrix; x (N,) or (N, k) -> FP32 CUDA tensor of the same shape."""
        xt = x if isinstance(x, torch.Tensor) else torch.as_tensor(x)
        squeeze = xt.dim() == 1
        X = as_fortran(xt.reshape(-1, 1) if squeeze else xt, torch.float32)
        k = X.shape[1]
        Y = fortran_empty(self.N, k, torch.float32)
        lib = N.load()
        wbytes = lib.mpdok_gemv_workspace_size(N.F32, self.N, self.N, k, 0)
        w = self._ws.get(wbytes)
        N.check(lib.mpdok_gemv(N.F32, 0, ptr(self.A_fp32), self.N, self.N, self.N, ptr(X), max(1, self.N), k,
                               ptr(Y), max(1, self.N), 1.0, 0.0, ptr(w), w.numel(), stream_handle()), "matvec")
        return Y.reshape(-1) if squeeze else Y

    def rmatvec(self, x) -> torch.Tensor:
        """A^T @ x with the FP32 matrix (used by the adjoint)."""
        X = as_fortran(torch.as_tensor(x).reshape(-1, 1), torch.float32)
        Y = fortran_empty(self.N, 1, torch.float32)
        lib = N.load()
        wbytes = lib.mpdok_gemv_workspace_size(N.F32, self.N, self.N, 1, 1)
        w = self._ws.get(wbytes)
        N.check(lib.mpdok_gemv(N.F32, 1, ptr(self.A_fp32), self.N, self.N, self.N, ptr(X), self.N, 1, ptr(Y),
                               self.N, 1.0, 0.0, ptr(w), w.numel(), stream_handle()), "rmatvec")
        return Y.reshape(-1)

    def residual_norm(self, x, b) -> float:
        """||b - A @ x||_2 in FP64 (a Python float); raises after free_fp64()."""
        if self.A_fp64 is None:
            raise RuntimeError(
                "FP64 copy was freed; residual_norm() is no longer available. "
                "Reconstruct the operator to recompute residuals.")
        x64 = as_vector(x, torch.float64)
        b64 = as_vector(b, torch.float64)
        r = torch.empty_like(x64)
        nrm2 = torch.empty(1, dtype=torch.float64, device=x64.device)
        lib = N.load()
        w = self._ws.get(lib.mpdok_gemv_workspace_size(N.F64, self.N, self.N, 1, 0))
        N.check(lib.mpdok_residual(ptr(self.A_fp64), self.N, self.N, ptr(b64), ptr(x64), ptr(r), ptr(nrm2), ptr(w),
                                   w.numel(), stream_handle()), "residual")
        return float(nrm2.item()) ** 0.5

    # -- memory management -------------------------------------------------
    def free_fp64(self):
        """Release the FP64 copy; matvec() keeps working, residual_norm() raises."""
        self.A_fp64 = None

    @property
    def shape(self):
        return (self.N, self.N)

    def vram_mb(self) -> float:
        total = self.A_fp32.numel() * 4
        if self.A_fp64 is not None:
            total += self.A_fp64.numel() * 8
        return total / 1e6

    def __repr__(self):
        fp64_state = f"{self.A_fp64.numel() * 8 / 1e6:.1f} MB" if self.A_fp64 is not None else "freed"
        return f"DenseLinearOperator(N={self.N:,}, fp32={self.A_fp32.numel() * 4 / 1e6:.1f} MB, fp64={fp64_state})"


def _require_fp64(op, what):
    if op.A_fp64 is None:
        raise RuntimeError(
            f"{what} requires op.A_fp64 for FP64 residual computation. "
            f"Do not call free_fp64() before {what}().")


def _krylov_ws(op, restart):
    return op._ws.get(N.load().mpdok_krylov_workspace_size(op.N, restart))


def cg(op, b, x0=None, tol: float = 1e-6, maxiter=None, check_every: int = 10, verbose: bool = False):
    """FP32 conjugate gradients with FP64 residual checks (dense_krylov.py:119-205).

    Returns ``(x_fp64, history, converged)``; history holds
    ``(iteration, fp64_relative_residual)`` at every check.
    """
    if getattr(op, "_matrix_free", False):
        return op.cg(b, x0=x0, tol=tol, maxiter=maxiter, check_every=check_every)
    _require_fp64(op, "cg")
    n = op.N
    maxiter = n if maxiter is None else int(maxiter)
    b64 = as_vector(b)
    x = torch.zeros(n, dtype=torch.float64, device=b64.device) if x0 is None else \
        as_vector(x0).to(torch.float32).to(torch.float64)
    info = N.SolveInfo()
    w = _krylov_ws(op, 1)
    N.check(N.load().mpdok_cg(ptr(op.A_fp32), n, ptr(op.A_fp64), n, n, ptr(b64), ptr(x), float(tol), maxiter,
                              int(check_every), ptr(w), w.numel(), ctypes.byref(info), stream_handle()), "cg")
    hist = info.history_list()
    if verbose:
        for it, r in hist:
            print(f"  CG iter {it:4d}  rel_res(FP64) = {r:.3e}")
    return x, hist, bool(info.converged)


def gmres(op, b, x0=None, tol: float = 1e-6, maxiter=None, restart: int = 50, verbose: bool = False):
    """Restarted FP32 GMRES(m) with FP64 checks at every restart (dense_krylov.py:212-331)."""
    _require_fp64(op, "gmres")
    n = op.N
    maxiter = n if maxiter is None else int(maxiter)
    b64 = as_vector(b)
    x = torch.zeros(n, dtype=torch.float64, device=b64.device) if x0 is None else \
        as_vector(x0).to(torch.float32).to(torch.float64)
    info = N.SolveInfo()
    w = _krylov_ws(op, restart)
    N.check(N.load().mpdok_gmres(ptr(op.A_fp32), n, ptr(op.A_fp64), n, n, ptr(b64), ptr(x), float(tol), maxiter,
                                 int(restart), ptr(w), w.numel(), ctypes.byref(info), stream_handle()), "gmres")
    hist = info.history_list()
    if verbose:
        for i, (it, r) in enumerate(hist):
            print(f"  GMRES restart {i + 1:3d}  iters={it:4d}  rel_res(FP64)={r:.3e}")
    return x, hist, bool(info.converged)


def gmres_ir(op, b, tol: float = 1e-11, maxiter_outer: int = 5, restart: int = 50, maxiter_inner=None,
             verbose: bool = False):
    """GMRES with iterative refinement (dense_krylov.py:338-421).

    Outer FP64 residual, inner FP32 GMRES to 1e-6, FP64 update; the history
    holds ``(outer_iter, relres)`` with a final entry at ``maxiter_outer``.
    """
    if getattr(op, "_matrix_free", False):
        return op.gmres_ir(b, tol=tol, maxiter_outer=maxiter_outer, restart=restart)
    _require_fp64(op, "GMRES-IR")
    n = op.N
    b64 = as_vector(b)
    x = torch.zeros(n, dtype=torch.float64, device=b64.device)
    info = N.SolveInfo()
    w = _krylov_ws(op, restart)
    mi = n if maxiter_inner is None else int(maxiter_inner)
    N.check(N.load().mpdok_dense_gmres_ir(ptr(op.A_fp32), n, ptr(op.A_fp64), n, n, ptr(b64), ptr(x), float(tol),
                                          int(maxiter_outer), int(restart), mi, ptr(w), w.numel(),
                                          ctypes.byref(info), stream_handle()), "gmres_ir")
    hist = info.history_list()
    if verbose:
        for it, r in hist:
            print(f"  GMRES-IR outer {it:2d}  rel_res(FP64) = {r:.3e}")
    return x, hist, bool(info.converged)


def cg_ir(op, B, tol: float = 1e-12, maxiter_outer: int = 10, inner_tol: float = 1e-6, inner_maxiter: int = 500,
          split: bool = False, precond=None):
    """Multi-RHS CG with FP64 refinement (the FP32 CG body of dense_krylov.py:119-205
    inside the refinement loop of :338-421).

    B: (N,) or (N, k<=8).  ``split=True`` stores A as two FP32 slices and forms
    every product with error-free FP32 arithmetic (FP64-level accuracy on the
    FP32 pipe) for both the inner operator and the residual.  ``precond``
    preconditions the inner CG, which an FP32 CG body needs once
    kappa(A) * 6e-8 >= 1: an ``mpdok_gb300.lu.LUFactorization`` (16/32-bit
    factors, for kappa up to about 1e7) or an
    ``mpdok_gb300.batch.CholeskyPreconditioner`` (FP64-accurate Cholesky, for
    the C2 family at kappa ~ 1e8).
    Returns ``(X_fp64, history, converged)``; history holds the worst column.
    """
    if getattr(op, "_matrix_free", False):
        return op.cg_ir(B, tol=tol, maxiter_outer=maxiter_outer, inner_tol=inner_tol, inner_maxiter=inner_maxiter,
                        precond=precond)
    _require_fp64(op, "cg_ir")
    from ._device import as_columns
    n = op.N
    Bc = as_columns(B, torch.float64)
    k = Bc.shape[1]
    if k > 8:
        raise ValueError("cg_ir handles up to 8 right-hand sides per call")
    X = fortran_empty(n, k, torch.float64)
    lib = N.load()
    mode = 1 if split else 0
    ld4 = (n + 3) // 4 * 4
    if mode == 0 and ld4 == n:
        opbuf, ready = op.A_fp32, 1
    else:
        cache = getattr(op, "_cgir_opbuf", None)
        if cache is None or cache[0] != mode:
            buf = torch.empty(lib.mpdok_cg_ir_operator_size(n, mode), dtype=torch.uint8, device=Bc.device)
            op._cgir_opbuf = (mode, buf)
            ready = 0
        else:
            buf, ready = cache[1], 1
        opbuf = buf
    info = N.SolveInfo()
    if precond is not None and hasattr(precond, "plan"):
        # FP64-accurate Cholesky (batch plan of one system) as the inner PCG's preconditioner
        if precond.n != n or precond.nrhs != k:
            raise ValueError(f"the Cholesky preconditioner holds n={precond.n}, nrhs={precond.nrhs}; "
                             f"this solve has n={n}, nrhs={k}")
        w = op._ws.get(lib.mpdok_chol_cg_ir_workspace_size(n, k, mode))
        N.check(lib.mpdok_chol_cg_ir(precond.plan, ptr(op.A_fp64), n, None, 0, 0, 0.0, 0.0, n, mode, ptr(opbuf), ready,
                                     k, ptr(Bc), n, ptr(X), n, float(tol), int(maxiter_outer), float(inner_tol),
                                     int(inner_maxiter), ptr(w), w.numel(), ctypes.byref(info), stream_handle()),
                "chol_cg_ir")
    elif precond is None:
        w = op._ws.get(lib.mpdok_cg_ir_workspace_size(n, k, mode))
        N.check(lib.mpdok_cg_ir(ptr(op.A_fp64), n, n, mode, ptr(opbuf), ready, k, ptr(Bc), n, ptr(X), n,
                                float(tol), int(maxiter_outer), float(inner_tol), int(inner_maxiter), ptr(w),
                                w.numel(), ctypes.byref(info), stream_handle()), "cg_ir")
    else:
        w = op._ws.get(lib.mpdok_lu_cg_ir_workspace_size(n, k, mode))
        N.check(lib.mpdok_lu_cg_ir(ptr(op.A_fp64), n, n, mode, ptr(opbuf), ready, ptr(precond.factors),
                                   precond.fdtype, k, ptr(Bc), n, ptr(X), n, float(tol), int(maxiter_outer),
                                   float(inner_tol), int(inner_maxiter), ptr(w), w.numel(), ctypes.byref(info),
                                   stream_handle()), "lu_cg_ir")
    hist = info.history_list()
    return (X.reshape(-1) if torch.as_tensor(B).dim() == 1 else X), hist, bool(info.converged)
