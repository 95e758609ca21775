"""Matrix-free RBF operator: entries recomputed on the fly, A never stored.

``MatrixFreeOperator(coords, gamma, reg, kernel)`` behaves like
``DenseLinearOperator`` (``matvec``, ``residual_norm``) for the RBF system
A = K(coords, coords) + reg I, and ``cg`` / ``gmres_ir`` of
``mpdok_gb300.dense_krylov`` accept it.  The FP32 evaluate-and-multiply
stages centre tiles into shared memory by TMA and recomputes exp / sqrt per
entry; the FP64 variant gives residual-accurate products (the reference's
matrix-free FP64 residual, mpdok_ooc.py:205-227).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _native as N
from ._device import Workspace, as_columns, as_vector, fortran_empty, ptr, require_cuda, stream_handle
from .rbf_kernel import KERNELS, _coords_device


class MatrixFreeOperator:
    """A = phi(||c_i - c_j||) + reg I, applied without storing A."""

    _matrix_free = True

    def __init__(self, coords, gamma: float, reg: float = 0.0, kernel: str = "gaussian"):
        self.coords = _coords_device(coords)
        self.N = int(self.coords.shape[0])
        self.dim = int(self.coords.shape[1])
        self.gamma = float(gamma)
        self.reg = float(reg)
        self.kernel = kernel
        self.kcode = KERNELS[kernel]
        self._ws = Workspace()
        self.A_fp64 = True  # residuals are available (computed matrix-free in FP64)

    @property
    def shape(self):
        return (self.N, self.N)

    def _apply(self, X, precision):
        squeeze = X.dim() == 1
        tdt = torch.float64 if precision == N.F64 else torch.float32
        Xc = as_columns(X, tdt)
        k = Xc.shape[1]
        if k > 8:
            return torch.cat([self._apply(Xc[:, i:i + 8], precision) for i in range(0, k, 8)], dim=1)
        ld = self.N if precision == N.F64 else (self.N + 3) // 4 * 4
        if ld != self.N:
            Xp = fortran_empty(ld, k, tdt)
            Xp[: self.N] = Xc
            Xc = Xp
        Y = fortran_empty(self.N, k, tdt)
        lib = N.load()
        w = self._ws.get(lib.mpdok_matfree_workspace_size(self.N, self.N, k, precision))
        N.check(lib.mpdok_matfree_apply(ptr(self.coords), self.N, ptr(self.coords), self.N, self.dim, self.kcode,
                                        self.gamma, self.reg, 0, precision, ptr(Xc), Xc.stride(1) if k > 1 else ld,
                                        k, ptr(Y), self.N, ptr(w), w.numel(), stream_handle()), "matfree_apply")
        return Y.reshape(-1) if squeeze else Y

    def matvec(self, x) -> torch.Tensor:
        """A @ x in FP32 (entries recomputed per product)."""
        return self._apply(torch.as_tensor(x, device=require_cuda()) if not isinstance(x, torch.Tensor) else x,
                           N.F32)

    def matvec64(self, x) -> torch.Tensor:
        """A @ x in FP64."""
        return self._apply(torch.as_tensor(x, device=require_cuda()) if not isinstance(x, torch.Tensor) else x,
                           N.F64)

    def residual_norm(self, x, b) -> float:
        x64 = as_vector(x)
        b64 = as_vector(b)
        r = b64 - self.matvec64(x64)
        return float(torch.linalg.vector_norm(r).item())

    def gmres_ir(self, b, tol=1e-11, maxiter_outer=5, restart=50, inner_tol=1e-6):
        b64 = as_vector(b)
        x = torch.zeros(self.N, dtype=torch.float64, device=b64.device)
        lib = N.load()
        w = self._ws.get(lib.mpdok_mf_krylov_workspace_size(self.N, restart))
        info = N.SolveInfo()
        N.check(lib.mpdok_mf_gmres_ir(ptr(self.coords), self.N, self.dim, self.kcode, self.gamma, self.reg,
                                      ptr(b64), ptr(x), float(tol), int(maxiter_outer), int(restart),
                                      float(inner_tol), ptr(w), w.numel(), ctypes.byref(info), stream_handle()),
                "mf_gmres_ir")
        return x, info.history_list(), bool(info.converged)

    def cg(self, b, x0=None, tol=1e-6, maxiter=None, check_every=10):
        b64 = as_vector(b)
        x = torch.zeros(self.N, dtype=torch.float64, device=b64.device) if x0 is None else \
            as_vector(x0).to(torch.float32).to(torch.float64)
        lib = N.load()
        w = self._ws.get(lib.mpdok_mf_krylov_workspace_size(self.N, 1))
        info = N.SolveInfo()
        mi = self.N if maxiter is None else int(maxiter)
        N.check(lib.mpdok_mf_cg(ptr(self.coords), self.N, self.dim, self.kcode, self.gamma, self.reg, ptr(b64),
                                ptr(x), float(tol), mi, int(check_every), ptr(w), w.numel(), ctypes.byref(info),
                                stream_handle()), "mf_cg")
        return x, info.history_list(), bool(info.converged)

    def cg_ir(self, B, tol=1e-12, maxiter_outer=10, inner_tol=1e-6, inner_maxiter=500, precond=None):
        """Multi-RHS CG-IR on the matrix-free operator, optionally preconditioned by LU
        factors or by a ``CholeskyPreconditioner`` (see ``dense_krylov.cg_ir``)."""
        Bc = as_columns(B, torch.float64)
        k = Bc.shape[1]
        if k > 8:
            raise ValueError("cg_ir handles up to 8 right-hand sides per call")
        X = fortran_empty(self.N, k, torch.float64)
        lib = N.load()
        info = N.SolveInfo()
        if precond is not None and hasattr(precond, "plan"):
            if precond.n != self.N or precond.nrhs != k:
                raise ValueError(f"the Cholesky preconditioner holds n={precond.n}, nrhs={precond.nrhs}; "
                                 f"this solve has n={self.N}, nrhs={k}")
            w = self._ws.get(lib.mpdok_chol_cg_ir_workspace_size(self.N, k, 2))
            N.check(lib.mpdok_chol_cg_ir(precond.plan, None, 0, ptr(self.coords), self.dim, self.kcode, self.gamma,
                                         self.reg, self.N, 2, None, 0, k, ptr(Bc), self.N, ptr(X), self.N,
                                         float(tol), int(maxiter_outer), float(inner_tol), int(inner_maxiter),
                                         ptr(w), w.numel(), ctypes.byref(info), stream_handle()), "mf_chol_cg_ir")
        elif precond is None:
            w = self._ws.get(lib.mpdok_mf_cg_ir_workspace_size(self.N, k))
            N.check(lib.mpdok_mf_cg_ir(ptr(self.coords), self.N, self.dim, self.kcode, self.gamma, self.reg, k,
                                       ptr(Bc), self.N, ptr(X), self.N, float(tol), int(maxiter_outer),
                                       float(inner_tol), int(inner_maxiter), ptr(w), w.numel(), ctypes.byref(info),
                                       stream_handle()), "mf_cg_ir")
        else:
            w = self._ws.get(lib.mpdok_lu_cg_ir_workspace_size(self.N, k, 2))
            N.check(lib.mpdok_mf_lu_cg_ir(ptr(self.coords), self.N, self.dim, self.kcode, self.gamma, self.reg,
                                          ptr(precond.factors), precond.fdtype, k, ptr(Bc), self.N, ptr(X), self.N,
                                          float(tol), int(maxiter_outer), float(inner_tol), int(inner_maxiter),
                                          ptr(w), w.numel(), ctypes.byref(info), stream_handle()), "mf_lu_cg_ir")
        squeeze = torch.as_tensor(B).dim() == 1 if not isinstance(B, torch.Tensor) else B.dim() == 1
        return (X.reshape(-1) if squeeze else X), info.history_list(), bool(info.converged)

    def evaluate(self, query, alpha, precision: str = "f64") -> torch.Tensor:
        """f(q) = sum_i alpha_i phi(||q - c_i||) at query points (no nugget)."""
        return rbf_evaluate(alpha, self.coords, query, self.gamma, kernel=self.kernel, precision=precision)

    def __repr__(self):
        return f"MatrixFreeOperator(N={self.N:,}, dim={self.dim}, kernel={self.kernel}, gamma={self.gamma:g})"


def rbf_evaluate(alpha, centres, query, gamma: float, kernel: str = "gaussian", precision: str = "f64",
                 chunk: int | None = None) -> torch.Tensor:
    """Interpolant at query points: f(q) = sum_i alpha_i phi(||q - c_i||).

    The evaluation step that consumes every solve (enkf_solver.py:162-200,
    ``reconstruct``): the reference assembles (chunk x N) FP64 blocks of K and
    multiplies; here the same evaluate-and-multiply kernel as the solvers
    recomputes phi from TMA-staged centre tiles, so nothing of size M x N is
    ever stored.  ``alpha`` is (N,) or (N, k); the result is (M,) or (M, k),
    FP64 (``precision='f64'``, the reference's output type) or FP32.
    ``chunk`` is accepted for signature compatibility; no chunking is needed.
    """
    del chunk
    if precision not in ("f64", "f32"):
        raise ValueError("precision must be 'f64' or 'f32'")
    c = _coords_device(centres)
    q = _coords_device(query)
    if q.shape[1] != c.shape[1]:
        raise ValueError(f"query dimension {q.shape[1]} != centre dimension {c.shape[1]}")
    n, m, dim = int(c.shape[0]), int(q.shape[0]), int(c.shape[1])
    pcode = N.F64 if precision == "f64" else N.F32
    tdt = torch.float64 if precision == "f64" else torch.float32
    if not isinstance(alpha, torch.Tensor):
        alpha = torch.as_tensor(np.asarray(alpha), device=require_cuda())
    squeeze = alpha.dim() == 1
    A = as_columns(alpha, tdt)
    if A.shape[0] != n:
        raise ValueError(f"alpha has {A.shape[0]} rows, expected {n}")
    k = A.shape[1]
    out = fortran_empty(m, k, torch.float64)
    if m == 0 or k == 0:
        return out.reshape(-1) if squeeze else out
    lib = N.load()
    ld = n if pcode == N.F64 else (n + 3) // 4 * 4
    ws = Workspace()
    for j0 in range(0, k, 8):
        kk = min(8, k - j0)
        Xc = fortran_empty(ld, kk, tdt)
        Xc[:n] = A[:, j0:j0 + kk]
        Y = fortran_empty(m, kk, tdt)
        w = ws.get(lib.mpdok_matfree_workspace_size(m, n, kk, pcode))
        N.check(lib.mpdok_matfree_apply(ptr(q), m, ptr(c), n, dim, KERNELS[kernel], float(gamma), 0.0, 0, pcode,
                                        ptr(Xc), ld, kk, ptr(Y), m, ptr(w), w.numel(), stream_handle()),
                "matfree_apply (evaluate)")
        out[:, j0:j0 + kk] = Y
    return out.reshape(-1) if squeeze else out
