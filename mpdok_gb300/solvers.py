"""High-level mixed-precision solve used by the benchmark and the examples.

``MixedSolver.solve(A, b)`` takes an (N, N) FP64 matrix (CUDA tensor in
column-major order, or host memory, which is uploaded) and returns
``(x, info)`` with x an FP64 CUDA tensor at the FP64 relative-residual
tolerance.  ``fp64_gpu_solve`` is the plain FP64 GPU reference solve used for
comparison (vendor FP64 LU through PyTorch, FP64 refinement with this
library's residual kernel); it is a baseline, never used by the product path.
"""
from __future__ import annotations

import ctypes
import time
import warnings

import torch

from . import _native as N
from ._device import Workspace, as_fortran, as_vector, fortran_empty, ptr, stream_handle, upload_fortran


def _info_dict(info: N.SolveInfo) -> dict:
    return {"converged": bool(info.converged), "outer_iters": int(info.outer_iters),
            "inner_iters": int(info.inner_iters), "relres": float(info.relres),
            "history": info.history_list(), "diverged": int(info.stagnated) == 2}


class MixedSolver:
    """FP64-accurate solve of a dense system with low-precision work on the GPU.

    method ``'lu-gmres-ir'`` (default): BF16/FP16 blocked LU of the diagonally
    scaled matrix on the tensor cores, used as the right preconditioner of FP32
    GMRES inside FP64 refinement (three-precision GMRES-IR).
    method ``'gmres-ir'``: the reference's unpreconditioned GMRES-IR
    (py_gmres_ir semantics).
    """

    def __init__(self, method: str = "lu-gmres-ir", factor_dtype: str = "fp16", restart: int = 30,
                 maxiter_outer: int = 20, inner_tol: float = 1e-6):
        self.method = method
        self.factor_dtype = factor_dtype
        self.restart = restart
        self.maxiter_outer = maxiter_outer
        self.inner_tol = inner_tol
        self._ws = Workspace()
        self._fws = Workspace()
        self._a32 = None
        self.last_timing = {}

    def describe(self) -> str:
        if self.method == "gmres-ir":
            return (f"GMRES-IR: FP32 A copy + FP32 GMRES({self.restart}) inner (CGS2, FP64 Givens, inner tol "
                    f"{self.inner_tol:g}), FP64 residual/update")
        return (f"LU-GMRES-IR: {self.factor_dtype.upper()} blocked LU (tcgen05 trailing update, FP32 panels, "
                f"diagonal scaling) preconditioning FP32 GMRES({self.restart}) (CGS2, FP64 Givens, inner tol "
                f"{self.inner_tol:g}); FP64 residual/update")

    def solve(self, A, b, tol: float = 1e-12):
        """x, info for A x = b.  A may live on the host: then it is uploaded
        straight into its device buffer, and for the LU method its FP32 copy
        is made block by block while the rest of A is still in flight."""
        t_host = time.perf_counter()
        b64 = as_vector(b, torch.float64)
        n = int(A.shape[0])
        if self._a32 is None or self._a32.shape[0] != n:
            self._a32 = fortran_empty(n, n, torch.float32)
        a32_ready = False
        up = None
        if isinstance(A, torch.Tensor) and not A.is_cuda and A.dtype == torch.float64 and A.dim() == 2 \
                and self.method != "gmres-ir":
            up = [torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)]
            up[0].record()
            A64 = upload_fortran(A, out32=self._a32)
            up[1].record()
            a32_ready = True
        else:
            A64 = as_fortran(A, torch.float64)
        x = torch.zeros(n, dtype=torch.float64, device=b64.device)
        lib = N.load()
        info = N.SolveInfo()
        if self.method == "gmres-ir":
            w = self._ws.get(lib.mpdok_krylov_workspace_size(n, self.restart))
            N.check(lib.mpdok_gmres_ir(ptr(A64), n, ptr(self._a32), n, 0, n, ptr(b64), ptr(x), float(tol),
                                       self.maxiter_outer, self.restart, self.inner_tol, ptr(w), w.numel(),
                                       ctypes.byref(info), stream_handle()), "gmres_ir")
            return x, _info_dict(info)
        from .lu import LUFactorization
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        ev[0].record()
        if not a32_ready:
            N.check(lib.mpdok_convert(ptr(A64), N.F64, ptr(self._a32), N.F32, n * n, stream_handle()), "convert")
        lu = LUFactorization(A64, dtype=self.factor_dtype, work=self._fws)
        ev[1].record()
        x, d = lu.gmres_ir(A64, b64, A32=self._a32, tol=tol, maxiter_outer=self.maxiter_outer,
                           restart=self.restart, inner_tol=self.inner_tol)
        ev[2].record()
        ev[2].synchronize()
        d["factor_ms"] = ev[0].elapsed_time(ev[1])
        d["refine_ms"] = ev[1].elapsed_time(ev[2])
        d["perturbed_pivots"] = lu.n_perturbed
        self.last_timing = {"factor_ms": d["factor_ms"], "refine_ms": d["refine_ms"],
                            "host_ms": (time.perf_counter() - t_host) * 1e3}
        if up is not None:
            self.last_timing["upload_ms"] = up[0].elapsed_time(up[1])
        if not d["converged"]:
            why = ("the FP64 residual diverged; the best iterate is returned" if d["diverged"]
                   else f"not converged in {self.maxiter_outer} outer steps")
            warnings.warn(f"MixedSolver ({self.factor_dtype} LU-GMRES-IR): {why} (relres {d['relres']:.2e}, "
                          f"{lu.n_perturbed} perturbed pivots)", RuntimeWarning, stacklevel=2)
        return x, d


def fp64_gpu_solve(A, b, tol: float = 1e-12, max_refine: int = 3):
    """Plain FP64 GPU solve: vendor FP64 LU (torch.linalg.lu_factor) + FP64 refinement."""
    A64 = as_fortran(A, torch.float64)
    b64 = as_vector(b, torch.float64)
    n = A64.shape[0]
    lib = N.load()
    ws = Workspace()
    w = ws.get(lib.mpdok_gemv_workspace_size(N.F64, n, n, 1, 0))
    r = torch.empty_like(b64)
    nrm2 = torch.empty(1, dtype=torch.float64, device=b64.device)
    bn = float(torch.linalg.norm(b64))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    LU, piv = torch.linalg.lu_factor(A64)
    x = torch.linalg.lu_solve(LU, piv, b64.reshape(-1, 1)).reshape(-1)
    rel = float("inf")
    for _ in range(max_refine + 1):
        N.check(lib.mpdok_residual(ptr(A64), n, n, ptr(b64), ptr(x), ptr(r), ptr(nrm2), ptr(w), w.numel(),
                                   stream_handle()), "residual")
        rel = float(nrm2.item()) ** 0.5 / bn
        if rel <= tol:
            break
        x = x + torch.linalg.lu_solve(LU, piv, r.reshape(-1, 1)).reshape(-1)
    torch.cuda.synchronize()
    secs = time.perf_counter() - t0
    del LU, piv
    return {"x": x, "seconds": secs, "relres": rel, "method": "torch.linalg.lu_factor FP64 + FP64 refinement"}
