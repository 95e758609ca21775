"""Gradients of one in-core RBF solve: a torch.autograd.Function over the LU path.

``rbf_solve(coords, eps, reg, b)`` assembles A = phi_eps(||c_i - c_j||) + reg I
on the GPU (FP64), factors it once (BF16 / FP16 / FP32 LU of the diagonally
scaled matrix, tcgen05 trailing update) and solves A x = b to the FP64
tolerance with the three-precision GMRES-IR (the headline solver).  Its
backward pass

* solves A^T lam = dL/dx with the SAME factors (A is symmetric, so A^T = A
  and the LU preconditions the adjoint solve exactly as it did the forward
  one): no second factorization;
* contracts lam^T (dA/dtheta) x for theta = centre coordinates, eps and the
  nugget in one fused FP64 kernel that recomputes phi and its derivatives
  from the coordinates (dA, N x N, is never formed);
* returns dL/db = lam.

The reference solves one system per call and has no gradients
(mpdok_ops.py:323-508); this is the differentiated form of its in-core solve.
"""
from __future__ import annotations

import ctypes

import torch

from . import _native as N
from ._device import Workspace, ptr, require_cuda, stream_handle
from .lu import LUFactorization
from .rbf_kernel import KERNELS, assemble


class _RBFSolveFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, coords, eps, reg, b, opts):
        dev = require_cuda()
        c = coords.detach().to(device=dev, dtype=torch.float64).contiguous()
        e = float(eps)
        r = float(reg)
        A = assemble(c, gamma=e * e, reg=r, kernel=opts["kernel"], dtype=torch.float64)
        lu = LUFactorization(A, dtype=opts["factor_dtype"])
        b64 = b.detach().to(device=dev, dtype=torch.float64).contiguous()
        x, info = lu.gmres_ir(A, b64, tol=opts["tol"], maxiter_outer=opts["maxiter_outer"], restart=opts["restart"])
        ctx.lu, ctx.A, ctx.opts, ctx.info = lu, A, opts, info
        ctx.save_for_backward(c, x)
        ctx.eps = e
        ctx.devs = (coords.device, eps.device, reg.device, b.device)
        opts["last_info"] = info
        return x

    @staticmethod
    def backward(ctx, gx):
        c, x = ctx.saved_tensors
        opts = ctx.opts
        g64 = gx.detach().to(dtype=torch.float64).contiguous()
        # A^T = A: the adjoint solve reuses the forward factors
        lam, info = ctx.lu.gmres_ir(ctx.A, g64, tol=opts["tol"], maxiter_outer=opts["maxiter_outer"],
                                    restart=opts["restart"])
        opts["last_adjoint_info"] = info
        n, dim = c.shape
        gc = torch.empty_like(c)
        ge = torch.empty(1, dtype=torch.float64, device=c.device)
        gr = torch.empty(1, dtype=torch.float64, device=c.device)
        lib = N.load()
        w = opts["ws"].get(lib.mpdok_rbf_adjoint_workspace_size(n))
        N.check(lib.mpdok_rbf_adjoint(ptr(c), n, dim, KERNELS[opts["kernel"]], ctx.eps, 1, ptr(x), ptr(lam), ptr(gc),
                                      ptr(ge), ptr(gr), ptr(w), w.numel(), stream_handle()), "rbf_adjoint")
        dc, de, dr, db = ctx.devs
        return gc.to(dc), ge.reshape(()).to(de), gr.reshape(()).to(dr), lam.to(db), None


def rbf_solve(coords, eps, reg, b, factor_dtype: str = "fp16", tol: float = 1e-12, kernel: str = "gaussian",
              restart: int = 30, maxiter_outer: int = 20, opts: dict | None = None) -> torch.Tensor:
    """x = A(coords, eps, reg)^-1 b, differentiable in coords, eps, reg and b.

    ``opts`` (optional dict) receives the forward and adjoint solve reports
    (``last_info``, ``last_adjoint_info``)."""
    o = opts if opts is not None else {}
    o.update(kernel=kernel, factor_dtype=factor_dtype, tol=float(tol), restart=int(restart),
             maxiter_outer=int(maxiter_outer))
    o.setdefault("ws", Workspace())
    eps_t = eps if isinstance(eps, torch.Tensor) else torch.tensor(float(eps), dtype=torch.float64)
    reg_t = reg if isinstance(reg, torch.Tensor) else torch.tensor(float(reg), dtype=torch.float64)
    return _RBFSolveFn.apply(coords, eps_t, reg_t, b, o)
