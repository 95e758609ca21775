"""RBF problem assembly on the GPU (Gaussian and multiquadric kernels).

Mirrors MPDOK's rbf_kernel.py API (``synthetic_coords``, ``_estimate_gamma``,
``build_rbf_kernel``, ``weather_front``) with the arithmetic in the fused
sm_103a assembly kernel (``mpdok_rbf_assemble``): one pass writes every entry
A[i, j] = phi(||c_i - c_j||) + reg * delta_ij, with no chunk temporaries.

Kernels: ``'gaussian'`` phi(r) = exp(-gamma r^2) (rbf_kernel.py:162) and
``'mq'`` phi(r) = sqrt(1 + gamma r^2) (multiquadric, gamma = eps^2).
"""
from __future__ import annotations

import numpy as np
import torch

from . import _native as N
from ._device import as_fortran, fortran_empty, ptr, require_cuda, stream_handle

KERNELS = {"gaussian": N.KERNEL_GAUSSIAN, "mq": N.KERNEL_MQ, "multiquadric": N.KERNEL_MQ}
_DT = {torch.float64: N.F64, torch.float32: N.F32, torch.bfloat16: N.BF16, torch.float16: N.F16}


def synthetic_coords(N_pts: int, D: int = 2, seed: int = 42, scale: float = 100.0) -> torch.Tensor:
    """N_pts uniform points in [0, scale]^D as an (N, D) FP64 CUDA tensor.

    rbf_kernel.py:41-54 draws them with CuPy's generator; this uses NumPy's
    ``default_rng(seed)`` (CuPy's stream is not reproducible without CuPy), so
    the points are the same on every machine.
    """
    rng = np.random.default_rng(seed)
    pts = rng.uniform(0.0, scale, size=(N_pts, D))
    return torch.from_numpy(pts).to(device=require_cuda(), dtype=torch.float64)


def _estimate_gamma(coords, max_sample: int = 512) -> float:
    """gamma = 1 / (2 * mean pairwise squared distance) over the first points.

    rbf_kernel.py:57-68.  The mean of ||c_i - c_j||^2 over all ordered pairs
    of the sample equals 2 (mean ||c||^2 - ||mean c||^2); it is evaluated on
    the (at most 512 x D) sample on the host in FP64.
    """
    c = coords[:max_sample]
    c = c.detach().cpu().numpy() if isinstance(c, torch.Tensor) else np.asarray(c, dtype=np.float64)
    c = np.asarray(c, dtype=np.float64)
    sq = np.sum(c * c, axis=1)
    d2 = sq[:, None] + sq[None, :] - 2.0 * (c @ c.T)
    np.maximum(d2, 0.0, out=d2)
    mean_d2 = float(np.mean(d2))
    return 1.0 / (2.0 * mean_d2) if mean_d2 > 1e-30 else 1.0


def _coords_device(coords) -> torch.Tensor:
    dev = require_cuda()
    if isinstance(coords, torch.Tensor):
        c = coords.to(device=dev, dtype=torch.float64)
    else:
        c = torch.from_numpy(np.asarray(coords, dtype=np.float64)).to(dev)
    if c.dim() == 1:
        c = c.reshape(-1, 1)
    return c.contiguous()


def assemble(rows, cols=None, gamma: float = 1.0, reg: float = 0.0, kernel: str = "gaussian",
             dtype=torch.float64, out: torch.Tensor | None = None, diag_offset: int = 0,
             col_major: bool = True) -> torch.Tensor:
    """Kernel block K(rows, cols) (+ reg on the entries with i + diag_offset == j)."""
    r = _coords_device(rows)
    c = r if cols is None else _coords_device(cols)
    if r.shape[1] != c.shape[1]:
        raise ValueError("rows and cols must have the same dimension")
    nr, nc, dim = r.shape[0], c.shape[0], r.shape[1]
    if out is None:
        out = fortran_empty(nr, nc, dtype) if col_major else torch.empty((nr, nc), dtype=dtype, device=r.device)
    if col_major:
        if out.stride(0) != 1:
            raise ValueError("out must be column-major")
        ld = out.stride(1) if nc > 1 else max(1, nr)
    else:
        if out.stride(1) != 1:
            raise ValueError("out must be row-major")
        ld = out.stride(0) if nr > 1 else max(1, nc)
    N.check(N.load().mpdok_rbf_assemble(ptr(r), nr, ptr(c), nc, dim, KERNELS[kernel], float(gamma), float(reg),
                                        int(diag_offset), _DT[out.dtype], ptr(out), ld, 1 if col_major else 0,
                                        stream_handle()), "rbf_assemble")
    return out


def build_rbf_kernel(coords, gamma=None, reg: float = 1e-6, out=None, chunk: int = 1024, verbose: bool = False,
                     kernel: str = "gaussian", dtype=torch.float64):
    """Build A = phi(||c_i - c_j||) + reg I on the GPU; returns ``(A, gamma)``.

    Same contract as rbf_kernel.py:158-227: A is (N, N), Fortran order, FP64
    by default; ``out`` may be a preallocated (N, N) array (including a
    managed array from ``alloc_managed``).  ``chunk`` is accepted for API
    compatibility; the fused kernel needs no row chunking.
    """
    c = _coords_device(coords)
    n = c.shape[0]
    if gamma is None:
        gamma = _estimate_gamma(c)
    target = out.array if hasattr(out, "array") else out
    if target is None:
        target = fortran_empty(n, n, dtype)
    elif not isinstance(target, torch.Tensor):
        raise TypeError("out must be a torch CUDA tensor or a managed array")
    assemble(c, None, gamma=gamma, reg=reg, kernel=kernel, dtype=target.dtype, out=target)
    if verbose:
        print(f"  build_rbf_kernel: N={n:,} kernel={kernel} gamma={gamma:.3e} reg={reg:.1e}")
    return (out if out is not None else target), gamma


def weather_front(coords, t: int, noise_std: float = 0.05, seed=None) -> torch.Tensor:
    """Moving thermal front RHS of rbf_kernel.py:230-252 (noise from NumPy's generator)."""
    c = _coords_device(coords)
    x, y = c[:, 0], c[:, 1]
    field = 15.0 + 5.0 * torch.sin((x + y) / 20.0 - 0.5 * t)
    if noise_std > 0:
        rng = np.random.default_rng(t if seed is None else seed)
        field = field + torch.from_numpy(rng.standard_normal(c.shape[0]) * noise_std).to(c.device)
    return field.to(torch.float64)
