"""Device-memory plumbing on PyTorch: streams, layouts and workspaces.

PyTorch provides device allocation and the current CUDA stream; all
arithmetic of the solvers runs in libmpdok_gb300.so.  Matrices are kept in
column-major (Fortran) order, the reference ABI's layout (mpdok_ops.py:363):
a torch tensor of shape (N, M) with strides (1, N).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch


def require_cuda() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("mpdok_gb300 needs a CUDA device (sm_103a); there is no CPU fallback")
    return torch.device("cuda", torch.cuda.current_device())


def stream_handle(stream: torch.cuda.Stream | None = None) -> ctypes.c_void_p:
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def ptr(t: torch.Tensor | None) -> ctypes.c_void_p:
    return ctypes.c_void_p(0 if t is None else t.data_ptr())


def is_fortran(t: torch.Tensor) -> bool:
    if t.dim() != 2:
        return False
    n, m = t.shape
    return t.stride(0) == 1 and (t.stride(1) == n or m <= 1)


def fortran_empty(n: int, m: int, dtype=torch.float64, device=None) -> torch.Tensor:
    device = device or require_cuda()
    return torch.empty_strided((n, m), (1, max(1, n)), dtype=dtype, device=device)


def as_fortran(A, dtype=torch.float64) -> torch.Tensor:
    """(N, M) array-like -> CUDA tensor of `dtype` in column-major layout (no copy when already so)."""
    dev = require_cuda()
    if isinstance(A, torch.Tensor):
        if A.dim() != 2:
            raise ValueError(f"A must be 2-D, got shape {tuple(A.shape)}")
        if A.is_cuda and A.dtype == dtype and is_fortran(A):
            return A
        if not A.is_cuda and A.dtype == torch.float64 and dtype == torch.float64:
            return upload_fortran(A)
        out = fortran_empty(A.shape[0], A.shape[1], dtype, dev)
        out.copy_(A.to(device=dev, dtype=dtype))
        return out
    arr = np.asarray(A)
    if arr.ndim != 2:
        raise ValueError(f"A must be 2-D, got shape {arr.shape}")
    arr = np.asfortranarray(arr, dtype=np.float64 if dtype == torch.float64 else None)
    host = torch.from_numpy(arr)
    out = fortran_empty(arr.shape[0], arr.shape[1], dtype, dev)
    out.copy_(host.to(dtype))
    return out


def upload_fortran(A_host: torch.Tensor, out: torch.Tensor | None = None, out32: torch.Tensor | None = None,
                   chunk_bytes: int = 256 << 20) -> torch.Tensor:
    """Host (N, M) FP64 matrix in column-major order -> CUDA column-major FP64 tensor.

    The host columns are copied straight into the device buffer (no device
    temporary), in blocks of whole columns on a side stream; when ``out32`` is
    given, each block is converted to FP32 on the current stream while the
    next block is still on the host link, so the FP32 copy of A costs no extra
    pass once the upload ends.  A pinned host tensor gives the full host-link
    rate; a pageable one is copied synchronously.  The current stream owns the
    result (it waits for every block)."""
    from . import _native as N
    if A_host.dim() != 2 or A_host.dtype != torch.float64 or A_host.is_cuda:
        raise ValueError("upload_fortran expects a host FP64 2-D tensor")
    n, m = A_host.shape
    if not is_fortran(A_host):
        A_host = A_host.t().contiguous().t()
    dev = require_cuda()
    if out is None:
        out = fortran_empty(n, m, torch.float64, dev)
    flat_h = A_host.t().reshape(-1)   # column-major storage as one contiguous run
    flat_d = out.t().reshape(-1)
    flat_32 = out32.t().reshape(-1) if out32 is not None else None
    cols = max(1, chunk_bytes // max(1, 8 * n))
    cur = torch.cuda.current_stream(dev)
    side = torch.cuda.Stream(dev)
    side.wait_stream(cur)
    lib = N.load() if out32 is not None else None
    for c0 in range(0, m, cols):
        c1 = min(m, c0 + cols)
        lo, hi = c0 * n, c1 * n
        with torch.cuda.stream(side):
            flat_d[lo:hi].copy_(flat_h[lo:hi], non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(side)
        cur.wait_event(ev)
        if out32 is not None:
            N.check(lib.mpdok_convert(ptr(flat_d[lo:hi]), N.F64, ptr(flat_32[lo:hi]), N.F32, hi - lo,
                                      ctypes.c_void_p(cur.cuda_stream)), "convert")
    flat_d.record_stream(side)
    return out


def as_vector(b, dtype=torch.float64) -> torch.Tensor:
    dev = require_cuda()
    if isinstance(b, torch.Tensor):
        t = b.to(device=dev, dtype=dtype)
    else:
        t = torch.from_numpy(np.ascontiguousarray(np.asarray(b, dtype=np.float64))).to(device=dev, dtype=dtype)
    return t.contiguous()


def as_columns(B, dtype=torch.float64) -> torch.Tensor:
    """(N,) or (N, k) -> column-major (N, k) CUDA tensor."""
    if isinstance(B, torch.Tensor):
        t = B
    else:
        t = torch.from_numpy(np.asarray(B, dtype=np.float64))
    if t.dim() == 1:
        t = t.reshape(-1, 1)
    return as_fortran(t, dtype)


class Workspace:
    """Growable device scratch buffer (bytes) owned by a solver object."""

    def __init__(self):
        self._buf: torch.Tensor | None = None

    def get(self, nbytes: int) -> torch.Tensor:
        nbytes = max(256, int(nbytes))
        if self._buf is None or self._buf.numel() < nbytes or self._buf.device != require_cuda():
            self._buf = torch.empty(nbytes, dtype=torch.uint8, device=require_cuda())
        return self._buf

    def release(self):
        self._buf = None
