"""Out-of-core GMRES-IR (drop-in for MPDOK's mpdok_ooc.py).

``MPDOKOOCSolver(tile_rows)`` keeps the FP32 RBF matrix outside HBM: in
pinned host RAM (``store='ram'``) or in a raw row-major FP32 file without a
header (``store='ssd'``, the reference's format).  Every inner product streams
the tiles to the GPU with double-buffered copies on a side stream; the outer
FP64 residual is recomputed matrix-free from the coordinates
(mpdok_ooc.py:205-227).  Same method names and defaults as the reference.
"""
from __future__ import annotations

import ctypes
import time
import warnings

import numpy as np
import torch

from . import _native as N
from ._device import Workspace, as_vector, ptr, require_cuda, stream_handle
from .rbf_kernel import KERNELS, _coords_device, _estimate_gamma


class MPDOKOOCSolver:
    """Out-of-core GMRES-IR for N beyond the HBM budget of the stored FP32 matrix."""

    def __init__(self, tile_rows: int = 4096):
        self.tile_rows = tile_rows
        self._store = None
        self._ssd_path = None
        self.N = None
        self.gamma = None
        self.reg = None
        self._coords = None
        self._h = None
        self._ws = Workspace()
        self.kernel = "gaussian"

    def build(self, coords, gamma=None, reg: float = 1e-6, store: str = "ram", path=None, verbose: bool = True,
              kernel: str = "gaussian"):
        """Assemble the FP32 matrix tile by tile on the GPU into the store; returns gamma."""
        if store not in ("ram", "ssd"):
            raise ValueError(f"store must be 'ram' or 'ssd', got {store!r}")
        if store == "ssd" and path is None:
            raise ValueError("store='ssd' requires a path argument")
        self.free()
        c = _coords_device(coords)
        n = int(c.shape[0])
        if gamma is None:
            gamma = _estimate_gamma(c)
        self.N, self.gamma, self.reg, self._store, self._ssd_path = n, float(gamma), float(reg), store, path
        self.kernel = kernel
        self._coords = c
        lib = N.load()
        h = ctypes.c_void_p()
        N.check(lib.mpdok_ooc_create(n, int(self.tile_rows), 0 if store == "ram" else 1,
                                     (path or "").encode(), ctypes.byref(h)), "ooc_create")
        self._h = h
        t0 = time.perf_counter()
        N.check(lib.mpdok_ooc_build(self._h, ptr(c), int(c.shape[1]), KERNELS[kernel], self.gamma, self.reg,
                                    stream_handle()), "ooc_build")
        if verbose:
            ntiles = (n + self.tile_rows - 1) // self.tile_rows
            print(f"  OOC build: N={n:,}  gamma={self.gamma:.3e}  FP32={n * n * 4 / 1024 ** 3:.2f} GB  "
                  f"tiles={ntiles}  store={store}  ({time.perf_counter() - t0:.1f} s)")
        return self.gamma

    # -- products (mpdok_ooc.py:158-227) ----------------------------------------
    def _tiled_sgemv(self, v_fp32) -> torch.Tensor:
        """y = A_fp32 v, streaming the tiles from the store."""
        v = as_vector(v_fp32, torch.float32)
        y = torch.empty_like(v)
        N.check(N.load().mpdok_ooc_matvec(self._h, ptr(v), ptr(y), stream_handle()), "ooc_matvec")
        return y

    def _tiled_dgemv_fp64(self, v_fp64) -> torch.Tensor:
        """y = A_fp64 v recomputed matrix-free from the coordinates (FP64)."""
        from .matfree import MatrixFreeOperator
        op = MatrixFreeOperator(self._coords, gamma=self.gamma, reg=self.reg, kernel=self.kernel)
        return op.matvec64(as_vector(v_fp64))

    def stored_matrix(self, row0: int = 0, rows=None) -> np.ndarray:
        """Rows [row0, row0 + rows) of the stored FP32 matrix, read back from the store."""
        if self._h is None:
            raise RuntimeError("Call build() first")
        rows = self.N - row0 if rows is None else rows
        out = np.empty((rows, self.N), dtype=np.float32)
        torch.cuda.synchronize()
        N.check(N.load().mpdok_ooc_read_rows(self._h, int(row0), int(rows), out.ctypes.data), "ooc_read_rows")
        return out

    def bytes_moved(self) -> float:
        return float(N.load().mpdok_ooc_bytes_moved(self._h)) if self._h else 0.0

    # -- solve --------------------------------------------------------------------
    def solve(self, b, tol: float = 1e-5, maxiter_outer: int = 20, restart: int = 50, verbose: bool = True,
              inner_tol: float = 1e-6):
        if self.N is None:
            raise RuntimeError("Call build() before solve()")
        b64 = as_vector(b)
        x = torch.zeros(self.N, dtype=torch.float64, device=b64.device)
        lib = N.load()
        w = self._ws.get(lib.mpdok_ooc_workspace_size(self.N, restart))
        info = N.SolveInfo()
        N.check(lib.mpdok_ooc_gmres_ir(self._h, ptr(self._coords), int(self._coords.shape[1]), KERNELS[self.kernel],
                                       self.gamma, self.reg, ptr(b64), ptr(x), float(tol), int(maxiter_outer),
                                       int(restart), float(inner_tol), ptr(w), w.numel(), ctypes.byref(info),
                                       stream_handle()), "ooc_gmres_ir")
        self.last_info = info
        hist = info.history_list()
        if verbose:
            for it, r in hist:
                print(f"  outer {it}: rel_res={r:.2e}")
        if not info.converged:
            warnings.warn(f"MPDOKOOCSolver did not converge within {maxiter_outer} outer iterations "
                          f"(final rel_res={info.relres:.2e})", RuntimeWarning, stacklevel=2)
        return x

    def free(self):
        """Release the store and the device buffers."""
        if getattr(self, "_h", None):
            N.load().mpdok_ooc_destroy(self._h)
        self._h = None
        self._coords = None
        self._ws.release()

    def __del__(self):
        # the pinned host store can be tens of GB: release it with the object
        try:
            self.free()
        except Exception:
            pass
