"""ctypes binding of libmpdok_gb300.so (the C ABI declared in include/mpdok_gb300.h).

The library is built in-tree by ``mpdok_gb300._build.build()``.  There is no
fallback: if the shared library is missing, importing the solver modules fails
with an explicit error, and every call that reaches the GPU goes through the
sm_103a kernels in the library.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libmpdok_gb300.so"

# Status codes (include/mpdok_gb300.h)
OK = 0
ERR_INVALID_ARG = -1
ERR_CUDA = -2
ERR_ALLOC = -3
ERR_NOT_FACTORED = -4
ERR_TIMEOUT = -5
ERR_UNSUPPORTED = -6
ERR_IO = -7
ERR_NONFINITE = -8

F64, F32, BF16, F16 = 0, 1, 2, 3
(PROF_GEMV_F32, PROF_GEMV_F64, PROF_ASSEMBLE, PROF_LU_GEMM, PROF_TRSV, PROF_MATFREE, PROF_OOC_COPY, PROF_LU_PANEL,
 PROF_LU_GEMM_DEEP) = range(9)
KERNEL_GAUSSIAN, KERNEL_MQ = 0, 1
ENGINE_TENSOR, ENGINE_SIMT = 0, 1
HISTORY_MAX = 256
DEBUG_WAIT_LIMIT, DEBUG_TRSV_FIRST_TICKET = 1, 2
NOALLOC_SCRATCH_BYTES = 16 << 20

c_void_p = ctypes.c_void_p
c_int = ctypes.c_int
c_ll = ctypes.c_longlong
c_double = ctypes.c_double
c_size_t = ctypes.c_size_t


class SolveInfo(ctypes.Structure):
    """mirror of mpdok_solve_info."""

    _fields_ = [
        ("converged", c_int),
        ("outer_iters", c_int),
        ("inner_iters", c_int),
        ("stagnated", c_int),
        ("relres", c_double),
        ("bnorm", c_double),
        ("n_history", c_int),
        ("hist_iter", c_int * HISTORY_MAX),
        ("history", c_double * HISTORY_MAX),
    ]

    def history_list(self):
        n = min(self.n_history, HISTORY_MAX)
        return [(int(self.hist_iter[i]), float(self.history[i])) for i in range(n)]


class MPDOKError(RuntimeError):
    """Raised when a native entry point returns an error status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"[{status}] {message}")
        self.status = status


# Signatures: name -> (restype, [argtypes]).
_SIGS = {
    "mpdok_version": (c_int, []),
    "mpdok_status_string": (ctypes.c_char_p, [c_int]),
    "mpdok_last_error": (ctypes.c_char_p, []),
    "mpdok_clear_error": (None, []),
    "mpdok_debug_set": (c_int, [c_int, c_ll]),
    "mpdok_rbf_assemble": (c_int, [c_void_p, c_ll, c_void_p, c_ll, c_int, c_int, c_double, c_double, c_ll,
                                   c_int, c_void_p, c_ll, c_int, c_void_p]),
    "mpdok_convert": (c_int, [c_void_p, c_int, c_void_p, c_int, c_ll, c_void_p]),
    "mpdok_gemv_workspace_size": (c_size_t, [c_int, c_ll, c_ll, c_int, c_int]),
    "mpdok_gemv": (c_int, [c_int, c_int, c_void_p, c_ll, c_ll, c_ll, c_void_p, c_ll, c_int, c_void_p, c_ll,
                           c_double, c_double, c_void_p, c_size_t, c_void_p]),
    "mpdok_gemv_noalloc": (c_int, [c_int, c_int, c_void_p, c_ll, c_ll, c_ll, c_void_p, c_ll, c_int, c_void_p, c_ll,
                                   c_double, c_double, c_void_p]),
    "mpdok_residual": (c_int, [c_void_p, c_ll, c_ll, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_size_t,
                               c_void_p]),
    "mpdok_krylov_workspace_size": (c_size_t, [c_ll, c_int]),
    "mpdok_gmres_ir": (c_int, [c_void_p, c_ll, c_void_p, c_ll, c_int, c_ll, c_void_p, c_void_p, c_double, c_int,
                               c_int, c_double, c_void_p, c_size_t, ctypes.POINTER(SolveInfo), c_void_p]),
    "mpdok_gmres": (c_int, [c_void_p, c_ll, c_void_p, c_ll, c_ll, c_void_p, c_void_p, c_double, c_int, c_int,
                            c_void_p, c_size_t, ctypes.POINTER(SolveInfo), c_void_p]),
    "mpdok_dense_gmres_ir": (c_int, [c_void_p, c_ll, c_void_p, c_ll, c_ll, c_void_p, c_void_p, c_double, c_int,
                                     c_int, c_int, c_void_p, c_size_t, ctypes.POINTER(SolveInfo), c_void_p]),
    "mpdok_cg": (c_int, [c_void_p, c_ll, c_void_p, c_ll, c_ll, c_void_p, c_void_p, c_double, c_int, c_int,
                         c_void_p, c_size_t, ctypes.POINTER(SolveInfo), c_void_p]),
    "mpdok_gemm_update": (c_int, [c_void_p, c_ll, c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_int, c_void_p,
                                  c_void_p]),
    "mpdok_lu_factor_size": (c_size_t, [c_ll, c_int]),
    "mpdok_lu_work_size": (c_size_t, [c_ll, c_int]),
    "mpdok_lu_factor": (c_int, [c_void_p, c_ll, c_ll, c_int, c_int, c_void_p, c_size_t, c_void_p, c_size_t,
                                c_void_p]),
    "mpdok_lu_export": (c_int, [c_void_p, c_ll, c_int, c_void_p, c_ll, c_void_p, c_void_p, c_void_p, c_void_p,
                                c_void_p]),
    "mpdok_lu_apply_work_size": (c_size_t, [c_ll]),
    "mpdok_lu_apply": (c_int, [c_void_p, c_ll, c_int, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    "mpdok_lu_ir_work_size": (c_size_t, [c_ll]),
    "mpdok_lu_ir_solve": (c_int, [c_void_p, c_ll, c_ll, c_void_p, c_int, c_void_p, c_void_p, c_double, c_int,
                                  c_void_p, c_size_t, ctypes.POINTER(SolveInfo), c_void_p]),
    "mpdok_lu_gmres_ir_work_size": (c_size_t, [c_ll, c_int]),
    "mpdok_lu_gmres_ir": (c_int, [c_void_p, c_ll, c_void_p, c_ll, c_ll, c_void_p, c_int, c_void_p, c_void_p,
                                  c_double, c_int, c_int, c_double, c_void_p, c_size_t, ctypes.POINTER(SolveInfo),
                                  c_void_p]),
    "mpdok_matfree_workspace_size": (c_size_t, [c_ll, c_ll, c_int, c_int]),
    "mpdok_matfree_apply": (c_int, [c_void_p, c_ll, c_void_p, c_ll, c_int, c_int, c_double, c_double, c_ll, c_int,
                                    c_void_p, c_ll, c_int, c_void_p, c_ll, c_void_p, c_size_t, c_void_p]),
    "mpdok_mf_krylov_workspace_size": (c_size_t, [c_ll, c_int]),
    "mpdok_mf_gmres_ir": (c_int, [c_void_p, c_ll, c_int, c_int, c_double, c_double, c_void_p, c_void_p, c_double,
                                  c_int, c_int, c_double, c_void_p, c_size_t, ctypes.POINTER(SolveInfo), c_void_p]),
    "mpdok_mf_cg": (c_int, [c_void_p, c_ll, c_int, c_int, c_double, c_double, c_void_p, c_void_p, c_double, c_int,
                            c_int, c_void_p, c_size_t, ctypes.POINTER(SolveInfo), c_void_p]),
    "mpdok_split_matrix": (c_int, [c_void_p, c_ll, c_ll, c_ll, c_void_p, c_void_p, c_ll, c_void_p]),
    "mpdok_split_gemv_workspace_size": (c_size_t, [c_ll, c_ll, c_int]),
    "mpdok_split_gemv": (c_int, [c_void_p, c_void_p, c_ll, c_ll, c_ll, c_void_p, c_ll, c_int, c_void_p, c_ll,
                                 c_double, c_double, c_void_p, c_ll, c_void_p, c_size_t, c_void_p]),
    "mpdok_cg_ir_operator_size": (c_size_t, [c_ll, c_int]),
    "mpdok_cg_ir_workspace_size": (c_size_t, [c_ll, c_int, c_int]),
    "mpdok_cg_ir": (c_int, [c_void_p, c_ll, c_ll, c_int, c_void_p, c_int, c_int, c_void_p, c_ll, c_void_p, c_ll,
                            c_double, c_int, c_double, c_int, c_void_p, c_size_t, ctypes.POINTER(SolveInfo),
                            c_void_p]),
    "mpdok_mf_cg_ir_workspace_size": (c_size_t, [c_ll, c_int]),
    "mpdok_mf_cg_ir": (c_int, [c_void_p, c_ll, c_int, c_int, c_double, c_double, c_int, c_void_p, c_ll, c_void_p,
                               c_ll, c_double, c_int, c_double, c_int, c_void_p, c_size_t, ctypes.POINTER(SolveInfo),
                               c_void_p]),
    "mpdok_chol_cg_ir_workspace_size": (c_size_t, [c_ll, c_int, c_int]),
    "mpdok_chol_cg_ir": (c_int, [c_void_p, c_void_p, c_ll, c_void_p, c_int, c_int, c_double, c_double, c_ll, c_int,
                                 c_void_p, c_int, c_int, c_void_p, c_ll, c_void_p, c_ll, c_double, c_int, c_double,
                                 c_int, c_void_p, c_size_t, ctypes.POINTER(SolveInfo), c_void_p]),
    "mpdok_lu_cg_ir_workspace_size": (c_size_t, [c_ll, c_int, c_int]),
    "mpdok_lu_cg_ir": (c_int, [c_void_p, c_ll, c_ll, c_int, c_void_p, c_int, c_void_p, c_int, c_int, c_void_p, c_ll,
                               c_void_p, c_ll, c_double, c_int, c_double, c_int, c_void_p, c_size_t,
                               ctypes.POINTER(SolveInfo), c_void_p]),
    "mpdok_mf_lu_cg_ir": (c_int, [c_void_p, c_ll, c_int, c_int, c_double, c_double, c_void_p, c_int, c_int, c_void_p,
                                  c_ll, c_void_p, c_ll, c_double, c_int, c_double, c_int, c_void_p, c_size_t,
                                  ctypes.POINTER(SolveInfo), c_void_p]),
    "mpdok_ooc_create": (c_int, [c_ll, c_int, c_int, ctypes.c_char_p, ctypes.POINTER(c_void_p)]),
    "mpdok_ooc_destroy": (c_int, [c_void_p]),
    "mpdok_ooc_build": (c_int, [c_void_p, c_void_p, c_int, c_int, c_double, c_double, c_void_p]),
    "mpdok_ooc_matvec": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "mpdok_ooc_bytes_moved": (c_double, [c_void_p]),
    "mpdok_ooc_read_rows": (c_int, [c_void_p, c_ll, c_ll, c_void_p]),
    "mpdok_ooc_workspace_size": (c_size_t, [c_ll, c_int]),
    "mpdok_ooc_gmres_ir": (c_int, [c_void_p, c_void_p, c_int, c_int, c_double, c_double, c_void_p, c_void_p,
                                   c_double, c_int, c_int, c_double, c_void_p, c_size_t, ctypes.POINTER(SolveInfo),
                                   c_void_p]),
    "mpdok_profile_skipped": (c_ll, [c_int]),
    "mpdok_managed_kind": (c_int, []),
    "mpdok_lu_ir_multi_work_size": (c_size_t, [c_ll, c_int]),
    "mpdok_lu_ir_solve_multi": (c_int, [c_void_p, c_ll, c_ll, c_void_p, c_int, c_int, c_void_p, c_ll, c_void_p, c_ll,
                                        c_double, c_int, c_void_p, c_size_t, ctypes.POINTER(SolveInfo), c_void_p]),
    "mpdok_profile_bytes": (c_double, [c_int]),
    "mpdok_profile_timeline": (c_ll, [ctypes.POINTER(c_double), c_ll]),
    "mpdok_lu_schedule": (c_ll, [c_ll, c_int, ctypes.POINTER(c_ll), c_ll]),
    "mpdok_batch_create": (c_int, [c_int, c_void_p, c_int, c_int, c_int, c_int, c_int, ctypes.POINTER(c_void_p)]),
    "mpdok_batch_destroy": (c_int, [c_void_p]),
    "mpdok_batch_bytes": (c_size_t, [c_void_p]),
    "mpdok_batch_load": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "mpdok_batch_factor": (c_int, [c_void_p, c_void_p]),
    "mpdok_batch_solve": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_void_p]),
    "mpdok_batch_relres": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "mpdok_batch_adjoint": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "mpdok_batch_perturbed": (c_int, [c_void_p, c_void_p]),
    "mpdok_batch_graph_build": (c_int, [c_void_p, c_void_p, c_void_p, c_int]),
    "mpdok_batch_graph_launch": (c_int, [c_void_p, c_void_p]),
    "mpdok_batch_graph_nodes": (c_ll, [c_void_p]),
    "mpdok_batch_schedule": (c_int, [c_void_p, c_int, c_int]),
    "mpdok_rbf_adjoint_workspace_size": (c_size_t, [c_ll]),
    "mpdok_rbf_adjoint": (c_int, [c_void_p, c_ll, c_int, c_int, c_double, c_int, c_void_p, c_void_p, c_void_p,
                                  c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    "mpdok_batch_step": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_void_p]),
    "mpdok_batch_dag_status": (c_int, [c_void_p, c_void_p]),
    "mpdok_launch_count": (c_ll, []),
    "mpdok_profile_enable": (c_int, [c_int]),
    "mpdok_profile_query": (c_int, [c_int, ctypes.POINTER(c_double), ctypes.POINTER(c_ll), ctypes.POINTER(c_double)]),
    # reference ctypes ABI (mpdok_ops.py:361-382)
    "py_gmres_ir": (None, [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_double, c_int, c_int,
                           ctypes.POINTER(c_int)]),
    "py_alloc_managed": (None, [c_int, ctypes.POINTER(c_void_p)]),
    "py_free_managed": (None, []),
    # reference ctypes ABI (lu_ir.so, mpdok_ops.py:101-141)
    "py_lu_ir": (None, [c_void_p, c_void_p, c_void_p, c_int, c_double, c_int, ctypes.POINTER(c_int)]),
    "py_lu_factor": (None, [c_void_p, c_int, ctypes.POINTER(c_int)]),
    "py_lu_solve_factored": (None, [c_void_p, c_void_p, c_void_p, c_int, c_double, c_int, ctypes.POINTER(c_int)]),
    "py_lu_free_factored": (None, []),
    "py_lu_alloc_managed": (None, [c_int, ctypes.POINTER(c_void_p)]),
    "py_lu_free_managed": (None, []),
}

_lib = None


def load(path: str | os.PathLike | None = None) -> ctypes.CDLL:
    """Load (once) and return the native library with its signatures set."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path is not None else LIB_PATH
    if not p.exists():
        raise FileNotFoundError(
            f"{p} not found. Build the sm_103a library first: "
            "python -c 'import __graft_entry__ as g; g.build()' (or python -m mpdok_gb300._build)")
    lib = ctypes.CDLL(str(p))
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def declared_symbols() -> list[str]:
    return list(_SIGS)


def last_error() -> str:
    msg = load().mpdok_last_error()
    return msg.decode(errors="replace") if msg else ""


def debug_set(key: int, value: int) -> None:
    """Failure-path test hooks (DEBUG_WAIT_LIMIT, DEBUG_TRSV_FIRST_TICKET); see the header."""
    check(int(load().mpdok_debug_set(int(key), int(value))), "debug_set")


def call_error(lib) -> str:
    """The library's error message for the call just made (empty when it raised none).

    The reference-compatible py_* entry points return no status, so callers
    clear the message before the call (``lib.mpdok_clear_error()``) and read it
    afterwards to tell an error from plain non-convergence."""
    fn = getattr(lib, "mpdok_last_error", None)
    if fn is None:
        return ""
    msg = fn()
    return msg.decode(errors="replace") if msg else ""


def check(status: int, what: str = "") -> int:
    """Raise MPDOKError for negative statuses; return the status otherwise."""
    if status < 0:
        lib = load()
        base = lib.mpdok_status_string(status).decode(errors="replace")
        raise MPDOKError(status, f"{what}: {base}: {last_error()}")
    return status


def dtype_code(dt) -> int:
    import torch

    table = {torch.float64: F64, torch.float32: F32, torch.bfloat16: BF16, torch.float16: F16,
             np.dtype(np.float64): F64, np.dtype(np.float32): F32, np.dtype(np.float16): F16}
    try:
        return table[dt]
    except KeyError as e:
        raise ValueError(f"unsupported dtype {dt}") from e


def profile_enable(on: bool = True):
    check(load().mpdok_profile_enable(1 if on else 0), "profile_enable")


def profile_query(cls: int):
    """(total_ms, launches, work) of one kernel class since profile_enable()."""
    t = c_double(0.0)
    n = c_ll(0)
    w = c_double(0.0)
    check(load().mpdok_profile_query(cls, ctypes.byref(t), ctypes.byref(n), ctypes.byref(w)), "profile_query")
    return t.value, n.value, w.value


def profile_bytes(cls: int) -> float:
    """Algorithmic bytes of a class whose work counts flops."""
    return float(load().mpdok_profile_bytes(cls))


def profile_skipped(cls: int) -> int:
    """Launches of one class that a device skip flag turned off."""
    return int(load().mpdok_profile_skipped(cls))


def lu_schedule(n: int, fdtype: int) -> np.ndarray:
    """(steps, 12) int64 array: the launch schedule of mpdok_lu_factor (host only)."""
    lib = load()
    cnt = check(int(lib.mpdok_lu_schedule(n, fdtype, None, 0)), "lu_schedule")
    out = np.zeros((max(cnt, 1), 12), dtype=np.int64)
    check(int(lib.mpdok_lu_schedule(n, fdtype, out.ctypes.data_as(ctypes.POINTER(c_ll)), cnt)), "lu_schedule")
    return out[:cnt]


def profile_timeline() -> np.ndarray:
    """(records, 4) array of (class, start ms, end ms, work) of every timed
    launch since profile_enable(), in launch order."""
    lib = load()
    n = check(int(lib.mpdok_profile_timeline(None, 0)), "profile_timeline")
    out = np.zeros((max(n, 1), 4), dtype=np.float64)
    check(int(lib.mpdok_profile_timeline(out.ctypes.data_as(ctypes.POINTER(c_double)), n)), "profile_timeline")
    return out[:n]


def launch_count() -> int:
    return int(load().mpdok_launch_count())
