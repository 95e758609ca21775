"""GPU: failure paths, each made on the host (the failure handling of the reference's solvers).

* a right-hand side with a NaN gives a clean MPDOK_ERR_NONFINITE status from
  every solver entry point, and the drop-in wrappers' warning names the error;
* a truncated out-of-core tile file gives MPDOK_ERR_IO;
* a device allocation that fails under a memory cap gives the reference's
  ResourceWarning and re-raises (mpdok_ops.py:270-282);
* a bounded device wait that runs out returns MPDOK_ERR_TIMEOUT: a test hook
  shortens the triangular solves' wait limit and raises their first ticket, so
  no block ever solves block 0 and the blocks that need it give up and return.
  The device stays usable, which the same test checks with a normal solve.

Nothing here faults, traps or hangs the GPU: every wait is bounded and the
failing inputs are rejected by the host or by the kernels' own checks.
"""
import ctypes
import os
import warnings

import numpy as np
import pytest
import torch

from oracle import krylov_ref as O

pytestmark = pytest.mark.gpu


def _ptr(t):
    return ctypes.c_void_p(0 if t is None else t.data_ptr())


def _system(n=300, seed=0):
    rng = np.random.default_rng(seed)
    X = rng.uniform(0, 1, (n, 2))
    A = O.rbf_matrix(X, gamma=200.0, reg=1e-2)
    b = rng.standard_normal(n)
    return A, b


def _fortran(A, dtype=torch.float64):
    from mpdok_gb300._device import as_fortran
    return as_fortran(A, dtype)


def _factor(lib, A64, n, fdtype):
    from mpdok_gb300 import _native as N
    fac = torch.empty(lib.mpdok_lu_factor_size(n, fdtype), dtype=torch.uint8, device="cuda")
    work = torch.empty(max(lib.mpdok_lu_work_size(n, fdtype), lib.mpdok_lu_ir_work_size(n),
                           lib.mpdok_lu_apply_work_size(n), lib.mpdok_lu_gmres_ir_work_size(n, 30)),
                       dtype=torch.uint8, device="cuda")
    st = lib.mpdok_lu_factor(_ptr(A64), n, n, fdtype, 0, _ptr(fac), fac.numel(), _ptr(work), work.numel(), None)
    assert st >= 0, N.last_error()
    return fac, work


def test_nan_rhs_is_reported_as_nonfinite(native_lib):
    from mpdok_gb300 import _native as N
    lib = native_lib
    A, b = _system()
    n = A.shape[0]
    A64 = _fortran(A)
    A32 = _fortran(A, torch.float32)
    bad = torch.tensor(b, device="cuda")
    bad[17] = float("nan")
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    info = N.SolveInfo()
    fac, work = _factor(lib, A64, n, N.F32)
    st = lib.mpdok_lu_ir_solve(_ptr(A64), n, n, _ptr(fac), N.F32, _ptr(bad), _ptr(x), 1e-12, 5, _ptr(work),
                               work.numel(), ctypes.byref(info), None)
    assert st == N.ERR_NONFINITE and "non-finite" in N.last_error()
    st = lib.mpdok_lu_gmres_ir(_ptr(A64), n, _ptr(A32), n, n, _ptr(fac), N.F32, _ptr(bad), _ptr(x), 1e-12, 5, 30,
                               1e-6, _ptr(work), work.numel(), ctypes.byref(info), None)
    assert st == N.ERR_NONFINITE
    kw = torch.empty(lib.mpdok_krylov_workspace_size(n, 30), dtype=torch.uint8, device="cuda")
    st = lib.mpdok_gmres_ir(_ptr(A64), n, _ptr(A32), n, 0, n, _ptr(bad), _ptr(x), 1e-12, 5, 30, 1e-6, _ptr(kw),
                            kw.numel(), ctypes.byref(info), None)
    assert st == N.ERR_NONFINITE
    st = lib.mpdok_cg(_ptr(A32), n, _ptr(A64), n, n, _ptr(bad), _ptr(x), 1e-12, 50, 10, _ptr(kw), kw.numel(),
                      ctypes.byref(info), None)
    assert st == N.ERR_NONFINITE
    # multi-RHS LU-IR: the second column carries the NaN
    B = torch.tensor(np.stack([b, b], axis=1), device="cuda").t().contiguous().t()
    B[5, 1] = float("inf")
    X = torch.zeros_like(B)
    mw = torch.empty(lib.mpdok_lu_ir_multi_work_size(n, 2), dtype=torch.uint8, device="cuda")
    st = lib.mpdok_lu_ir_solve_multi(_ptr(A64), n, n, _ptr(fac), N.F32, 2, _ptr(B), n, _ptr(X), n, 1e-12, 5,
                                     _ptr(mw), mw.numel(), ctypes.byref(info), None)
    assert st == N.ERR_NONFINITE and "right-hand side 1" in N.last_error()
    # the drop-in wrappers turn the swallowed status into a warning that names it
    from mpdok_gb300.mpdok_ops import MPDOKSolver
    with pytest.warns(RuntimeWarning, match="library error: .*non-finite"):
        MPDOKSolver().solve(A64, bad, tol=1e-12)
    # a clean solve afterwards warns about nothing and converges
    with warnings.catch_warnings():
        warnings.simplefilter("error")
        xs = MPDOKSolver().solve(A64, torch.tensor(b, device="cuda"), tol=1e-12, maxiter_outer=20, restart=40)
    assert O.relres(A, xs.cpu().numpy(), b) < 1e-11


def test_truncated_tile_file_is_an_io_error(native_lib, tmp_path):
    from mpdok_gb300 import _native as N
    lib = native_lib
    rng = np.random.default_rng(3)
    n, rows = 600, 128
    X = torch.tensor(rng.uniform(0, 1, (n, 2)), device="cuda")
    path = str(tmp_path / "A_fp32.bin")
    h = ctypes.c_void_p()
    assert lib.mpdok_ooc_create(n, rows, 1, path.encode(), ctypes.byref(h)) == 0
    try:
        assert lib.mpdok_ooc_build(h, _ptr(X), 2, N.KERNEL_GAUSSIAN, 50.0, 1e-2, None) == 0
        torch.cuda.synchronize()
        assert os.path.getsize(path) == n * n * 4
        x = torch.ones(n, dtype=torch.float32, device="cuda")
        y = torch.empty(n, dtype=torch.float32, device="cuda")
        assert lib.mpdok_ooc_matvec(h, _ptr(x), _ptr(y), None) == 0
        torch.cuda.synchronize()
        # cut the file inside its last tile: the product must fail loudly
        os.truncate(path, (n - 10) * n * 4)
        st = lib.mpdok_ooc_matvec(h, _ptr(x), _ptr(y), None)
        torch.cuda.synchronize()
        assert st == N.ERR_IO
        assert "short file" in N.last_error()
        buf = np.empty((20, n), dtype=np.float32)
        st = lib.mpdok_ooc_read_rows(h, n - 20, 20, buf.ctypes.data_as(ctypes.c_void_p))
        assert st == N.ERR_IO
    finally:
        lib.mpdok_ooc_destroy(h)


def test_out_of_memory_warns_and_reraises():
    from mpdok_gb300.mpdok_ops import MPDOKSolver
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    total = torch.cuda.get_device_properties(0).total_memory
    n = 12000  # A in FP64 is 1.15 GB; the solver's FP32 scratch (a torch allocation) another 0.58 GB
    A = torch.empty((n, n), dtype=torch.float64, device="cuda").t()
    b = torch.ones(n, dtype=torch.float64, device="cuda")
    # cap this process at what it already holds plus 64 MB: the next large
    # allocation (the FP32 copy of A) fails inside solve()
    frac = (torch.cuda.memory_reserved() + (64 << 20)) / total
    torch.cuda.set_per_process_memory_fraction(frac, 0)
    try:
        with pytest.warns(ResourceWarning, match="VRAM insufficient"):
            with pytest.raises(torch.cuda.OutOfMemoryError):
                MPDOKSolver().solve(A, b)
    finally:
        torch.cuda.set_per_process_memory_fraction(1.0, 0)
        del A
        torch.cuda.empty_cache()


def test_bounded_wait_reports_timeout_and_device_recovers(native_lib):
    from mpdok_gb300 import _native as N
    lib = native_lib
    A, b = _system(n=700, seed=1)
    n = A.shape[0]
    A64 = _fortran(A)
    fac, work = _factor(lib, A64, n, N.F16)
    v = torch.tensor(b, dtype=torch.float32, device="cuda")
    z = torch.empty(n, dtype=torch.float32, device="cuda")
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    info = N.SolveInfo()
    aw = torch.empty(lib.mpdok_lu_apply_work_size(n), dtype=torch.uint8, device="cuda")
    try:
        N.debug_set(N.DEBUG_WAIT_LIMIT, 2048)
        N.debug_set(N.DEBUG_TRSV_FIRST_TICKET, 1)
        st = lib.mpdok_lu_apply(_ptr(fac), n, N.F16, _ptr(v), _ptr(z), _ptr(aw), aw.numel(), None)
        assert st == N.ERR_TIMEOUT, (st, N.last_error())
        assert "ran out" in N.last_error()
        st = lib.mpdok_lu_ir_solve(_ptr(A64), n, n, _ptr(fac), N.F16, _ptr(torch.tensor(b, device="cuda")), _ptr(x),
                                   1e-12, 3, _ptr(work), work.numel(), ctypes.byref(info), None)
        assert st == N.ERR_TIMEOUT
    finally:
        N.debug_set(N.DEBUG_TRSV_FIRST_TICKET, 0)
        N.debug_set(N.DEBUG_WAIT_LIMIT, 0)
    torch.cuda.synchronize()
    # the context is intact: the same solve now converges (from x = 0: the
    # timed-out solve left NaN in x, which the solver rejects as a start)
    bt = torch.tensor(b, device="cuda")
    st = lib.mpdok_lu_gmres_ir(_ptr(A64), n, _ptr(_fortran(A, torch.float32)), n, n, _ptr(fac), N.F16, _ptr(bt),
                               _ptr(x), 1e-12, 10, 30, 1e-6, _ptr(work), work.numel(), ctypes.byref(info), None)
    assert st == N.ERR_NONFINITE and "initial guess" in N.last_error()
    x.zero_()
    st = lib.mpdok_lu_gmres_ir(_ptr(A64), n, _ptr(_fortran(A, torch.float32)), n, n, _ptr(fac), N.F16, _ptr(bt),
                               _ptr(x), 1e-12, 10, 30, 1e-6, _ptr(work), work.numel(), ctypes.byref(info), None)
    assert st == 0 and info.converged == 1
    assert O.relres(A, x.cpu().numpy(), b) < 1e-11
