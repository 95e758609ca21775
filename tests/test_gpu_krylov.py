"""GPU parity: the device-resident Krylov solvers against the oracle and the
reference's golden outputs (dense_krylov.py / mpdok_ooc.py / mpdok_ops.py)."""
import warnings

import numpy as np
import pytest
import torch

from oracle import krylov_ref as O

pytestmark = pytest.mark.gpu


def _np(t):
    return t.detach().cpu().numpy()


def test_operator_matvec_and_residual_norm(golden):
    from mpdok_gb300.dense_krylov import DenseLinearOperator
    g = golden("dense_krylov")
    op = DenseLinearOperator(g["A_ns"], verbose=False)
    y = op.matvec(torch.from_numpy(g["b"].astype(np.float32)).cuda())
    assert y.dtype == torch.float32
    np.testing.assert_allclose(_np(y), g["y32"], rtol=1e-5, atol=1e-4)
    rn = op.residual_norm(torch.from_numpy(g["x_ir"]).cuda(), g["b"])
    assert rn == pytest.approx(float(g["rn"]), rel=1e-6, abs=1e-13)
    op.free_fp64()
    with pytest.raises(RuntimeError):
        op.residual_norm(g["x_ir"], g["b"])


def test_cg_matches_reference(golden):
    from mpdok_gb300.dense_krylov import DenseLinearOperator, cg
    g = golden("dense_krylov")
    op = DenseLinearOperator(g["A_spd"], verbose=False)
    x, h, c = cg(op, g["b"], tol=1e-6)
    assert c == bool(g["c_cg"])
    assert len(h) == len(g["h_cg"])
    np.testing.assert_allclose(_np(x), g["x_cg"], rtol=0, atol=1e-5 * np.abs(g["x_cg"]).max())


def test_gmres_matches_reference(golden):
    from mpdok_gb300.dense_krylov import DenseLinearOperator, gmres
    g = golden("dense_krylov")
    op = DenseLinearOperator(g["A_ns"], verbose=False)
    x, h, c = gmres(op, g["b"], tol=1e-6, restart=20)
    assert c == bool(g["c_gm"])
    assert [i for i, _ in h] == [int(i) for i in g["h_gm"][:, 0]]
    np.testing.assert_allclose(_np(x), g["x_gm"], rtol=0, atol=1e-5 * np.abs(g["x_gm"]).max())


@pytest.mark.parametrize("key", ["", "_spd"])
def test_gmres_ir_matches_reference(golden, key):
    from mpdok_gb300.dense_krylov import DenseLinearOperator, gmres_ir
    g = golden("dense_krylov")
    A = g["A_ns"] if key == "" else g["A_spd"]
    op = DenseLinearOperator(A, verbose=False)
    x, h, c = gmres_ir(op, g["b"], tol=1e-11, restart=20)
    assert c == bool(g["c_ir" + key]) and c
    assert len(h) == len(g["h_ir" + key])
    ref = g["x_ir" + key]
    np.testing.assert_allclose(_np(x), ref, rtol=0, atol=1e-10 * np.abs(ref).max())


def _rbf_system(n, gamma, reg, seed=0, dim=2):
    rng = np.random.default_rng(seed)
    X = rng.uniform(0, 1, size=(n, dim))
    b = rng.standard_normal(n)
    return X, O.rbf_matrix(X, gamma=gamma, reg=reg), b


def test_mpdok_solver_gmres_ir_on_rbf():
    """The reference algorithm (unpreconditioned inner GMRES) on a kappa ~ 5e3
    RBF system contracts ~3x per outer step: same trajectory as the oracle."""
    import ctypes
    from mpdok_gb300 import _native as N
    from mpdok_gb300.mpdok_ops import MPDOKSolver
    from mpdok_gb300.rbf_kernel import build_rbf_kernel
    X, A64, b = _rbf_system(1500, 100.0, 1e-2)
    A, _ = build_rbf_kernel(X, gamma=100.0, reg=1e-2)
    lib = N.load()
    A32 = torch.empty_strided((1500, 1500), (1, 1500), dtype=torch.float32, device="cuda")
    x = torch.zeros(1500, dtype=torch.float64, device="cuda")
    db = torch.from_numpy(b).cuda()
    ws = torch.empty(lib.mpdok_krylov_workspace_size(1500, 50), dtype=torch.uint8, device="cuda")
    info = N.SolveInfo()
    assert lib.mpdok_gmres_ir(ctypes.c_void_p(A.data_ptr()), 1500, ctypes.c_void_p(A32.data_ptr()), 1500, 0, 1500,
                              ctypes.c_void_p(db.data_ptr()), ctypes.c_void_p(x.data_ptr()), 1e-12, 8, 50, 1e-6,
                              ctypes.c_void_p(ws.data_ptr()), ws.numel(), ctypes.byref(info), None) == 0
    x_or, hist_or, conv_or, _ = O.gmres_ir_native(A64, b, tol=1e-12, maxiter_outer=8, restart=50)
    h = info.history_list()
    assert len(h) == len(hist_or) and not conv_or and not info.converged
    for (i, r), (io, ro) in zip(h, hist_or):
        assert i == io and 0.7 < r / ro < 1.4
    # better conditioned: converges to FP64 accuracy through the reference ABI
    X, A64, b = _rbf_system(1500, 900.0, 1e-1, seed=5)
    A, _ = build_rbf_kernel(X, gamma=900.0, reg=1e-1)
    xs = MPDOKSolver().solve(A, b, tol=1e-12, maxiter_outer=20, restart=50).cpu().numpy()
    x_lu = O.fp64_solve(A64, b)
    assert O.relres(A64, xs, b) <= max(1e-12, 10 * O.relres(A64, x_lu, b))
    assert np.linalg.norm(xs - x_lu) / np.linalg.norm(x_lu) < 1e-9


def test_gmres_ir_native_api_history_and_status():
    import ctypes
    from mpdok_gb300 import _native as N
    lib = N.load()
    X, A64, b = _rbf_system(800, 900.0, 1e-1, seed=3)
    dA = torch.from_numpy(A64.T.copy()).cuda().t()
    A32 = torch.empty_strided((800, 800), (1, 800), dtype=torch.float32, device="cuda")
    db = torch.from_numpy(b).cuda()
    x = torch.zeros(800, dtype=torch.float64, device="cuda")
    ws = torch.empty(lib.mpdok_krylov_workspace_size(800, 30), dtype=torch.uint8, device="cuda")
    info = N.SolveInfo()
    st = lib.mpdok_gmres_ir(ctypes.c_void_p(dA.data_ptr()), 800, ctypes.c_void_p(A32.data_ptr()), 800, 0, 800,
                            ctypes.c_void_p(db.data_ptr()), ctypes.c_void_p(x.data_ptr()), 1e-12, 6, 30, 1e-6,
                            ctypes.c_void_p(ws.data_ptr()), ws.numel(), ctypes.byref(info), None)
    assert st == 0, N.last_error()
    assert info.converged == 1
    h = info.history_list()
    assert h[0] == (0, pytest.approx(1.0))
    assert all(h[i + 1][1] < h[i][1] for i in range(len(h) - 1))
    x_or, hist_or, _, steps = O.gmres_ir_native(A64, b, tol=1e-12, maxiter_outer=6, restart=30)
    assert len(h) == len(hist_or)
    assert abs(info.inner_iters - steps) <= 2
    np.testing.assert_allclose(A32.cpu().numpy(), A64.astype(np.float32), rtol=0, atol=0)


def test_solver_edge_cases():
    from mpdok_gb300.mpdok_ops import MPDOKSolver
    s = MPDOKSolver()
    A = np.eye(5) * 3.0
    x = s.solve(A, np.zeros(5))
    assert torch.count_nonzero(x) == 0
    x = s.solve(A, np.ones(5), tol=1e-14)
    np.testing.assert_allclose(_np(x), np.ones(5) / 3.0, rtol=1e-15)
    x = s.solve(np.array([[2.0]]), np.array([4.0]))
    assert float(x[0]) == 2.0
    with pytest.raises(ValueError):
        s.solve(np.eye(3), np.ones(4))
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        X, A64, b = _rbf_system(400, 9.0, 1e-8, seed=1)
        s.solve(A64, b, tol=1e-15, maxiter_outer=1, restart=5)
        assert any(issubclass(i.category, RuntimeWarning) for i in w)


def test_cg_on_spd_rbf_reaches_fp32_floor():
    from mpdok_gb300.dense_krylov import DenseLinearOperator, cg
    X, A64, b = _rbf_system(2000, 400.0, 1e-1, seed=2, dim=3)
    op = DenseLinearOperator(A64, verbose=False)
    x, h, c = cg(op, b, tol=1e-5, check_every=5)
    x_or, h_or, c_or = O.cg(A64, b, tol=1e-5, check_every=5)
    assert c and c_or
    assert abs(len(h) - len(h_or)) <= 1
    assert O.relres(A64, _np(x), b) < 1e-5


def test_alloc_managed_is_device_memory_and_solves():
    """py_alloc_managed / py_lu_alloc_managed keep the reference's API but hand
    out device memory (no page migration); the solvers run on it."""
    from mpdok_gb300 import _native as N
    from mpdok_gb300.mpdok_ops import LUIRSolver, MPDOKSolver
    rng = np.random.default_rng(12)
    n = 700
    X = rng.uniform(0, 1, (n, 2))
    A64 = O.rbf_matrix(X, gamma=400.0, reg=1e-2)
    b = rng.standard_normal(n)
    for cls in (MPDOKSolver, LUIRSolver):
        s = cls()
        M = s.alloc_managed(n)
        assert N.load().mpdok_managed_kind() == 0
        M[:, :] = torch.from_numpy(A64).cuda()
        kw = {"maxiter_outer": 20, "restart": 50} if cls is MPDOKSolver else {"maxiter_outer": 5}
        x = s.solve(M.array, torch.from_numpy(b).cuda(), tol=1e-12, **kw).cpu().numpy()
        assert O.relres(A64, x, b) < 1e-11
        s.free_managed()
