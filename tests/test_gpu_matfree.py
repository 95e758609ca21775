"""GPU parity: matrix-free evaluate-and-multiply (TMA-staged centre tiles) and
the Krylov solves on it, against the oracle's dense products and FP64 LU."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import krylov_ref as O

pytestmark = pytest.mark.gpu


def _apply(rows, cols, gamma, reg, kernel, diag_off, X, precision):
    from mpdok_gb300 import _native as N
    lib = N.load()
    nr, nc, dim = rows.shape[0], cols.shape[0], rows.shape[1]
    tdt = torch.float64 if precision == N.F64 else torch.float32
    k = X.shape[1]
    ldx = nc if precision == N.F64 else (nc + 3) // 4 * 4
    dX = torch.zeros((k, ldx), dtype=tdt, device="cuda")
    dX[:, :nc] = torch.from_numpy(X.T.copy()).to(tdt)
    dY = torch.empty((k, nr), dtype=tdt, device="cuda")
    dr = torch.from_numpy(np.ascontiguousarray(rows)).cuda()
    dc = torch.from_numpy(np.ascontiguousarray(cols)).cuda()
    w = torch.empty(lib.mpdok_matfree_workspace_size(nr, nc, k, precision), dtype=torch.uint8, device="cuda")
    st = lib.mpdok_matfree_apply(ctypes.c_void_p(dr.data_ptr()), nr, ctypes.c_void_p(dc.data_ptr()), nc, dim,
                                 {"gaussian": 0, "mq": 1}[kernel], gamma, reg, diag_off, precision,
                                 ctypes.c_void_p(dX.data_ptr()), ldx, k, ctypes.c_void_p(dY.data_ptr()), nr,
                                 ctypes.c_void_p(w.data_ptr()), w.numel(), None)
    assert st == 0, N.last_error()
    return dY.double().cpu().numpy().T


@pytest.mark.parametrize("kernel,gamma", [("gaussian", 25.0), ("gaussian", 1600.0), ("mq", 4.0)])
@pytest.mark.parametrize("dim", [1, 2, 3])
@pytest.mark.parametrize("k", [1, 3, 8])
def test_matfree_f32_matches_dense(kernel, gamma, dim, k):
    from mpdok_gb300 import _native as N
    rng = np.random.default_rng(dim * 10 + k)
    rows = rng.uniform(0, 1, (1000, dim))
    cols = rng.uniform(0, 1, (1500, dim))
    X = rng.standard_normal((1500, k))
    A = O.rbf_matrix(rows, cols, gamma=gamma, reg=0.3, kernel=kernel, diag_offset=200)
    got = _apply(rows, cols, gamma, 0.3, kernel, 200, X, N.F32)
    ref = A @ X
    scale = np.abs(A) @ np.abs(X)
    assert np.all(np.abs(got - ref) <= 2e-5 * scale + 1e-6)


@pytest.mark.parametrize("kernel,gamma", [("gaussian", 100.0), ("mq", 4.0)])
def test_matfree_f64_matches_dense(kernel, gamma):
    from mpdok_gb300 import _native as N
    rng = np.random.default_rng(7)
    X3 = rng.uniform(0, 1, (777, 3))
    x = rng.standard_normal((777, 2))
    A = O.rbf_matrix(X3, gamma=gamma, reg=1e-3, kernel=kernel)
    got = _apply(X3, X3, gamma, 1e-3, kernel, 0, x, N.F64)
    ref = A @ x
    assert np.all(np.abs(got - ref) <= 1e-13 * (np.abs(A) @ np.abs(x)))


def test_matfree_operator_matvec_vs_stored():
    from mpdok_gb300.dense_krylov import DenseLinearOperator
    from mpdok_gb300.matfree import MatrixFreeOperator
    rng = np.random.default_rng(3)
    X = rng.uniform(0, 1, (3000, 2))
    A = O.rbf_matrix(X, gamma=400.0, reg=1e-2)
    v = rng.standard_normal(3000).astype(np.float32)
    mf = MatrixFreeOperator(X, gamma=400.0, reg=1e-2)
    st = DenseLinearOperator(A, verbose=False)
    y1 = mf.matvec(torch.from_numpy(v).cuda()).double().cpu().numpy()
    y2 = st.matvec(torch.from_numpy(v).cuda()).double().cpu().numpy()
    assert np.allclose(y1, y2, rtol=0, atol=1e-5 * np.abs(y2).max())


def test_matfree_gmres_ir_and_cg_solve():
    from mpdok_gb300.dense_krylov import cg, gmres_ir
    from mpdok_gb300.matfree import MatrixFreeOperator
    rng = np.random.default_rng(5)
    X = rng.uniform(0, 1, (1500, 2))
    b = rng.standard_normal(1500)
    A = O.rbf_matrix(X, gamma=900.0, reg=1e-1)
    mf = MatrixFreeOperator(X, gamma=900.0, reg=1e-1)
    x, h, c = gmres_ir(mf, b, tol=1e-12, maxiter_outer=20, restart=50)
    x_lu = O.fp64_solve(A, b)
    assert c and O.relres(A, x.cpu().numpy(), b) <= max(1e-12, 10 * O.relres(A, x_lu, b))
    assert np.linalg.norm(x.cpu().numpy() - x_lu) / np.linalg.norm(x_lu) < 1e-9
    x2, h2, c2 = cg(mf, b, tol=1e-5, check_every=5)
    x3, h3, c3 = O.cg(A, b, tol=1e-5, check_every=5)
    assert c2 and c3 and abs(len(h2) - len(h3)) <= 1


@pytest.mark.parametrize("m,n,k", [(1, 1, 1), (3001, 1234, 1), (257, 4096, 3), (64, 513, 11)])
@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_rbf_evaluate_at_query_points(m, n, k, precision):
    """f(q) = sum_i alpha_i phi(||q - c_i||) (enkf_solver.py:162-200) against the dense oracle."""
    from mpdok_gb300.matfree import rbf_evaluate
    rng = np.random.default_rng(m + n + k)
    C = rng.uniform(0, 1, (n, 2))
    Q = rng.uniform(-0.1, 1.1, (m, 2))
    alpha = rng.standard_normal((n, k)) if k > 1 else rng.standard_normal(n)
    K = O.rbf_matrix(Q, C, gamma=30.0, reg=0.0)
    ref = K @ alpha
    got = rbf_evaluate(alpha, C, Q, 30.0, precision=precision).cpu().numpy()
    assert got.shape == ref.shape and got.dtype == np.float64
    bound = np.abs(K) @ np.abs(alpha)
    tol = 1e-13 if precision == "f64" else 2e-5
    assert np.all(np.abs(got - ref) <= tol * bound + (0 if precision == "f64" else 1e-6))


def test_rbf_evaluate_reconstructs_solved_field():
    """Solve on the centres, evaluate back at the centres: reproduces b up to the nugget term."""
    from mpdok_gb300.matfree import MatrixFreeOperator
    rng = np.random.default_rng(5)
    C = rng.uniform(0, 1, (800, 2))
    b = np.sin(2 * np.pi * C[:, 0]) * np.cos(2 * np.pi * C[:, 1])
    A = O.rbf_matrix(C, gamma=400.0, reg=1e-3)
    alpha = O.fp64_solve(A, b)
    op = MatrixFreeOperator(C, gamma=400.0, reg=1e-3)
    f = op.evaluate(C, alpha).cpu().numpy()
    np.testing.assert_allclose(f + 1e-3 * alpha, b, atol=1e-10)
