"""GPU parity: split (two-slice FP32) GEMV and multi-RHS CG-IR (C2 family:
SPD Gaussian systems, several right-hand sides), stored, split and matrix-free,
unpreconditioned and preconditioned by the tensor-core LU."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import krylov_ref as O

pytestmark = pytest.mark.gpu


def test_split_gemv_is_fp64_accurate():
    from mpdok_gb300 import _native as N
    lib = N.load()
    rng = np.random.default_rng(2)
    m, n, k = 3001, 2999, 3
    A = O.rbf_matrix(rng.uniform(0, 1, (m, 3)), rng.uniform(0, 1, (n, 3)), gamma=25.0)
    X = rng.standard_normal((n, k))
    B = rng.standard_normal((m, k))
    ld = (m + 3) // 4 * 4
    dA = torch.zeros((n, ld), dtype=torch.float64, device="cuda")
    dA[:, :m] = torch.from_numpy(A.T.copy())
    hi = torch.empty((n, ld), dtype=torch.float32, device="cuda")
    lo = torch.empty((n, ld), dtype=torch.float32, device="cuda")
    P = ctypes.c_void_p
    assert lib.mpdok_split_matrix(P(dA.data_ptr()), ld, m, n, P(hi.data_ptr()), P(lo.data_ptr()), ld, None) == 0
    dX = torch.from_numpy(X.T.copy()).cuda()
    dB = torch.from_numpy(B.T.copy()).cuda()
    Y = torch.empty((k, m), dtype=torch.float64, device="cuda")
    w = torch.empty(lib.mpdok_split_gemv_workspace_size(m, n, k), dtype=torch.uint8, device="cuda")
    assert lib.mpdok_split_gemv(P(hi.data_ptr()), P(lo.data_ptr()), ld, m, n, P(dX.data_ptr()), n, k,
                                P(Y.data_ptr()), m, -1.0, 1.0, P(dB.data_ptr()), m, P(w.data_ptr()), w.numel(),
                                None) == 0, N.last_error()
    ref = B - A @ X
    got = Y.cpu().numpy().T
    scale = np.abs(A) @ np.abs(X) + np.abs(B)
    assert np.all(np.abs(got - ref) <= 1e-13 * scale)


def _spd(n, gamma, reg, seed, dim=3, k=4):
    rng = np.random.default_rng(seed)
    X = rng.uniform(0, 1, (n, dim))
    return X, O.rbf_matrix(X, gamma=gamma, reg=reg), rng.standard_normal((n, k))


@pytest.mark.parametrize("split", [False, True])
def test_cg_ir_well_conditioned_reaches_fp64(split):
    from mpdok_gb300.dense_krylov import DenseLinearOperator, cg_ir
    X, A, B = _spd(2000, 900.0, 1e-1, seed=4)
    op = DenseLinearOperator(A, verbose=False)
    Xs, hist, conv = cg_ir(op, B, tol=1e-12, maxiter_outer=10, split=split)
    assert conv and hist[0] == (0, pytest.approx(1.0))
    Xs = Xs.cpu().numpy()
    Xlu = np.linalg.solve(A, B)
    for j in range(B.shape[1]):
        assert O.relres(A, Xs[:, j], B[:, j]) < 1e-12
    assert np.linalg.norm(Xs - Xlu) / np.linalg.norm(Xlu) < 1e-10


def test_matfree_cg_ir_well_conditioned():
    from mpdok_gb300.matfree import MatrixFreeOperator
    X, A, B = _spd(2000, 900.0, 1e-1, seed=6)
    mf = MatrixFreeOperator(X, gamma=900.0, reg=1e-1)
    Xs, hist, conv = mf.cg_ir(B, tol=1e-12, maxiter_outer=10)
    assert conv and hist[0] == (0, pytest.approx(1.0)) and hist[-1][1] < 1e-12
    Xs = Xs.cpu().numpy()
    Xlu = np.linalg.solve(A, B)
    for j in range(B.shape[1]):
        # the solver's own (matrix-free FP64) residual met 1e-12; a second FP64
        # evaluation (dense, other summation order) differs by ~n u |A||x|
        noise = 2 * A.shape[0] * 1.1e-16 * np.linalg.norm(np.abs(A) @ np.abs(Xs[:, j])) / np.linalg.norm(B[:, j])
        assert O.relres(A, Xs[:, j], B[:, j]) < 1e-12 + noise
    assert np.linalg.norm(Xs - Xlu) / np.linalg.norm(Xlu) < 1e-10


@pytest.mark.parametrize("variant", ["stored", "split", "matfree"])
def test_lu_preconditioned_cg_ir(variant):
    """PCG inner (z = (LU)^-1 r) with FP32 factors on a kappa ~ 6e3 Gaussian
    family member (kappa * u_f < 1): converges to the FP64 LU oracle's level."""
    from mpdok_gb300.dense_krylov import DenseLinearOperator, cg_ir
    from mpdok_gb300.lu import LUFactorization
    from mpdok_gb300.matfree import MatrixFreeOperator
    X, A, B = _spd(2000, 1600.0, 1e-2, seed=9, dim=2)
    lu = LUFactorization(A, dtype="fp32")
    Xlu = np.linalg.solve(A, B)
    floor = max(O.relres(A, Xlu[:, j], B[:, j]) for j in range(B.shape[1]))
    if variant == "matfree":
        Xs, hist, conv = MatrixFreeOperator(X, gamma=1600.0, reg=1e-2).cg_ir(B, tol=1e-12, maxiter_outer=8,
                                                                             precond=lu)
    else:
        op = DenseLinearOperator(A, verbose=False)
        Xs, hist, conv = cg_ir(op, B, tol=1e-12, maxiter_outer=8, split=variant == "split", precond=lu)
    Xs = Xs.cpu().numpy()
    worst = max(O.relres(A, Xs[:, j], B[:, j]) for j in range(B.shape[1]))
    assert conv and hist[0] == (0, pytest.approx(1.0))
    assert worst <= max(2e-12, 10 * floor)
    assert np.linalg.norm(Xs - Xlu) / np.linalg.norm(Xlu) < 1e-9


def test_cg_ir_c2_family_reports_infeasibility():
    """C2 family (3-D, eps = 5, nugget 1e-6): kappa ~ 7e7 already at N = 2000, so
    kappa * u_32 > 1 and an FP32 CG body cannot converge; the FP64 LU oracle's
    own relres is ~2e-9 > 1e-12.  The solver must stop cleanly and say so."""
    from mpdok_gb300.dense_krylov import DenseLinearOperator, cg_ir
    X, A, B = _spd(2000, 25.0, 1e-6, seed=1)
    op = DenseLinearOperator(A, verbose=False)
    Xs, hist, conv = cg_ir(op, B, tol=1e-12, maxiter_outer=3, inner_maxiter=100, split=True)
    assert not conv
    assert len(hist) == 4 and hist[0] == (0, pytest.approx(1.0))
    assert np.all(np.isfinite(Xs.cpu().numpy()))


@pytest.mark.parametrize("variant", ["stored", "split", "matfree"])
def test_c2_family_through_cholesky_preconditioned_cg_ir(variant):
    """C2's family (3-D Gaussian eps=5, nugget 1e-6, 4 RHS; kappa ~ 1e8 at this
    N): every FP32 CG body stalls here (kappa * 6e-8 > 1).  With the inner CG
    preconditioned by the FP64-accurate Cholesky factor, CG-IR reaches the
    FP64 LU oracle's own floor on every column (relres <= 10x the oracle's)."""
    from mpdok_gb300.batch import CholeskyPreconditioner
    from mpdok_gb300.dense_krylov import DenseLinearOperator, cg_ir
    from mpdok_gb300.matfree import MatrixFreeOperator
    n = 5000
    X, A, B = _spd(n, 25.0, 1e-6, seed=1)
    pc = CholeskyPreconditioner(X, eps=5.0, reg=1e-6, nrhs=4)
    if variant == "matfree":
        op = MatrixFreeOperator(X, gamma=25.0, reg=1e-6)
        Xs, hist, conv = op.cg_ir(B, tol=1e-12, maxiter_outer=8, inner_tol=1e-6, inner_maxiter=6, precond=pc)
    else:
        op = DenseLinearOperator(A, verbose=False)
        Xs, hist, conv = cg_ir(op, B, tol=1e-12, maxiter_outer=8, inner_tol=1e-6, inner_maxiter=6,
                               split=(variant == "split"), precond=pc)
    Xs = Xs.cpu().numpy()
    for j in range(B.shape[1]):
        x_lu = O.fp64_solve(A, B[:, j])
        floor = O.relres(A, x_lu, B[:, j])
        rel = O.relres(A, Xs[:, j], B[:, j])
        assert rel <= max(1e-12, 10 * floor), (variant, j, rel, floor, hist)
        assert np.linalg.norm(Xs[:, j] - x_lu) / np.linalg.norm(x_lu) < 1e3 * max(floor, 1e-13) * 1e4
    # a handful of preconditioned steps per refinement, not hundreds
    assert hist[-1][0] <= 8
