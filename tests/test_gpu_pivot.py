"""GPU parity: LU with partial pivoting (the reference's Sgetrf semantics).

The reference's LU-IR factors with cusolverDnSgetrf (L, U and P,
benchmark_mpdok.ipynb:989-990) and ``LUIRSolver.factor`` raises on LAPACK's
info != 0 (mpdok_ops.py:195-202).  These tests run matrices that cannot be
factored without row exchanges (a dense N(0,1) matrix and one with an exactly
zero diagonal) through the drop-in ``LUIRSolver`` and the factor API, and
compare with the oracle (oracle/lu_ref.py): the same power-of-two
equilibration, LAPACK dgetrf's pivot rows, P W = L U to FP32 rounding, |L| <= 1,
LAPACK's info on a singular matrix, and LU-IR reaching <= 10x the relres of
SciPy's FP64 lu_factor / lu_solve with refinement.
"""
import numpy as np
import pytest
import torch

from oracle import lu_ref as R

pytestmark = pytest.mark.gpu


def _factor(A, dtype="fp32"):
    from mpdok_gb300.lu import LUFactorization
    return LUFactorization(torch.tensor(A, device="cuda").t().contiguous().t(), dtype=dtype, pivoting=True)


@pytest.mark.parametrize("n", [1, 5, 129, 300, 1000, 2100])
@pytest.mark.parametrize("kind", ["gaussian", "zero_diagonal"])
def test_factor_matches_lapack_getrf(n, kind):
    if kind == "zero_diagonal" and n % 2:
        n += 1  # the anti-diagonal misses the diagonal only for even n
    A = R.test_matrices(n, seed=n)[kind]
    lu = _factor(A, "fp32")
    assert lu.info == 0
    LU, ipiv, perm, dr, dc = (t.cpu().numpy() for t in lu.export())
    lu_ref, piv_ref, info_ref, dr_ref, dc_ref = R.getrf(A)
    assert info_ref == 0
    # the equilibration is exact powers of two, computed the same way
    np.testing.assert_array_equal(dr, dr_ref)
    np.testing.assert_array_equal(dc, dc_ref)
    W = A * dr.astype(np.float64)[:, None] * dc.astype(np.float64)[None, :]
    L = np.tril(LU.astype(np.float64), -1) + np.eye(n)
    U = np.triu(LU.astype(np.float64))
    # partial pivoting bounds the multipliers
    assert np.max(np.abs(L)) <= 1.0 + 1e-6
    # P W = L U to FP32 rounding, with P from the factorization's own exchanges
    np.testing.assert_array_equal(perm, R.perm_from_ipiv(ipiv))
    rel = np.linalg.norm(W[perm] - L @ U) / np.linalg.norm(W)
    assert rel < 2e-6 * max(1.0, np.log2(n)), rel
    # the same pivot rows as LAPACK dgetrf on the same scaled matrix, up to the
    # first step where FP32 and FP64 elimination meet a near tie: there the two
    # candidates' exact (FP64) Schur-complement magnitudes agree to FP32 rounding
    diff = np.nonzero(ipiv != piv_ref)[0]
    if diff.size == 0:
        assert np.linalg.norm(LU - lu_ref) / np.linalg.norm(lu_ref) < 1e-4
        return
    d = int(diff[0])
    Wd = W.copy()
    for i in range(d):  # the first d exchanges, identical in both
        Wd[[i, ipiv[i]]] = Wd[[ipiv[i], i]]
    col = Wd[d:, d] - Wd[d:, :d] @ np.linalg.solve(Wd[:d, :d], Wd[:d, d]) if d else Wd[:, 0]
    mine, ref = abs(col[ipiv[d] - d]), abs(col[piv_ref[d] - d])
    assert mine >= ref * (1 - 1e-4), (n, d, mine, ref)
    # the leading d x d factors (rows fixed before the tie) agree
    if d:
        assert np.linalg.norm(LU[:d, :d] - lu_ref[:d, :d]) <= 1e-4 * np.linalg.norm(lu_ref[:d, :d])


@pytest.mark.parametrize("n", [1000, 2048])
@pytest.mark.parametrize("kind", ["gaussian", "zero_diagonal"])
def test_dropin_luirsolver_needs_pivoting(n, kind):
    import warnings
    from mpdok_gb300.mpdok_ops import LUIRSolver
    A = R.test_matrices(n, seed=7 + n)[kind]
    b = np.random.default_rng(n).standard_normal(n)
    ref = R.lu_ir_relres(A, b)
    Ad = torch.tensor(A, device="cuda").t().contiguous().t()
    s = LUIRSolver()
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")  # tol below the floor: the non-convergence warning is expected
        x = s.solve(Ad, b, tol=1e-16, maxiter_outer=4).cpu().numpy()
    rel = np.linalg.norm(b - A @ x) / np.linalg.norm(b)
    assert rel <= 10 * ref, (rel, ref)
    # factor once, solve twice (the reference's solve_factored)
    s.factor(Ad)
    for k in range(2):
        bk = np.random.default_rng(100 + k).standard_normal(n)
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            xk = s.solve_factored(bk, tol=1e-16, maxiter_outer=4).cpu().numpy()
        assert np.linalg.norm(bk - A @ xk) / np.linalg.norm(bk) <= 10 * R.lu_ir_relres(A, bk)
    s.free_factored()


def test_singular_matrix_reports_lapack_info():
    from scipy.linalg import lapack
    from mpdok_gb300.mpdok_ops import LUIRSolver
    n = 400
    A = R.test_matrices(n, seed=3)["gaussian"]
    A[:, 37] = 0.0
    _, _, info_ref = lapack.dgetrf(A)
    assert info_ref == 38
    lu = _factor(A, "fp32")
    assert lu.info == info_ref
    with pytest.raises(RuntimeError, match="info=38"):
        LUIRSolver().factor(torch.tensor(A, device="cuda").t().contiguous().t())


@pytest.mark.parametrize("dtype", ["fp16", "bf16"])
def test_pivoted_16bit_factors_precondition_gmres_ir(dtype):
    n = 1536
    A = R.test_matrices(n, seed=11)["gaussian"]
    b = np.random.default_rng(12).standard_normal(n)
    ref = R.lu_ir_relres(A, b)
    lu = _factor(A, dtype)
    assert lu.info == 0
    Ad = torch.tensor(A, device="cuda").t().contiguous().t()
    x, info = lu.gmres_ir(Ad, b, tol=1e-12, maxiter_outer=20, restart=30)
    rel = np.linalg.norm(b - A @ x.cpu().numpy()) / np.linalg.norm(b)
    assert info["converged"] and rel <= max(1e-12, 10 * ref), (rel, ref, info)


def test_pivoted_factors_many_rhs_and_large_panel():
    """n = 5000: the panel spans more rows than one CTA per SM at 32 rows each;
    three right-hand sides through the multi-RHS triangular sweeps."""
    n = 5000
    A = R.test_matrices(n, seed=5)["gaussian"]
    B = np.random.default_rng(6).standard_normal((n, 3))
    lu = _factor(A, "fp32")
    Ad = torch.tensor(A, device="cuda").t().contiguous().t()
    X, info = lu.solve_ir_many(Ad, B, tol=1e-13, maxiter_outer=5)
    Xh = X.cpu().numpy()
    rel = np.linalg.norm(B - A @ Xh, axis=0) / np.linalg.norm(B, axis=0)
    for k in range(3):
        assert rel[k] <= 10 * R.lu_ir_relres(A, B[:, k]), (k, rel[k])
