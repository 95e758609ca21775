"""CPU: the design claim behind the unpivoted blocked LU on multiquadric
systems (C3 family).  MQ matrices are conditionally negative definite (one
positive eigenvalue), so their Schur complements stay definite and Gaussian
elimination without pivoting is backward stable on them: the growth factor
stays modest (< 200 from flat to sharp shape parameters) and the backward
error stays within 50x of partial pivoting.  What pivoting would bound and
this does not: the multipliers, |L| up to 1e9 for flat kernels, which
overflows FP16 storage (BF16 and FP32 factors hold them)."""
import numpy as np
import scipy.linalg as sl

from mpdok_gb300 import configs
from oracle import krylov_ref as O


def _lu_nopiv(A):
    M = A.copy()
    n = len(M)
    growth = 0.0
    for k in range(n - 1):
        M[k + 1:, k] /= M[k, k]
        M[k + 1:, k + 1:] -= np.outer(M[k + 1:, k], M[k, k + 1:])
        growth = max(growth, np.abs(M[k + 1:, k + 1:]).max())
    return np.tril(M, -1) + np.eye(n), np.triu(M), growth / np.abs(A).max()


def test_unpivoted_lu_on_mq_is_backward_stable():
    for n, gamma in [(400, 4.0), (400, 1e2), (400, 1e4), (600, 1.0)]:
        X = configs.stratified_jitter(n, 2)
        A = O.rbf_matrix(X, gamma=gamma, reg=0.0, kernel="mq")
        L, U, growth = _lu_nopiv(A)
        berr = np.linalg.norm(L @ U - A) / np.linalg.norm(A)
        P, Lp, Up = sl.lu(A)
        berr_p = np.linalg.norm(P @ Lp @ Up - A) / np.linalg.norm(A)
        assert growth < 200, (n, gamma, growth)
        assert berr < 50 * max(berr_p, 1e-16) and berr < 1e-14, (n, gamma, berr, berr_p)


def test_unpivoted_multipliers_leave_fp16_range_for_flat_mq():
    X = configs.stratified_jitter(400, 2)
    L, _, _ = _lu_nopiv(O.rbf_matrix(X, gamma=4.0, reg=0.0, kernel="mq"))
    assert np.abs(L).max() > 65504.0
