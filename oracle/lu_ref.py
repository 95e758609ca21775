"""Oracle of the pivoted LU: power-of-two equilibration + LAPACK getrf (FP64).

TEST INFRASTRUCTURE ONLY (imported by tests/, never by the product).

The reference's LU-IR factors with cusolverDnSgetrf, i.e. LAPACK getrf with
partial pivoting by rows (benchmark_mpdok.ipynb:989-990), and its
``LUIRSolver.factor`` raises on LAPACK's info != 0 (mpdok_ops.py:195-202).
The GPU factorization first scales rows and then columns by powers of two
(exact) so that every row and column of W = Dr A Dc has its largest entry in
[0.5, 1); ``equilibrate`` restates that scaling and ``getrf`` runs SciPy's
LAPACK dgetrf on W, giving the pivot rows and L\\U the GPU result is compared
with.
"""
from __future__ import annotations

import numpy as np
import scipy.linalg as sla
from scipy.linalg import lapack


def pow2_inv_scale(m: np.ndarray) -> np.ndarray:
    """2^-e with m * 2^-e in [0.5, 1) (frexp's exponent, clamped to +-120); 1 for 0 / non-finite."""
    m = np.asarray(m, dtype=np.float64)
    out = np.ones_like(m)
    ok = (m > 0) & np.isfinite(m)
    _, e = np.frexp(m[ok])
    e = np.clip(e, -120, 120)
    out[ok] = np.ldexp(1.0, -e)
    return out.astype(np.float32)


def equilibrate(A: np.ndarray):
    """(dr, dc) of the GPU factorization: rows first, then columns of Dr A."""
    A = np.asarray(A, dtype=np.float64)
    dr = pow2_inv_scale(np.max(np.abs(A), axis=1))
    dc = pow2_inv_scale(np.max(np.abs(A) * dr.astype(np.float64)[:, None], axis=0))
    return dr, dc


def getrf(A: np.ndarray):
    """(LU, ipiv 0-based, info) of LAPACK dgetrf on the equilibrated matrix, with (dr, dc)."""
    dr, dc = equilibrate(A)
    W = np.asarray(A, dtype=np.float64) * dr.astype(np.float64)[:, None] * dc.astype(np.float64)[None, :]
    lu, piv, info = lapack.dgetrf(W)
    return lu, piv, info, dr, dc


def perm_from_ipiv(ipiv: np.ndarray) -> np.ndarray:
    """Gather form of LAPACK's row exchanges: (P x)_i = x[perm[i]]."""
    perm = np.arange(len(ipiv))
    for i, p in enumerate(ipiv):
        perm[i], perm[p] = perm[p], perm[i]
    return perm


def lu_ir_relres(A: np.ndarray, b: np.ndarray, steps: int = 3) -> float:
    """SciPy FP64 lu_factor / lu_solve + refinement: the relres the GPU LU-IR is held to."""
    lu = sla.lu_factor(A, check_finite=False)
    x = sla.lu_solve(lu, b, check_finite=False)
    for _ in range(steps):
        x = x + sla.lu_solve(lu, b - A @ x, check_finite=False)
    return float(np.linalg.norm(b - A @ x) / np.linalg.norm(b))


def test_matrices(n: int, seed: int):
    """Matrices that need row exchanges: a dense N(0,1) matrix (not diagonally
    dominant) and one with an exactly zero diagonal whose large entries sit on
    the anti-diagonal (n even)."""
    rng = np.random.default_rng(seed)
    G = rng.standard_normal((n, n))
    Z = rng.standard_normal((n, n))
    Z[np.arange(n), n - 1 - np.arange(n)] += 4.0 * np.sqrt(n)
    np.fill_diagonal(Z, 0.0)
    return {"gaussian": G, "zero_diagonal": Z}
