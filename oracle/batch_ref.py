"""Oracle for the batched RBF solves and their gradients (test infrastructure).

FP64 NumPy/SciPy restatements, used only by tests, smoke() and the bench's CPU
baseline.  The batched workload is not in the reference (its solvers take one
system per call: mpdok_ops.py:101-141, dense_krylov.py:338-421); its ground
truth is SciPy's FP64 Cholesky per system (cho_factor / cho_solve), the same
FP64 factorization the reference's SciPy path uses (lu_factor / lu_solve on
an SPD matrix).

Gradients of L(X) with X = A^{-1} B, A = phi(eps * r_ij) + reg I:
lam = A^{-1} dL/dX, dL/dB = lam, dL/dtheta = -sum_r lam_r^T (dA/dtheta) x_r,
with dA/dtheta formed densely here (the product path never stores it).
"""
from __future__ import annotations

import numpy as np
import scipy.linalg as sl


def rbf(X, eps, reg, kernel="gaussian"):
    d2 = ((X[:, None, :] - X[None, :, :]) ** 2).sum(-1)
    g = eps * eps
    A = np.exp(-g * d2) if kernel == "gaussian" else np.sqrt(1.0 + g * d2)
    return A + reg * np.eye(len(X))


def solve(X, eps, reg, B, kernel="gaussian"):
    """FP64 Cholesky solve and its relative residual (max over RHS)."""
    A = rbf(X, eps, reg, kernel)
    Bm = B.reshape(len(X), -1)
    x = sl.cho_solve(sl.cho_factor(A, lower=True), Bm)
    rel = np.max(np.linalg.norm(Bm - A @ x, axis=0) / np.linalg.norm(Bm, axis=0))
    return x, rel


def grads(X, eps, reg, B, dLdX, kernel="gaussian"):
    """(dL/dcoords (n, dim), dL/deps, dL/dreg, dL/dB) by dense FP64 formulas."""
    n, dim = X.shape
    A = rbf(X, eps, reg, kernel)
    Bm = B.reshape(n, -1)
    x = np.linalg.solve(A, Bm)
    lam = np.linalg.solve(A.T, dLdX.reshape(n, -1))
    diff = X[:, None, :] - X[None, :, :]
    d2 = (diff ** 2).sum(-1)
    g = eps * eps
    if kernel == "gaussian":
        phi = np.exp(-g * d2)
        dphi_dd2 = -g * phi
        dphi_dg = -d2 * phi
    else:
        phi = np.sqrt(1.0 + g * d2)
        dphi_dd2 = g / (2 * phi)
        dphi_dg = d2 / (2 * phi)
    M = lam @ x.T                      # M_ij = sum_r lam_ir x_jr = -dL/dA_ij
    d_eps = -np.sum(M * dphi_dg * 2 * eps)
    d_reg = -np.trace(M)
    W = M + M.T                        # symmetric in (k, j)
    d_c = -2.0 * np.einsum("kj,kj,kjd->kd", W, dphi_dd2, diff)
    return d_c, d_eps, d_reg, lam
