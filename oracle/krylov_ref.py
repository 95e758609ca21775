"""CPU oracle: NumPy/SciPy restatement of MPDOK's dense-operator Krylov path.

TEST INFRASTRUCTURE ONLY.  This module is the oracle of the sm_103a
implementation: only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline / reference arm import it.  The product never routes through it.

Each function cites the reference file:line whose algorithm it restates.
Pinning: tests/test_oracle_golden.py checks these functions against golden
vectors produced by running the reference's own modules (dense_krylov.py,
mpdok_ooc.py, rbf_kernel.py) under a NumPy stand-in for CuPy
(tests/golden/make_golden.py), and against SciPy's FP64 LU.

Precisions follow the reference: FP32 operator and Krylov vectors, FP64
residual / update / Hessenberg / Givens.
"""
from __future__ import annotations

import numpy as np
import scipy.linalg as sla

F32 = np.float32
F64 = np.float64


# ----------------------------------------------------------------- assembly
def estimate_gamma(coords, max_sample=512):
    """rbf_kernel.py:57-68: gamma = 1 / (2 mean ||c_i - c_j||^2) over the first points."""
    c = np.asarray(coords, F64)[:max_sample]
    sq = np.sum(c ** 2, axis=1)
    d2 = sq[:, None] + sq[None, :] - 2.0 * (c @ c.T)
    np.maximum(d2, 0.0, out=d2)
    m = float(np.mean(d2))
    return 1.0 / (2.0 * m) if m > 1e-30 else 1.0


def rbf_matrix(rows, cols=None, gamma=1.0, reg=0.0, kernel="gaussian", diag_offset=0):
    """A[i,j] = phi(||r_i - c_j||) + reg [i + diag_offset == j]  (rbf_kernel.py:158-227).

    d^2 is summed from coordinate differences; the reference's GEMM identity
    (rbf_kernel.py:219-220) agrees to ~1e-15 for coordinates in [0, 1].
    """
    r = np.asarray(rows, F64)
    c = r if cols is None else np.asarray(cols, F64)
    d2 = np.zeros((r.shape[0], c.shape[0]), F64)
    for k in range(r.shape[1]):
        t = r[:, k][:, None] - c[:, k][None, :]
        d2 += t * t
    if kernel == "gaussian":
        A = np.exp(-gamma * d2)
    elif kernel in ("mq", "multiquadric"):
        A = np.sqrt(1.0 + gamma * d2)
    else:
        raise ValueError(kernel)
    if reg:
        i = np.arange(r.shape[0])
        j = i + diag_offset
        ok = (j >= 0) & (j < c.shape[0])
        A[i[ok], j[ok]] += reg
    return A


def rbf_matrix_identity(coords, gamma, reg):
    """The reference's own GEMM-identity build (rbf_kernel.py:215-224), for pinning."""
    c = np.asarray(coords, F64)
    sq = np.sum(c ** 2, axis=1)
    d2 = sq[:, None] + sq[None, :] - 2.0 * (c @ c.T)
    np.maximum(d2, 0.0, out=d2)
    A = np.exp(-gamma * d2)
    A[np.arange(len(c)), np.arange(len(c))] += reg
    return A


# ----------------------------------------------------------------- GEMV
def gemv_exact(A32, x32):
    """FP64 value of the FP32 product A32 @ x32 (dense_krylov.py:61-63 target)."""
    return np.asarray(A32, F64) @ np.asarray(x32, F64)


# ------------------------------------------------- inner GMRES (native port)
def inner_gmres(A32, rhs64, restart, tol_rel=1e-6):
    """mpdok_ooc.py:231-311: FP32 Arnoldi with two Gram-Schmidt passes (DGKS),
    FP64 Hessenberg and Givens rotations, early stop |g_{k+1}| / beta < tol_rel.

    One deliberate difference: on a lucky breakdown (|w| <= 1e-12) the
    reference leaves column k unrotated before back substitution
    (mpdok_ooc.py:278-282); here the rotations are applied first, which is
    the mathematically consistent least-squares solution.
    Returns (e32, steps).
    """
    A32 = np.asarray(A32, F32)
    n = A32.shape[0]
    rhs = np.asarray(rhs64, F64).astype(F32)
    beta = float(np.sqrt(np.dot(rhs.astype(F64), rhs.astype(F64))))
    if beta < 1e-30:
        return np.zeros(n, F32), 0
    V = np.empty((n, restart + 1), F32, order="F")
    V[:, 0] = rhs * F32(1.0 / beta)
    H = np.zeros((restart + 1, restart), F64)
    cs = np.zeros(restart, F64)
    sn = np.zeros(restart, F64)
    g = np.zeros(restart + 1, F64)
    g[0] = beta
    m = restart
    for k in range(restart):
        w = (A32 @ V[:, k]).astype(F32)
        h = (V[:, :k + 1].astype(F64).T @ w.astype(F64))
        H[:k + 1, k] = h
        w = (w - (V[:, :k + 1] @ h.astype(F32))).astype(F32)
        h2 = (V[:, :k + 1].astype(F64).T @ w.astype(F64))
        H[:k + 1, k] += h2
        w = (w - (V[:, :k + 1] @ h2.astype(F32))).astype(F32)
        nrm = float(np.sqrt(np.dot(w.astype(F64), w.astype(F64))))
        H[k + 1, k] = nrm
        breakdown = not nrm > 1e-12
        if not breakdown:
            V[:, k + 1] = w * F32(1.0 / nrm)
        for j in range(k):
            tmp = cs[j] * H[j, k] + sn[j] * H[j + 1, k]
            H[j + 1, k] = -sn[j] * H[j, k] + cs[j] * H[j + 1, k]
            H[j, k] = tmp
        rho = np.hypot(H[k, k], H[k + 1, k])
        cs[k], sn[k] = (H[k, k] / rho, H[k + 1, k] / rho) if rho != 0 else (1.0, 0.0)
        if rho != 0:
            H[k, k] = rho
        H[k + 1, k] = 0.0
        g[k + 1] = -sn[k] * g[k]
        g[k] = cs[k] * g[k]
        if breakdown or abs(g[k + 1]) / beta < tol_rel:
            m = k + 1
            break
    y = np.zeros(m, F64)
    for j in range(m - 1, -1, -1):
        s = g[j] - np.dot(H[j, j + 1:m], y[j + 1:m])
        y[j] = s / H[j, j] if H[j, j] != 0 else 0.0
    e = (V[:, :m] @ y.astype(F32)).astype(F32)
    return e, m


def gmres_ir_native(A64, b, tol=1e-11, maxiter_outer=5, restart=50, inner_tol=1e-6, A32=None):
    """MPDOKSolver.solve / py_gmres_ir semantics: mpdok_ooc.py:315-373 outer loop
    (FP64 residual, inner_gmres, FP64 update) plus the final residual of
    dense_krylov.py:414-419.  Returns (x, history, converged, inner_steps)."""
    A64 = np.asarray(A64, F64)
    A32 = A64.astype(F32) if A32 is None else A32
    b = np.asarray(b, F64)
    n = len(b)
    bnorm = float(np.linalg.norm(b))
    if bnorm == 0.0:
        return np.zeros(n), [(0, 0.0)], True, 0
    x = np.zeros(n, F64)
    hist, conv, steps = [], False, 0
    for outer in range(maxiter_outer):
        r = b - A64 @ x
        rel = float(np.linalg.norm(r)) / bnorm
        hist.append((outer, rel))
        if rel < tol:
            conv = True
            break
        e, m = inner_gmres(A32, r, restart, inner_tol)
        steps += m
        x = x + e.astype(F64)
    if not conv:
        rel = float(np.linalg.norm(b - A64 @ x)) / bnorm
        hist.append((maxiter_outer, rel))
        conv = rel < tol
    return x, hist, conv, steps


# --------------------------------------------- dense_krylov.py restatements
def _arnoldi_cgs1_cycle(A32, r32, m):
    """One GMRES(m) cycle with a single classical Gram-Schmidt pass
    (dense_krylov.py:270-312); least squares by Givens (same minimiser as
    the reference's lstsq at :308).  Returns (update32, steps, beta)."""
    n = A32.shape[0]
    beta = float(np.sqrt(np.dot(r32.astype(F64), r32.astype(F64))))
    if beta == 0.0:
        return np.zeros(n, F32), 0, 0.0
    V = np.empty((n, m + 1), F32, order="F")
    V[:, 0] = r32 * F32(1.0 / beta)
    H = np.zeros((m + 1, m), F64)
    steps = 0
    for k in range(m):
        w = (A32 @ V[:, k]).astype(F32)
        h = V[:, :k + 1].astype(F64).T @ w.astype(F64)
        H[:k + 1, k] = h
        w = (w - V[:, :k + 1] @ h.astype(F32)).astype(F32)
        nw = float(np.sqrt(np.dot(w.astype(F64), w.astype(F64))))
        H[k + 1, k] = nw
        steps = k + 1
        if nw < 1e-12:
            break
        V[:, k + 1] = w * F32(1.0 / nw)
    e1 = np.zeros(steps + 1)
    e1[0] = beta
    y = np.linalg.lstsq(H[:steps + 1, :steps], e1, rcond=None)[0]
    return (V[:, :steps] @ y.astype(F32)).astype(F32), steps, beta


def gmres(A64, b, x0=None, tol=1e-6, maxiter=None, restart=50, A32=None):
    """dense_krylov.py:212-331: restarted FP32 GMRES with FP64 checks per restart."""
    A64 = np.asarray(A64, F64)
    A32 = A64.astype(F32) if A32 is None else A32
    b64 = np.asarray(b, F64)
    n = len(b64)
    maxiter = n if maxiter is None else maxiter
    b32 = b64.astype(F32)
    bnorm = float(np.linalg.norm(b64))
    if bnorm == 0.0:
        return np.zeros(n), [(0, 0.0)], True
    x = np.zeros(n, F32) if x0 is None else np.asarray(x0, F32)
    hist, conv, total, prev = [], False, 0, float("inf")
    for _ in range((maxiter + restart - 1) // restart):
        r = (b32 - (A32 @ x).astype(F32)).astype(F32)
        mm = min(restart, maxiter - total)
        if mm <= 0:
            break
        upd, steps, beta = _arnoldi_cgs1_cycle(A32, r, mm)
        if beta == 0.0:
            conv = True
            break
        x = (x + upd).astype(F32)
        total += steps
        rel = float(np.linalg.norm(b64 - A64 @ x.astype(F64))) / bnorm
        hist.append((total, rel))
        if rel < tol:
            conv = True
            break
        if rel > prev * (1.0 - 1e-2):
            break
        prev = rel
    return x.astype(F64), hist, conv


def gmres_ir(A64, b, tol=1e-11, maxiter_outer=5, restart=50, maxiter_inner=None, A32=None):
    """dense_krylov.py:338-421."""
    A64 = np.asarray(A64, F64)
    A32 = A64.astype(F32) if A32 is None else A32
    b64 = np.asarray(b, F64)
    n = len(b64)
    bnorm = float(np.linalg.norm(b64))
    if bnorm == 0.0:
        return np.zeros(n), [(0, 0.0)], True
    x = np.zeros(n, F64)
    hist, conv = [], False
    for outer in range(maxiter_outer):
        r = b64 - A64 @ x
        rel = float(np.linalg.norm(r)) / bnorm
        hist.append((outer, rel))
        if rel < tol:
            conv = True
            break
        e, _, _ = gmres(A64, r, tol=1e-6, restart=restart, maxiter=maxiter_inner, A32=A32)
        x = x + e
    rel = float(np.linalg.norm(b64 - A64 @ x)) / bnorm
    hist.append((maxiter_outer, rel))
    return x, hist, conv or rel < tol


def cg(A64, b, x0=None, tol=1e-6, maxiter=None, check_every=10, A32=None):
    """dense_krylov.py:119-205: FP32 CG, FP64 residual every check_every iterations,
    1 % stagnation stop."""
    A64 = np.asarray(A64, F64)
    A32 = A64.astype(F32) if A32 is None else A32
    b64 = np.asarray(b, F64)
    n = len(b64)
    maxiter = n if maxiter is None else maxiter
    b32 = b64.astype(F32)
    bnorm = float(np.linalg.norm(b64))
    if bnorm == 0.0:
        return np.zeros(n), [(0, 0.0)], True
    x = np.zeros(n, F32) if x0 is None else np.asarray(x0, F32)
    r = (b32 - (A32 @ x).astype(F32)).astype(F32)
    p = r.copy()
    rs = float(np.float32(np.dot(r.astype(F64), r.astype(F64))))
    hist, conv, prev, k = [], False, float("inf"), -1
    for k in range(maxiter):
        if k % check_every == 0:
            rel = float(np.linalg.norm(b64 - A64 @ x.astype(F64))) / bnorm
            hist.append((k, rel))
            if rel < tol:
                conv = True
                break
            if rel > prev * (1.0 - 1e-2):
                break
            prev = rel
        Ap = (A32 @ p).astype(F32)
        pap = float(np.float32(np.dot(p.astype(F64), Ap.astype(F64))))
        if pap == 0.0:
            break
        alpha = rs / pap
        x = (x + F32(alpha) * p).astype(F32)
        r = (r - F32(alpha) * Ap).astype(F32)
        rs_new = float(np.float32(np.dot(r.astype(F64), r.astype(F64))))
        beta = rs_new / rs if rs != 0 else 0.0
        p = (r + F32(beta) * p).astype(F32)
        rs = rs_new
    if not conv:
        rel = float(np.linalg.norm(b64 - A64 @ x.astype(F64))) / bnorm
        hist.append((k + 1, rel))
        conv = rel < tol
    return x.astype(F64), hist, conv


# ------------------------------------------------------------------ LU-IR
def lu_ir(A64, b, tol=1e-11, maxiter_outer=3, factor_dtype=F32):
    """LU-IR steps of benchmark_mpdok.ipynb:982-993: cast A, LU with partial
    pivoting in `factor_dtype` (SciPy getrf), initial solve, then FP64
    residual / low-precision correction solve / FP64 update.
    Returns (x, history, converged)."""
    A64 = np.asarray(A64, F64)
    b64 = np.asarray(b, F64)
    lu, piv = sla.lu_factor(A64.astype(factor_dtype), check_finite=False)
    bnorm = float(np.linalg.norm(b64))
    x = sla.lu_solve((lu, piv), b64.astype(factor_dtype)).astype(F64)
    hist, conv = [], False
    for it in range(maxiter_outer):
        r = b64 - A64 @ x
        rel = float(np.linalg.norm(r)) / bnorm
        hist.append((it, rel))
        if rel < tol:
            conv = True
            break
        d = sla.lu_solve((lu, piv), r.astype(factor_dtype)).astype(F64)
        x = x + d
    if not conv:
        rel = float(np.linalg.norm(b64 - A64 @ x)) / bnorm
        hist.append((maxiter_outer, rel))
        conv = rel < tol
    return x, hist, conv


def fp64_solve(A64, b):
    """The FP64 LU ground truth (SciPy lu_factor / lu_solve)."""
    lu = sla.lu_factor(np.asarray(A64, F64), check_finite=False)
    return sla.lu_solve(lu, np.asarray(b, F64))


def relres(A64, x, b):
    b = np.asarray(b, F64)
    return float(np.linalg.norm(b - np.asarray(A64, F64) @ np.asarray(x, F64)) / np.linalg.norm(b))
