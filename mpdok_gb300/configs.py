"""Seeded synthetic RBF systems of the five benchmark configurations (host NumPy, FP64).

All inputs come from ``numpy.random.default_rng(seed)`` on the host, so the
same arrays feed the CPU oracle, the CPU baseline and the GPU solvers.

* C1  N=2000, U[0,1]^2 (seed 0), Gaussian eps=3 (gamma=9), nugget 1e-10,
      b = sin(2 pi x1) cos(2 pi x2) + N(0, 1e-3^2).
* C2  N=20000, U[0,1]^3 (seed 1), Gaussian eps=5 (gamma=25), nugget 1e-6, 4 RHS ~ N(0,1).
* C3  N=32768, 2-D stratified jitter (seed 2), multiquadric sqrt(1+(2r)^2) (gamma=4), no nugget,
      b = sin(2 pi x1) cos(2 pi x2).
* HEADLINE  the same N=32768 centres (seed 2) with a Gaussian eps=40 (gamma=1600), nugget 1e-2,
      b ~ N(0,1): kappa ~ 6e3, FP64 LU + refinement relres ~ 2e-13, so relres <= 1e-12 is attainable.
* C4  256 Gaussian systems, N ~ U{500..8000} (seed 3), U[0,1]^2, eps ~ U(2,8), nugget 1e-8, 8 RHS.
* C5  N=250000, U[0,1]^3 (seed 4), Gaussian eps=10 (gamma=100), nugget 1e-6, 1 RHS.

Stratified jitter: a 182 x 182 grid of cells over [0,1]^2; one point uniformly
inside each cell; N of the 33124 cells chosen without replacement and kept
in cell (row-major) order.  Every draw comes from one generator in the order
written here.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class RBFSystem:
    name: str
    coords: np.ndarray            # (N, D) FP64
    kernel: str                   # 'gaussian' | 'mq'
    gamma: float                  # eps^2
    reg: float                    # nugget on the diagonal
    b: np.ndarray                 # (N,) or (N, k) FP64
    tol: float = 1e-12
    extra: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.coords.shape[0])


def stratified_jitter(n: int, seed: int, grid: int = 182) -> np.ndarray:
    if n > grid * grid:
        raise ValueError("n exceeds the number of cells")
    rng = np.random.default_rng(seed)
    ii, jj = np.meshgrid(np.arange(grid), np.arange(grid), indexing="ij")
    pts = np.stack([(ii.ravel() + rng.uniform(size=grid * grid)) / grid,
                    (jj.ravel() + rng.uniform(size=grid * grid)) / grid], axis=1)
    idx = np.sort(rng.choice(grid * grid, n, replace=False))
    return np.ascontiguousarray(pts[idx])


def c1(n: int = 2000) -> RBFSystem:
    rng = np.random.default_rng(0)
    X = rng.uniform(0.0, 1.0, size=(n, 2))
    noise = rng.normal(0.0, 1e-3, size=n)
    b = np.sin(2 * np.pi * X[:, 0]) * np.cos(2 * np.pi * X[:, 1]) + noise
    return RBFSystem("C1", X, "gaussian", 9.0, 1e-10, b, tol=1e-12, extra={"restart": 50})


def c2(n: int = 20000, nrhs: int = 4) -> RBFSystem:
    rng = np.random.default_rng(1)
    X = rng.uniform(0.0, 1.0, size=(n, 3))
    B = rng.standard_normal(size=(n, nrhs))
    return RBFSystem("C2", X, "gaussian", 25.0, 1e-6, B, tol=1e-12)


def c3(n: int = 32768) -> RBFSystem:
    X = stratified_jitter(n, 2)
    b = np.sin(2 * np.pi * X[:, 0]) * np.cos(2 * np.pi * X[:, 1])
    return RBFSystem("C3", X, "mq", 4.0, 0.0, b, tol=1e-12, extra={"restart": 30})


def headline(n: int = 32768) -> RBFSystem:
    X = stratified_jitter(n, 2)
    rng = np.random.default_rng(20)
    b = rng.standard_normal(n)
    return RBFSystem("HEADLINE", X, "gaussian", 1600.0, 1e-2, b, tol=1e-12, extra={"restart": 30})


HARD_EPS = 100.0


def hard_headline(n: int = 32768, eps: float = HARD_EPS) -> RBFSystem:
    """The headline centres with C5's nugget (1e-6): kappa ~ lambda_max / 1e-6.

    With a white-noise right-hand side the solution's components along the
    eigenvectors at the nugget grow by 1e6 and the FP64 LU floor itself sits
    near u * kappa; the right-hand side is therefore the smooth field of C1 /
    C3, sin(2 pi x1) cos(2 pi x2), for which the FP64 solve reaches 1e-12."""
    X = stratified_jitter(n, 2)
    b = np.sin(2 * np.pi * X[:, 0]) * np.cos(2 * np.pi * X[:, 1])
    return RBFSystem("HARD", X, "gaussian", eps * eps, 1e-6, b, tol=1e-12, extra={"restart": 30})


def c4(n_systems: int = 256, nrhs: int = 8, n_lo: int = 500, n_hi: int = 8000) -> list[RBFSystem]:
    rng = np.random.default_rng(3)
    sizes = rng.integers(n_lo, n_hi + 1, size=n_systems)
    eps = rng.uniform(2.0, 8.0, size=n_systems)
    out = []
    for i, (n, e) in enumerate(zip(sizes, eps)):
        X = rng.uniform(0.0, 1.0, size=(int(n), 2))
        B = rng.standard_normal(size=(int(n), nrhs))
        out.append(RBFSystem(f"C4[{i}]", X, "gaussian", float(e) ** 2, 1e-8, B, tol=1e-12))
    return out


def c5(n: int = 250000) -> RBFSystem:
    rng = np.random.default_rng(4)
    X = rng.uniform(0.0, 1.0, size=(n, 3))
    b = rng.standard_normal(n)
    return RBFSystem("C5", X, "gaussian", 100.0, 1e-6, b, tol=1e-10)


def by_name(name: str, **kw):
    return {"C1": c1, "C2": c2, "C3": c3, "HEADLINE": headline, "C4": c4, "C5": c5}[name.upper()](**kw)


def time_series_fields(n: int = 8192, steps: int = 24, seed: int = 42):
    """Factor-once / many-RHS workload: n sensors uniform in a 100 x 100 square
    (seed), three smooth fields sampled at `steps` times (3 * steps RHS).

    Seeded synthetic stand-in with the shape of the reference's time-series
    demo (rbf_demo.ipynb cells 3-7: N=8192, 3 fields x 24 steps, reg 1e-2,
    tol 1e-5); the field formulas are this module's own.
    """
    rng = np.random.default_rng(seed)
    X = rng.uniform(0.0, 100.0, size=(n, 2))
    x, y = X[:, 0] / 100.0, X[:, 1] / 100.0
    cols = []
    for t in range(steps):
        ph = 2.0 * np.pi * t / steps
        temp = 15.0 + 5.0 * np.sin(2 * np.pi * x + ph) * np.cos(2 * np.pi * y) + 0.1 * rng.standard_normal(n)
        pres = 10.0 * np.cos(2 * np.pi * (x + y) - ph) + 0.05 * rng.standard_normal(n)
        hum = 40.0 + 30.0 * np.exp(-((x - 0.5 - 0.2 * np.sin(ph)) ** 2 + (y - 0.5) ** 2) / 0.08) \
            + 0.5 * rng.standard_normal(n)
        cols += [temp, pres, hum]
    return X, np.stack(cols, axis=1)
