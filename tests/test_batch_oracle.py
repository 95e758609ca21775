"""CPU: the batched oracle's gradient formulas against central finite
differences, and the autotuner's cache logic."""
import json

import numpy as np
import pytest

from oracle import batch_ref as R


def _loss(X, eps, reg, B, Xstar, kernel):
    x, _ = R.solve(X, eps, reg, B, kernel)
    return float(np.sum((x - Xstar) ** 2))


@pytest.mark.parametrize("kernel,eps,reg", [("gaussian", 4.0, 1e-3), ("gaussian", 7.0, 1e-2)])
def test_oracle_gradients_match_finite_differences(kernel, eps, reg):
    rng = np.random.default_rng(11)
    n, k = 40, 3
    X = rng.uniform(0, 1, (n, 2))
    B = rng.standard_normal((n, k))
    Xs = rng.standard_normal((n, k))
    x, _ = R.solve(X, eps, reg, B, kernel)
    dc, de, dr, lam = R.grads(X, eps, reg, B, 2 * (x - Xs), kernel)
    h = 1e-6
    fd_e = (_loss(X, eps + h, reg, B, Xs, kernel) - _loss(X, eps - h, reg, B, Xs, kernel)) / (2 * h)
    assert de == pytest.approx(fd_e, rel=1e-5)
    hr = 1e-7 * reg
    fd_r = (_loss(X, eps, reg + hr, B, Xs, kernel) - _loss(X, eps, reg - hr, B, Xs, kernel)) / (2 * hr)
    assert dr == pytest.approx(fd_r, rel=1e-5)
    for (i, d) in [(0, 0), (7, 1), (n - 1, 0)]:
        Xp, Xm = X.copy(), X.copy()
        Xp[i, d] += h
        Xm[i, d] -= h
        fd = (_loss(Xp, eps, reg, B, Xs, kernel) - _loss(Xm, eps, reg, B, Xs, kernel)) / (2 * h)
        assert dc[i, d] == pytest.approx(fd, rel=1e-4, abs=1e-6 * np.abs(dc).max())
    e = 1e-7
    Bp = B.copy()
    Bp[3, 1] += e
    Bm = B.copy()
    Bm[3, 1] -= e
    fd_b = (_loss(X, eps, reg, Bp, Xs, kernel) - _loss(X, eps, reg, Bm, Xs, kernel)) / (2 * e)
    assert lam[3, 1] == pytest.approx(fd_b, rel=1e-5)


def test_autotune_cache_roundtrip(tmp_path, monkeypatch):
    from mpdok_gb300 import batch as Bt
    monkeypatch.setenv("MPDOK_GB300_AUTOTUNE", str(tmp_path / "tune.json"))
    k1 = Bt.tune_key("GB300", [500, 800, 700], 2, 8, "gaussian", "df32")
    k2 = Bt.tune_key("GB300", [800, 700, 500], 2, 8, "gaussian", "df32")
    k3 = Bt.tune_key("GB300", [800, 700, 501], 2, 8, "gaussian", "df32")
    assert k1 == k2 and k1 != k3
    assert Bt.cache_get(k1) is None
    Bt.cache_put(k1, {"grid_mult": 4})
    Bt.cache_put(k3, {"grid_mult": 1})
    assert Bt.cache_get(k1)["grid_mult"] == 4
    data = json.loads((tmp_path / "tune.json").read_text())
    assert set(data) == {k1, k3}
    best, times = Bt.choose((1, 2, 4), lambda c: {1: 3.0, 2: 1.0, 4: 2.0}[c], reps=3)
    assert best == 2 and times[2] == 1.0
