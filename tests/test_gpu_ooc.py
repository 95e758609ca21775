"""GPU parity: out-of-core store (pinned RAM and raw file) and streamed
GMRES-IR against the reference's own MPDOKOOCSolver outputs (golden) and the
oracle."""
import os

import numpy as np
import pytest
import torch

from oracle import krylov_ref as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("store", ["ram", "ssd"])
def test_ooc_tiled_products_match_reference(golden, store, tmp_path):
    from mpdok_gb300.mpdok_ooc import MPDOKOOCSolver
    g = golden("mpdok_ooc")
    s = MPDOKOOCSolver(tile_rows=40)
    path = str(tmp_path / "A_fp32.bin") if store == "ssd" else None
    gam = s.build(g["pts"], gamma=9.0, reg=1e-2, store=store, path=path, verbose=False)
    assert gam == 9.0
    if store == "ram":
        np.testing.assert_array_max_ulp(s.stored_matrix(), g["A32"], maxulp=1)
    y = s._tiled_sgemv(g["b"].astype(np.float32)).cpu().numpy()
    np.testing.assert_allclose(y, g["y_sgemv"], rtol=1e-5, atol=1e-5)
    yd = s._tiled_dgemv_fp64(g["b"]).cpu().numpy()
    np.testing.assert_allclose(yd, g["y_dgemv"], rtol=1e-12, atol=1e-12)
    if store == "ssd":
        torch.cuda.synchronize()
        raw = np.fromfile(path, dtype=np.float32)
        assert raw.size == g["ssd_raw"].size  # raw row-major FP32, no header
        # FP64 math rounded once, nugget added in FP32: the reference's bytes up to
        # one ulp (its distances use the |x|^2 + |y|^2 - 2 x.y identity)
        np.testing.assert_array_max_ulp(raw, g["ssd_raw"], maxulp=1)
    assert s.bytes_moved() == pytest.approx(150 * 150 * 4)
    s.free()


def test_ooc_solve_follows_reference_trajectory(golden):
    import warnings
    from mpdok_gb300.mpdok_ooc import MPDOKOOCSolver
    g = golden("mpdok_ooc")
    A64 = O.rbf_matrix(g["pts"], gamma=9.0, reg=1e-2)
    s = MPDOKOOCSolver(tile_rows=40)
    s.build(g["pts"], gamma=9.0, reg=1e-2, store="ram", verbose=False)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        x = s.solve(g["b"], tol=1e-10, maxiter_outer=8, restart=20, verbose=False).cpu().numpy()
    ref_rel = O.relres(A64, g["x"], g["b"])
    rel = O.relres(A64, x, g["b"])
    assert 0.5 < rel / ref_rel < 2.0  # restart 20 stalls near 2e-5 in the reference too
    assert np.linalg.norm(x - g["x"]) / np.linalg.norm(g["x"]) < 1e-3
    s.free()


def test_ooc_converges_on_well_conditioned_system():
    from mpdok_gb300.mpdok_ooc import MPDOKOOCSolver
    rng = np.random.default_rng(4)
    X = rng.uniform(0, 1, (3000, 3))
    b = rng.standard_normal(3000)
    A = O.rbf_matrix(X, gamma=400.0, reg=1e-1)
    s = MPDOKOOCSolver(tile_rows=1000)
    s.build(X, gamma=400.0, reg=1e-1, store="ram", verbose=False)
    x = s.solve(b, tol=1e-11, maxiter_outer=10, restart=30, verbose=False).cpu().numpy()
    x_lu = O.fp64_solve(A, b)
    assert O.relres(A, x, b) < 1e-11
    assert np.linalg.norm(x - x_lu) / np.linalg.norm(x_lu) < 1e-9
    s.free()


def test_ooc_missing_file_directory_is_an_io_error(tmp_path):
    from mpdok_gb300 import _native as N
    from mpdok_gb300.mpdok_ooc import MPDOKOOCSolver
    s = MPDOKOOCSolver(tile_rows=16)
    with pytest.raises(N.MPDOKError):
        s.build(np.random.default_rng(0).uniform(0, 1, (64, 2)), gamma=4.0, store="ssd",
                path=str(tmp_path / "no" / "such" / "dir.bin"), verbose=False)
