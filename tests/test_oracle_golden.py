"""CPU: the oracle restatement reproduces the reference's own outputs.

Golden vectors come from running the reference modules (rbf_kernel.py,
dense_krylov.py, mpdok_ooc.py) on CPU via tests/golden/make_golden.py.
"""
import numpy as np
import pytest

from oracle import krylov_ref as O


def test_estimate_gamma_matches_reference(golden):
    g = golden("rbf_assembly")
    assert O.estimate_gamma(g["coords"]) == pytest.approx(float(g["gamma_est"]), rel=1e-14)
    assert float(g["gamma_auto"]) == pytest.approx(float(g["gamma_est"]), rel=1e-14)


def test_rbf_matrix_matches_reference_build(golden):
    g = golden("rbf_assembly")
    A = O.rbf_matrix(g["coords"], gamma=9.0, reg=1e-6)
    np.testing.assert_allclose(A, g["A_gauss"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(O.rbf_matrix_identity(g["coords"], 9.0, 1e-6), g["A_gauss"], rtol=0, atol=1e-15)
    np.testing.assert_allclose(A, g["A_cpu"], rtol=0, atol=1e-14)
    A2 = O.rbf_matrix(g["coords"], gamma=float(g["gamma_auto"]), reg=1e-3)
    np.testing.assert_allclose(A2, g["A_auto"], rtol=0, atol=1e-14)


def test_fp32_tile_matches_reference(golden):
    g = golden("rbf_assembly")
    c3 = g["coords3"]
    tile = O.rbf_matrix(c3[16:56], c3, gamma=25.0).astype(np.float32)
    # the reference adds no nugget inside _build_fp32_tile (mpdok_ooc.py:39-46)
    np.testing.assert_array_max_ulp(tile, g["tile3"], maxulp=2)


def test_ooc_ram_buffer_is_assembly_plus_nugget(golden):
    g = golden("mpdok_ooc")
    A = O.rbf_matrix(g["pts"], gamma=9.0, reg=1e-2).astype(np.float32)
    np.testing.assert_allclose(A, g["A32"], rtol=2e-7, atol=2e-7)
    # SSD store = the same matrix as raw row-major FP32 without a header
    np.testing.assert_array_equal(g["ssd_raw"], g["A32"].reshape(-1))


def test_tiled_gemvs_match(golden):
    g = golden("mpdok_ooc")
    A32 = g["A32"]
    b = g["b"]
    np.testing.assert_allclose(O.gemv_exact(A32, b.astype(np.float32)), g["y_sgemv"], rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(O.rbf_matrix(g["pts"], gamma=9.0, reg=1e-2) @ b, g["y_dgemv"], rtol=1e-12, atol=1e-12)


def test_inner_gmres_matches_reference_port(golden):
    g = golden("mpdok_ooc")
    e, m = O.inner_gmres(g["A32"], g["b"], 20)
    np.testing.assert_allclose(e, g["e_inner"], rtol=2e-4, atol=2e-4 * np.abs(g["e_inner"]).max())
    assert 1 <= m <= 20


def test_native_gmres_ir_matches_ooc_solve(golden):
    """restart 20 on this kappa ~ 4e3 system stalls at ~2e-5 after 8 outer
    steps in the reference too; the oracle must follow the same trajectory."""
    g = golden("mpdok_ooc")
    A64 = O.rbf_matrix(g["pts"], gamma=9.0, reg=1e-2)
    x, hist, conv, _ = O.gmres_ir_native(A64, g["b"], tol=1e-10, maxiter_outer=8, restart=20, A32=g["A32"])
    ref_rel = O.relres(A64, g["x"], g["b"])
    assert not conv and ref_rel > 1e-10
    assert 0.5 < hist[-1][1] / ref_rel < 2.0
    assert [h[0] for h in hist] == list(range(9))
    # each outer step contracts the residual by the same factor (+-30 %)
    rates = [hist[i + 1][1] / hist[i][1] for i in range(8)]
    assert all(0.1 < r < 0.4 for r in rates)
    assert np.linalg.norm(x - g["x"]) / np.linalg.norm(g["x"]) < 1e-3


def test_dense_krylov_cg_gmres_match(golden):
    g = golden("dense_krylov")
    x, h, c = O.cg(g["A_spd"], g["b"], tol=1e-6)
    assert c == bool(g["c_cg"])
    np.testing.assert_allclose(x, g["x_cg"], rtol=0, atol=1e-5 * np.abs(g["x_cg"]).max())
    assert len(h) == len(g["h_cg"])
    x, h, c = O.gmres(g["A_ns"], g["b"], tol=1e-6, restart=20)
    assert c == bool(g["c_gm"])
    np.testing.assert_allclose(x, g["x_gm"], rtol=0, atol=1e-5 * np.abs(g["x_gm"]).max())
    assert [int(i) for i, _ in h] == [int(i) for i in g["h_gm"][:, 0]]


def test_dense_gmres_ir_matches(golden):
    g = golden("dense_krylov")
    for A, key in ((g["A_ns"], ""), (g["A_spd"], "_spd")):
        x, h, c = O.gmres_ir(A, g["b"], tol=1e-11, restart=20)
        assert c == bool(g["c_ir" + key])
        ref = g["x_ir" + key]
        np.testing.assert_allclose(x, ref, rtol=0, atol=1e-10 * np.abs(ref).max())
        assert len(h) == len(g["h_ir" + key])
        assert h[-1][1] < 1e-11


def test_matvec_and_residual_norm(golden):
    g = golden("dense_krylov")
    y = O.gemv_exact(g["A_ns"].astype(np.float32), g["b"].astype(np.float32))
    np.testing.assert_allclose(y, g["y32"], rtol=1e-5)
    rn = np.linalg.norm(g["b"] - g["A_ns"] @ g["x_ir"])
    assert rn == pytest.approx(float(g["rn"]), rel=1e-6, abs=1e-14)


def test_lu_ir_reaches_fp64():
    rng = np.random.default_rng(3)
    n = 200
    A = rng.standard_normal((n, n)) + n * np.eye(n)
    b = rng.standard_normal(n)
    x, hist, conv = O.lu_ir(A, b, tol=1e-13)
    assert conv
    np.testing.assert_allclose(x, O.fp64_solve(A, b), rtol=1e-12, atol=1e-14)


def test_oracle_edge_cases():
    A = np.eye(4) * 2.0
    x, h, c, _ = O.gmres_ir_native(A, np.zeros(4))
    assert c and np.all(x == 0)
    x, h, c = O.cg(A, np.zeros(4))
    assert c and h == [(0, 0.0)]
    e, m = O.inner_gmres(A.astype(np.float32), np.ones(4), 5)
    np.testing.assert_allclose(e, 0.5 * np.ones(4), rtol=1e-6)   # breakdown after one step
    assert m == 1
