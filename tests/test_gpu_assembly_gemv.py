"""GPU parity: fused RBF assembly and the streaming GEMV against the CPU oracle."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import krylov_ref as O

pytestmark = pytest.mark.gpu


def _lib():
    from mpdok_gb300 import _native
    return _native, _native.load()


@pytest.mark.parametrize("kernel", ["gaussian", "mq"])
@pytest.mark.parametrize("dim", [1, 2, 3])
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32, torch.bfloat16, torch.float16])
@pytest.mark.parametrize("col_major", [True, False])
def test_assembly_matches_oracle(kernel, dim, dtype, col_major):
    from mpdok_gb300 import rbf_kernel as R
    rng = np.random.default_rng(dim)
    rows = rng.uniform(0, 1, size=(203, dim))
    cols = rng.uniform(0, 1, size=(131, dim))
    gamma = 9.0 if kernel == "gaussian" else 4.0
    A = R.assemble(rows, cols, gamma=gamma, reg=1e-3, kernel=kernel, dtype=dtype, diag_offset=5,
                   col_major=col_major)
    torch.cuda.synchronize()
    ref = O.rbf_matrix(rows, cols, gamma=gamma, reg=1e-3, kernel=kernel, diag_offset=5)
    got = A.to(torch.float64).cpu().numpy()
    tol = {torch.float64: (1e-14, 1e-14), torch.float32: (3e-7, 3e-7),
           torch.bfloat16: (8e-3, 1e-6), torch.float16: (1e-3, 1e-7)}[dtype]
    np.testing.assert_allclose(got, ref, rtol=tol[0], atol=tol[1])


def test_build_rbf_kernel_matches_reference_golden(golden):
    from mpdok_gb300 import rbf_kernel as R
    g = golden("rbf_assembly")
    A, gamma = R.build_rbf_kernel(g["coords"], gamma=9.0, reg=1e-6)
    assert A.stride() == (1, 128) and A.dtype == torch.float64
    # the reference builds d^2 by the GEMM identity (|a|^2+|b|^2-2ab), whose
    # cancellation error is ~gamma * u * (|a|^2+|b|^2) ~ 4e-15 here
    np.testing.assert_allclose(A.cpu().numpy(), g["A_gauss"], rtol=0, atol=1e-14)
    A2, g2 = R.build_rbf_kernel(g["coords"], reg=1e-3)
    assert g2 == pytest.approx(float(g["gamma_auto"]), rel=1e-14)
    np.testing.assert_allclose(A2.cpu().numpy(), g["A_auto"], rtol=0, atol=1e-14)


def test_fp32_tile_matches_reference_golden(golden):
    from mpdok_gb300 import rbf_kernel as R
    g = golden("rbf_assembly")
    c3 = g["coords3"]
    t = R.assemble(c3[16:56], c3, gamma=25.0, reg=0.0, dtype=torch.float32, col_major=False)
    np.testing.assert_allclose(t.cpu().numpy(), g["tile3"], rtol=4e-7, atol=4e-7)


def test_assembly_edge_sizes():
    from mpdok_gb300 import rbf_kernel as R
    one = R.assemble(np.array([[0.5, 0.5]]), gamma=3.0, reg=0.25)
    assert float(one[0, 0]) == 1.25
    empty = R.assemble(np.zeros((0, 2)), np.zeros((4, 2)), gamma=1.0)
    assert empty.shape == (0, 4)


def _bound(A64, X64, n):
    return 2.0 * n * np.finfo(np.float32).eps * (np.abs(A64) @ np.abs(X64)) + 1e-30


@pytest.mark.parametrize("m,n", [(1, 1), (7, 5), (100, 257), (1000, 999), (4099, 3001), (33, 20000)])
@pytest.mark.parametrize("nrhs", [1, 3, 4, 8])
@pytest.mark.parametrize("trans", [0, 1])
def test_gemv_f32_matches_exact_product(m, n, nrhs, trans):
    N, lib = _lib()
    rng = np.random.default_rng(m * 7 + n)
    A = np.asfortranarray(rng.standard_normal((m, n)).astype(np.float32))
    k_in = m if trans else n
    k_out = n if trans else m
    X = np.asfortranarray(rng.standard_normal((k_in, nrhs)).astype(np.float32))
    dA = torch.from_numpy(A.T.copy()).cuda().t()  # column-major view
    dX = torch.from_numpy(X.T.copy()).cuda().t()
    dY = torch.empty_strided((k_out, nrhs), (1, k_out), dtype=torch.float32, device="cuda")
    ws = torch.empty(lib.mpdok_gemv_workspace_size(N.F32, m, n, nrhs, trans), dtype=torch.uint8, device="cuda")
    st = lib.mpdok_gemv(N.F32, trans, ctypes.c_void_p(dA.data_ptr()), m, m, n, ctypes.c_void_p(dX.data_ptr()),
                        k_in, nrhs, ctypes.c_void_p(dY.data_ptr()), k_out, 1.0, 0.0,
                        ctypes.c_void_p(ws.data_ptr()), ws.numel(), None)
    assert st == 0, N.last_error()
    torch.cuda.synchronize()
    A64 = A.astype(np.float64).T if trans else A.astype(np.float64)
    exact = A64 @ X.astype(np.float64)
    got = dY.cpu().numpy().astype(np.float64)
    assert np.all(np.abs(got - exact) <= _bound(A64, X.astype(np.float64), k_in))


@pytest.mark.parametrize("dt", ["f64", "bf16", "f16"])
def test_gemv_other_dtypes(dt):
    N, lib = _lib()
    m, n = 3000, 2051
    rng = np.random.default_rng(5)
    A = rng.standard_normal((m, n))
    tdt = {"f64": torch.float64, "bf16": torch.bfloat16, "f16": torch.float16}[dt]
    code = {"f64": N.F64, "bf16": N.BF16, "f16": N.F16}[dt]
    dA = torch.from_numpy(A.T.copy()).to("cuda", tdt).t()
    xdt = torch.float64 if dt == "f64" else torch.float32
    x = torch.from_numpy(rng.standard_normal(n)).to("cuda", xdt)
    y = torch.empty(m, dtype=xdt, device="cuda")
    ws = torch.empty(lib.mpdok_gemv_workspace_size(code, m, n, 1, 0), dtype=torch.uint8, device="cuda")
    assert lib.mpdok_gemv(code, 0, ctypes.c_void_p(dA.data_ptr()), m, m, n, ctypes.c_void_p(x.data_ptr()), n, 1,
                          ctypes.c_void_p(y.data_ptr()), m, 1.0, 0.0, ctypes.c_void_p(ws.data_ptr()), ws.numel(),
                          None) == 0
    A_used = dA.to(torch.float64).cpu().numpy()
    exact = A_used @ x.to(torch.float64).cpu().numpy()
    u = 1.2e-16 if dt == "f64" else 6e-8
    bound = 2 * n * u * (np.abs(A_used) @ np.abs(x.to(torch.float64).cpu().numpy()))
    assert np.all(np.abs(y.to(torch.float64).cpu().numpy() - exact) <= bound)


def test_gemv_unaligned_lda_and_alpha_beta():
    N, lib = _lib()
    m, n, lda = 1001, 777, 1003
    rng = np.random.default_rng(9)
    store = torch.from_numpy(rng.standard_normal((n, lda)).astype(np.float32)).cuda()  # column j at row j
    A = store.t()[:m, :]  # (m, n) with column stride lda, base + 0
    Aoff = store.reshape(-1)[1:]  # misaligned base pointer
    x = torch.from_numpy(rng.standard_normal(n).astype(np.float32)).cuda()
    y0 = torch.from_numpy(rng.standard_normal(m).astype(np.float32)).cuda()
    for base in (store.reshape(-1), Aoff):
        y = y0.clone()
        ws = torch.empty(lib.mpdok_gemv_workspace_size(N.F32, m, n, 1, 0), dtype=torch.uint8, device="cuda")
        assert lib.mpdok_gemv(N.F32, 0, ctypes.c_void_p(base.data_ptr()), lda, m, n, ctypes.c_void_p(x.data_ptr()),
                              n, 1, ctypes.c_void_p(y.data_ptr()), m, 2.0, -0.5, ctypes.c_void_p(ws.data_ptr()),
                              ws.numel(), None) == 0
        flat = base.cpu().numpy()
        Am = np.stack([flat[j * lda: j * lda + m] for j in range(n)], axis=1).astype(np.float64)
        exact = 2.0 * (Am @ x.cpu().numpy().astype(np.float64)) - 0.5 * y0.cpu().numpy().astype(np.float64)
        bound = 4 * n * 6e-8 * (np.abs(Am) @ np.abs(x.cpu().numpy())) + 1e-6
        assert np.all(np.abs(y.cpu().numpy() - exact) <= bound)


def test_gemv_is_deterministic():
    N, lib = _lib()
    n = 6000
    A = torch.randn(n, n, device="cuda").t()
    x = torch.randn(n, device="cuda")
    ws = torch.empty(lib.mpdok_gemv_workspace_size(N.F32, n, n, 1, 0), dtype=torch.uint8, device="cuda")
    outs = []
    for _ in range(3):
        y = torch.empty(n, device="cuda")
        lib.mpdok_gemv(N.F32, 0, ctypes.c_void_p(A.data_ptr()), n, n, n, ctypes.c_void_p(x.data_ptr()), n, 1,
                       ctypes.c_void_p(y.data_ptr()), n, 1.0, 0.0, ctypes.c_void_p(ws.data_ptr()), ws.numel(), None)
        outs.append(y.cpu())
    assert torch.equal(outs[0], outs[1]) and torch.equal(outs[1], outs[2])


def test_fp64_residual_and_norm():
    N, lib = _lib()
    n = 2500
    rng = np.random.default_rng(12)
    A = rng.standard_normal((n, n))
    x = rng.standard_normal(n)
    b = rng.standard_normal(n)
    dA = torch.from_numpy(A.T.copy()).cuda().t()
    dx, db = torch.from_numpy(x).cuda(), torch.from_numpy(b).cuda()
    r = torch.empty(n, dtype=torch.float64, device="cuda")
    nrm2 = torch.empty(1, dtype=torch.float64, device="cuda")
    ws = torch.empty(lib.mpdok_gemv_workspace_size(N.F64, n, n, 1, 0), dtype=torch.uint8, device="cuda")
    for _ in range(2):  # the ordered reduction re-arms its ticket
        assert lib.mpdok_residual(ctypes.c_void_p(dA.data_ptr()), n, n, ctypes.c_void_p(db.data_ptr()),
                                  ctypes.c_void_p(dx.data_ptr()), ctypes.c_void_p(r.data_ptr()),
                                  ctypes.c_void_p(nrm2.data_ptr()), ctypes.c_void_p(ws.data_ptr()), ws.numel(),
                                  None) == 0
        ref = b - A @ x
        bound = 2 * n * 1.2e-16 * (np.abs(A) @ np.abs(x) + np.abs(b))
        assert np.all(np.abs(r.cpu().numpy() - ref) <= bound)
        assert float(nrm2.item()) == pytest.approx(float(ref @ ref), rel=1e-12)
