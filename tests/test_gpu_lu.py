"""GPU parity: tcgen05 trailing update, blocked LU, LU-IR and LU-preconditioned GMRES-IR."""
import warnings

import numpy as np
import pytest
import torch

from oracle import krylov_ref as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dt", [torch.bfloat16, torch.float16])
@pytest.mark.parametrize("M,Nn,K", [(128, 256, 128), (300, 520, 128), (1000, 777, 64), (257, 1029, 256),
                                    (129, 100, 192),
                                    # K >= 256 with ldc % 4 == 0: the warp-specialised kernel (strips of
                                    # four tiles, two TMEM accumulators, TMA reduce-add epilogue)
                                    (1000, 777, 256), (512, 1100, 512), (4096, 4100, 1024), (132, 2048, 320)])
def test_tensor_core_update_matches_cuda_cores(dt, M, Nn, K):
    from mpdok_gb300.lu import gemm_update
    g = torch.Generator(device="cuda").manual_seed(M + Nn + K)
    A = torch.randn(M, K, device="cuda", generator=g).to(dt)
    B = torch.randn(Nn, K, device="cuda", generator=g).to(dt)
    C0 = torch.randn(Nn, M, device="cuda", generator=g).t()  # column-major (M, Nn)
    C_tc = gemm_update(C0.clone().t().contiguous().t(), A, B, engine="tensor")
    C_sc = gemm_update(C0.clone().t().contiguous().t(), A, B, engine="simt")
    ref = C0.double() - A.double() @ B.double().t()
    torch.cuda.synchronize()
    scale = (A.double().abs() @ B.double().abs().t()) + C0.double().abs()
    assert torch.all((C_tc.double() - ref).abs() <= 4 * K * 6e-8 * scale + 1e-6)
    assert torch.all((C_sc.double() - ref).abs() <= 4 * K * 6e-8 * scale + 1e-6)


def _rbf(n, gamma, reg, seed=0, dim=2):
    rng = np.random.default_rng(seed)
    X = rng.uniform(0, 1, size=(n, dim))
    return X, O.rbf_matrix(X, gamma=gamma, reg=reg), rng.standard_normal(n)


@pytest.mark.parametrize("dtype", ["fp32", "fp16", "bf16"])
@pytest.mark.parametrize("n", [128, 1000, 1100])
def test_lu_factor_apply_inverts(dtype, n):
    from mpdok_gb300.lu import LUFactorization
    X, A, b = _rbf(n, 400.0, 1e-1, seed=n)
    lu = LUFactorization(A, dtype=dtype)
    assert lu.n_perturbed == 0
    z = lu.apply(torch.from_numpy(b).cuda().float()).double().cpu().numpy()
    x_true = O.fp64_solve(A, b)
    err = np.linalg.norm(z - x_true) / np.linalg.norm(x_true)
    kappa = np.linalg.cond(A)
    u = {"fp32": 6e-8, "fp16": 4.9e-4, "bf16": 3.9e-3}[dtype]
    assert err < max(1e-3, 50 * kappa * u) if dtype != "fp32" else err < 1e-4 * kappa + 1e-5


@pytest.mark.parametrize("dtype,tol", [("fp32", 5e-6), ("fp16", 3e-3), ("bf16", 2e-2)])
@pytest.mark.parametrize("n", [1, 128, 131, 300, 1077, 2100])
def test_unpivoted_factors_reproduce_the_scaled_matrix(dtype, tol, n):
    """L U = D A D for the unpivoted factorization (diagonal LU two steps per
    barrier, block-substitution panel solves, tensor-core or CUDA-core
    updates), with an odd last block (n = 131, 1077) included."""
    from mpdok_gb300.lu import LUFactorization
    X, A, b = _rbf(n, 400.0, 1e-1, seed=n + 11)
    lu = LUFactorization(A, dtype=dtype)
    assert lu.n_perturbed == 0
    LU, ipiv, perm, dr, dc = (t.cpu().numpy() for t in lu.export())
    np.testing.assert_array_equal(perm, np.arange(n))
    W = A * dr.astype(np.float64)[:, None] * dc.astype(np.float64)[None, :]
    L = np.tril(LU.astype(np.float64), -1) + np.eye(n)
    U = np.triu(LU.astype(np.float64))
    rel = np.linalg.norm(W - L @ U) / np.linalg.norm(W)
    assert rel < tol * max(1.0, np.log2(n)), rel


def test_lu_apply_is_deterministic():
    from mpdok_gb300.lu import LUFactorization
    X, A, b = _rbf(2000, 900.0, 1e-2, seed=4)
    lu = LUFactorization(A, dtype="fp16")
    v = torch.from_numpy(b).cuda().float()
    z1 = lu.apply(v)
    z2 = lu.apply(v)
    assert torch.equal(z1, z2)


def test_lu_ir_solver_matches_reference(golden):
    from mpdok_gb300.mpdok_ops import LUIRSolver
    g = golden("dense_krylov")
    for A in (g["A_ns"], g["A_spd"]):
        s = LUIRSolver()
        x = s.solve(A, g["b"], tol=1e-12, maxiter_outer=3)
        xo, ho, co = O.lu_ir(A, g["b"], tol=1e-12, maxiter_outer=3)
        assert co
        assert O.relres(A, x.cpu().numpy(), g["b"]) < 1e-12
        np.testing.assert_allclose(x.cpu().numpy(), O.fp64_solve(A, g["b"]), rtol=1e-11, atol=1e-14)


def test_lu_ir_factor_once_solve_many():
    from mpdok_gb300.mpdok_ops import LUIRSolver
    X, A, _ = _rbf(1500, 2500.0, 1e-2, seed=8)
    s = LUIRSolver()
    s.factor(A)
    rng = np.random.default_rng(1)
    for _ in range(3):
        b = rng.standard_normal(1500)
        x = s.solve_factored(b, tol=1e-12, maxiter_outer=5)
        assert O.relres(A, x.cpu().numpy(), b) < 1e-12
    s.free_factored()
    with pytest.raises(RuntimeError):
        s.solve_factored(b)


@pytest.mark.parametrize("dtype", ["fp16", "bf16"])
def test_lu_gmres_ir_reaches_fp64(dtype):
    from mpdok_gb300.lu import LUFactorization
    X, A, b = _rbf(3000, 1600.0, 1e-2, seed=2)
    lu = LUFactorization(A, dtype=dtype)
    x, info = lu.gmres_ir(A, b, tol=1e-12, maxiter_outer=10, restart=30)
    assert info["converged"]
    xs = x.cpu().numpy()
    rel = O.relres(A, xs, b)
    x_lu = O.fp64_solve(A, b)
    assert rel <= max(1e-12, 10 * O.relres(A, x_lu, b))
    assert np.linalg.norm(xs - x_lu) / np.linalg.norm(x_lu) < 1e-9
    assert info["inner_iters"] < 200


def test_mixed_solver_headline_family_small():
    from mpdok_gb300 import configs
    from mpdok_gb300.rbf_kernel import assemble
    from mpdok_gb300.solvers import MixedSolver
    s = configs.headline(n=4096)
    A = assemble(s.coords, gamma=s.gamma, reg=s.reg)
    x, info = MixedSolver().solve(A, s.b, tol=1e-12)
    A64 = O.rbf_matrix(s.coords, gamma=s.gamma, reg=s.reg)
    assert info["converged"]
    assert O.relres(A64, x.cpu().numpy(), s.b) < 1e-12


def test_hard_family_fp32_factors_reach_the_fp64_floor():
    """The hard family (the headline's centres, C5's nugget 1e-6, smooth
    right-hand side) at N = 4096, with eps scaled to the point density,
    100 * sqrt(4096 / 32768): kappa ~ 1.5e7.  FP32 factors precondition the
    GMRES-IR to <= max(1e-12, 10 x) the FP64 LU oracle's relres, and the
    solution agrees with the oracle's to within kappa times the residual floor.
    FP16 factors have kappa * u > 1 here; their outcome is only reported."""
    import math
    import warnings
    from mpdok_gb300 import configs
    from mpdok_gb300.rbf_kernel import assemble
    from mpdok_gb300.solvers import MixedSolver
    n = 4096
    s = configs.hard_headline(n=n, eps=configs.HARD_EPS * math.sqrt(n / 32768))
    A64 = O.rbf_matrix(s.coords, gamma=s.gamma, reg=s.reg)
    x_ref = O.fp64_solve(A64, s.b)
    floor = O.relres(A64, x_ref, s.b)
    A = assemble(s.coords, gamma=s.gamma, reg=s.reg, dtype=torch.float64)
    b = torch.from_numpy(s.b).cuda()
    x, info = MixedSolver(factor_dtype="fp32").solve(A, b, tol=1e-12)
    assert info["converged"]
    xs = x.cpu().numpy()
    assert O.relres(A64, xs, s.b) <= max(1e-12, 10 * floor)
    assert np.linalg.norm(xs - x_ref) / np.linalg.norm(x_ref) < 1e-6
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        x16, info16 = MixedSolver(factor_dtype="fp16").solve(A, b, tol=1e-12)
    assert torch.isfinite(x16).all() and info16["relres"] <= 1.0 + 1e-12


def test_lu_not_factored_status():
    import ctypes
    from mpdok_gb300 import _native as N
    lib = N.load()
    n = 256
    fac = torch.zeros(lib.mpdok_lu_factor_size(n, N.F16), dtype=torch.uint8, device="cuda")
    w = torch.empty(lib.mpdok_lu_ir_work_size(n), dtype=torch.uint8, device="cuda")
    A = torch.eye(n, dtype=torch.float64, device="cuda")
    b = torch.ones(n, dtype=torch.float64, device="cuda")
    x = torch.zeros_like(b)
    info = N.SolveInfo()
    st = lib.mpdok_lu_ir_solve(ctypes.c_void_p(A.data_ptr()), n, n, ctypes.c_void_p(fac.data_ptr()), N.F16,
                               ctypes.c_void_p(b.data_ptr()), ctypes.c_void_p(x.data_ptr()), 1e-12, 3,
                               ctypes.c_void_p(w.data_ptr()), w.numel(), ctypes.byref(info), None)
    assert st == N.ERR_NOT_FACTORED


def test_mixed_solver_guard_on_singular_c3():
    """C3 as specified (MQ, eps=2, no nugget) is singular to working precision:
    the pivoted FP64 LU reaches relres ~1e2.  The guarded mixed solve returns
    its best iterate (relres <= 1, finite) with a RuntimeWarning."""
    import warnings
    from mpdok_gb300 import configs
    from mpdok_gb300.rbf_kernel import assemble
    from mpdok_gb300.solvers import MixedSolver
    c3 = configs.c3(n=4096)
    A = assemble(c3.coords, gamma=c3.gamma, reg=c3.reg, kernel=c3.kernel, dtype=torch.float64)
    b = torch.from_numpy(c3.b).cuda()
    for fd in ("fp16", "bf16"):
        with warnings.catch_warnings(record=True) as w:
            warnings.simplefilter("always")
            x, info = MixedSolver(factor_dtype=fd).solve(A, b, tol=1e-12)
        assert not info["converged"]
        assert any(issubclass(m.category, RuntimeWarning) for m in w)
        assert torch.isfinite(x).all()
        rel = float(torch.linalg.norm(b - A @ x) / torch.linalg.norm(b))
        assert rel <= 1.0 + 1e-12 and abs(rel - info["relres"]) <= 1e-6 * max(rel, 1e-30)


def test_mixed_solver_fp32_factors_on_moderate_mq():
    """MQ with a sharp shape parameter (gamma = 1e4, N = 2048, kappa ~ 1.7e8,
    one positive eigenvalue): the unpivoted FP32-factor LU-GMRES-IR reaches the
    FP64 LU oracle's own residual floor."""
    import warnings
    from mpdok_gb300 import configs
    from mpdok_gb300.rbf_kernel import assemble
    from mpdok_gb300.solvers import MixedSolver
    X = configs.stratified_jitter(2048, 2)
    b = np.random.default_rng(7).standard_normal(2048)
    A64 = O.rbf_matrix(X, gamma=1e4, reg=0.0, kernel="mq")
    x_ref = O.fp64_solve(A64, b)
    floor = O.relres(A64, x_ref, b)
    A = assemble(X, gamma=1e4, reg=0.0, kernel="mq", dtype=torch.float64)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        x, info = MixedSolver(factor_dtype="fp32").solve(A, torch.from_numpy(b).cuda(), tol=1e-12)
    xh = x.cpu().numpy()
    assert O.relres(A64, xh, b) <= 10 * floor
    assert np.linalg.norm(xh - x_ref) / np.linalg.norm(x_ref) < 1e-8


@pytest.mark.parametrize("fdtype", ["fp32", "bf16"])
@pytest.mark.parametrize("n,k", [(1000, 1), (1500, 8), (777, 19)])
def test_lu_ir_many_rhs_matches_single_rhs_and_oracle(fdtype, n, k):
    """Multi-RHS LU-IR (one triangular sweep pair for up to 8 columns) against
    the FP64 LU oracle, and column by column against the single-RHS LU-IR."""
    from mpdok_gb300.lu import LUFactorization
    rng = np.random.default_rng(n + k)
    X = rng.uniform(0, 1, (n, 2))
    A64 = O.rbf_matrix(X, gamma=1600.0, reg=1e-1)  # kappa ~ 20: plain refinement converges with BF16 factors
    B = rng.standard_normal((n, k))
    A = torch.from_numpy(np.asfortranarray(A64)).cuda()
    lu = LUFactorization(A, dtype=fdtype)
    Xg, info = lu.solve_ir_many(A, torch.from_numpy(B).cuda(), tol=1e-12, maxiter_outer=10)
    assert info["converged"]
    Xh = Xg.cpu().numpy().reshape(n, k)
    Xref = np.linalg.solve(A64, B)
    for j in range(k):
        rel = O.relres(A64, Xh[:, j], B[:, j])
        assert rel < 1e-12
        assert np.linalg.norm(Xh[:, j] - Xref[:, j]) / np.linalg.norm(Xref[:, j]) < 1e-10
    xs, d = lu.solve_ir(A, torch.from_numpy(B[:, 0].copy()).cuda(), tol=1e-12, maxiter_outer=10)
    assert d["converged"]
    np.testing.assert_allclose(Xh[:, 0], xs.cpu().numpy(), rtol=1e-9, atol=1e-12 * np.abs(Xh[:, 0]).max())


def test_profile_timeline_matches_class_totals():
    """The per-launch timeline of an LU factorization (chain, strip and far
    streams) agrees with the per-class totals of the same records."""
    from mpdok_gb300 import _native as N
    from mpdok_gb300.lu import LUFactorization
    X, A, b = _rbf(3000, 1600.0, 1e-2, seed=5)
    N.profile_enable(True)
    try:
        LUFactorization(A, dtype="fp16")
        torch.cuda.synchronize()
        tl = N.profile_timeline()
        totals = {c: N.profile_query(c) for c in range(9)}
    finally:
        N.profile_enable(False)
    assert len(tl) == sum(cnt for _, cnt, _ in totals.values())
    assert np.all(tl[:, 2] >= tl[:, 1]) and np.all(tl[:, 1] >= 0.0)
    assert totals[N.PROF_LU_PANEL][1] > 0 and totals[N.PROF_LU_GEMM_DEEP][1] > 0
    for c in (N.PROF_LU_PANEL, N.PROF_LU_GEMM, N.PROF_LU_GEMM_DEEP):
        rows = tl[tl[:, 0] == c]
        ms, cnt, work = totals[c]
        assert len(rows) == cnt
        assert np.isclose(rows[:, 3].sum(), work, rtol=1e-12)
        assert np.isclose((rows[:, 2] - rows[:, 1]).sum(), ms, rtol=1e-3, atol=1e-3)
    # a record per 128-column panel on the chain stream (its diagonal LU and
    # its solve inside the super-panel), and one on the below stream while
    # super-panels follow
    s = N.lu_schedule(16384, N.F16)
    spw = sorted({int(j) for j in s[s[:, 0] == 0][:, 2]})[1]
    n, expect = 3000, 0
    for jp in range(0, n, 128):
        jend = min(n, (jp // spw + 1) * spw)
        expect += 1 + (n > spw and jend < n)
    assert len(tl[tl[:, 0] == N.PROF_LU_PANEL]) == expect
