"""GPU parity: batched Cholesky solves of uneven RBF systems, CUDA-graph
replay, and the adjoint gradients, against the FP64 oracle (SciPy Cholesky
per system, dense gradient formulas), torch FP64 autograd and finite
differences."""
import numpy as np
import pytest
import torch

from oracle import batch_ref as R

pytestmark = pytest.mark.gpu


def _batch(sizes, dim, nrhs, seed, eps_lo=2.0, eps_hi=8.0):
    rng = np.random.default_rng(seed)
    Xs = [rng.uniform(0, 1, (n, dim)) for n in sizes]
    eps = rng.uniform(eps_lo, eps_hi, len(sizes))
    Bs = [rng.standard_normal((n, nrhs)) for n in sizes]
    return Xs, eps, Bs


@pytest.mark.parametrize("arith", ["df32", "f64"])
@pytest.mark.parametrize("dim,nrhs", [(2, 3), (3, 8), (1, 1)])
def test_batch_solve_matches_fp64_cholesky(arith, dim, nrhs):
    from mpdok_gb300.batch import BatchedRBFSolver, unpack_rhs
    sizes = [1, 63, 64, 65, 130, 257, 511, 40, 200]
    Xs, eps, Bs = _batch(sizes, dim, nrhs, seed=dim * 10 + nrhs, eps_lo=3.0, eps_hi=6.0)
    reg = 1e-4
    s = BatchedRBFSolver(sizes, dim=dim, nrhs=nrhs, arith=arith, grid_mult=2)
    s.load(Xs, eps, reg).factor()
    assert s.perturbed_pivots() == 0
    X = s.solve(Bs, refine=2)
    rel = s.relres(Bs, X).cpu().numpy()
    for i, (Xc, B, xg) in enumerate(zip(Xs, Bs, unpack_rhs(X, sizes, nrhs))):
        x_ref, rel_ref = R.solve(Xc, eps[i], reg, B)
        A = R.rbf(Xc, eps[i], reg)
        rel_true = np.max(np.linalg.norm(B - A @ xg.cpu().numpy(), axis=0) / np.linalg.norm(B, axis=0))
        assert rel_true <= max(1e-13, 10 * rel_ref), (i, sizes[i], rel_true, rel_ref)
        assert rel[i] == pytest.approx(rel_true, rel=0.5, abs=1e-14)  # both at FP64 rounding level
        err = np.linalg.norm(xg.cpu().numpy() - x_ref) / np.linalg.norm(x_ref)
        cond = np.linalg.cond(A)
        assert err <= max(1e-12, 50 * cond * 1.1e-16), (i, err, cond)


def test_batch_c4_shape_reaches_the_fp64_floor():
    """C4-shaped (reduced): N in [500, 1500], eps ~ U(2, 8), nugget 1e-8, 8 RHS;
    kappa 1e9 - 1e11.  relres within 10x of the FP64 Cholesky oracle's own."""
    from mpdok_gb300.batch import BatchedRBFSolver, unpack_rhs
    rng = np.random.default_rng(3)
    sizes = list(rng.integers(500, 1501, size=6))
    Xs, eps, Bs = _batch(sizes, 2, 8, seed=3)
    s = BatchedRBFSolver(sizes, dim=2, nrhs=8, arith="df32", grid_mult=2)
    s.load(Xs, eps, 1e-8).factor()
    X = s.solve(Bs, refine=3)
    for i, (Xc, B, xg) in enumerate(zip(Xs, Bs, unpack_rhs(X, sizes, 8))):
        x_ref, rel_ref = R.solve(Xc, eps[i], 1e-8, B)
        A = R.rbf(Xc, eps[i], 1e-8)
        rel = np.max(np.linalg.norm(B - A @ xg.cpu().numpy(), axis=0) / np.linalg.norm(B, axis=0))
        assert rel <= 10 * rel_ref + 1e-14, (i, rel, rel_ref)


def test_batch_graph_replay_is_identical_to_direct_calls():
    from mpdok_gb300.batch import BatchedRBFSolver
    sizes = [300, 129, 64, 700, 5]
    Xs, eps, Bs = _batch(sizes, 2, 4, seed=9)
    s = BatchedRBFSolver(sizes, dim=2, nrhs=4, grid_mult=1)
    s.load(Xs, eps, 1e-6).factor()
    X_direct = s.solve(Bs, refine=2).clone()
    Bbuf, Xbuf = s.build_graph(Bs, refine=2)
    assert s.graph_nodes > 10
    for _ in range(2):
        Xbuf.zero_()
        s.run_graph()
        torch.cuda.synchronize()
        assert torch.equal(Xbuf, X_direct)


def test_batch_adjoint_matches_oracle_and_torch_autograd():
    from mpdok_gb300.batch import BatchedRBFSolver, pack_coords, pack_rhs, rbf_batch_solve, unpack_rhs
    sizes = [90, 33, 150, 64]
    nrhs = 3
    Xs, eps, Bs = _batch(sizes, 2, nrhs, seed=21, eps_lo=3.0, eps_hi=7.0)
    reg = 1e-3
    rng = np.random.default_rng(5)
    Xstar = [rng.standard_normal((n, nrhs)) for n in sizes]
    s = BatchedRBFSolver(sizes, dim=2, nrhs=nrhs, arith="f64", grid_mult=1)
    C = pack_coords(Xs).requires_grad_(True)
    E = torch.tensor(eps, dtype=torch.float64, device="cuda", requires_grad=True)
    G = torch.tensor(reg, dtype=torch.float64, device="cuda", requires_grad=True)
    B = pack_rhs(Bs, nrhs).requires_grad_(True)
    Xp = rbf_batch_solve(C, E, G, B, s, refine=2)
    T = pack_rhs(Xstar, nrhs)
    loss = ((Xp - T) ** 2).sum()
    loss.backward()
    gC = C.grad.cpu().numpy()
    o = 0
    tot_reg = 0.0
    for i, n in enumerate(sizes):
        x = unpack_rhs(Xp.detach(), sizes, nrhs)[i].cpu().numpy()
        dc, de, dr, lam = R.grads(Xs[i], eps[i], reg, Bs[i], 2 * (x - Xstar[i]))
        np.testing.assert_allclose(gC[o:o + n], dc, rtol=1e-7, atol=1e-9 * np.abs(dc).max())
        assert E.grad[i].item() == pytest.approx(de, rel=1e-8)
        lam_g = unpack_rhs(B.grad, sizes, nrhs)[i].cpu().numpy()
        np.testing.assert_allclose(lam_g, lam, rtol=1e-8, atol=1e-10 * np.abs(lam).max())
        tot_reg += dr
        o += n
    assert G.grad.item() == pytest.approx(tot_reg, rel=1e-8)

    # torch FP64 autograd through torch.linalg.solve on the first system
    c0 = torch.tensor(Xs[0], dtype=torch.float64, device="cuda", requires_grad=True)
    e0 = torch.tensor(eps[0], dtype=torch.float64, device="cuda", requires_grad=True)
    r0 = torch.tensor(reg, dtype=torch.float64, device="cuda", requires_grad=True)
    b0 = torch.tensor(Bs[0], dtype=torch.float64, device="cuda", requires_grad=True)
    d2 = ((c0[:, None, :] - c0[None, :, :]) ** 2).sum(-1)
    A0 = torch.exp(-(e0 ** 2) * d2) + r0 * torch.eye(sizes[0], dtype=torch.float64, device="cuda")
    x0 = torch.linalg.solve(A0, b0)
    l0 = ((x0 - torch.tensor(Xstar[0], dtype=torch.float64, device="cuda")) ** 2).sum()
    l0.backward()
    np.testing.assert_allclose(gC[:sizes[0]], c0.grad.cpu().numpy(), rtol=1e-6,
                               atol=1e-8 * c0.grad.abs().max().item())
    assert E.grad[0].item() == pytest.approx(e0.grad.item(), rel=1e-7)
    np.testing.assert_allclose(unpack_rhs(B.grad, sizes, nrhs)[0].cpu().numpy(), b0.grad.cpu().numpy(),
                               rtol=1e-7, atol=1e-9 * b0.grad.abs().max().item())


def test_batch_adjoint_central_differences_in_eps_and_centres():
    from mpdok_gb300.batch import BatchedRBFSolver, pack_coords, pack_rhs, rbf_batch_solve
    sizes = [70, 120]
    nrhs = 2
    Xs, eps, Bs = _batch(sizes, 2, nrhs, seed=33, eps_lo=4.0, eps_hi=5.0)
    reg = 1e-2
    T = pack_rhs([np.ones((n, nrhs)) for n in sizes], nrhs)
    s = BatchedRBFSolver(sizes, dim=2, nrhs=nrhs, arith="f64", grid_mult=1)
    B = pack_rhs(Bs, nrhs)

    def L(C, E):
        with torch.no_grad():
            X = rbf_batch_solve(C, E, torch.tensor(reg, dtype=torch.float64, device="cuda"), B, s, refine=2)
            return ((X - T) ** 2).sum().item()

    C = pack_coords(Xs).requires_grad_(True)
    E = torch.tensor(eps, dtype=torch.float64, device="cuda", requires_grad=True)
    X = rbf_batch_solve(C, E, torch.tensor(reg, dtype=torch.float64, device="cuda"), B, s, refine=2)
    ((X - T) ** 2).sum().backward()
    gE, gC = E.grad.clone(), C.grad.clone()
    h = 1e-6
    for i in range(2):
        Ep, Em = E.detach().clone(), E.detach().clone()
        Ep[i] += h
        Em[i] -= h
        fd = (L(C.detach(), Ep) - L(C.detach(), Em)) / (2 * h)
        assert gE[i].item() == pytest.approx(fd, rel=1e-5)
    for (r, d) in [(3, 0), (75, 1), (189, 0)]:
        Cp, Cm = C.detach().clone(), C.detach().clone()
        Cp[r, d] += h
        Cm[r, d] -= h
        fd = (L(Cp, E.detach()) - L(Cm, E.detach())) / (2 * h)
        assert gC[r, d].item() == pytest.approx(fd, rel=1e-4, abs=1e-6 * gC.abs().max().item())


def test_batch_autotune_picks_and_caches(tmp_path, monkeypatch):
    from mpdok_gb300 import batch as Bt
    monkeypatch.setenv("MPDOK_GB300_AUTOTUNE", str(tmp_path / "t.json"))
    sizes = [400, 300, 200]
    Xs, eps, Bs = _batch(sizes, 2, 2, seed=1)
    s = Bt.BatchedRBFSolver(sizes, dim=2, nrhs=2)
    s.load(Xs, eps, 1e-6)
    rec = s.autotune(candidates=("levels:1", "levels:2", "dag:2", "dag:3"), reps=1)
    assert rec["config"] in ("levels:1", "levels:2", "dag:2", "dag:3") and s.config == rec["config"]
    assert set(rec["seconds"]) == {"levels:1", "levels:2", "dag:2", "dag:3"} and rec["tile"] == 64
    s2 = Bt.BatchedRBFSolver(sizes, dim=2, nrhs=2)
    assert s2.tuned is not None and s2.config == rec["config"]
    s2.load(Xs, eps, 1e-6).factor()
    X = s2.solve(Bs)
    rel = s2.relres(Bs, X).cpu().numpy()
    for i in range(3):
        _, rel_ref = R.solve(Xs[i], eps[i], 1e-6, Bs[i])
        assert rel[i] <= 10 * rel_ref + 1e-14


def test_batch_rejects_bad_arguments():
    from mpdok_gb300 import _native as N
    from mpdok_gb300.batch import BatchedRBFSolver
    with pytest.raises(N.MPDOKError):
        BatchedRBFSolver([10, 20], dim=2, nrhs=9)
    with pytest.raises(ValueError):
        BatchedRBFSolver([10, 0], dim=2, nrhs=1)
    s = BatchedRBFSolver([10, 20], dim=2, nrhs=1)
    with pytest.raises(RuntimeError):
        s.factor()
    with pytest.raises(ValueError):
        s.load([np.zeros((10, 2)), np.zeros((19, 2))], 3.0, 1e-6)


def test_c1_as_specified_reaches_the_fp64_floor():
    """C1 (N=2000, eps=3, nugget 1e-10, kappa ~ 5e12): 1e-12 is out of reach even
    for FP64 LU (its relres ~ 2e-7).  The double-float Cholesky with FP64
    refinement reaches the oracle's own floor."""
    from mpdok_gb300 import configs
    from mpdok_gb300.batch import BatchedRBFSolver
    c1 = configs.c1()
    s = BatchedRBFSolver([c1.n], dim=2, nrhs=1, grid_mult=2)
    s.load([c1.coords], [3.0], c1.reg).factor()
    x = s.solve([np.asarray(c1.b).reshape(-1, 1)], refine=3).cpu().numpy()
    x_ref, rel_ref = R.solve(c1.coords, 3.0, c1.reg, np.asarray(c1.b))
    A = R.rbf(c1.coords, 3.0, c1.reg)
    rel = np.linalg.norm(c1.b - A @ x) / np.linalg.norm(c1.b)
    assert rel <= 10 * rel_ref, (rel, rel_ref)


def test_c2_family_reaches_the_fp64_floor_with_four_rhs():
    """C2 family at N=5000 (3-D, eps=5, nugget 1e-6, 4 RHS, kappa ~ 1.8e8): no FP32
    Krylov body converges here; the batched Cholesky reaches the FP64 floor."""
    from mpdok_gb300 import configs
    from mpdok_gb300.batch import BatchedRBFSolver, unpack_rhs
    c2 = configs.c2(n=5000)
    B = np.asarray(c2.b)
    s = BatchedRBFSolver([c2.n], dim=3, nrhs=4, grid_mult=2)
    s.load([c2.coords], [5.0], c2.reg).factor()
    X = unpack_rhs(s.solve([B], refine=3), [c2.n], 4)[0].cpu().numpy()
    x_ref, rel_ref = R.solve(c2.coords, 5.0, c2.reg, B)
    A = R.rbf(c2.coords, 5.0, c2.reg)
    rel = np.max(np.linalg.norm(B - A @ X, axis=0) / np.linalg.norm(B, axis=0))
    assert rel <= 10 * rel_ref, (rel, rel_ref)
    assert np.linalg.norm(X - x_ref) / np.linalg.norm(x_ref) < 1e-3


@pytest.mark.parametrize("arith", ["df32", "f64"])
def test_task_graph_step_is_bit_identical_to_level_schedule(arith):
    """The persistent task-graph step (one launch: assembly, Cholesky, solve and
    two FP64 refinements of every system) runs each tile task with the
    arithmetic and the update order of the level-scheduled launches, so X is
    bit-identical; and it reaches the FP64 Cholesky oracle's floor."""
    from mpdok_gb300.batch import BatchedRBFSolver, unpack_rhs
    sizes = [700, 129, 64, 300, 5, 1000, 77]
    Xs, eps, Bs = _batch(sizes, 2, 3, seed=21)
    s = BatchedRBFSolver(sizes, dim=2, nrhs=3, arith=arith, grid_mult=2)
    s.load(Xs, eps, 1e-8)
    X_lev = s.step(Bs, refine=2).clone()
    for ctas in (1, 3):
        s.configure(f"dag:{ctas}")
        X_dag = s.step(Bs, refine=2)
        torch.cuda.synchronize()
        s.dag_status()
        assert torch.equal(X_dag, X_lev), ctas
    for i, (Xc, B, xg) in enumerate(zip(Xs, Bs, unpack_rhs(X_dag, sizes, 3))):
        _, rel_ref = R.solve(Xc, eps[i], 1e-8, B)
        A = R.rbf(Xc, eps[i], 1e-8)
        rel = np.max(np.linalg.norm(B - A @ xg.cpu().numpy(), axis=0) / np.linalg.norm(B, axis=0))
        assert rel <= 10 * rel_ref + 1e-14, (i, rel, rel_ref)


def test_task_graph_is_one_kernel_in_the_captured_graph():
    from mpdok_gb300.batch import BatchedRBFSolver
    sizes = [300, 129, 64, 700, 5]
    Xs, eps, Bs = _batch(sizes, 2, 4, seed=9)
    s = BatchedRBFSolver(sizes, dim=2, nrhs=4, grid_mult=1)
    s.load(Xs, eps, 1e-6)
    X_ref = s.step(Bs, refine=2).clone()
    s.configure("dag:3")
    Bbuf, Xbuf = s.build_graph(Bs, refine=2)
    assert s.graph_nodes <= 4  # the state resets (memsets) and ONE kernel node
    for _ in range(2):
        Xbuf.zero_()
        s.run_graph()
        torch.cuda.synchronize()
        s.dag_status()
        assert torch.equal(Xbuf, X_ref)
