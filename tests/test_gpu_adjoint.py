"""GPU parity: gradients of one in-core RBF solve (rbf_solve, the differentiated
three-precision GMRES-IR) against FP64 torch.linalg.solve autograd and
central finite differences.

The backward pass solves A^T lam = dL/dx with the forward LU factors (A is
symmetric) and contracts lam^T (dA/dtheta) x in one fused FP64 kernel that
recomputes phi from the coordinates.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _torch_reference(X, eps, reg, b, w, kernel):
    c = torch.tensor(X, dtype=torch.float64, requires_grad=True)
    e = torch.tensor(eps, dtype=torch.float64, requires_grad=True)
    r = torch.tensor(reg, dtype=torch.float64, requires_grad=True)
    bb = torch.tensor(b, dtype=torch.float64, requires_grad=True)
    d2 = ((c[:, None, :] - c[None, :, :]) ** 2).sum(-1)
    A = torch.exp(-(e * e) * d2) if kernel == "gaussian" else torch.sqrt(1.0 + (e * e) * d2)
    A = A + r * torch.eye(len(X), dtype=torch.float64)
    x = torch.linalg.solve(A, bb)
    L = (torch.tensor(w) * x).sum() + 0.5 * (x * x).sum()
    L.backward()
    return x.detach().numpy(), c.grad.numpy(), float(e.grad), float(r.grad), bb.grad.numpy()


@pytest.mark.parametrize("factor_dtype", ["fp16", "fp32"])
def test_rbf_solve_gradients_match_fp64_autograd(factor_dtype):
    from mpdok_gb300.adjoint import rbf_solve
    rng = np.random.default_rng(5)
    n = 400
    X = rng.uniform(0, 1, (n, 2))
    eps, reg = 20.0, 1e-3
    b = rng.standard_normal(n)
    w = rng.standard_normal(n)
    coords = torch.tensor(X, device="cuda", requires_grad=True)
    e = torch.tensor(eps, dtype=torch.float64, requires_grad=True)
    r = torch.tensor(reg, dtype=torch.float64, requires_grad=True)
    bt = torch.tensor(b, device="cuda", requires_grad=True)
    opts = {}
    x = rbf_solve(coords, e, r, bt, factor_dtype=factor_dtype, tol=1e-13, opts=opts)
    L = (torch.tensor(w, device="cuda") * x).sum() + 0.5 * (x * x).sum()
    L.backward()
    assert opts["last_info"]["converged"] and opts["last_adjoint_info"]["converged"]
    x_ref, gc_ref, ge_ref, gr_ref, gb_ref = _torch_reference(X, eps, reg, b, w, "gaussian")
    np.testing.assert_allclose(x.detach().cpu().numpy(), x_ref, rtol=0, atol=1e-9 * np.abs(x_ref).max())
    rel = lambda a, b: np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300)
    assert rel(bt.grad.cpu().numpy(), gb_ref) < 1e-8
    assert rel(coords.grad.cpu().numpy(), gc_ref) < 1e-8
    assert abs(float(e.grad) - ge_ref) <= 1e-8 * abs(ge_ref)
    assert abs(float(r.grad) - gr_ref) <= 1e-8 * abs(gr_ref)


def test_rbf_solve_eps_gradient_matches_central_differences():
    from mpdok_gb300.adjoint import rbf_solve
    rng = np.random.default_rng(8)
    n = 300
    X = rng.uniform(0, 1, (n, 2))
    b = rng.standard_normal(n)
    coords = torch.tensor(X, device="cuda")
    bt = torch.tensor(b, device="cuda")

    def loss(eps, reg):
        x = rbf_solve(coords, eps, reg, bt, factor_dtype="fp32", tol=1e-14)
        return float(0.5 * (x * x).sum())

    e = torch.tensor(15.0, dtype=torch.float64, requires_grad=True)
    r = torch.tensor(1e-2, dtype=torch.float64, requires_grad=True)
    x = rbf_solve(coords, e, r, bt, factor_dtype="fp32", tol=1e-14)
    (0.5 * (x * x).sum()).backward()
    h = 1e-5
    fd_e = (loss(15.0 + h, 1e-2) - loss(15.0 - h, 1e-2)) / (2 * h)
    fd_r = (loss(15.0, 1e-2 + 1e-7) - loss(15.0, 1e-2 - 1e-7)) / 2e-7
    assert float(e.grad) == pytest.approx(fd_e, rel=1e-5)
    assert float(r.grad) == pytest.approx(fd_r, rel=1e-5)
