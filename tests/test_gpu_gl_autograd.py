"""GPU: the unrolled GL adjoint (reg_drot.autograd.group_lasso_drot_fn).

Reference: the FP64 unrolled map of oracle/adjoint.gl_unrolled (pinned to the
oracle's GL loop and to finite differences on the CPU) differentiated by
torch autograd, for the same number of iterations the GPU solve ran.  The
GPU backward recomputes each segment's states from checkpoints (segment
lengths below force several segments, one of them partial) and applies
drot_gl_adjoint_step once per iteration.  Tolerance 1e-4 relative
(Frobenius; measured 2e-7..7e-5): FP32 forward and FP32 adjoint recursion
over the iterations.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from oracle import adjoint as A  # noqa: E402

TOL = 1e-4


def _problem(nr, nc, seed):
    rng = np.random.default_rng(seed)
    xs = rng.normal(size=(nr, 2)) + np.where(np.arange(nr)[:, None] < nr // 2, -2.0, 2.0) * [1, 0]
    yt = rng.normal(size=(nc, 2)) @ (np.eye(2) + 0.3 * rng.normal(size=(2, 2))) + rng.normal(size=2)
    c = A.sqeuclidean(xs, yt)
    c = (c / c.max()).astype(np.float32)
    p = np.full(nr, 1.0 / nr, np.float32)
    q = np.full(nc, 1.0 / nc, np.float32)
    W = rng.normal(size=(nc, nr)).astype(np.float32)
    return c, p, q, W


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _reference(c, p, q, W, G, rw, T, convention="torch", last_k=None):
    ct = torch.tensor(c, dtype=torch.float64, requires_grad=True)
    pt = torch.tensor(p, dtype=torch.float64, requires_grad=True)
    qt = torch.tensor(q, dtype=torch.float64, requires_grad=True)
    X = A.gl_unrolled(ct, pt, qt, G, 2.0, rw, T, convention=convention, last_k=last_k)
    (X * torch.tensor(W, dtype=torch.float64)).sum().backward()
    return X.detach().numpy(), ct.grad.numpy(), pt.grad.numpy(), qt.grad.numpy()


@pytest.mark.parametrize("nr,nc,G,rw,T,seg", [(60, 40, 2, 1e-3, 25, 8), (90, 70, 3, 5e-3, 40, 16),
                                               (300, 200, 2, 1e-3, 30, 32)])
def test_gl_gradient_fixed_iterations(cuda, solver_lib, nr, nc, G, rw, T, seg):
    from reg_drot.autograd import group_lasso_drot_fn
    c, p, q, W = _problem(nr, nc, nr + G)
    ct = torch.tensor(c, device=cuda, requires_grad=True)
    pt = torch.tensor(p, device=cuda, requires_grad=True)
    qt = torch.tensor(q, device=cuda, requires_grad=True)
    x = group_lasso_drot_fn(ct, pt, qt, G, 2.0, rw, T, 0.0, segment=seg)
    (x * torch.tensor(W, device=cuda)).sum().backward()
    X64, gc, gp, gq = _reference(c, p, q, W, G, rw, T)
    assert _rel(x.detach().cpu().numpy(), X64) <= 1e-4
    assert _rel(ct.grad.cpu().numpy(), gc) <= TOL, _rel(ct.grad.cpu().numpy(), gc)
    assert _rel(pt.grad.cpu().numpy(), gp) <= TOL, _rel(pt.grad.cpu().numpy(), gp)
    assert _rel(qt.grad.cpu().numpy(), gq) <= TOL, _rel(qt.grad.cpu().numpy(), gq)


def test_gl_gradient_of_a_converged_solve(cuda, solver_lib):
    from reg_drot.autograd import GroupLassoDROTFn, group_lasso_drot_fn  # noqa: F401
    nr, nc, G, rw = 80, 60, 2, 1e-3
    c, p, q, W = _problem(nr, nc, 7)
    ct = torch.tensor(c, device=cuda, requires_grad=True)
    x = group_lasso_drot_fn(ct, torch.tensor(p, device=cuda), torch.tensor(q, device=cuda), G, 2.0,
                            rw, 20000, 1e-4, segment=16)
    T = x.grad_fn.info["n_iter"]  # iterations over all segments
    assert x.grad_fn.info["converged"] == 1 and T > 16
    (x * torch.tensor(W, device=cuda)).sum().backward()
    X64, gc, _, _ = _reference(c, p, q, W, G, rw, T)
    assert _rel(ct.grad.cpu().numpy(), gc) <= TOL


def test_gl_forward_equals_operator(cuda, solver_lib):
    import reg_drot
    from reg_drot.autograd import group_lasso_drot_fn
    c, p, q, W = _problem(150, 100, 3)
    args = (torch.tensor(c, device=cuda), torch.tensor(p, device=cuda), torch.tensor(q, device=cuda))
    x1 = reg_drot.group_lasso_drot(*args, 2, 2.0, 1e-3, 20000, 1e-4)
    x2 = group_lasso_drot_fn(*args, 2, 2.0, 1e-3, 20000, 1e-4, segment=7)
    assert torch.equal(x1, x2)


@pytest.mark.parametrize("last_k,seg,conv", [(20, 8, "operator"), (33, 16, "wrapper"),
                                             (64, 32, "wrapper")])
def test_gl_truncated_adjoint_matches_fp64(cuda, solver_lib, last_k, seg, conv):
    """The truncated adjoint (last_k iterations unrolled, the state before
    them held fixed) against the FP64 unrolled map truncated the same way;
    both lambda conventions (operator r * sqrt(n/G), C++ wrapper r / sqrt(n/G))."""
    from reg_drot.autograd import group_lasso_drot_fn
    nr, nc, G, rw, T = 300, 200, 2, 1e-3, 90
    c, p, q, W = _problem(nr, nc, 17)
    ct = torch.tensor(c, device=cuda, requires_grad=True)
    pt = torch.tensor(p, device=cuda, requires_grad=True)
    qt = torch.tensor(q, device=cuda, requires_grad=True)
    x = group_lasso_drot_fn(ct, pt, qt, G, 2.0, rw, T, 0.0, segment=seg, convention=conv,
                            last_k=last_k)
    (x * torch.tensor(W, device=cuda)).sum().backward()
    X64, gc, gp, gq = _reference(c, p, q, W, G, rw, T, "torch" if conv == "operator" else conv,
                                 last_k)
    assert _rel(x.detach().cpu().numpy(), X64) <= 1e-4
    assert _rel(ct.grad.cpu().numpy(), gc) <= TOL, _rel(ct.grad.cpu().numpy(), gc)
    assert _rel(pt.grad.cpu().numpy(), gp) <= TOL, _rel(pt.grad.cpu().numpy(), gp)
    assert _rel(qt.grad.cpu().numpy(), gq) <= TOL, _rel(qt.grad.cpu().numpy(), gq)
