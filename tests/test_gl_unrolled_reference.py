"""CPU: the FP64 unrolled GL reference (oracle/adjoint.gl_unrolled).

Its forward is pinned to the oracle's FP64 GL loop (itself pinned to the
reference's numpy implementation by the golden tests), so its autograd
gradient is the exact gradient of the iterations the GPU backward reverses;
a central finite difference in C confirms it.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import adjoint as A  # noqa: E402
from oracle import oracle as O  # noqa: E402


def _problem(nr, nc, seed):
    rng = np.random.default_rng(seed)
    xs = rng.normal(size=(nr, 2)) + np.where(np.arange(nr)[:, None] < nr // 2, -2.0, 2.0) * [1, 0]
    yt = rng.normal(size=(nc, 2))
    c = A.sqeuclidean(xs, yt)
    return c / c.max(), np.full(nr, 1.0 / nr), np.full(nc, 1.0 / nc)


@pytest.mark.parametrize("nr,nc,G,rw,T", [(40, 30, 2, 1e-3, 25), (33, 17, 3, 5e-3, 40)])
def test_unrolled_forward_matches_oracle(nr, nc, G, rw, T):
    c, p, q = _problem(nr, nc, nr)
    X = A.gl_unrolled(torch.tensor(c), torch.tensor(p), torch.tensor(q), G, 2.0, rw, T)
    o = O.group_lasso_drot(c, p, q, G, 2.0, rw, T, 0.0, dtype=np.float64)
    assert o["n_iter"] == T
    assert np.abs(X.numpy() - o["x"]).max() <= 1e-12 * max(1.0, np.abs(o["x"]).max())


def test_unrolled_gradient_matches_finite_differences():
    nr, nc, G, rw, T = 40, 30, 2, 1e-3, 25
    c, p, q = _problem(nr, nc, 5)
    rng = np.random.default_rng(1)
    W = torch.tensor(rng.normal(size=(nc, nr)))
    ct = torch.tensor(c, requires_grad=True)
    loss = (A.gl_unrolled(ct, torch.tensor(p), torch.tensor(q), G, 2.0, rw, T) * W).sum()
    loss.backward()
    E = rng.normal(size=c.shape)
    h = 1e-7

    def L(cc):
        with torch.no_grad():
            return float((A.gl_unrolled(torch.tensor(cc), torch.tensor(p), torch.tensor(q), G, 2.0,
                                        rw, T) * W).sum())
    fd = (L(c + h * E) - L(c - h * E)) / (2 * h)
    an = float((ct.grad.numpy() * E).sum())
    assert abs(fd - an) <= 1e-5 * max(1.0, abs(fd)), (fd, an)


def test_truncated_unrolled_gradient_is_the_last_steps_gradient():
    """gl_unrolled(last_k=K): the gradient of the last K steps from the state
    they start at -- equal to differentiating a K-step run started at that
    (detached) state; the forward value does not change."""
    nr, nc, G, rw, T, K = 40, 30, 2, 1e-3, 25, 9
    c, p, q = _problem(nr, nc, 6)
    rng = np.random.default_rng(2)
    W = torch.tensor(rng.normal(size=(nc, nr)))
    ct = torch.tensor(c, requires_grad=True)
    X = A.gl_unrolled(ct, torch.tensor(p), torch.tensor(q), G, 2.0, rw, T, last_k=K)
    Xf = A.gl_unrolled(torch.tensor(c), torch.tensor(p), torch.tensor(q), G, 2.0, rw, T)
    assert torch.equal(X.detach(), Xf)
    (X * W).sum().backward()
    # finite difference in C of the last K steps only: perturb C in those
    # steps, keep the state at T - K from the unperturbed run
    E = rng.normal(size=c.shape)
    h = 1e-7

    def L(eps_):
        with torch.no_grad():
            out = A.gl_unrolled(torch.tensor(c), torch.tensor(p), torch.tensor(q), G, 2.0, rw, T,
                                last_k=K, c_last=torch.tensor(c + eps_ * E))
        return float((out * W).sum())
    fd = (L(h) - L(-h)) / (2 * h)
    an = float((ct.grad.numpy() * E).sum())
    assert abs(fd - an) <= 1e-5 * max(1.0, abs(fd)), (fd, an)
