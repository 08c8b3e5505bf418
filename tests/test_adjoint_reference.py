"""CPU: the FP64 reference gradient of the QR plan against finite differences.

oracle/adjoint.py states the implicit gradient of the problem the reference's
QR iteration solves (its fixed point, core/drot_qr.hpp:159-234).  Here it is
pinned by central finite differences of FP64 oracle solves (tight stop,
1e-13): directional derivatives in C, in the marginals (directions that keep
the masses equal), and through squared-Euclidean costs of point clouds in
R^16 with h = 1e-3.  The GPU adjoint is then checked against this reference.
"""
import numpy as np
import pytest

from oracle import adjoint as A

RHO = 2.0


def _problem(nr, nc, seed):
    rng = np.random.default_rng(seed)
    xs = rng.normal(size=(nr, 16))
    yt = rng.normal(size=(nc, 16))
    c = A.sqeuclidean(xs, yt)
    scale = c.max()
    p = rng.dirichlet(np.ones(nr))
    q = rng.dirichlet(np.ones(nc))
    return xs / np.sqrt(scale), yt / np.sqrt(scale), c / scale, p, q, rng


@pytest.mark.parametrize("nr,nc,rw,w", [(12, 15, 1e-2, 0.3), (20, 9, 1e-3, 0.0), (7, 7, 5e-2, 1.0)])
def test_gradient_in_cost_matches_finite_differences(nr, nc, rw, w):
    xs, yt, c, p, q, rng = _problem(nr, nc, nr * 100 + nc)
    L, gc, a, b, o = A.loss_and_grads(c, p, q, RHO, rw, w)
    assert o["residual"] < 1e-12
    for _ in range(3):
        E = rng.normal(size=c.shape)
        h = 1e-6
        fd = (A.loss_and_grads(c + h * E, p, q, RHO, rw, w)[0] -
              A.loss_and_grads(c - h * E, p, q, RHO, rw, w)[0]) / (2 * h)
        assert abs(fd - (gc * E).sum()) <= 1e-6 * max(1.0, abs(fd)), (fd, (gc * E).sum())


@pytest.mark.parametrize("nr,nc,rw", [(12, 15, 1e-2), (20, 9, 1e-3)])
def test_gradient_in_marginals_matches_finite_differences(nr, nc, rw):
    xs, yt, c, p, q, rng = _problem(nr, nc, 7 + nr)
    L, gc, a, b, o = A.loss_and_grads(c, p, q, RHO, rw, 0.5)
    assert abs(a.sum() - b.sum()) < 1e-10
    dp = rng.normal(size=nr)
    dp -= dp.mean()
    dq = rng.normal(size=nc)
    dq -= dq.mean()
    h = 1e-6
    fd = (A.loss_and_grads(c, p + h * dp, q + h * dq, RHO, rw, 0.5)[0] -
          A.loss_and_grads(c, p - h * dp, q - h * dq, RHO, rw, 0.5)[0]) / (2 * h)
    assert abs(fd - (a @ dp + b @ dq)) <= 1e-6 * max(1.0, abs(fd))


def test_gradient_through_point_clouds_h_1e_3():
    xs, yt, c, p, q, rng = _problem(12, 15, 3)
    w = 0.3

    def loss(x_, y_):
        return A.loss_and_grads(A.sqeuclidean(x_, y_), p, q, RHO, 1e-2, w)

    L, gc, *_ = loss(xs, yt)
    gx, gy = A.point_grads(xs, yt, gc)
    h = 1e-3
    for (i, d) in [(0, 0), (3, 5), (7, 15), (11, 2)]:
        e = np.zeros_like(xs)
        e[i, d] = h
        fd = (loss(xs + e, yt)[0] - loss(xs - e, yt)[0]) / (2 * h)
        assert abs(fd - gx[i, d]) <= 1e-5 * max(1.0, abs(fd)), (i, d, fd, gx[i, d])
    for (j, d) in [(0, 1), (14, 9)]:
        e = np.zeros_like(yt)
        e[j, d] = h
        fd = (loss(xs, yt + e)[0] - loss(xs, yt - e)[0]) / (2 * h)
        assert abs(fd - gy[j, d]) <= 1e-5 * max(1.0, abs(fd)), (j, d, fd, gy[j, d])


def test_support_from_duals_not_from_positive_entries():
    # A finite solve leaves tiny positive entries off the support; the dual
    # test S = {phi1 + phi2 - sC > 0} excludes them.
    xs, yt, c, p, q, rng = _problem(12, 15, 0)
    o = A.solve64(c, p, q, RHO, 1e-2)
    S = A.support(o, c, A.O.step_size(RHO, 12, 15))
    X = o["x"]
    assert (X[S] > 1e-9).all()
    assert (X[~S] < 1e-12).all()


def test_sparse_adjoint_matches_dense_least_squares():
    """The sparse FP64 CG form of the adjoint (used at sizes where the dense
    least-squares system does not fit) gives the dense solution."""
    rng = np.random.default_rng(12)
    xs, yt = rng.normal(size=(90, 4)), rng.normal(size=(70, 4))
    c = A.sqeuclidean(xs, yt)
    c /= c.max()
    p, q = rng.dirichlet(np.ones(90)), rng.dirichlet(np.ones(70))
    o = A.solve64(c, p, q, 2.0, 1e-2)
    _, gd, ad, bd = A.grads_at_state(o, c, 2.0, 1e-2, 0.3, sparse=False)
    _, gs, as_, bs = A.grads_at_state(o, c, 2.0, 1e-2, 0.3, sparse=True)
    assert np.abs(gs - gd).max() <= 1e-10 * np.abs(gd).max()
    assert np.abs(as_ - ad).max() <= 1e-10 * np.abs(ad).max()
    assert np.abs(bs - bd).max() <= 1e-10 * np.abs(bd).max()
