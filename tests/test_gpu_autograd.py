"""GPU: gradients of the QR plan (reg_drot.autograd) against the FP64 reference.

The reference operators have no backward (pytorch/src/drot_cuda.cpp:26-44);
the gradient checked here is that of the problem their QR iteration solves,
stated in FP64 by oracle/adjoint.py and pinned there against central finite
differences (tests/test_adjoint_reference.py).  The GPU path: the CUDA solve
(forward), then drot_qr_adjoint_prepare (support bitmasks from the final
duals) and drot_qr_adjoint_solve (masked Jacobi-PCG, one persistent launch).

Loss: L = <C, X*> + w ||X*||_F^2.  Tolerances: the forward runs in FP32 to
a marginal residual of 1e-7 and CG to 1e-7 relative residual (at 1e-6 a
weakly regularised case is off by 7e-4); measured
dL/dC errors against the FP64 reference are 5e-6..6e-5 relative
(Frobenius), and the bar is 1e-4 for dL/dC (and for the point-cloud chain
rule and the batch-vs-single comparison), 5e-3 for dL/dp, dL/dq.
The forward tolerance matters for dL/dp, dL/dq: at 1e-6 a weakly
regularised case (200 x 150, r_weight 1e-3) leaves one support entry of 359
undecided, which moves dL/dp by a few percent while dL/dC stays within
1e-4 (measured with the FP32 oracle on the CPU).

dL/dp, dL/dq are unique up to one constant per connected component of the
support graph.  An entry whose FP64 margin phi1_i + phi2_j - s C_ij is
within 1e-5 of s max C is not decided by an FP32 forward at 1e-7 (the
1000 x 64 case has one at 4e-6 that bridges two components).  Flipping one
such bridge leaves the adjoint solution the same up to the constants of the
two components it joins (the bridge only adds the relation a_i + b_j =
G_ij), so dL/dC is unchanged and dL/dp, dL/dq are compared in the gauge of
the components of the support without the undecided entries.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from oracle import adjoint as A  # noqa: E402

RHO = 2.0
TOL_C = 1e-4
TOL_PQ = 5e-3
EPS_FWD = 1e-7


def _points(nr, nc, seed, dim=16):
    rng = np.random.default_rng(seed)
    xs = rng.normal(size=(nr, dim))
    yt = rng.normal(size=(nc, dim))
    scale = np.sqrt(A.sqeuclidean(xs, yt).max())
    xs, yt = xs / scale, yt / scale
    p = rng.dirichlet(np.ones(nr))
    q = rng.dirichlet(np.ones(nc))
    return xs, yt, p, q


def _component_gauge(S, a, b):
    """a, b shifted per connected component of the bipartite support graph so
    that each component has sum(a) = sum(b): dL/dp, dL/dq are unique only up
    to one constant per component (a + t, b - t), so both sides are compared
    in this gauge."""
    from scipy.sparse import coo_matrix
    from scipy.sparse.csgraph import connected_components
    nc, nr = S.shape
    j, i = np.nonzero(S)
    g = coo_matrix((np.ones(len(i)), (i, nr + j)), shape=(nr + nc, nr + nc))
    _, lab = connected_components(g, directed=False)
    a = np.asarray(a, np.float64).copy()
    b = np.asarray(b, np.float64).copy()
    for comp in np.unique(lab):
        ra = lab[:nr] == comp
        cb = lab[nr:] == comp
        t = (b[cb].sum() - a[ra].sum()) / (ra.sum() + cb.sum())
        a[ra] += t
        b[cb] -= t
    return a, b


def _decided_support(o, c, s, rel=1e-5):
    """The FP64 support minus the entries an FP32 forward cannot decide
    (|margin| below rel * s * max C)."""
    c = np.asarray(c, np.float64)
    m = o["phi1"][None, :] + o["phi2"][:, None] - s * c
    return (m > 0) & (np.abs(m) >= rel * s * np.abs(c).max())


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("nr,nc,rw,w", [(30, 40, 1e-2, 0.3), (200, 150, 1e-3, 0.0),
                                        (513, 300, 1e-2, 1.0), (1000, 64, 1e-2, 0.5)])
def test_qr_gradient_matches_fp64_reference(cuda, solver_lib, nr, nc, rw, w):
    from reg_drot.autograd import quadratic_drot_fn
    xs, yt, p, q = _points(nr, nc, nr + 3 * nc)
    c64 = A.sqeuclidean(xs, yt)
    c = torch.tensor(c64, dtype=torch.float32, device=cuda, requires_grad=True)
    pt = torch.tensor(p, dtype=torch.float32, device=cuda, requires_grad=True)
    qt = torch.tensor(q, dtype=torch.float32, device=cuda, requires_grad=True)
    x = quadratic_drot_fn(c, pt, qt, RHO, rw, 200000, EPS_FWD)
    loss = (c * x).sum() + w * (x * x).sum()
    loss.backward()
    # the reference on the same (FP32-rounded) inputs
    L, gc, ga, gb, o = A.loss_and_grads(c.detach().double().cpu().numpy(),
                                        pt.detach().double().cpu().numpy(),
                                        qt.detach().double().cpu().numpy(), RHO, rw, w)
    assert abs(loss.item() - L) <= 1e-4 * abs(L)
    assert _rel(c.grad.cpu().numpy(), gc) <= TOL_C, _rel(c.grad.cpu().numpy(), gc)
    assert abs(float(pt.grad.sum() - qt.grad.sum())) <= 1e-5 * float(pt.grad.abs().sum())
    S = _decided_support(o, c.detach().double().cpu().numpy(), A.O.step_size(RHO, nr, nc))
    ga_g, gb_g = _component_gauge(S, pt.grad.cpu().numpy(), qt.grad.cpu().numpy())
    ga_r, gb_r = _component_gauge(S, ga, gb)
    assert _rel(ga_g, ga_r) <= TOL_PQ, _rel(ga_g, ga_r)
    assert _rel(gb_g, gb_r) <= TOL_PQ, _rel(gb_g, gb_r)


def test_qr_gradient_through_point_clouds(cuda, solver_lib):
    from reg_drot.autograd import quadratic_drot_fn
    nr, nc, rw, w = 300, 257, 1e-2, 0.3
    xs, yt, p, q = _points(nr, nc, 11)
    xt = torch.tensor(xs, dtype=torch.float32, device=cuda, requires_grad=True)
    yq = torch.tensor(yt, dtype=torch.float32, device=cuda, requires_grad=True)
    pt = torch.tensor(p, dtype=torch.float32, device=cuda)
    qt = torch.tensor(q, dtype=torch.float32, device=cuda)
    c = ((yq[:, None, :] - xt[None, :, :]) ** 2).sum(-1)
    x = quadratic_drot_fn(c, pt, qt, RHO, rw, 200000, EPS_FWD)
    loss = (c * x).sum() + w * (x * x).sum()
    loss.backward()
    x64 = xt.detach().double().cpu().numpy()
    y64 = yq.detach().double().cpu().numpy()
    L, gc, *_ = A.loss_and_grads(A.sqeuclidean(x64, y64), p.astype(np.float32).astype(np.float64),
                                 q.astype(np.float32).astype(np.float64), RHO, rw, w)
    gx, gy = A.point_grads(x64, y64, gc)
    assert _rel(xt.grad.cpu().numpy(), gx) <= TOL_C
    assert _rel(yq.grad.cpu().numpy(), gy) <= TOL_C


def test_support_mask_matches_fp64_duals(cuda, solver_lib):
    from reg_drot.autograd import _Adjoint, quadratic_drot_fn, QuadraticDROTFn  # noqa: F401
    import reg_drot.autograd as AG
    nr, nc = 400, 300
    xs, yt, p, q = _points(nr, nc, 5)
    c = torch.tensor(A.sqeuclidean(xs, yt), dtype=torch.float32, device=cuda)
    pt = torch.tensor(p, dtype=torch.float32, device=cuda)
    qt = torch.tensor(q, dtype=torch.float32, device=cuda)
    seen = {}
    orig = AG._Adjoint.__init__

    def spy(self, *a, **k):
        orig(self, *a, **k)
        seen["mask"] = self.mask.cpu().numpy()
    AG._Adjoint.__init__ = spy
    try:
        cr = c.clone().requires_grad_(True)
        x = quadratic_drot_fn(cr, pt, qt, RHO, 1e-2, 200000, EPS_FWD)
        x.sum().backward()
    finally:
        AG._Adjoint.__init__ = orig
    o = A.solve64(c.double().cpu().numpy(), pt.double().cpu().numpy(), qt.double().cpu().numpy(),
                  RHO, 1e-2)
    S = A.support(o, c.double().cpu().numpy(), A.O.step_size(RHO, nr, nc))
    mism = (seen["mask"] != S).sum()
    assert mism <= 1e-3 * S.sum(), (mism, S.sum())
    # the dual support is far smaller than the positive entries of X
    assert S.sum() < (x.detach().cpu().numpy() > 0).sum()


def test_batch_gradients_match_single_instance(cuda, solver_lib):
    from reg_drot.autograd import batch_quadratic_drot_fn, quadratic_drot_fn
    from reg_drot.batch import QRBatch
    shapes = [(64, 96), (300, 257), (513, 200), (128, 1100)]
    rw, w = 1e-2, 0.3
    insts = [_points(nr, nc, 40 + k) for k, (nr, nc) in enumerate(shapes)]
    costs = [torch.tensor(A.sqeuclidean(xs, yt), dtype=torch.float32, device=cuda)
             for xs, yt, _, _ in insts]
    ps = [torch.tensor(p, dtype=torch.float32) for _, _, p, _ in insts]
    qs = [torch.tensor(q, dtype=torch.float32) for _, _, _, q in insts]
    B = QRBatch(shapes, RHO, rw, EPS_FWD, device=cuda, cols_per_tile=64)
    leaves = [c.clone().requires_grad_(True) for c in costs]
    cp = B.pack_c(leaves)
    p, q = B.pack_marginals(ps, qs)
    x = batch_quadratic_drot_fn(B, cp, p, q, 200000)
    loss = sum((B.view(cp, k) * xk).sum() + w * (xk * xk).sum() for k, xk in enumerate(B.unpack(x)))
    loss.backward()
    for k in range(len(shapes)):
        c1 = costs[k].clone().requires_grad_(True)
        x1 = quadratic_drot_fn(c1, ps[k].to(cuda), qs[k].to(cuda), RHO, rw, 200000, EPS_FWD)
        ((c1 * x1).sum() + w * (x1 * x1).sum()).backward()
        # two FP32 results, each within TOL_C of the FP64 reference
        assert _rel(leaves[k].grad.cpu().numpy(), c1.grad.cpu().numpy()) <= 2 * TOL_C
        L, gc, *_ = A.loss_and_grads(costs[k].double().cpu().numpy(), ps[k].double().numpy(),
                                     qs[k].double().numpy(), RHO, rw, w)
        assert _rel(leaves[k].grad.cpu().numpy(), gc) <= TOL_C, k


def test_zero_upstream_gives_zero_gradient(cuda, solver_lib):
    from reg_drot.autograd import quadratic_drot_fn
    xs, yt, p, q = _points(50, 60, 2)
    c = torch.tensor(A.sqeuclidean(xs, yt), dtype=torch.float32, device=cuda, requires_grad=True)
    x = quadratic_drot_fn(c, torch.tensor(p, dtype=torch.float32, device=cuda),
                          torch.tensor(q, dtype=torch.float32, device=cuda), RHO, 1e-2, 100000, EPS_FWD)
    (x * 0.0).sum().backward()
    assert float(c.grad.abs().max()) == 0.0
