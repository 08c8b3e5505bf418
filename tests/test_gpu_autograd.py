"""GPU: gradients of the QR plan (reg_drot.autograd) against the FP64 reference.

The reference operators have no backward (pytorch/src/drot_cuda.cpp:26-44);
the gradient checked here is that of the problem their QR iteration solves,
stated in FP64 by oracle/adjoint.py and pinned there against central finite
differences (tests/test_adjoint_reference.py).  The GPU path: the CUDA solve
(forward), then drot_qr_adjoint_prepare (support bitmasks from the final
duals), drot_qr_adjoint_solve (right-hand side from the upstream gradient,
masked Jacobi-PCG in FP64, one persistent launch) and drot_qr_adjoint_grad
(dL/dC, dL/dp, dL/dq).

Loss: L = <C, X*> + w ||X*||_F^2.  Tolerances: the forward runs in FP32 to
a marginal residual of 1e-7 and CG to 1e-10 relative residual; measured
dL/dC errors against the FP64 reference are 5e-6..6e-5 relative
(Frobenius), and the bar is 1e-4 for dL/dC (and for the point-cloud chain
rule and the batch-vs-single comparison) and for dL/dp, dL/dq (measured
7e-7..7e-6 in the component gauge below).
The forward tolerance matters for dL/dp, dL/dq: at 1e-6 a weakly
regularised case (200 x 150, r_weight 1e-3) leaves one support entry of 359
undecided, which moves dL/dp by a few percent while dL/dC stays within
1e-4 (measured with the FP32 oracle on the CPU).  Tests that stop the
forward earlier compare with the FP64 oracle run to the same stop.

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
TOL_PQ = 1e-4
EPS_FWD = 1e-7
MAX_ITERS = 1_000_000


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
    print(f"\n[grad] {nr}x{nc} rw {rw:g}: dL/dC {_rel(c.grad.cpu().numpy(), gc):.2e}, "
          f"dL/dp {_rel(ga_g, ga_r):.2e}, dL/dq {_rel(gb_g, gb_r):.2e}")
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
    from reg_drot.autograd import _Adjoint, quadratic_drot_fn
    nr, nc = 400, 300
    xs, yt, p, q = _points(nr, nc, 5)
    c = torch.tensor(A.sqeuclidean(xs, yt), dtype=torch.float32, device=cuda)
    pt = torch.tensor(p, dtype=torch.float32, device=cuda)
    qt = torch.tensor(q, dtype=torch.float32, device=cuda)
    cr = c.clone().requires_grad_(True)
    x = quadratic_drot_fn(cr, pt, qt, RHO, 1e-2, 200000, EPS_FWD)
    _, phi1, phi2 = x.grad_fn.saved_tensors
    s = A.O.step_size(RHO, nr, nc)
    adj = _Adjoint(c, phi1, phi2, [(nr, nc, nr, 0, 0, 0, 0, s, A.qr_lambda(RHO, 1e-2, nr, nc))],
                   byte_mask=True)
    mask = adj.mask.cpu().numpy()
    o = A.solve64(c.double().cpu().numpy(), pt.double().cpu().numpy(), qt.double().cpu().numpy(),
                  RHO, 1e-2)
    S = A.support(o, c.double().cpu().numpy(), s)
    mism = (mask != S).sum()
    assert mism <= 1e-3 * S.sum(), (mism, S.sum())
    # the dual support is far smaller than the positive entries of X
    assert S.sum() < (x.detach().cpu().numpy() > 0).sum()


def test_batch_gradients_match_single_instance(cuda, solver_lib):
    """The batched backward against the single-instance one and against the
    FP64 gradient of the same computation.  The forward stops at the absolute
    residual 1e-6 (1e-7 is below the FP32 floor of the (513, 200) instance:
    its duals near 0.56 move by less than their FP32 ulp, so no FP32 solve
    gets there -- the reference's FP32 loop has the same floor), and every
    solve must reach its stop.  The FP64 reference runs the oracle to the GPU
    solve's own stop iteration (oracle.quadratic_drot_at) and differentiates
    there."""
    from reg_drot.autograd import batch_quadratic_drot_fn, quadratic_drot_fn
    from reg_drot.batch import QRBatch
    shapes = [(64, 96), (300, 257), (513, 200), (128, 1100)]
    rw, w, eps = 1e-2, 0.3, 1e-6
    insts = [_points(nr, nc, 40 + k) for k, (nr, nc) in enumerate(shapes)]
    costs = [torch.tensor(A.sqeuclidean(xs, yt), dtype=torch.float32, device=cuda)
             for xs, yt, _, _ in insts]
    ps = [torch.tensor(p, dtype=torch.float32) for _, _, p, _ in insts]
    qs = [torch.tensor(q, dtype=torch.float32) for _, _, _, q in insts]
    B = QRBatch(shapes, RHO, rw, eps, device=cuda, cols_per_tile=64)
    leaves = [c.clone().requires_grad_(True) for c in costs]
    cp = B.pack_c(leaves)
    p, q = B.pack_marginals(ps, qs)
    x = batch_quadratic_drot_fn(B, cp, p, q, MAX_ITERS)
    # the implicit gradient is that of the optimal plan: every solve must
    # have reached its stop
    info = x.grad_fn.info
    assert all(r["converged"] == 1 for r in info), info
    loss = sum((B.view(cp, k) * xk).sum() + w * (xk * xk).sum() for k, xk in enumerate(B.unpack(x)))
    loss.backward()
    for k, (nr, nc) in enumerate(shapes):
        c1 = costs[k].clone().requires_grad_(True)
        x1 = quadratic_drot_fn(c1, ps[k].to(cuda), qs[k].to(cuda), RHO, rw, MAX_ITERS, eps)
        assert x1.grad_fn.info["converged"] == 1, (k, x1.grad_fn.info)
        ((c1 * x1).sum() + w * (x1 * x1).sum()).backward()
        ck = costs[k].double().cpu().numpy()
        refs = {}
        for name, n_iter in (("batch", info[k]["n_iter"]), ("single", x1.grad_fn.info["n_iter"])):
            if n_iter not in refs:
                o = A.O.quadratic_drot_at(ck, ps[k].double().numpy(), qs[k].double().numpy(),
                                          RHO, rw, n_iter, dtype=np.float64)
                refs[n_iter] = A.grads_at_state(o, ck, RHO, rw, w)[1]
        e_b = _rel(leaves[k].grad.cpu().numpy(), refs[info[k]["n_iter"]])
        e_s = _rel(c1.grad.cpu().numpy(), refs[x1.grad_fn.info["n_iter"]])
        print(f"\n[grad-batch] {nr}x{nc}: n_iter {info[k]['n_iter']} / "
              f"{x1.grad_fn.info['n_iter']}, dL/dC batch {e_b:.2e}, single {e_s:.2e}")
        assert e_b <= TOL_C and e_s <= TOL_C, (k, e_b, e_s)
        if info[k]["n_iter"] == x1.grad_fn.info["n_iter"]:
            assert _rel(leaves[k].grad.cpu().numpy(), c1.grad.cpu().numpy()) <= 2 * TOL_C


def test_zero_upstream_gives_zero_gradient(cuda, solver_lib):
    from reg_drot.autograd import quadratic_drot_fn
    xs, yt, p, q = _points(50, 60, 2)
    c = torch.tensor(A.sqeuclidean(xs, yt), dtype=torch.float32, device=cuda, requires_grad=True)
    x = quadratic_drot_fn(c, torch.tensor(p, dtype=torch.float32, device=cuda),
                          torch.tensor(q, dtype=torch.float32, device=cuda), RHO, 1e-2, 100000, EPS_FWD)
    (x * 0.0).sum().backward()
    assert float(c.grad.abs().max()) == 0.0


# The differentiable workload's operating point: shapes from its range (m, n
# in 512..4096), points in R^16 ~ N(0, 1), C = |x - y|^2 / 64 on the tensor
# cores, alpha 1e-3, forward stopped at the relative marginal residual 1e-4
# (the benchmark's stop), loss sum_k <C_k, X_k> + w |X_k|^2.
OP_SHAPES = [(2048, 3072), (3584, 1024), (512, 4096)]
OP_SCALE = 1.0 / 64


def test_batch_gradients_at_the_relative_1e4_stop(cuda, solver_lib):
    """Gradients at the benchmark's stop (relative marginal residual 1e-4)
    against the FP64 reference of the same computation: the FP64 oracle run
    to the GPU's stop iteration (oracle.quadratic_drot_at), its FP64 implicit
    adjoint at its own duals (sparse CG to 1e-13) and the FP64 chain rule to
    the points, on the cost the GPU built.  Bar: 1e-4 relative for dL/dC,
    dL/dx, dL/dy and for dL/dp, dL/dq (in the gauge of the support's
    components).  Measured on the CPU at 1024 x 1536 with the FP32 oracle in
    the GPU's place: dL/dC 5e-6, dL/dx, dL/dy 1e-5, dL/dp, dL/dq 3e-8.  The
    distance to the gradient at the exact optimum is not this test's subject:
    a plan stopped at relative 1e-4 is itself about 4e-4 from the optimum,
    and so is its gradient (3.8e-4 for dL/dC, 3.3e-4 for dL/dx at 1024 x 1536,
    FP64 run to 9e-10 absolute residual)."""
    from reg_drot.autograd import batch_quadratic_drot_fn
    from reg_drot.batch import QRBatch
    from reg_drot.cost import packed_sqeuclidean_cost
    rw, w = 1e-3, 0.3
    rng = np.random.default_rng(2024)
    xs = [rng.normal(size=(m, 16)).astype(np.float32) for m, _ in OP_SHAPES]
    ys = [rng.normal(size=(n, 16)).astype(np.float32) for _, n in OP_SHAPES]
    eps = [1e-4 * np.sqrt(1.0 / m + 1.0 / n) for m, n in OP_SHAPES]
    B = QRBatch(OP_SHAPES, RHO, rw, eps, device=cuda, cols_per_tile=256)
    xc = torch.tensor(np.concatenate(xs), device=cuda, requires_grad=True)
    yc = torch.tensor(np.concatenate(ys), device=cuda, requires_grad=True)
    pb, qb = B.pack_marginals([torch.full((m,), 1.0 / m) for m, _ in OP_SHAPES],
                              [torch.full((n,), 1.0 / n) for _, n in OP_SHAPES])
    pb.requires_grad_(True)
    qb.requires_grad_(True)
    cb = packed_sqeuclidean_cost(B, xc, yc, OP_SCALE)
    cb.retain_grad()
    X = batch_quadratic_drot_fn(B, cb, pb, qb, MAX_ITERS)
    info = X.grad_fn.info
    assert all(r["converged"] == 1 for r in info), info
    ((cb * X).sum() + w * (X * X).sum()).backward()
    cg_rel = X.grad_fn.cg_residuals
    assert all(r <= 1e-7 for r in cg_rel), cg_rel
    po = qo = 0
    for k, (m, n) in enumerate(OP_SHAPES):
        ck = B.view(cb, k).detach().cpu().numpy()
        p = np.full(m, 1.0 / m, np.float32)
        q = np.full(n, 1.0 / n, np.float32)
        o64 = A.O.quadratic_drot_at(ck, p, q, RHO, rw, info[k]["n_iter"], dtype=np.float64)
        _, gc, ga, gb = A.grads_at_state(o64, ck, RHO, rw, w)
        gx, gy = A.point_grads(xs[k].astype(np.float64), ys[k].astype(np.float64), gc * OP_SCALE)
        e_c = _rel(B.view(cb.grad, k).cpu().numpy(), gc)
        e_x = _rel(xc.grad[po:po + m].cpu().numpy(), gx)
        e_y = _rel(yc.grad[qo:qo + n].cpu().numpy(), gy)
        S = _decided_support(o64, ck, A.O.step_size(RHO, m, n))
        ga_g, gb_g = _component_gauge(S, pb.grad[po:po + m].cpu().numpy(),
                                      qb.grad[qo:qo + n].cpu().numpy())
        ga_r, gb_r = _component_gauge(S, ga, gb)
        e_p, e_q = _rel(ga_g, ga_r), _rel(gb_g, gb_r)
        print(f"\n[grad-op] {m}x{n}: n_iter {info[k]['n_iter']}, CG {X.grad_fn.cg_iters[k]} "
              f"iterations to {cg_rel[k]:.1e}; dL/dC {e_c:.2e}, dL/dx {e_x:.2e}, "
              f"dL/dy {e_y:.2e}, dL/dp {e_p:.2e}, dL/dq {e_q:.2e}")
        assert e_c <= 1e-4 and e_x <= 1e-4 and e_y <= 1e-4, (k, e_c, e_x, e_y)
        assert e_p <= 1e-4 and e_q <= 1e-4, (k, e_p, e_q)
        po += m
        qo += n


def test_batch_cg_stops_each_instance_on_its_own(cuda, solver_lib):
    """The adjoint CG stops every instance at its own relative residual: the
    iteration counts differ across instances of different shapes, and each
    final relative residual is at or below the tolerance (an instance that
    stopped early stays stopped while the others continue)."""
    from reg_drot.autograd import batch_quadratic_drot_fn
    from reg_drot.batch import QRBatch
    shapes = [(64, 96), (300, 257), (513, 200), (1500, 900), (128, 1100)]
    insts = [_points(nr, nc, 70 + k) for k, (nr, nc) in enumerate(shapes)]
    B = QRBatch(shapes, RHO, 1e-2, EPS_FWD, device=cuda, cols_per_tile=64)
    leaves = [torch.tensor(A.sqeuclidean(xs, yt), dtype=torch.float32, device=cuda,
                           requires_grad=True) for xs, yt, _, _ in insts]
    cp = B.pack_c(leaves)
    p, q = B.pack_marginals([torch.tensor(i[2], dtype=torch.float32) for i in insts],
                            [torch.tensor(i[3], dtype=torch.float32) for i in insts])
    x = batch_quadratic_drot_fn(B, cp, p, q, MAX_ITERS, cg_tol=1e-7)
    ((cp * x).sum() + 0.3 * (x * x).sum()).backward()
    iters, rel = x.grad_fn.cg_iters, x.grad_fn.cg_residuals
    print(f"\n[cg] iterations {iters}, final relative residuals {rel}")
    assert len(set(iters)) > 1, iters
    assert all(0 < r <= 1e-7 for r in rel), rel
