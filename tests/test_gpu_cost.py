"""GPU: tensor-core cost matrices (reg_drot.cost, drot_sqeuclidean_cost).

Against an FP64 torch reference of the same formula,
    C[j, i] = scale * max(|x_i|^2 + |y_j|^2 - 2 <x_i, y_j>, 0).
Bound: the Gram term is split TF32 (hi.hi + hi.lo + lo.hi, FP32 accumulate),
whose error is about 2^-22 |x_i||y_j| per product term; with FP32 norms the
error of an entry stays below 4e-6 (|x_i|^2 + |y_j|^2) * scale -- a plain
single-pass TF32 product would miss this bound by about three orders of
magnitude.  Gradients (drot_sqeuclidean_cost_grad: FP32 sums in a fixed
order) against FP64 autograd: 1e-5 relative.
"""
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _ref(x, y, scale=1.0, clamp=True):
    x = x.double()
    y = y.double()
    c = (y * y).sum(1)[:, None] + (x * x).sum(1)[None, :] - 2.0 * (y @ x.t())
    if clamp:
        c = c.clamp_min(0.0)
    return c * scale


def _bound(x, y, scale):
    return 4e-6 * ((y.double() ** 2).sum(1)[:, None] + (x.double() ** 2).sum(1)[None, :]) * scale


@pytest.mark.parametrize("m,n,d", [(1, 1, 8), (127, 255, 16), (128, 256, 16), (300, 517, 16),
                                   (1000, 700, 32), (64, 3000, 24), (4096, 130, 8)])
def test_cost_matches_fp64(cuda, solver_lib, m, n, d):
    from reg_drot.cost import sqeuclidean_cost
    g = torch.Generator(device=cuda).manual_seed(m * 7 + n + d)
    x = torch.randn(m, d, generator=g, device=cuda)
    y = torch.randn(n, d, generator=g, device=cuda) * 0.5 + 0.1
    for scale in (1.0, 1.0 / 64):
        c = sqeuclidean_cost(x, y, scale)
        assert c.shape == (n, m)
        err = (c.double() - _ref(x, y, scale)).abs()
        assert bool((err <= _bound(x, y, scale) + 1e-30).all()), float((err / _bound(x, y, scale)).max())
        assert float(c.min()) >= 0.0


def test_cost_identical_points_and_no_clamp(cuda, solver_lib):
    from reg_drot.cost import sqeuclidean_cost
    g = torch.Generator(device=cuda).manual_seed(1)
    x = torch.randn(200, 16, generator=g, device=cuda)
    c = sqeuclidean_cost(x, x)
    assert float(c.diagonal().abs().max()) <= float(_bound(x, x, 1.0).diagonal().max())
    c2 = sqeuclidean_cost(x, x, clamp=False)
    err = (c2.double() - _ref(x, x, 1.0, clamp=False)).abs()
    assert bool((err <= _bound(x, x, 1.0)).all())


@pytest.mark.parametrize("m,n,d", [(300, 257, 16), (301, 257, 8), (517, 64, 24), (129, 700, 32)])
def test_cost_backward_matches_fp64_autograd(cuda, solver_lib, m, n, d):
    """drot_sqeuclidean_cost_grad (hand-written chain rule) against FP64
    autograd of the same formula; n_rows % 4 != 0 takes the scalar loads."""
    from reg_drot.cost import sqeuclidean_cost
    g = torch.Generator(device=cuda).manual_seed(3 + m)
    x = torch.randn(m, d, generator=g, device=cuda, requires_grad=True)
    y = torch.randn(n, d, generator=g, device=cuda, requires_grad=True)
    G = torch.randn(n, m, generator=g, device=cuda)
    (sqeuclidean_cost(x, y, 0.25) * G).sum().backward()
    xd = x.detach().double().requires_grad_(True)
    yd = y.detach().double().requires_grad_(True)
    (_ref(xd, yd, 0.25) * G.double()).sum().backward()
    for a, b in ((x.grad, xd.grad), (y.grad, yd.grad)):
        rel = float((a.double() - b).norm() / b.norm())
        assert rel <= 1e-5, rel


def test_packed_cost_for_a_batch(cuda, solver_lib):
    from reg_drot.batch import QRBatch
    from reg_drot.cost import packed_sqeuclidean_cost
    shapes = [(64, 96), (300, 257), (513, 200), (7, 1100)]
    g = torch.Generator(device=cuda).manual_seed(9)
    xs = [torch.randn(m, 16, generator=g, device=cuda) for m, _ in shapes]
    ys = [torch.randn(n, 16, generator=g, device=cuda) for _, n in shapes]
    B = QRBatch(shapes, 2.0, 1e-3, 1e-4, device=cuda, cols_per_tile=64)
    c = packed_sqeuclidean_cost(B, torch.cat(xs), torch.cat(ys), 1.0 / 64)
    ref = B.pack_c([_ref(x, y, 1.0 / 64).float() for x, y in zip(xs, ys)])
    for k in range(len(shapes)):
        err = (B.view(c, k).double() - _ref(xs[k], ys[k], 1.0 / 64)).abs()
        assert bool((err <= _bound(xs[k], ys[k], 1.0 / 64)).all()), k
    mask = torch.ones_like(c, dtype=torch.bool)
    for k in range(len(shapes)):
        B.view(mask, k).fill_(False)
    assert float(c[mask].abs().max()) == 0.0 and float(ref[mask].abs().max()) == 0.0


def test_packed_cost_backward_for_a_batch(cuda, solver_lib):
    from reg_drot.batch import QRBatch
    from reg_drot.cost import packed_sqeuclidean_cost
    shapes = [(64, 96), (300, 257), (513, 200), (7, 1100), (1030, 333)]
    g = torch.Generator(device=cuda).manual_seed(19)
    xc = torch.randn(sum(m for m, _ in shapes), 16, generator=g, device=cuda, requires_grad=True)
    yc = torch.randn(sum(n for _, n in shapes), 16, generator=g, device=cuda, requires_grad=True)
    B = QRBatch(shapes, 2.0, 1e-3, 1e-4, device=cuda, cols_per_tile=64)
    c = packed_sqeuclidean_cost(B, xc, yc, 1.0 / 64)
    G = torch.randn(c.shape, generator=g, device=cuda)
    (c * G).sum().backward()
    xo = yo = 0
    for k, (m, n) in enumerate(shapes):
        xd = xc[xo:xo + m].detach().double().requires_grad_(True)
        yd = yc[yo:yo + n].detach().double().requires_grad_(True)
        (_ref(xd, yd, 1.0 / 64) * B.view(G, k).double()).sum().backward()
        for a, b in ((xc.grad[xo:xo + m], xd.grad), (yc.grad[yo:yo + n], yd.grad)):
            rel = float((a.double() - b).norm() / b.norm())
            assert rel <= 1e-5, (k, rel)
        xo += m
        yo += n


def test_cost_rejects_bad_inputs(cuda, solver_lib):
    from reg_drot.cost import sqeuclidean_cost
    x = torch.randn(10, 12, device=cuda)
    with pytest.raises(RuntimeError):
        sqeuclidean_cost(x, x)
    with pytest.raises(RuntimeError):
        sqeuclidean_cost(torch.randn(10, 16, device=cuda), torch.randn(10, 8, device=cuda))
