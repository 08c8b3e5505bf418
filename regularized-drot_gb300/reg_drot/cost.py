"""Squared-Euclidean cost matrices of point clouds on the tensor cores.

The reference's callers build C on the host before calling the solver
(benchmark/utils/compute_w2_dist.py:68-94).  Here the cost of point clouds x
(m x d) and y (n x d) is one CUDA kernel (drot_sqeuclidean_cost: the Gram
term on tcgen05 tensor cores in split TF32, FP32-level accuracy):

    C[j, i] = scale * max(|x_i|^2 + |y_j|^2 - 2 <x_i, y_j>, 0)

in the solver's layout ([n, m] = column-major m x n, p over the x points,
q over the y points), with autograd:

    dL/dx_i = 2 scale (x_i sum_j G'_ji - sum_j G'_ji y_j)
    dL/dy_j = 2 scale (y_j sum_i G'_ji - sum_i G'_ji x_i)

(G' = dL/dC where C > 0; drot_sqeuclidean_cost_grad: one pass over G' and C,
FP32 sums in a fixed order).
``sqeuclidean_cost(x, y)`` builds one cost; ``packed_sqeuclidean_cost(batch,
x_cat, y_cat)`` builds every instance of a QRBatch straight into its packed
C buffer (x_cat, y_cat: the instances' points concatenated in order).
"""
import torch

from ._lib import DrotCostInstance, check, lib

DIMS = (8, 16, 24, 32)


def _check_points(t, name):
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise RuntimeError(f"{name} must be a CUDA tensor")
    if t.dtype != torch.float32 or t.dim() != 2:
        raise RuntimeError(f"{name} must be a 2-D float32 tensor [points, dim]")
    if t.size(1) not in DIMS:
        raise RuntimeError(f"point dimension must be one of {DIMS}")


def _launch(descs, x, y, scale, clamp, c):
    n = len(descs)
    arr = (DrotCostInstance * n)()
    for k, (m, nn, ld, xo, yo, co) in enumerate(descs):
        a = arr[k]
        a.m, a.n, a.ld, a.x_offset, a.y_offset, a.c_offset = m, nn, ld, xo, yo, co
    with torch.cuda.device(x.device):
        rc = lib().drot_sqeuclidean_cost(n, arr, x.data_ptr(), y.data_ptr(), x.size(1),
                                         float(scale), int(clamp), c.data_ptr(),
                                         torch.cuda.current_stream(x.device).cuda_stream)
    check(rc, "sqeuclidean_cost")


def _chain_rule(descs, x, y, scale, c, g, clamp):
    """dL/dx, dL/dy of C = scale * max(|x|^2 + |y|^2 - 2 x.y, 0) for g = dL/dC
    (the layout of c) through drot_sqeuclidean_cost_grad."""
    n = len(descs)
    arr = (DrotCostInstance * n)()
    for k, (m, nn, ld, xo, yo, co) in enumerate(descs):
        a = arr[k]
        a.m, a.n, a.ld, a.x_offset, a.y_offset, a.c_offset = m, nn, ld, xo, yo, co
    gx = torch.empty_like(x)
    gy = torch.empty_like(y)
    with torch.cuda.device(x.device):
        nbytes = int(lib().drot_sqeuclidean_cost_grad_workspace_bytes(n, arr, x.size(1)))
        if nbytes == 0:
            raise RuntimeError("drot_sqeuclidean_cost_grad_workspace_bytes: invalid instances")
        ws = torch.empty(nbytes, dtype=torch.uint8, device=x.device)
        rc = lib().drot_sqeuclidean_cost_grad(n, arr, x.data_ptr(), y.data_ptr(), x.size(1),
                                              float(scale), c.data_ptr() if clamp else None,
                                              g.data_ptr(), gx.data_ptr(), gy.data_ptr(),
                                              ws.data_ptr(), nbytes,
                                              torch.cuda.current_stream(x.device).cuda_stream)
    check(rc, "sqeuclidean_cost_grad")
    return gx, gy


class SqEuclideanCostFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, y, scale, clamp):
        _check_points(x, "x")
        _check_points(y, "y")
        if x.size(1) != y.size(1) or x.device != y.device:
            raise RuntimeError("x and y must have the same dimension and device")
        x = x.detach().contiguous()
        y = y.detach().contiguous()
        m, n = x.size(0), y.size(0)
        c = torch.empty(n, m, dtype=torch.float32, device=x.device)
        _launch([(m, n, m, 0, 0, 0)], x, y, scale, clamp, c)
        ctx.save_for_backward(x, y, c)
        ctx.scale, ctx.clamp = scale, clamp
        return c

    @staticmethod
    def backward(ctx, gc):
        x, y, c = ctx.saved_tensors
        m, n = x.size(0), y.size(0)
        G = gc.float().contiguous()
        gx, gy = _chain_rule([(m, n, m, 0, 0, 0)], x, y, ctx.scale, c, G, ctx.clamp)
        return gx, gy, None, None


def sqeuclidean_cost(x, y, scale=1.0, clamp=True):
    """Cost [n, m] between x (m x d) and y (n x d); differentiable in x and y."""
    return SqEuclideanCostFn.apply(x, y, float(scale), bool(clamp))


class PackedSqEuclideanCostFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x_cat, y_cat, batch, scale, clamp, dtype):
        _check_points(x_cat, "x")
        _check_points(y_cat, "y")
        x = x_cat.detach().contiguous()
        y = y_cat.detach().contiguous()
        descs, xo, yo = [], 0, 0
        for k, (m, n) in enumerate(batch.shapes):
            descs.append((m, n, batch.lds[k], xo, yo, batch.offsets[k]))
            xo += m
            yo += n
        if xo != x.size(0) or yo != y.size(0):
            raise RuntimeError("x_cat / y_cat must hold every instance's points in order")
        c = torch.zeros(batch.total, dtype=torch.float32, device=x.device)
        for s in range(0, len(descs), 256):
            _launch(descs[s:s + 256], x, y, scale, clamp, c)
        ctx.save_for_backward(x, y, c)
        ctx.batch, ctx.scale, ctx.clamp, ctx.descs = batch, scale, clamp, descs
        return c if dtype == torch.float32 else c.to(dtype)

    @staticmethod
    def backward(ctx, gc):
        x, y, c = ctx.saved_tensors
        G = gc.float().contiguous()
        gx = torch.empty_like(x)
        gy = torch.empty_like(y)
        for s in range(0, len(ctx.descs), 256):
            part = ctx.descs[s:s + 256]
            gxs, gys = _chain_rule(part, x, y, ctx.scale, c, G, ctx.clamp)
            # each call writes the rows of its own instances only
            x0, x1 = part[0][3], part[-1][3] + part[-1][0]
            y0, y1 = part[0][4], part[-1][4] + part[-1][1]
            gx[x0:x1] = gxs[x0:x1]
            gy[y0:y1] = gys[y0:y1]
        return gx, gy, None, None, None, None


def packed_sqeuclidean_cost(batch, x_cat, y_cat, scale=1.0, clamp=True, dtype=torch.float32):
    """The packed C buffer of a QRBatch from concatenated point clouds;
    differentiable in x_cat and y_cat.  dtype=torch.bfloat16 gives the
    BF16-stored cost (rounded from the FP32 result)."""
    return PackedSqEuclideanCostFn.apply(x_cat, y_cat, batch, float(scale), bool(clamp), dtype)


__all__ = ["sqeuclidean_cost", "packed_sqeuclidean_cost", "DIMS"]
