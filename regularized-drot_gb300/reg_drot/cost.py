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

(G' = dL/dC where C > 0; two FP32 cuBLAS GEMMs per instance).
``sqeuclidean_cost(x, y)`` builds one cost; ``packed_sqeuclidean_cost(batch,
x_cat, y_cat)`` builds every instance of a QRBatch straight into its packed
C buffer (x_cat, y_cat: the instances' points concatenated in order).
"""
import ctypes

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


def _point_grads(G, x, y, scale):
    """Chain rule of C = scale * (|x|^2 + |y|^2 - 2 x.y) for G = dL/dC ([n, m])."""
    gx = 2.0 * scale * (x * G.sum(0)[:, None] - G.t() @ y)
    gy = 2.0 * scale * (y * G.sum(1)[:, None] - G @ x)
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
        G = gc.float()
        if ctx.clamp:
            G = G * (c > 0)
        gx, gy = _point_grads(G, x, y, ctx.scale)
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
        B = ctx.batch
        G = gc.float()
        gx = torch.empty_like(x)
        gy = torch.empty_like(y)
        for k, (m, n, ld, xo, yo, co) in enumerate(ctx.descs):
            Gk = B.view(G, k)
            if ctx.clamp:
                Gk = Gk * (B.view(c, k) > 0)
            gxk, gyk = _point_grads(Gk, x[xo:xo + m], y[yo:yo + n], ctx.scale)
            gx[xo:xo + m] = gxk
            gy[yo:yo + n] = gyk
        return gx, gy, None, None, None, None


def packed_sqeuclidean_cost(batch, x_cat, y_cat, scale=1.0, clamp=True, dtype=torch.float32):
    """The packed C buffer of a QRBatch from concatenated point clouds;
    differentiable in x_cat and y_cat.  dtype=torch.bfloat16 gives the
    BF16-stored cost (rounded from the FP32 result)."""
    return PackedSqEuclideanCostFn.apply(x_cat, y_cat, batch, float(scale), bool(clamp), dtype)


__all__ = ["sqeuclidean_cost", "packed_sqeuclidean_cost", "DIMS"]
