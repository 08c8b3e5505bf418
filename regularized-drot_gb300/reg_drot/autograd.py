"""Differentiable DROT plans (torch.autograd).

The reference's operators return plans without gradients
(pytorch/src/drot_cuda.cpp:26-44: outputs have requires_grad=False).  Here:

  quadratic_drot_fn(c, p, q, rho, r_weight, max_iters, eps)   -> x (differentiable)
  batch_quadratic_drot_fn(batch, c, p, q, max_iters)          -> packed x (differentiable)
  group_lasso_drot_fn(c, p, q, n_class, rho, r_weight, max_iters, eps) -> x (differentiable)

Group lasso: the gradient is the unrolled adjoint of the iterations the
solve ran (drot_gl_adjoint_step, one reverse step per iteration), with the
states recomputed segment by segment from checkpoints of the forward.

Forward: the CUDA solver (single instance or QRBatch).  Backward: the
implicit adjoint of the regularised problem
    min <C, X> + (lambda / 2) ||X||_F^2  s.t.  X 1 = p, X^T 1 = q, X >= 0,
lambda = (kappa - 1) / s (= r_weight * (n_rows + n_cols) with the operator's
parameters, pytorch/src/qr_drot_cuda_kernel.cu:100-102): on the support S,
    dL/dC = (a_i + b_j - G_ij) / lambda,  dL/dp = a,  dL/dq = b,
where [a; b] solves the masked Laplacian system built from the support
(drot_qr_adjoint_prepare / _solve / _grad: bit-packed masks, the right-hand
side from the upstream gradient, Jacobi-preconditioned CG in FP64 in one
persistent launch, and one kernel for dL/dC, dL/dp, dL/dq).  The support is S = {phi1_i + phi2_j - s C_ij
> 0} from the solve's final duals: a finite solve leaves tiny, geometrically
decaying positive entries of X off S, so X > 0 would overstate it.  a and b
are unique up to a + t, b - t (the marginals' masses are tied) -- one such
constant per connected component of the bipartite support graph; the
returned pair has sum(a) = sum(b) overall.  The gradient is
that of the exact solution on a locally fixed support, so it assumes the
forward solve converged (a warning is raised otherwise) and r_weight > 0.
"""
import ctypes
import math
import warnings

import numpy as np
import torch

from ._lib import DrotAdjointInstance, check, lib

C_F32, C_BF16 = 0, 1
CG_TOL = 1e-10
CG_MAX_ITERS = 5000

f32 = np.float32


def qr_lambda(rho, r_weight, n_rows, n_cols):
    """lambda = (kappa - 1) / s with the FP32 s and kappa of the operator."""
    s = f32(rho) / (f32(n_rows) + f32(n_cols))
    t = f32(s * f32(r_weight))
    t = f32(t * f32(n_rows + n_cols))
    kappa = f32(f32(1.0) + t)
    return (float(kappa) - 1.0) / float(s)


def step_and_kappa(rho, r_weight, n_rows, n_cols):
    s = f32(rho) / (f32(n_rows) + f32(n_cols))
    t = f32(s * f32(r_weight))
    t = f32(t * f32(n_rows + n_cols))
    return float(s), float(f32(f32(1.0) + t))


class _Adjoint:
    """Support masks, CG solve and gradient assembly of one or more instances
    (drot_qr_adjoint_prepare / _solve / _grad / _residuals)."""

    def __init__(self, c, phi1, phi2, descs, byte_mask=False):
        # descs: (n_rows, n_cols, ld, c_offset, v_offset, phi1_offset, phi2_offset, s, lambda)
        n = len(descs)
        self.n = n
        self.arr = (DrotAdjointInstance * n)()
        self.nv = 0
        for k, (nr, nc, ld, co, vo, o1, o2, st, lam) in enumerate(descs):
            d = self.arr[k]
            d.n_rows, d.n_cols, d.ld, d.c_offset, d.v_offset = nr, nc, ld, co, vo
            d.phi1_offset, d.phi2_offset, d.step_size, d.lambda_ = o1, o2, st, lam
            self.nv = max(self.nv, vo + nr + nc)
        self.device = c.device
        self.mask = None
        with torch.cuda.device(c.device):
            self.nbytes = int(lib().drot_qr_adjoint_workspace_bytes(n, self.arr))
            if self.nbytes == 0:
                raise RuntimeError("drot_qr_adjoint_workspace_bytes: unsupported shapes")
            self.ws = torch.empty(self.nbytes + 256, dtype=torch.uint8, device=c.device)
            self.ptr = self.ws.data_ptr() + (-self.ws.data_ptr()) % 256
            if byte_mask:
                self.mask = torch.zeros(c.shape, dtype=torch.uint8, device=c.device)
            rc = lib().drot_qr_adjoint_prepare(
                n, self.arr, c.data_ptr(), C_BF16 if c.dtype == torch.bfloat16 else C_F32,
                phi1.data_ptr(), phi2.data_ptr(),
                self.mask.data_ptr() if byte_mask else None, self.ptr, self.nbytes,
                self._stream())
        check(rc, "qr_adjoint_prepare")
        if byte_mask:
            self.mask = self.mask.bool()

    def _stream(self):
        return torch.cuda.current_stream(self.device).cuda_stream

    def solve(self, g, tol, max_iters):
        """z = [a; b] (FP64) of every instance for the upstream gradient g
        (float32, layout of C); returns (z, CG iterations, final relative
        residuals)."""
        z = torch.empty(self.nv, dtype=torch.float64, device=self.device)
        iters = (ctypes.c_int * self.n)()
        rel = (ctypes.c_double * self.n)()
        with torch.cuda.device(self.device):
            rc = lib().drot_qr_adjoint_solve(self.n, self.arr, g.data_ptr(), z.data_ptr(),
                                             float(tol), int(max_iters), self.ptr, self.nbytes,
                                             iters, self._stream())
            check(rc, "qr_adjoint_solve")
            rc = lib().drot_qr_adjoint_residuals(self.n, self.arr, self.ptr, self.nbytes, rel,
                                                 self._stream())
        check(rc, "qr_adjoint_residuals")
        return z, list(iters), list(rel)

    def grad(self, g, z, gc, gp, gq):
        """dL/dC into gc (layout of C), dL/dp into gp, dL/dq into gq."""
        with torch.cuda.device(self.device):
            rc = lib().drot_qr_adjoint_grad(self.n, self.arr, g.data_ptr(), z.data_ptr(),
                                            gc.data_ptr(), gp.data_ptr(), gq.data_ptr(),
                                            self.ptr, self.nbytes, self._stream())
        check(rc, "qr_adjoint_grad")


class QuadraticDROTFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, c, p, q, rho, r_weight, max_iters, eps, cg_tol, cg_max_iters):
        from . import _check_input, _check_shapes, DrotResult
        _check_input(c, "c", allow_bf16=True)
        for t, n in ((p, "p"), (q, "q")):
            _check_input(t, n)
        nr, nc = _check_shapes(c, p, q)
        s, kappa = step_and_kappa(rho, r_weight, nr, nc)
        dev = c.device
        x = torch.empty(c.shape, dtype=torch.float32, device=dev)
        a = torch.empty(nr, device=dev)
        b = torch.empty(nc, device=dev)
        phi1 = torch.empty(nr, device=dev)
        phi2 = torch.empty(nc, device=dev)
        alpha = torch.empty(1, device=dev)
        res = DrotResult()
        with torch.cuda.device(dev):
            st = torch.cuda.current_stream(dev).cuda_stream
            check(lib().drot_init_state(nr, nc, s, 1, p.data_ptr(), q.data_ptr(), x.data_ptr(),
                                        a.data_ptr(), b.data_ptr(), phi1.data_ptr(),
                                        phi2.data_ptr(), alpha.data_ptr(), st), "init_state")
            nbytes = int(lib().drot_qr_workspace_bytes(nr, nc))
            ws = torch.empty(nbytes + 256, dtype=torch.uint8, device=dev)
            wptr = ws.data_ptr() + (-ws.data_ptr()) % 256
            check(lib().drot_qr_solve_ex(c.data_ptr(), C_BF16 if c.dtype == torch.bfloat16 else C_F32,
                                         p.data_ptr(), q.data_ptr(), nr, nc, s, kappa,
                                         int(max_iters), float(eps), x.data_ptr(), a.data_ptr(),
                                         b.data_ptr(), phi1.data_ptr(), phi2.data_ptr(),
                                         alpha.data_ptr(), wptr, nbytes, ctypes.byref(res), st),
                  "qr_solve")
        info = res.as_dict()
        if not info["converged"]:
            warnings.warn("quadratic_drot_fn: the solve did not converge; the implicit "
                          "gradient assumes the optimal plan")
        ctx.save_for_backward(c, phi1, phi2)
        ctx.meta = (nr, nc, s, (kappa - 1.0) / s)
        ctx.cg = (cg_tol, cg_max_iters)
        ctx.info = info
        return x

    @staticmethod
    def backward(ctx, gx):
        c, phi1, phi2 = ctx.saved_tensors
        nr, nc, s, lam = ctx.meta
        G = gx.detach().float().contiguous()
        adj = _Adjoint(c.detach(), phi1, phi2, [(nr, nc, nr, 0, 0, 0, 0, s, lam)])
        z, iters, rel = adj.solve(G, *ctx.cg)
        ctx.cg_iters = iters
        ctx.cg_residuals = rel
        gc = torch.empty(c.shape, dtype=torch.float32, device=c.device)
        gp = torch.empty(nr, dtype=torch.float32, device=c.device)
        gq = torch.empty(nc, dtype=torch.float32, device=c.device)
        adj.grad(G, z, gc, gp, gq)
        return gc.to(c.dtype), gp, gq, None, None, None, None, None, None


def quadratic_drot_fn(c, p, q, rho, r_weight, max_iters, eps, *, cg_tol=CG_TOL,
                      cg_max_iters=CG_MAX_ITERS):
    """reg_drot.quadratic_drot with a backward (implicit adjoint)."""
    if not r_weight > 0:
        raise RuntimeError("quadratic_drot_fn needs r_weight > 0 (the gradient divides by lambda)")
    return QuadraticDROTFn.apply(c, p, q, float(rho), float(r_weight), int(max_iters), float(eps),
                                 float(cg_tol), int(cg_max_iters))


class BatchQuadraticDROTFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, c, p, q, batch, max_iters, cg_tol, cg_max_iters, points):
        if points is None:
            x, info = batch.solve(c.detach(), p.detach(), q.detach(), max_iters)
        else:  # the same cost recomputed from the clouds inside the solve
            xs, ys, scale = points
            x, info = batch.solve_points(xs, ys, p.detach(), q.detach(), max_iters, scale)
        if not all(r["converged"] for r in info):
            warnings.warn("batch_quadratic_drot_fn: some instances did not converge; the "
                          "implicit gradient assumes optimal plans")
        phi1, phi2 = batch.duals()
        ctx.save_for_backward(c, phi1, phi2)
        ctx.batch = batch
        ctx.cg = (cg_tol, cg_max_iters)
        ctx.info = info
        return x

    @staticmethod
    def backward(ctx, gx):
        c, phi1, phi2 = ctx.saved_tensors
        B = ctx.batch
        G = gx.detach().float().contiguous()
        steps = B.step_sizes()
        descs, vo, prow, pcol = [], 0, 0, 0
        for k, (nr, nc) in enumerate(B.shapes):
            lam = (step_and_kappa(B.rho[k], B.r_weight[k], nr, nc)[1] - 1.0) / steps[k]
            descs.append((nr, nc, B.lds[k], B.offsets[k], vo, prow, pcol, steps[k], lam))
            vo += nr + nc
            prow += nr
            pcol += nc
        adj = _Adjoint(c.detach(), phi1, phi2, descs)
        z, iters, rel = adj.solve(G, *ctx.cg)
        ctx.cg_iters = iters
        ctx.cg_residuals = rel
        gc = torch.zeros_like(G)  # the padding rows of every block stay zero
        gp = torch.empty(prow, dtype=torch.float32, device=G.device)
        gq = torch.empty(pcol, dtype=torch.float32, device=G.device)
        adj.grad(G, z, gc, gp, gq)
        return gc.to(c.dtype), gp, gq, None, None, None, None, None


def batch_quadratic_drot_fn(batch, c, p, q, max_iters, *, cg_tol=CG_TOL,
                            cg_max_iters=CG_MAX_ITERS, points=None):
    """QRBatch.solve with a backward; c, p, q packed (QRBatch.pack_c /
    pack_marginals), returns the packed plans (QRBatch.unpack gives views).
    points=(x_cat, y_cat, scale): the forward recomputes the cost from the
    clouds inside the solve (QRBatch.solve_points, on the tensor cores) -- c
    must hold the same cost (packed_sqeuclidean_cost of the clouds: the
    values the solve recomputes); the backward reads it once."""
    if not all(r > 0 for r in batch.r_weight):
        raise RuntimeError("batch_quadratic_drot_fn needs r_weight > 0 for every instance")
    return BatchQuadraticDROTFn.apply(c, p, q, batch, int(max_iters), float(cg_tol),
                                      int(cg_max_iters), points)


def gl_step_and_lambda(rho, r_weight, n_rows, n_cols, n_class, convention="operator"):
    """s and the group threshold lambda: the GL operator's r * sqrt(n_rows //
    n_class) (pytorch/src/glr_drot_cuda_kernel.cu:255-257) or, with
    convention="wrapper", the C++ wrapper's r / sqrt(n_rows // n_class)
    (core/drot_glr.hpp:385), both rounded from FP64 to FP32."""
    import math
    s = f32(rho) / (f32(n_rows) + f32(n_cols))
    k = math.sqrt(n_rows // n_class)
    if convention == "operator":
        lam = f32(float(f32(r_weight)) * k)
    elif convention == "wrapper":
        lam = f32(float(f32(r_weight)) / k)
    else:
        raise RuntimeError("convention must be 'operator' or 'wrapper'")
    return float(s), float(lam)


class _GLState:
    """Solver state (X, a, b, phi1, phi2, alpha) on the device and the
    one-call GL solve from it (drot_gl_solve_ex: state in / state out)."""

    def __init__(self, c, p, q, n_class, s, lam):
        self.c, self.p, self.q, self.G, self.s, self.lam = c, p, q, n_class, s, lam
        self.nc, self.nr = c.shape
        dev = c.device
        self.t = {"x": torch.empty(c.shape, dtype=torch.float32, device=dev),
                  "a": torch.empty(self.nr, device=dev), "b": torch.empty(self.nc, device=dev),
                  "phi1": torch.empty(self.nr, device=dev),
                  "phi2": torch.empty(self.nc, device=dev),
                  "alpha": torch.empty(1, device=dev)}
        with torch.cuda.device(dev):
            self.nbytes = int(lib().drot_gl_workspace_bytes(self.nr, self.nc, n_class))
        if self.nbytes == 0:
            raise RuntimeError("group_lasso_drot_fn: unsupported shape")
        self.ws = torch.empty(self.nbytes + 256, dtype=torch.uint8, device=dev)
        self.wptr = self.ws.data_ptr() + (-self.ws.data_ptr()) % 256

    def stream(self):
        return torch.cuda.current_stream(self.c.device).cuda_stream

    def warm_start(self):
        t = self.t
        with torch.cuda.device(self.c.device):
            check(lib().drot_init_state(self.nr, self.nc, self.s, 1, self.p.data_ptr(),
                                        self.q.data_ptr(), t["x"].data_ptr(), t["a"].data_ptr(),
                                        t["b"].data_ptr(), t["phi1"].data_ptr(),
                                        t["phi2"].data_ptr(), t["alpha"].data_ptr(),
                                        self.stream()), "init_state")

    def run(self, iters, eps):
        from . import DrotResult
        t = self.t
        res = DrotResult()
        with torch.cuda.device(self.c.device):
            check(lib().drot_gl_solve_ex(
                self.c.data_ptr(), C_BF16 if self.c.dtype == torch.bfloat16 else C_F32,
                self.p.data_ptr(), self.q.data_ptr(), self.nr, self.nc, self.G, self.s, self.lam,
                int(iters), float(eps), t["x"].data_ptr(), t["a"].data_ptr(), t["b"].data_ptr(),
                t["phi1"].data_ptr(), t["phi2"].data_ptr(), t["alpha"].data_ptr(), self.wptr,
                self.nbytes, ctypes.byref(res), self.stream()), "gl_solve")
        return res.as_dict()

    def snapshot(self):
        return {k: v.clone() for k, v in self.t.items()}

    def restore(self, snap):
        for k, v in snap.items():
            self.t[k].copy_(v)



class GroupLassoDROTFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, c, p, q, n_class, rho, r_weight, max_iters, eps, segment, convention,
                last_k):
        from . import _check_input, _check_shapes
        _check_input(c, "c", allow_bf16=True)
        for t, n in ((p, "p"), (q, "q")):
            _check_input(t, n)
        nr, nc = _check_shapes(c, p, q)
        s, lam = gl_step_and_lambda(rho, r_weight, nr, nc, n_class, convention)
        st = _GLState(c.detach(), p.detach(), q.detach(), n_class, s, lam)
        st.warm_start()
        # Checkpoints (segment index, state); with last_k only the newest
        # ceil(last_k / segment) + 1 are kept -- those the truncated backward reads.
        keep = None if last_k is None else (last_k + segment - 1) // segment + 1
        checkpoints, T, info, si = [], 0, None, 0
        while T < max_iters:
            checkpoints.append((si, st.snapshot()))
            if keep is not None and len(checkpoints) > keep:
                checkpoints.pop(0)
            info = st.run(min(segment, max_iters - T), eps)
            T += info["iters_run"]
            si += 1
            if info["converged"] or info["iters_run"] == 0:
                break
        ctx.save_for_backward(c, p, q)
        t_lo = 0 if last_k is None else max(0, T - int(last_k))
        ctx.meta = (nr, nc, int(n_class), s, lam, int(segment), T, t_lo)
        ctx.checkpoints = checkpoints
        ctx.info = dict(info, n_iter=T, iters_run=T)  # totals over the segments
        return st.t["x"].clone()

    @staticmethod
    def backward(ctx, gx):
        c, p, q = ctx.saved_tensors
        nr, nc, G, s, lam, seg, T, t_lo = ctx.meta
        cbar, pbar, qbar = _gl_unrolled_backward(c, p, q, G, s, lam, seg, ctx.checkpoints, T,
                                                 t_lo, gx.detach().float().contiguous())
        return cbar.to(c.dtype), pbar, qbar, None, None, None, None, None, None, None, None


def _gl_unrolled_backward(c, p, q, G, s, lam, seg, checkpoints, T, t_lo, xbar):
    """Adjoint of GL iterations [t_lo, T) (checkpoints: (segment index,
    state) of the segments covering them, every `seg` iterations from 0)
    applied to xbar = dL/dX at T; returns (dL/dC, dL/dp, dL/dq)."""
    nc, nr = c.shape
    dev = c.device
    st = _GLState(c.detach(), p.detach(), q.detach(), G, s, lam)
    xbar = xbar.clone()
    vbar = torch.zeros(2 * (nr + nc) + 1, device=dev)
    cbar = torch.zeros(c.shape, dtype=torch.float32, device=dev)
    pbar = torch.zeros(nr, device=dev)
    qbar = torch.zeros(nc, device=dev)
    with torch.cuda.device(dev):
        abytes = int(lib().drot_gl_adjoint_workspace_bytes(nr, nc, G))
    if abytes == 0:
        raise RuntimeError("group_lasso_drot_fn: shape unsupported by the adjoint")
    aws = torch.empty(abytes + 256, dtype=torch.uint8, device=dev)
    aptr = aws.data_ptr() + (-aws.data_ptr()) % 256
    cdt = C_BF16 if c.dtype == torch.bfloat16 else C_F32
    states = torch.empty(seg * (nr * nc + nr + nc), device=dev)
    t = st.t
    for si, snap in reversed(checkpoints):
        k0 = si * seg
        k1 = min(k0 + seg, T)
        if k1 <= t_lo:
            break
        st.restore(snap)
        if k0 < t_lo:
            # truncated adjoint: advance to its first iteration without it
            st.run(t_lo - k0, -1.0)
            k0 = t_lo
        with torch.cuda.device(dev):
            rc = lib().drot_gl_adjoint_segment(
                c.data_ptr(), cdt, p.data_ptr(), q.data_ptr(), nr, nc, G, s, lam,
                t["x"].data_ptr(), t["a"].data_ptr(), t["b"].data_ptr(), t["phi1"].data_ptr(),
                t["phi2"].data_ptr(), t["alpha"].data_ptr(), k1 - k0, states.data_ptr(),
                st.wptr, st.nbytes, xbar.data_ptr(), vbar.data_ptr(), cbar.data_ptr(),
                pbar.data_ptr(), qbar.data_ptr(), aptr, abytes, st.stream())
        check(rc, "gl_adjoint_segment")
    return cbar, pbar, qbar


class _GlAdjointBatch:
    """The batched GL adjoint of a GLBatch (drot_gl_adjoint_batch_*): one set
    of launches per reverse iteration for every instance."""

    def __init__(self, batch):
        from ._lib import DrotGlAdjointBatchInstance
        B = batch
        self.n = B.n
        self.desc = (DrotGlAdjointBatchInstance * B.n)()
        steps = B.step_sizes()
        prow = pcol = 0
        self.vlen = 0
        for k, (nr, nc) in enumerate(B.shapes):
            d = self.desc[k]
            d.n_rows, d.n_cols, d.ld, d.n_groups = nr, nc, B.lds[k], B.n_class[k]
            d.x_offset = d.c_offset = B.offsets[k]
            d.row_offset, d.col_offset = prow, pcol
            d.step_size, d.lambda_ = steps[k], B.lambdas[k]
            prow += nr
            pcol += nc
            self.vlen += 2 * (nr + nc) + 1
        self.h = ctypes.c_void_p()
        with torch.cuda.device(B.device):
            check(lib().drot_gl_adjoint_batch_plan_create(B.n, self.desc, ctypes.byref(self.h)),
                  "gl_adjoint_batch_plan_create")
        self.nbytes = int(lib().drot_gl_adjoint_batch_workspace_bytes(self.h))
        self.ws = torch.empty(self.nbytes + 256, dtype=torch.uint8, device=B.device)
        self.ptr = self.ws.data_ptr() + (-self.ws.data_ptr()) % 256

    def setup(self, c, xbar, vbar, cbar, pbar, qbar, stream):
        check(lib().drot_gl_adjoint_batch_setup(
            self.h, self.desc, c.data_ptr(), C_BF16 if c.dtype == torch.bfloat16 else C_F32,
            xbar.data_ptr(), vbar.data_ptr(), cbar.data_ptr(), pbar.data_ptr(), qbar.data_ptr(),
            self.ptr, self.nbytes, stream), "gl_adjoint_batch_setup")

    def step(self, x, phi1, phi2, stream):
        check(lib().drot_gl_adjoint_batch_step(self.h, x.data_ptr(), phi1.data_ptr(),
                                               phi2.data_ptr(), self.ptr, self.nbytes, stream),
              "gl_adjoint_batch_step")

    def __del__(self):
        try:
            if self.h:
                lib().drot_gl_adjoint_batch_plan_destroy(self.h)
        except Exception:
            pass


class BatchGroupLassoDROTFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, c, p, q, batch, max_iters, last_k, segment):
        x, info = batch.solve(c.detach(), p.detach(), q.detach(), max_iters)
        if not all(r["converged"] for r in info):
            warnings.warn("batch_group_lasso_drot_fn: some instances did not converge; the "
                          "adjoint is taken at the last iterate")
        ctx.save_for_backward(c, p, q)
        ctx.batch, ctx.last_k, ctx.seg = batch, int(last_k), int(segment)
        # the packed final state (alpha of each instance's own parity in slot 0)
        v = batch.state_views()
        par = torch.tensor([int(r["iters_run"]) & 1 for r in info], device=x.device)
        ctx.snap = {"x": x.detach().clone(), "a": v["a"].clone(), "b": v["b"].clone(),
                    "phi1": v["phi1"].clone(), "phi2": v["phi2"].clone(),
                    "alpha": v["alpha"].gather(0, par.view(1, -1)).view(-1).clone()}
        ctx.info = info
        ctx.state = batch.state(info)
        return x

    @staticmethod
    def backward(ctx, gx):
        """Every instance's unrolled adjoint of last_k GL iterations taken
        from its solution, batched: the iterations are recomputed for all
        instances at once (drot_batch_resume, checkpoints every `segment`
        iterations, the segment's states kept), then each reverse iteration
        is one set of launches over all instances
        (drot_gl_adjoint_batch_step).  The recomputation runs in the
        batch's own workspace: afterwards GLBatch.results() describes those
        launches; the forward's per-instance outcomes stay in
        grad_fn.info."""
        c, p, q = ctx.saved_tensors
        B = ctx.batch
        dev = c.device
        stream = torch.cuda.current_stream(dev).cuda_stream
        cd, pd, qd = c.detach(), p.detach(), q.detach()
        xw = B.empty_x()
        views = B.state_views()

        def load(snap):
            xw.copy_(snap["x"])
            for k in ("a", "b", "phi1", "phi2"):
                views[k].copy_(snap[k])
            views["alpha"][0].copy_(snap["alpha"])

        def save():
            return {"x": xw.clone(), "a": views["a"].clone(), "b": views["b"].clone(),
                    "phi1": views["phi1"].clone(), "phi2": views["phi2"].clone(),
                    "alpha": views["alpha"][0].clone()}

        # checkpoints at the start of every segment of the last_k iterations
        K, seg = ctx.last_k, ctx.seg
        load(ctx.snap)
        checkpoints = []
        T = 0
        while T < K:
            checkpoints.append((T, save()))
            n = min(seg, K - T)
            if T + n < K:
                B.resume(cd, pd, qd, xw, n)
            T += n
        adj = getattr(B, "_gl_adjoint", None)
        if adj is None:
            adj = B._gl_adjoint = _GlAdjointBatch(B)
        xbar = gx.detach().float().contiguous().clone()
        vbar = torch.zeros(adj.vlen, device=dev)
        cbar = torch.zeros(B.total, dtype=torch.float32, device=dev)
        pbar = torch.zeros(B.total_rows, device=dev)
        qbar = torch.zeros(B.total_cols, device=dev)
        adj.setup(cd, xbar, vbar, cbar, pbar, qbar, stream)
        sx = torch.empty(min(seg, K), B.total, device=dev)
        s1 = torch.empty(min(seg, K), B.total_rows, device=dev)
        s2 = torch.empty(min(seg, K), B.total_cols, device=dev)
        for T0, snap in reversed(checkpoints):
            n = min(seg, K - T0)
            load(snap)
            for i in range(n):
                sx[i].copy_(xw)
                s1[i].copy_(views["phi1"])
                s2[i].copy_(views["phi2"])
                if i + 1 < n:
                    B.resume(cd, pd, qd, xw, 1)
            for i in reversed(range(n)):
                adj.step(sx[i], s1[i], s2[i], stream)
        return cbar.to(c.dtype), pbar, qbar, None, None, None, None


def batch_group_lasso_drot_fn(batch, c, p, q, max_iters, *, last_k=64, segment=None):
    """GLBatch.solve with a backward: for every instance, the unrolled
    adjoint of last_k GL iterations taken from its solution (the state the
    batched solve stopped at, held fixed) -- the truncated adjoint at the
    fixed point, where last_k more iterations leave the plan within the stop
    tolerance.  c, p, q packed (GLBatch.pack_c / pack_marginals).
    segment: checkpoint spacing of the recomputation; the backward holds
    about last_k / segment checkpoints and segment stored iterates of the
    packed plans, so the default ceil(sqrt(last_k)) keeps both near their
    minimum (8 + 8 plan copies for last_k = 64).  The gradient does not
    depend on it."""
    if int(last_k) <= 0:
        raise RuntimeError("last_k must be positive")
    if segment is None:
        segment = max(1, int(math.ceil(math.sqrt(int(last_k)))))
    if int(segment) <= 0:
        raise RuntimeError("segment must be positive")
    return BatchGroupLassoDROTFn.apply(c, p, q, batch, int(max_iters), int(last_k),
                                       int(segment))


def group_lasso_drot_fn(c, p, q, n_class, rho, r_weight, max_iters, eps, *, segment=32,
                        convention="operator", last_k=None):
    """reg_drot.group_lasso_drot with a backward: the unrolled adjoint of the
    iterations the solve ran, recomputed from checkpoints taken every
    ``segment`` iterations (memory: one state per segment plus ``segment``
    plans during the backward).  last_k: unroll only the last last_k
    iterations (the truncated adjoint: the gradient of the last last_k steps
    with the state before them held fixed; memory: ceil(last_k / segment) + 1
    states).  convention: "operator" (lambda = r_weight * sqrt(n_rows //
    n_class), the PyTorch operator) or "wrapper" (r_weight / sqrt(n_rows //
    n_class), the C++ wrapper)."""
    if last_k is not None and int(last_k) <= 0:
        raise RuntimeError("last_k must be positive")
    if int(segment) <= 0:
        raise RuntimeError("segment must be positive")
    return GroupLassoDROTFn.apply(c, p, q, int(n_class), float(rho), float(r_weight),
                                  int(max_iters), float(eps), int(segment), str(convention),
                                  None if last_k is None else int(last_k))


__all__ = ["quadratic_drot_fn", "batch_quadratic_drot_fn", "group_lasso_drot_fn",
           "batch_group_lasso_drot_fn", "qr_lambda",
           "step_and_kappa", "gl_step_and_lambda"]
