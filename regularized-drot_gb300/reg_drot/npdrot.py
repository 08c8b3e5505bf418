"""GPU backend with the API of the reference's numpy solvers.

Same names and arguments as ``npdrot`` (numpy/npdrot/solver.py:191-290):

    quaddrot(init, C, p, q, reg, numba=False, incl_dual_offset=False, **kwargs) -> x [, log]
    l1l2drot(init, C, p, q, reg, groups, numba=False, **kwargs)                 -> x [, log]
    drot(init, C, p, q, numba=False, **kwargs)                                   -> x [, log]

numpy arrays in and out (C and init m x n, Fortran order as the reference
asserts; p of length m, q of length n); the iterations run on the GPU in
FP32 through the C ABI (drot_np_solve).  The loop is the one of regdrot
(solver.py:7-189): prox, marginal residual, dual correction; stop when the
primal residual is <= eps_abs (tested every iteration) or after max_iters
iterations; then one final prox.  Keyword arguments as regdrot: max_iters
(100), eps_abs (1e-6), step (2 / (m + n)), compute_r_primal / compute_r_dual
(the stop test needs one of them, as in the reference), init_strategy,
return_log, verbose.

Mapping to the device solver's state (the CUDA solver and the numpy loop
run the same map): X = init, a = X 1 - p, b = X^T 1 - q, phi1 = phi2 = 0,
alpha = sum(X) + sum(p) - 2; QR divisor 1 + step * reg; GL threshold
reg * step over the row groups.

Differences, stated: ``groups`` must tile the rows 0..m-1 with contiguous
(start, stop) pairs (every row in exactly one group); the GPU group shrink
adds 1e-9 to the group norm like the reference's CUDA kernels (numpy adds
nothing); ``callbacks`` are not supported (they need the host every
iteration); ``log["primal"]`` holds the final residual only (the
per-iteration history stays on the device); numpy's dual-gap and dual
residual terms (compute_r_dual, dual_offset, dual_resid) contribute 0 in
the reference as well and are accepted.
"""
import ctypes
import time

import numpy as np
import torch

from ._lib import DrotResult, check, lib

MODE_QR, MODE_GL = 0, 1
C_F32 = 0


def initial_state(init, p, q, init_strategy=False):
    """The device solver's state (FP64, numpy) equivalent to regdrot's start
    from ``init``, including its init_strategy (solver.py:75-93)."""
    x = np.array(init, dtype=np.float64, order="F")
    p = np.asarray(p, dtype=np.float64)
    q = np.asarray(q, dtype=np.float64)
    m, n = x.shape
    if init_strategy:
        w = 4.0 * m * n / (m + n)
        yy = -w * p - w / (m + n)
        xx = -w * q - w / (m + n)
        x += (-1.0 / n) * yy[:, None] + (-1.0 / m) * xx[None, :]
    return {"x": x, "a": x.sum(1) - p, "b": x.sum(0) - q, "phi1": np.zeros(m),
            "phi2": np.zeros(n), "alpha": np.array([x.sum() + p.sum() - 2.0])}


def group_bounds_from_pairs(groups, m):
    """Boundaries [0, ..., m] of contiguous row groups given as (start, stop)
    pairs that tile 0..m-1."""
    pairs = sorted((int(a), int(b)) for a, b in groups)
    bounds = [0]
    for a, b in pairs:
        if a != bounds[-1] or b <= a:
            raise NotImplementedError("groups must tile the rows 0..m-1 with contiguous "
                                      "(start, stop) pairs")
        bounds.append(b)
    if bounds[-1] != m:
        raise NotImplementedError("groups must cover every row")
    return bounds


def _regdrot_gpu(mode, init, C, p, q, coef, groups=None, device=None, **kwargs):
    max_iters = int(kwargs.pop("max_iters", 100))
    eps_abs = float(kwargs.pop("eps_abs", 1e-6))
    m, n = np.shape(init)
    step = float(kwargs.pop("step", 2.0 / (len(p) + len(q))))
    verbose = kwargs.pop("verbose", False)
    kwargs.pop("print_every", None)
    compute = kwargs.pop("compute_r_primal", False) or kwargs.pop("compute_r_dual", False)
    return_log = kwargs.pop("return_log", False)
    if kwargs.pop("callbacks", None) is not None:
        raise NotImplementedError("callbacks run on the host every iteration; not supported")
    init_strategy = kwargs.pop("init_strategy", False)
    for k in ("dual_offset", "dual_resid", "n_rows", "n_cols", "compute_r_dual"):
        kwargs.pop(k, None)
    if not np.isfortran(np.asarray(C)) and np.asarray(C).ndim == 2 and min(np.shape(C)) > 1:
        raise AssertionError("C must be F-contiguous (as the reference asserts)")
    if np.shape(C) != (m, n) or len(p) != m or len(q) != n:
        raise ValueError("shapes of init, C, p, q do not match")

    G = 0
    barr = None
    if mode == MODE_GL:  # validated before any device work
        bounds = group_bounds_from_pairs(groups, m)
        G = len(bounds) - 1
        barr = (ctypes.c_int * (G + 1))(*bounds)
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else \
        torch.device(device)
    st0 = initial_state(init, p, q, init_strategy)
    f32 = dict(dtype=torch.float32, device=dev)
    c_t = torch.tensor(np.ascontiguousarray(np.asarray(C, dtype=np.float32).T), **f32)
    p_t = torch.tensor(np.asarray(p, dtype=np.float32), **f32)
    q_t = torch.tensor(np.asarray(q, dtype=np.float32), **f32)
    t = {"x": torch.tensor(np.ascontiguousarray(st0["x"].T), **f32),
         "a": torch.tensor(st0["a"], **f32), "b": torch.tensor(st0["b"], **f32),
         "phi1": torch.zeros(m, **f32), "phi2": torch.zeros(n, **f32),
         "alpha": torch.tensor(st0["alpha"], **f32)}
    with torch.cuda.device(dev):
        nbytes = int(lib().drot_np_workspace_bytes(mode, m, n, G, barr))
        if nbytes == 0:
            raise RuntimeError("drot_np_workspace_bytes: unsupported problem")
        ws = torch.empty(nbytes + 256, dtype=torch.uint8, device=dev)
        wptr = ws.data_ptr() + (-ws.data_ptr()) % 256
        stream = torch.cuda.current_stream(dev).cuda_stream

        def run(iters, eps):
            res = DrotResult()
            rc = lib().drot_np_solve(mode, c_t.data_ptr(), C_F32, p_t.data_ptr(), q_t.data_ptr(),
                                     m, n, G, barr, step, coef, int(iters), float(eps),
                                     t["x"].data_ptr(), t["a"].data_ptr(), t["b"].data_ptr(),
                                     t["phi1"].data_ptr(), t["phi2"].data_ptr(),
                                     t["alpha"].data_ptr(), wptr, nbytes, ctypes.byref(res),
                                     stream)
            check(rc, "np_solve")
            return res

        t0 = time.time()
        # regdrot's loop runs at least once; without a residual it runs max_iters.
        res = run(max(max_iters, 1), eps_abs if compute else -1.0)
        k = res.iters_run
        dual = (t["phi1"].double().cpu().numpy(), t["phi2"].double().cpu().numpy())
        run(1, float(np.finfo(np.float32).max))  # the final prox
        elapsed = time.time() - t0
    x = np.asfortranarray(t["x"].double().cpu().numpy().T)
    if verbose:
        print(f"GPU DROT terminated at iteration {k - 1} (residual {res.residual:.5e})")
    if return_log:
        resid = np.array([res.residual])
        return x, {"dual_sol": dual, "primal": resid, "gap": resid, "dual": np.zeros(1),
                   "num_iters": k, "solve_time": elapsed}
    return x


def quaddrot(init, C, p, q, reg, numba=False, incl_dual_offset=False, **kwargs):
    """Quadratic-regularised OT (npdrot.quaddrot, solver.py:258-290) on the GPU."""
    step = float(kwargs.get("step", 2.0 / (len(p) + len(q))))
    kappa = float(np.float32(1.0) + np.float32(step) * np.float32(reg))
    return _regdrot_gpu(MODE_QR, init, C, p, q, kappa, **kwargs)


def drot(init, C, p, q, numba=False, **kwargs):
    """Unregularised OT (npdrot.drot, solver.py:191-210) on the GPU."""
    return _regdrot_gpu(MODE_QR, init, C, p, q, 1.0, **kwargs)


def l1l2drot(init, C, p, q, reg, groups, numba=False, **kwargs):
    """Group-lasso OT (npdrot.l1l2drot, solver.py:212-239) on the GPU; groups
    are (start, stop) row ranges tiling the rows."""
    step = float(kwargs.get("step", 2.0 / (len(p) + len(q))))
    lam = float(np.float32(reg) * np.float32(step))
    return _regdrot_gpu(MODE_GL, init, C, p, q, lam, groups=groups, **kwargs)


__all__ = ["quaddrot", "drot", "l1l2drot", "initial_state", "group_bounds_from_pairs"]
