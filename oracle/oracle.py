"""ctypes front end of the oracle -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs use this
module, and only as the checker / the timed CPU restatement.  The solver
library never imports it.

The functions mirror the reference's two entry points:
  * ``qr_solve``  -- core/drot_qr.hpp:159-234 (quadratic_regularizer_drot)
  * ``gl_solve``  -- core/drot_glr.hpp:242-355 (group_lasso_regularizer_drot)
and the host-side parameter mapping of pytorch/src/*_drot_cuda_kernel.cu and
the C++ wrappers (core/drot_qr.hpp:241-347, core/drot_glr.hpp:362-474).
Arrays are numpy, column-major X/C given as a [n_cols, n_rows] C-order array
(the reference's PyTorch layout).
"""
import ctypes

import numpy as np

from . import build_oracle

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = ctypes.CDLL(path)
        f32p = ctypes.POINTER(ctypes.c_float)
        f64p = ctypes.POINTER(ctypes.c_double)
        i32p = ctypes.POINTER(ctypes.c_int)
        c_int, c_float, c_double = ctypes.c_int, ctypes.c_float, ctypes.c_double
        L.oracle_step_size.restype = c_float
        L.oracle_step_size.argtypes = [c_float, c_int, c_int]
        for n in ("oracle_qr_scale_torch", "oracle_qr_scale_wrapper"):
            getattr(L, n).restype = c_float
            getattr(L, n).argtypes = [c_float, c_float, c_int, c_int]
        for n in ("oracle_gl_lambda_torch", "oracle_gl_lambda_wrapper"):
            getattr(L, n).restype = c_float
            getattr(L, n).argtypes = [c_float, c_int, c_int]
        L.oracle_group_bounds.restype = None
        L.oracle_group_bounds.argtypes = [c_int, c_int, i32p]
        L.oracle_warm_start.restype = None
        L.oracle_warm_start.argtypes = [c_float, c_int, c_int, f32p]
        L.oracle_max_threads.restype = c_int
        for sfx, rp, rt in (("_f32", f32p, c_float), ("_f64", f64p, c_double)):
            f = getattr(L, "oracle_qr_solve" + sfx)
            f.restype = c_int
            f.argtypes = [rp, rp, rp, c_int, c_int, rt, rt, c_int, rt,
                          rp, rp, rp, rp, rp, rp, i32p, rp, f64p, c_int]
            g = getattr(L, "oracle_gl_solve" + sfx)
            g.restype = c_int
            g.argtypes = [rp, rp, rp, c_int, c_int, c_int, i32p, rt, rt, c_double,
                          c_int, rt, rp, rp, rp, rp, rp, rp, i32p, rp, f64p, c_int]
        _lib = L
    return _lib


def _ptr(a, ct):
    return a.ctypes.data_as(ctypes.POINTER(ct))


def step_size(rho, nr, nc):
    return float(lib().oracle_step_size(rho, nr, nc))


def qr_scale(s, r_weight, nr, nc, convention="torch"):
    f = lib().oracle_qr_scale_torch if convention == "torch" else lib().oracle_qr_scale_wrapper
    return float(f(s, r_weight, nr, nc))


def gl_lambda(r_weight, nr, G, convention="torch"):
    f = lib().oracle_gl_lambda_torch if convention == "torch" else lib().oracle_gl_lambda_wrapper
    return float(f(r_weight, nr, G))


def group_bounds(nr, G):
    out = np.zeros(G + 1, dtype=np.int32)
    lib().oracle_group_bounds(nr, G, _ptr(out, ctypes.c_int))
    return out


def warm_start(s, nr, nc):
    """Return dict(phi1, phi2, a, b, alpha) of the reference warm start (float32 constants)."""
    out = np.zeros(5, dtype=np.float32)
    lib().oracle_warm_start(s, nr, nc, _ptr(out, ctypes.c_float))
    return dict(phi1=out[0], phi2=out[1], a=out[2], b=out[3], alpha=out[4])


def initial_state(nr, nc, s, p=None, q=None, warm=True, dtype=np.float32):
    """State arrays (x, a, b, phi1, phi2, alpha) for the warm start or the cold start X = p q^T."""
    dt = np.dtype(dtype)
    if warm:
        w = warm_start(s, nr, nc)
        x = np.zeros((nc, nr), dtype=dt)
        a = np.full(nr, w["a"], dtype=dt)
        b = np.full(nc, w["b"], dtype=dt)
        phi1 = np.full(nr, w["phi1"], dtype=dt)
        phi2 = np.full(nc, w["phi2"], dtype=dt)
        alpha = np.array([w["alpha"]], dtype=dt)
    else:
        # init_x: X = p q^T (kernel_qr.hpp:7-40); a = b = phi = 0; alpha = 0.
        x = (np.asarray(q, dtype=dt)[:, None] * np.asarray(p, dtype=dt)[None, :]).astype(dt)
        a = np.zeros(nr, dtype=dt)
        b = np.zeros(nc, dtype=dt)
        phi1 = np.zeros(nr, dtype=dt)
        phi2 = np.zeros(nc, dtype=dt)
        alpha = np.zeros(1, dtype=dt)
    return dict(x=np.ascontiguousarray(x), a=a, b=b, phi1=phi1, phi2=phi2, alpha=alpha)


def _solve(kind, c, p, q, state, dtype, threads, **kw):
    dt = np.dtype(dtype)
    ct = ctypes.c_float if dt == np.float32 else ctypes.c_double
    sfx = "_f32" if dt == np.float32 else "_f64"
    nc, nr = c.shape
    c = np.ascontiguousarray(c, dtype=dt)
    p = np.ascontiguousarray(p, dtype=dt)
    q = np.ascontiguousarray(q, dtype=dt)
    st = {k: np.ascontiguousarray(v, dtype=dt).copy() for k, v in state.items()}
    n_iter = ctypes.c_int(0)
    obj = np.zeros(1, dtype=dt)
    res = ctypes.c_double(-1.0)
    if threads is None:
        threads = lib().oracle_max_threads()
    L = lib()
    common_tail = [_ptr(st["x"], ct), _ptr(st["a"], ct), _ptr(st["b"], ct),
                   _ptr(st["phi1"], ct), _ptr(st["phi2"], ct), _ptr(st["alpha"], ct),
                   ctypes.byref(n_iter), _ptr(obj, ct), ctypes.byref(res), int(threads)]
    if kind == "qr":
        rc = getattr(L, "oracle_qr_solve" + sfx)(
            _ptr(c, ct), _ptr(p, ct), _ptr(q, ct), nr, nc, kw["s"], kw["kappa"],
            kw["max_iters"], kw["eps"], *common_tail)
    else:
        bounds = np.ascontiguousarray(kw["bounds"], dtype=np.int32)
        rc = getattr(L, "oracle_gl_solve" + sfx)(
            _ptr(c, ct), _ptr(p, ct), _ptr(q, ct), nr, nc, len(bounds) - 1,
            _ptr(bounds, ctypes.c_int), kw["s"], kw["lam"], kw.get("norm_eps", 1e-9),
            kw["max_iters"], kw["eps"], *common_tail)
    if rc != 0:
        raise MemoryError("oracle allocation failed")
    st["n_iter"] = n_iter.value
    st["objective"] = float(obj[0])
    st["residual"] = res.value
    return st


def qr_solve(c, p, q, s, kappa, max_iters, eps, state=None, dtype=np.float32, threads=None):
    """Reference QR loop; returns the final state dict (x, a, b, phi1, phi2, alpha, n_iter, objective, residual)."""
    nc, nr = c.shape
    if state is None:
        state = initial_state(nr, nc, s, dtype=dtype)
    return _solve("qr", c, p, q, state, dtype, threads, s=s, kappa=kappa,
                  max_iters=max_iters, eps=eps)


def gl_solve(c, p, q, bounds, s, lam, max_iters, eps, state=None, dtype=np.float32,
             threads=None, norm_eps=1e-9):
    """Reference GL loop; returns the final state dict."""
    nc, nr = c.shape
    if state is None:
        state = initial_state(nr, nc, s, dtype=dtype)
    return _solve("gl", c, p, q, state, dtype, threads, s=s, lam=lam, bounds=bounds,
                  max_iters=max_iters, eps=eps, norm_eps=norm_eps)


def quadratic_drot(c, p, q, rho, r_weight, max_iters, eps, dtype=np.float32, threads=None):
    """Oracle of reg_drot.quadratic_drot (pytorch/src/qr_drot_cuda_kernel.cu:142-210)."""
    nc, nr = c.shape
    s = step_size(rho, nr, nc)
    kappa = qr_scale(s, r_weight, nr, nc, "torch")
    return qr_solve(c, p, q, s, kappa, max_iters, eps, dtype=dtype, threads=threads)


def qr_solve_stopped_at(c, p, q, s, kappa, n_iter, dtype=np.float32, threads=None):
    """The QR loop as though its stop test had passed at iteration n_iter - 1.

    The reference tests even iterations only and reports the last index + 1
    (core/drot_qr.hpp:200-233), so n_iter - 1 must be even.  The loop runs
    iterations 0 .. n_iter - 1 with the test disabled, then applies fix_x
    (kernel_qr.hpp:469-482: X <- max(X + sC, 0), one rounding of s*C + X):
    the state, objective and residual the reference returns when its test
    passes there.  A solve whose stop moved by one check (a tie at the
    threshold between two summation orders) is compared with this."""
    k = int(n_iter) - 1
    if k < 0 or k % 2:
        raise ValueError("n_iter - 1 must be a non-negative even iteration index")
    st = qr_solve(c, p, q, s, kappa, k + 1, -1.0, dtype=dtype, threads=threads)
    dt = np.dtype(dtype)
    sv = float(np.asarray(s, dtype=dt))
    x = st["x"].astype(np.float64) + sv * np.asarray(c, dtype=dt).astype(np.float64)
    st["x"] = np.maximum(x, 0.0).astype(dt)
    st["n_iter"] = int(n_iter)
    return st


def quadratic_drot_at(c, p, q, rho, r_weight, n_iter, dtype=np.float32, threads=None):
    """quadratic_drot stopped (converged) at the reference count n_iter."""
    nc, nr = c.shape
    s = step_size(rho, nr, nc)
    kappa = qr_scale(s, r_weight, nr, nc, "torch")
    return qr_solve_stopped_at(c, p, q, s, kappa, n_iter, dtype=dtype, threads=threads)


def quadratic_drot_matching(n_iter, o, c, p, q, rho, r_weight, dtype=np.float32, threads=None):
    """The oracle solve `o` when it stopped at n_iter, else the oracle
    stopped at n_iter (quadratic_drot_at): the reference result to compare a
    converged solve that reported n_iter with."""
    if o["n_iter"] == n_iter:
        return o
    return quadratic_drot_at(c, p, q, rho, r_weight, n_iter, dtype=dtype, threads=threads)


def group_lasso_drot(c, p, q, n_class, rho, r_weight, max_iters, eps, dtype=np.float32,
                     threads=None):
    """Oracle of reg_drot.group_lasso_drot (pytorch/src/glr_drot_cuda_kernel.cu:299-381)."""
    nc, nr = c.shape
    s = step_size(rho, nr, nc)
    lam = gl_lambda(r_weight, nr, n_class, "torch")
    return gl_solve(c, p, q, group_bounds(nr, n_class), s, lam, max_iters, eps,
                    dtype=dtype, threads=threads)
