"""FP64 reference gradients of the quadratic-regularised plan -- TEST
INFRASTRUCTURE ONLY (tests/ use it as the checker; the solver never does).

The reference has no backward (pytorch/src/drot_cuda.cpp:26-44 returns plans
without autograd), so there is nothing of it to restate here; the gradient
follows from the problem the reference's QR iteration solves.  Its fixed
point (core/drot_qr.hpp:159-234 with the operator's parameters,
pytorch/src/qr_drot_cuda_kernel.cu:100-102: X = max(X + phi1 + phi2 - sC, 0)
/ kappa) is the solution of
    min <C, X> + (lambda / 2) ||X||_F^2  s.t.  X 1 = p, X^T 1 = q, X >= 0
with lambda = (kappa - 1) / s.  On the support S the plan is
X_ij = (u_i + v_j - C_ij) / lambda, and differentiating the constraints on a
fixed support gives the adjoint system, solved here densely (least squares,
FP64):
    [diag(D_r) M^T_rows; M diag(D_c)] [a; b] = [rowsum(G o M); colsum(G o M)]
    dL/dC = X (explicit, for L = <C, X> + w ||X||^2) + (a_i + b_j - G_ij) / lambda on S
    dL/dp = a, dL/dq = b   (gauge: shifted so that sum(a) = sum(b)).
S is read off the final duals, S = {phi1_i + phi2_j - s C_ij > 0}: at the
fixed point X > 0 exactly there, but a finite solve still carries tiny
positive entries of X elsewhere (decaying by 1/kappa per iteration).
Arrays use the reference's PyTorch layout [n_cols, n_rows].
"""
import numpy as np

from . import oracle as O

f32 = np.float32


def qr_lambda(rho, r_weight, n_rows, n_cols):
    s = O.step_size(rho, n_rows, n_cols)
    kappa = O.qr_scale(s, r_weight, n_rows, n_cols, "torch")
    return (kappa - 1.0) / s


def solve64(c, p, q, rho, r_weight, eps=1e-13, max_iters=300_000):
    """Tight FP64 solve with the reference iteration (the oracle's FP64 loop).
    Weakly regularised cases may stop on max_iters short of eps (rounding
    floor); their support and duals are settled long before."""
    return O.quadratic_drot(np.asarray(c, np.float64), np.asarray(p, np.float64),
                            np.asarray(q, np.float64), rho, r_weight, max_iters, eps,
                            dtype=np.float64)


def support(o, c, s):
    """S = {phi1_i + phi2_j - s C_ij > 0} from a solve's final state."""
    return (o["phi1"][None, :] + o["phi2"][:, None] - s * np.asarray(c, np.float64)) > 0


def implicit_adjoint(M, G, lam):
    """(dL/dC implicit part, a, b) for upstream G = dL/dX on support M ([nc, nr])."""
    nc, nr = M.shape
    Mf = M.astype(np.float64)
    A = np.zeros((nr + nc, nr + nc))
    A[:nr, :nr] = np.diag(Mf.sum(0))
    A[nr:, nr:] = np.diag(Mf.sum(1))
    A[:nr, nr:] = Mf.T
    A[nr:, :nr] = Mf
    Gm = G * Mf
    rhs = np.concatenate([Gm.sum(0), Gm.sum(1)])
    z = np.linalg.lstsq(A, rhs, rcond=None)[0]
    a, b = z[:nr], z[nr:]
    t = (b.sum() - a.sum()) / (nr + nc)
    a, b = a + t, b - t
    gc = np.where(M, (a[None, :] + b[:, None] - G) / lam, 0.0)
    return gc, a, b


def implicit_adjoint_sparse(M, G, lam, rtol=1e-13):
    """implicit_adjoint for large supports: the same system, FP64, as a
    sparse matrix solved by conjugate gradients (it is positive
    semidefinite and the right-hand side is consistent, so CG converges to
    a solution; the gauge a + t, b - t is fixed as in implicit_adjoint)."""
    from scipy.sparse import bmat, coo_matrix, diags
    from scipy.sparse.linalg import cg
    nc, nr = M.shape
    Mf = M.astype(np.float64)
    j, i = np.nonzero(M)
    off = coo_matrix((np.ones(len(i)), (i, j)), shape=(nr, nc)).tocsr()
    A = bmat([[diags(Mf.sum(0)), off], [off.T, diags(Mf.sum(1))]], format="csr")
    Gm = G * Mf
    rhs = np.concatenate([Gm.sum(0), Gm.sum(1)])
    deg = np.asarray(A.diagonal())
    pre = diags(np.where(deg > 0, 1.0 / np.maximum(deg, 1.0), 0.0))
    try:
        z, info = cg(A, rhs, rtol=rtol, atol=0.0, maxiter=100000, M=pre)
    except TypeError:  # scipy before 1.12 names the relative tolerance `tol`
        z, info = cg(A, rhs, tol=rtol, atol=0.0, maxiter=100000, M=pre)
    if info != 0:
        raise RuntimeError(f"implicit_adjoint_sparse: CG did not converge ({info})")
    a, b = z[:nr], z[nr:]
    t = (b.sum() - a.sum()) / (nr + nc)
    a, b = a + t, b - t
    gc = np.where(M, (a[None, :] + b[:, None] - G) / lam, 0.0)
    return gc, a, b


def grads_at_state(o, c, rho, r_weight, w, sparse=True):
    """Loss L = <C, X> + w ||X||_F^2 and its implicit gradients (dL/dC, dL/dp,
    dL/dq), FP64, at the plan and duals of a finished solve `o` (the support
    read off o's duals): the gradient the implicit adjoint gives for that
    solve."""
    X = np.asarray(o["x"], np.float64)
    c = np.asarray(c, np.float64)
    nc, nr = X.shape
    lam = qr_lambda(rho, r_weight, nr, nc)
    L = float((c * X).sum() + w * (X * X).sum())
    G = c + 2.0 * w * X
    M = support(o, c, O.step_size(rho, nr, nc))
    gi, a, b = (implicit_adjoint_sparse if sparse else implicit_adjoint)(M, G, lam)
    return L, X + gi, a, b


def loss_and_grads(c, p, q, rho, r_weight, w, eps=1e-13):
    """L = <C, X*> + w ||X*||_F^2 and its FP64 gradients w.r.t. C, p, q."""
    o = solve64(c, p, q, rho, r_weight, eps)
    X = o["x"]
    c = np.asarray(c, np.float64)
    nc, nr = X.shape
    lam = qr_lambda(rho, r_weight, nr, nc)
    L = float((c * X).sum() + w * (X * X).sum())
    G = c + 2.0 * w * X
    gi, a, b = implicit_adjoint(support(o, c, O.step_size(rho, nr, nc)), G, lam)
    return L, X + gi, a, b, o


def sqeuclidean(xs, yt):
    """C[j, i] = ||xs_i - yt_j||^2 ([n_cols = len(yt), n_rows = len(xs)])."""
    xs = np.asarray(xs, np.float64)
    yt = np.asarray(yt, np.float64)
    return ((yt[:, None, :] - xs[None, :, :]) ** 2).sum(-1)


def point_grads(xs, yt, gc):
    """Chain rule of C = sqeuclidean(xs, yt) for dL/dC = gc."""
    gx = 2.0 * (xs * gc.sum(0)[:, None] - gc.T @ yt)
    gy = 2.0 * (yt * gc.sum(1)[:, None] - gc @ xs)
    return gx, gy


def gl_unrolled(c, p, q, n_class, rho, r_weight, iters, norm_eps=1e-9, convention="torch",
                last_k=None, c_last=None, state=None, lam=None):
    """X after `iters` GL iterations from the warm start, in FP64 torch (CPU)
    so that autograd gives the exact gradient of the unrolled map.  Restates
    the oracle's GL loop (oracle_gl_solve: core/drot_glr.hpp:242-355,
    kernel_glr.hpp:59-161, 461-526) with the operator's parameters
    (pytorch/src/glr_drot_cuda_kernel.cu:255-257; convention="wrapper": the
    C++ wrapper's threshold, core/drot_glr.hpp:385).  last_k: the first
    iters - last_k iterations run without autograd, so the gradient is that
    of the last last_k steps with the state before them held fixed (the
    truncated unrolled adjoint); c_last, if given, is the cost those last
    steps use (c the earlier ones).  state: start there (a dict of x, a, b,
    phi1, phi2, alpha tensors, held fixed) instead of the warm start; lam:
    the threshold itself instead of the convention's.  c, p, q: torch
    float64 tensors ([n_cols, n_rows], [n_rows], [n_cols])."""
    import torch
    nc, nr = c.shape
    s = O.step_size(rho, nr, nc)
    if lam is None:
        lam = O.gl_lambda(r_weight, nr, n_class, convention)
    w = O.warm_start(s, nr, nc)
    bounds = [int(v) for v in O.group_bounds(nr, n_class)]
    f64 = dict(dtype=torch.float64)
    if state is None:
        X = torch.zeros(nc, nr, **f64)
        phi1 = torch.full((nr,), float(w["phi1"]), **f64)
        phi2 = torch.full((nc,), float(w["phi2"]), **f64)
        a = torch.full((nr,), float(w["a"]), **f64)
        b = torch.full((nc,), float(w["b"]), **f64)
        alpha = torch.tensor(float(w["alpha"]), **f64)
    else:
        X, phi1, phi2, a, b = (torch.as_tensor(state[k], **f64).detach().clone()
                               for k in ("x", "phi1", "phi2", "a", "b"))
        alpha = torch.as_tensor(state["alpha"], **f64).detach().reshape(())
    t_free = iters - last_k if last_k is not None else 0
    for it in range(iters):
        if it == t_free and last_k is not None:
            X, phi1, phi2, a, b, alpha = (v.detach() for v in (X, phi1, phi2, a, b, alpha))
        cc = c_last if (c_last is not None and it >= t_free) else c
        y = (X + phi1[None, :] + phi2[:, None] - s * cc).clamp_min(0.0)
        parts = []
        for g in range(n_class):
            yg = y[:, bounds[g]:bounds[g + 1]]
            n2 = (yg * yg).sum(1)
            pos = n2 > 0
            n = torch.sqrt(torch.where(pos, n2, torch.ones_like(n2))) * pos
            sig = (1.0 - lam / (n + norm_eps)).clamp_min(0.0)
            parts.append(sig[:, None] * yg)
        X = torch.cat(parts, 1)
        r, cs_, sigma = X.sum(0), X.sum(1), X.sum()
        gamma = (2.0 * (sigma - 1.0) - alpha) / (nr + nc)
        rs = r - p
        a = a - rs
        phi1 = (a - rs + gamma) / nc
        cs = cs_ - q
        b = b - cs
        phi2 = (b - cs + gamma) / nr
        alpha = alpha + 1.0 - sigma
    return X
