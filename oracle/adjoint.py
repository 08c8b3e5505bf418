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
