"""Generate the golden vectors that pin the oracle to the reference.

Imports the reference's own numpy implementation (numpy/npdrot in
WangZesen/Regularized-DROT) from a local checkout and records, for seeded
inputs, the iterates it produces.  The reference CUDA solver and the numpy
solver run the same Douglas-Rachford map; they start from the same point when

  * the CUDA cold start X = p q^T (core/kernel_qr.hpp:7-40, a = b = phi = 0,
    alpha = 0) is given to numpy as ``init = p q^T``, or
  * the CUDA warm start (X = 0, phi1 + phi2 = s, core/drot_qr.hpp:321-346) is
    given to numpy as ``init = s * ones`` -- valid for uniform marginals,
    where the warm-start dual a = (k+1)/n_rows equals numpy's row sums of
    the init minus p.

Parameter mapping (numpy/npdrot/solver.py, proximal.py):
  QR: numpy ``reg = r_weight * (n_rows + n_cols)`` gives the CUDA divisor
      kappa = 1 + s * r_weight * (n_rows + n_cols).
  GL: numpy ``reg = lambda / s`` gives the CUDA shrink 1 - lambda/||Y_g||
      (the CUDA kernels add 1e-9 to the norm; the oracle takes that constant
      as a parameter and is run with 0 against these vectors).

numpy's loop applies ``max_iters`` prox steps plus a final prox, so its
output after ``max_iters = T - 1`` is the CUDA iterate after T iterations,
and its primal residual log entry k is the CUDA residual of iteration k.

Usage (in a container that has the reference checkout):
    python tests/golden/gen_golden.py /path/to/Regularized-DROT
writes tests/golden/npdrot_golden.npz.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "npdrot_golden.npz")


def _import_npdrot(ref_root):
    sys.path.insert(0, os.path.join(HERE, "numba_standin"))
    sys.path.insert(0, os.path.join(ref_root, "numpy"))
    from npdrot.solver import regdrot  # noqa: E402
    from npdrot.proximal import (trace_nonnegative_quad_prox,  # noqa: E402
                                 trace_nonnegative_l1l2_prox)
    return regdrot, trace_nonnegative_quad_prox, trace_nonnegative_l1l2_prox


def _bounds(nr, G):
    """Reference group boundaries, restated with numpy float32 (kernel_glr.hpp:79-80, 185-186)."""
    off = 0.49 if -(-nr // G) <= 256 else 0.49999
    per = np.float32(nr) / np.float32(G)
    return [int(float(per * np.float32(k)) + off) for k in range(G + 1)]


def main(ref_root):
    regdrot, quad_prox, l1l2_prox = _import_npdrot(ref_root)
    rng = np.random.default_rng(20240605)
    arrays = {}
    manifest = []

    def add(name, meta, **arrs):
        for k, v in arrs.items():
            arrays[f"{name}/{k}"] = np.asarray(v)
        meta = dict(meta)
        meta["name"] = name
        manifest.append(meta)

    shapes = [(7, 5), (33, 20), (64, 65), (130, 67)]
    for (nr, nc) in shapes:
        iter_counts = [1, 2, 5, 40] if nr < 100 else [3, 40]
        C = rng.random((nr, nc)) + 1e-3
        C = C / C.max()
        pd = rng.dirichlet(np.ones(nr))
        qd = rng.dirichlet(np.ones(nc))
        pu = np.full(nr, 1.0 / nr)
        qu = np.full(nc, 1.0 / nc)
        rho = 2.0
        s = rho / (nr + nc)
        for kind in ("qr", "gl"):
            for start in ("cold", "warm"):
                p, q = (pd, qd) if start == "cold" else (pu, qu)
                if kind == "qr":
                    r_weight = 1e-2
                    prox = quad_prox
                    kw = dict(reg=r_weight * (nr + nc))
                    meta_extra = dict(r_weight=r_weight)
                else:
                    G = 2 if nr < 40 else 3
                    bounds = _bounds(nr, G)
                    lam = 2e-3
                    prox = l1l2_prox
                    groups = [(bounds[k], bounds[k + 1]) for k in range(G)]
                    kw = dict(reg=lam / s, groups=groups, n_rows=nr, n_cols=nc)
                    meta_extra = dict(lam=lam, bounds=bounds)
                init = np.outer(p, q) if start == "cold" else np.full((nr, nc), s)
                for T in iter_counts:
                    if T == 1:
                        # numpy's loop always runs at least once; the first iterate is
                        # one prox of the init.
                        x = np.array(init, order="F")
                        prox(x.T.reshape(-1), np.asfortranarray(C).T.reshape(-1), step=s, **kw)
                        resid = np.zeros(0)
                    else:
                        x, log = regdrot(np.asfortranarray(init), np.asfortranarray(C), p, q,
                                         prox, max_iters=T - 1, eps_abs=-1.0, step=s,
                                         compute_r_primal=True, return_log=True, **kw)
                        resid = log["primal"]
                    name = f"{kind}_{start}_{nr}x{nc}_T{T}"
                    add(name, dict(kind=kind, start=start, nr=nr, nc=nc, T=T, rho=rho,
                                   s=s, inputs=f"in_{start}_{nr}x{nc}", **meta_extra),
                        x=np.asarray(x).T.copy(), resid=resid)
                arrays[f"in_{start}_{nr}x{nc}/C"] = C.T.copy()
                arrays[f"in_{start}_{nr}x{nc}/p"] = p
                arrays[f"in_{start}_{nr}x{nc}/q"] = q

    # Fixed points for non-uniform marginals from an arbitrary init: the QR
    # problem is strongly convex, so the solution is unique.
    for (nr, nc) in [(12, 9), (40, 31)]:
        C = rng.random((nr, nc))
        p = rng.dirichlet(np.ones(nr))
        q = rng.dirichlet(np.ones(nc))
        rho, r_weight = 2.0, 5e-2
        s = rho / (nr + nc)
        x, log = regdrot(np.asfortranarray(np.outer(p, q)), np.asfortranarray(C), p, q, quad_prox,
                         max_iters=200000, eps_abs=1e-13, step=s, compute_r_primal=True,
                         return_log=True, reg=r_weight * (nr + nc))
        name = f"qr_fixedpoint_{nr}x{nc}"
        add(name, dict(kind="qr_fixedpoint", nr=nr, nc=nc, rho=rho, s=s, r_weight=r_weight,
                       iters=int(log["num_iters"])),
            C=C.T.copy(), p=p, q=q, x=np.asarray(x).T.copy())

    arrays["manifest"] = np.frombuffer(json.dumps(manifest).encode(), dtype=np.uint8)
    np.savez_compressed(OUT, **arrays)
    print(f"wrote {OUT}: {len(manifest)} cases")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: gen_golden.py /path/to/Regularized-DROT (the reference checkout)")
    main(sys.argv[1])
