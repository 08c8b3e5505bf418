"""Time the reference's own numpy solver beside the oracle port on the
CPU-runnable QR workload -- a measurement recipe, run where the reference
checkout exists (its sources do not travel to the GPU host, so this CPU
baseline is measured in the build container).

Workload: QR DROT, m = n = 1000, x_i, y_j ~ N(0, I_2) from numpy
default_rng(1234), C = squared Euclidean / max(C), p = q = 1/1000,
alpha (r_weight) = 1e-3, rho = 2, stop at the absolute marginal residual
1e-4 * ||(p; q)||_2 (relative 1e-4).

  reference  npdrot.quaddrot (numpy/npdrot/solver.py:262-290, loop 7-189)
             with numba=False (numba is not installed; a stand-in module
             makes the package importable, as for the golden vectors),
             reg = alpha * (m + n) and init = s * ones -- the CUDA warm start
             for uniform marginals (tests/golden/gen_golden.py explains the
             mapping); numpy/BLAS threads as the environment sets them.
  port       the oracle's FP32 loop (C, OpenMP on every core) on the same
             problem: oracle.quadratic_drot.

Usage: python oracle/time_reference_numpy.py /path/to/Regularized-DROT
Prints one JSON line.
"""
import json
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, REPO)


def problem():
    rng = np.random.default_rng(1234)
    xs = rng.normal(size=(1000, 2))
    yt = rng.normal(size=(1000, 2))
    c = ((yt[:, None, :] - xs[None, :, :]) ** 2).sum(-1)  # [n_cols, n_rows]
    c = c / c.max()
    p = np.full(1000, 1e-3)
    eps = 1e-4 * math.sqrt(2 * 1000 * 1e-6)
    return c, p, p.copy(), eps


def main(ref_root):
    from oracle import oracle as O
    sys.path.insert(0, os.path.join(REPO, "tests", "golden", "numba_standin"))
    sys.path.insert(0, os.path.join(ref_root, "numpy"))
    from npdrot.solver import quaddrot  # noqa: E402

    c, p, q, eps = problem()
    m, n = len(p), len(q)
    rho, alpha = 2.0, 1e-3
    s = rho / (m + n)
    C = np.asfortranarray(c.T)  # numpy's layout: rows = p, F-contiguous
    init = np.asfortranarray(np.full((m, n), s))
    t0 = time.perf_counter()
    x, log = quaddrot(init, C, p, q, alpha * (m + n), numba=False, max_iters=100000,
                      eps_abs=eps, step=s, compute_r_primal=True, return_log=True)
    t_ref = time.perf_counter() - t0
    it_ref = int(log["num_iters"])

    c32, p32 = c.astype(np.float32), p.astype(np.float32)
    O.quadratic_drot(c32, p32, p32, rho, alpha, 10, eps)  # page in, spin up threads
    t0 = time.perf_counter()
    o = O.quadratic_drot(c32, p32, p32, rho, alpha, 10 ** 6, eps)
    t_port = time.perf_counter() - t0
    err = float(np.linalg.norm(o["x"].T - x) / np.linalg.norm(x))
    print(json.dumps({
        "workload": "QR-DROT 1000x1000, N(0,I_2) clouds, C = sq. Euclidean / max, uniform "
                    "marginals, alpha 1e-3, rho 2, relative eps 1e-4",
        "reference_numpy": {"s_per_solve": t_ref, "iterations": it_ref,
                            "ms_per_iteration": 1e3 * t_ref / it_ref,
                            "threads": os.environ.get("OMP_NUM_THREADS", "default")},
        "oracle_port": {"s_per_solve": t_port, "iterations": o["n_iter"],
                        "ms_per_iteration": 1e3 * t_port / o["n_iter"],
                        "threads": int(O.lib().oracle_max_threads())},
        "plans_relative_difference": err, "cpu_count": os.cpu_count()}))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: time_reference_numpy.py /path/to/Regularized-DROT")
    main(sys.argv[1])
