"""GPU: the dense quadratic-regularised workloads against the FP64 oracle.

Workload: m = n = 3000 and 10000, C ~ U[0,1) float32, p, q ~ Dirichlet(1)
(numpy default_rng(1234)), rho = 2, r_weight (alpha) in {1e-4, 1e-3, 1e-2},
C stored in FP32 and in BF16 (FP32 iterates; the solve is the FP32 solve of
the BF16-rounded cost, so the oracles run on that rounded cost).  Seeded
synthetic inputs stand in for the reference's data.

Fixed-length cells.  Each (size, alpha, storage) cell runs T DR iterations
from the warm start (T = 2000 at 3000^2, T = 200 at 10000^2; the oracle's
cost bounds them) with the stop test off, on the GPU (the drop-in operator's
C-ABI entry point drot_quadratic_drot_ex, reg_drot.solve_qr) and in the FP32
and FP64 oracles (core/drot_qr.hpp:159-234 restated).  T is even, so the
last iteration is odd and X is returned unfolded.  The bars, with e32 the
FP32 oracle's own relative error against FP64 (the reference's FP32
arithmetic drifts 1.3e-5 .. 2.4e-5 from FP64 over 2000 iterations at
3000^2):
  * ||X - X64||_F / ||X64||_F       <= max(1e-5, 2 e32)
  * ||X - X32||_F / ||X32||_F       <= max(1e-5, 2 e32)
  * |obj - obj64| / |obj64|          <= max(1e-5, 2 x the FP32 oracle's)
  * |res - res64| / res64            <= max(1e-4, 2 x the FP32 oracle's)
                                       (the absolute marginal residual of the
                                       last stop check, here iteration T-2;
                                       near the stop it is a small difference
                                       of large sums, so FP32 holds fewer of
                                       its digits)
Each error is printed (pytest -s) so the measured figures can be quoted.

Converged cell.  3000^2, alpha = 1e-2, FP32 C, stopped at the relative
marginal residual 1e-4 (absolute eps = 1e-4 ||(p; q)||_2): the GPU solve
against the FP32 and FP64 oracles stopped at the GPU's iteration
(oracle.quadratic_drot_at), with the same bars, and the GPU's residual below
eps (reported and recomputed from X).
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from oracle import oracle as O  # noqa: E402

RHO = 2.0
SEED = 1234
REL_EPS = 1e-4
ITERS = {3000: 2000, 10000: 200}

_cache = {}


def _problem(n):
    """C ~ U[0,1) [n, n] float32 (layout [n_cols, n_rows]), p, q ~ Dirichlet(1)."""
    if n not in _cache:
        rng = np.random.default_rng(SEED)
        c = rng.random((n, n), dtype=np.float32)
        p = rng.dirichlet(np.ones(n)).astype(np.float32)
        q = rng.dirichlet(np.ones(n)).astype(np.float32)
        _cache.clear()
        _cache[n] = (c, p, q)
    return _cache[n]


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _check_cell(tag, x, info, o32, o64):
    e32 = _rel(o32["x"], o64["x"])
    e_gpu = _rel(x, o64["x"])
    e_gpu32 = _rel(x, o32["x"])
    obj32 = abs(o32["objective"] - o64["objective"]) / abs(o64["objective"])
    obj_gpu = abs(info["objective_f64"] - o64["objective"]) / abs(o64["objective"])
    res_gpu = abs(info["residual"] - o64["residual"]) / o64["residual"]
    res32 = abs(o32["residual"] - o64["residual"]) / o64["residual"]
    print(f"\n[config2] {tag}: X vs FP64 {e_gpu:.3e} (FP32 oracle {e32:.3e}), X vs FP32 oracle "
          f"{e_gpu32:.3e}, objective vs FP64 {obj_gpu:.3e} (FP32 oracle {obj32:.3e}), "
          f"residual {info['residual']:.6e} vs FP64 {o64['residual']:.6e} ({res_gpu:.2e}; FP32 "
          f"oracle {res32:.2e})")
    bar = max(1e-5, 2.0 * e32)
    assert e_gpu <= bar, (e_gpu, e32)
    assert e_gpu32 <= bar, (e_gpu32, e32)
    assert obj_gpu <= max(1e-5, 2.0 * obj32), (obj_gpu, obj32)
    assert res_gpu <= max(1e-4, 2.0 * res32), (res_gpu, res32)


@pytest.mark.parametrize("store", ["fp32", "bf16"])
@pytest.mark.parametrize("alpha", [1e-4, 1e-3, 1e-2])
@pytest.mark.parametrize("n", [3000, 10000])
def test_fixed_length_solve_against_fp64_oracle(cuda, solver_lib, n, alpha, store):
    import reg_drot
    c, p, q = _problem(n)
    T = ITERS[n]
    cd = torch.from_numpy(c).to(cuda)
    if store == "bf16":
        cd = cd.to(torch.bfloat16)
        c = cd.float().cpu().numpy()  # the cost the BF16 solve uses
    pd, qd = torch.from_numpy(p).to(cuda), torch.from_numpy(q).to(cuda)
    x, info, _ = reg_drot.solve_qr(cd, pd, qd, RHO, alpha, T, 0.0)
    assert info["status"] == 0 and info["iters_run"] == T and info["converged"] == 0
    xh = x.cpu().numpy()
    del x, cd
    o32 = O.quadratic_drot(c, p, q, RHO, alpha, T, 0.0)
    o64 = O.quadratic_drot(c, p, q, RHO, alpha, T, 0.0, dtype=np.float64)
    _check_cell(f"{n}^2 alpha {alpha:g} {store}, {T} iterations", xh, info, o32, o64)


def test_converged_solve_against_fp64_oracle(cuda, solver_lib):
    import reg_drot
    n, alpha = 3000, 1e-2
    c, p, q = _problem(n)
    eps = REL_EPS * math.sqrt(float((p.astype(np.float64) ** 2).sum() +
                                    (q.astype(np.float64) ** 2).sum()))
    cd, pd, qd = (torch.from_numpy(a).to(cuda) for a in (c, p, q))
    x, info, _ = reg_drot.solve_qr(cd, pd, qd, RHO, alpha, 10 ** 7, eps)
    assert info["status"] == 0 and info["converged"] == 1
    assert info["residual"] < eps
    resid = torch.sqrt(torch.sum((pd.double() - x.double().sum(0)) ** 2) +
                       torch.sum((qd.double() - x.double().sum(1)) ** 2)).item()
    assert resid <= eps * 1.001, (resid, eps)
    xh = x.cpu().numpy()
    o32 = O.quadratic_drot_at(c, p, q, RHO, alpha, info["n_iter"])
    o64 = O.quadratic_drot_at(c, p, q, RHO, alpha, info["n_iter"], dtype=np.float64)
    print(f"\n[config2] converged 3000^2 alpha 1e-2: n_iter {info['n_iter']}, residual "
          f"{info['residual']:.4e} (eps {eps:.4e}, recomputed {resid:.4e})")
    _check_cell(f"3000^2 alpha 1e-2 fp32, converged at {info['n_iter']}", xh, info, o32, o64)
