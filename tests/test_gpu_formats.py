"""GPU: the benchmark pipeline's W2 evaluation through the GPU solver.

benchmark/utils/compute_w2_dist.py:59-94 adapts the source domain with a
plan and scores it by the within-class W2 distance, solving one
unregularised OT problem per class with reg_drot.quadratic_drot
(compute_w2_dist.py:86).  reg_drot.formats.group_w2_distance does the same
with the GPU solver by default; here it is run that way and against the
oracle as the solver, on plans from the GPU group-lasso solver for the
domain-adaptation problem (2-class Gaussian mixture source, affine-mapped
target, as benchmark/generate_da.py draws them; seeded synthetic data).
The two W2 totals must agree to 1e-4 relative: the per-class solves stop
on the same residual (2e-6) and their objectives agree to FP32 rounding.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from oracle import oracle as O  # noqa: E402


def _oracle_solver(c, p, q):
    from reg_drot import formats as F
    o = O.quadratic_drot(np.asarray(c, np.float32), np.asarray(p, np.float32),
                         np.asarray(q, np.float32), F.W2_RHO, 0.0, F.W2_MAX_ITERS, F.W2_EPS)
    return o["x"]


def _da_problem(ns, nt, seed):
    rng = np.random.default_rng(seed)
    xs = rng.normal(size=(ns, 2)) + np.where(np.arange(ns)[:, None] < ns // 2, -2.0, 2.0) * [1, 0]
    xt0 = rng.normal(size=(nt, 2)) + np.where(np.arange(nt)[:, None] < nt // 2, -2.0, 2.0) * [1, 0]
    A = np.eye(2) + 0.3 * rng.normal(size=(2, 2))
    xt = xt0 @ A.T + rng.normal(size=2)
    return xs.astype(np.float32), xt.astype(np.float32)


@pytest.mark.parametrize("gl_weight", [1e-3, 5e-3])
def test_w2_of_a_gpu_gl_plan_matches_oracle_evaluation(cuda, solver_lib, gl_weight):
    import reg_drot
    from reg_drot import formats as F
    ns, nt = 120, 80
    xs, xt = _da_problem(ns, nt, 31)
    c = ((xs[:, None, :].astype(np.float64) - xt[None, :, :]) ** 2).sum(-1)
    c = (c / c.max()).astype(np.float32)                 # [n_rows = source, n_cols = target]
    # GL solve in the reference wrapper's convention (drot_glr.hpp:385):
    # r_weight / sqrt(n_rows / G) = the operator's r' * sqrt(n_rows / G)
    k = ns // 2
    r_op = gl_weight / k
    ct = torch.tensor(np.ascontiguousarray(c.T), device=cuda)   # [n_cols, n_rows]
    p = torch.full((ns,), 1.0 / ns, device=cuda)
    q = torch.full((nt,), 1.0 / nt, device=cuda)
    x, info, _ = reg_drot.solve_gl(ct, p, q, 2, 2.0, r_op, 20000, 1e-6)
    assert info["converged"] == 1
    plan = x.cpu().numpy()                                # [n_target, n_source]
    total_gpu, norm_gpu = F.group_w2_distance(xt, plan, 2)
    total_cpu, norm_cpu = F.group_w2_distance(xt, plan, 2, solver=_oracle_solver)
    assert total_gpu == pytest.approx(total_cpu, rel=1e-4)
    assert norm_gpu == pytest.approx(norm_cpu, rel=1e-4)
    assert total_gpu > 0.0
