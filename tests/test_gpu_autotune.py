"""GPU: the single-instance autotuner (reg_drot.tune, drot_set_launch_choice).

tune() times the candidate launch shapes on the caller's data and pins the
fastest; a pinned shape changes only how the FP32 partial sums are grouped,
so the tuned solve meets the parity bars against the oracle (X within 1e-5
relative, the same stop within one check) and pinned shapes that the
planner cannot use are refused on the host.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from oracle import oracle as O  # noqa: E402


def _problem(nr, nc, seed):
    g = torch.Generator().manual_seed(seed)
    c = torch.rand(nc, nr, generator=g) + 1e-3
    c = c / c.max()
    rng = np.random.default_rng(seed)
    p = torch.from_numpy(rng.dirichlet(np.ones(nr)).astype(np.float32))
    q = torch.from_numpy(rng.dirichlet(np.ones(nc)).astype(np.float32))
    return c, p, q


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("kind", ["qr", "gl"])
def test_tuned_solve_matches_oracle(cuda, solver_lib, kind):
    import reg_drot
    from reg_drot import autotune
    nr, nc = 1200, 800
    c, p, q = _problem(nr, nc, 3)
    cd, pd, qd = c.to(cuda), p.to(cuda), q.to(cuda)
    try:
        best, timings = reg_drot.tune(kind, cd, pd, qd, 2.0, 1e-3, n_class=2, iters=40)
        assert len(timings) >= 9 and best in [t[0] for t in timings]
        if kind == "qr":
            x, info, _ = reg_drot.solve_qr(cd, pd, qd, 2.0, 1e-3, 200000, 1e-5)
            o = O.quadratic_drot(c.numpy(), p.numpy(), q.numpy(), 2.0, 1e-3, 200000, 1e-5)
            assert abs(info["n_iter"] - o["n_iter"]) <= 2
            o = O.quadratic_drot_matching(info["n_iter"], o, c.numpy(), p.numpy(), q.numpy(),
                                          2.0, 1e-3)
            assert _rel(x.cpu().numpy(), o["x"]) <= 1e-5
        else:
            x, info, _ = reg_drot.solve_gl(cd, pd, qd, 2, 2.0, 1e-3, 20000, 1e-4)
            o32 = O.group_lasso_drot(c.numpy(), p.numpy(), q.numpy(), 2, 2.0, 1e-3, 20000, 1e-4)
            o64 = O.group_lasso_drot(c.numpy(), p.numpy(), q.numpy(), 2, 2.0, 1e-3, 20000, 1e-4,
                                     dtype=np.float64)
            ref = _rel(o32["x"], o64["x"])
            assert _rel(x.cpu().numpy(), o64["x"]) <= max(1e-5, 2 * ref)
        assert info["converged"] == 1
    finally:
        autotune.clear()


def test_every_pinned_shape_solves_the_same_problem(cuda, solver_lib):
    """Fixed-iteration solves under several pinned shapes agree with the
    default plan to FP32 rounding of the regrouped partial sums."""
    import reg_drot
    from reg_drot import autotune
    nr, nc = 1000, 600
    c, p, q = (t.to(cuda) for t in _problem(nr, nc, 8))
    x0, _, _ = reg_drot.solve_qr(c, p, q, 2.0, 1e-3, 300, 0.0)
    x0 = x0.clone()
    try:
        for kv, w, path, ct in ((1, 4, 0, 0), (2, 16, 0, 0), (4, 8, 1, 1), (4, 16, 1, 2)):
            autotune.pin("qr", nr, nc, vectors_per_lane=kv, warps_per_cta=w, data_path=path,
                         ctas_per_sm=ct)
            x, info, _ = reg_drot.solve_qr(c, p, q, 2.0, 1e-3, 300, 0.0)
            assert info["iters_run"] == 300
            assert _rel(x.cpu().numpy(), x0.cpu().numpy()) <= 1e-5, (kv, w, path, ct)
    finally:
        autotune.clear()


def test_invalid_pins_are_refused(cuda, solver_lib):
    from reg_drot import autotune
    with pytest.raises(RuntimeError):
        autotune.pin("qr", 100, 100, vectors_per_lane=8)   # QR has no 8-vector kernel
    with pytest.raises(RuntimeError):
        autotune.pin("qr", 100, 100, warps_per_cta=3)
    with pytest.raises(RuntimeError):
        autotune.pin("gl", 100, 0, 2)                       # one of n_rows, n_cols zero
    autotune.clear()
