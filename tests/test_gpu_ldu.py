"""GPU: the single-barrier kernels (DROT_LDU=1, QR and GL) against the oracle.

These kernels are opt-in and not yet measured, so this module runs only when
DROT_TEST_LDU=1 is set.  The bars are those of the default kernels
(tests/test_gpu_parity.py): the element arithmetic is the same; the row and
column sums are the same partials added in a different fixed order, so the
iterates agree to FP32 rounding, the objective to 1e-5 relative and the
iteration count within one stop check.  Runs are bitwise repeatable and
match the two-barrier kernels to the same bars.
"""
import os

import numpy as np
import pytest

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(os.environ.get("DROT_TEST_LDU") != "1",
                                 reason="single-barrier kernels: set DROT_TEST_LDU=1")]

torch = pytest.importorskip("torch")

from oracle import oracle as O  # noqa: E402

RTOL_X = 1e-5
RTOL_XMAX = 1e-4
RTOL_OBJ = 1e-5


def _problem(nr, nc, seed):
    g = torch.Generator().manual_seed(seed)
    c = torch.rand(nc, nr, generator=g, dtype=torch.float32) + 1e-3
    c = c / c.max()
    rng = np.random.default_rng(seed)
    p = torch.from_numpy(rng.dirichlet(np.ones(nr)).astype(np.float32))
    q = torch.from_numpy(rng.dirichlet(np.ones(nc)).astype(np.float32))
    return c, p, q


def _close(x, xo):
    x = np.asarray(x, np.float64)
    xo = np.asarray(xo, np.float64)
    assert np.linalg.norm(x - xo) <= RTOL_X * np.linalg.norm(xo)
    assert np.abs(x - xo).max() <= RTOL_XMAX * np.abs(xo).max()


@pytest.fixture(params=["4", "2"])
def ldu(request, monkeypatch):
    monkeypatch.setenv("DROT_LDU", "1")
    monkeypatch.setenv("DROT_QR_KV", request.param)  # 512- and 256-row bands
    return request.param


@pytest.mark.parametrize("nr,nc", [(1000, 700), (3000, 3000), (512, 2049), (4096, 100)])
def test_ldu_converged_matches_oracle(cuda, solver_lib, ldu, nr, nc):
    import reg_drot
    c, p, q = _problem(nr, nc, nr + nc)
    x, info, _ = reg_drot.solve_qr(c.to(cuda), p.to(cuda), q.to(cuda), 2.0, 1e-3, 20000, 1e-6)
    o = O.quadratic_drot(c.numpy(), p.numpy(), q.numpy(), 2.0, 1e-3, 20000, 1e-6)
    assert info["converged"] == 1
    assert abs(info["n_iter"] - o["n_iter"]) <= 2
    if info["n_iter"] == o["n_iter"]:
        _close(x.cpu().numpy(), o["x"])
        assert abs(info["objective"] - o["objective"]) <= RTOL_OBJ * abs(o["objective"])


@pytest.mark.parametrize("mi", [1, 2, 7, 30])
def test_ldu_fixed_iterations_match_oracle(cuda, solver_lib, ldu, mi):
    import reg_drot
    c, p, q = _problem(1000, 700, 5)
    x, info, _ = reg_drot.solve_qr(c.to(cuda), p.to(cuda), q.to(cuda), 2.0, 1e-3, mi, 0.0)
    o = O.quadratic_drot(c.numpy(), p.numpy(), q.numpy(), 2.0, 1e-3, mi, 0.0)
    assert info["iters_run"] == mi and info["n_iter"] == mi + 1
    floor = float(np.linalg.norm(p.numpy()) * np.linalg.norm(q.numpy()))
    xg = x.cpu().numpy().astype(np.float64)
    xo = np.asarray(o["x"], np.float64)
    assert np.linalg.norm(xg - xo) <= RTOL_X * max(np.linalg.norm(xo), floor)


def test_ldu_is_deterministic_and_matches_two_barrier_kernels(cuda, solver_lib, ldu, monkeypatch):
    import reg_drot
    c, p, q = (t.to(cuda) for t in _problem(1200, 900, 11))
    x1, i1, _ = reg_drot.solve_qr(c, p, q, 2.0, 1e-3, 20000, 1e-6)
    x2, i2, _ = reg_drot.solve_qr(c, p, q, 2.0, 1e-3, 20000, 1e-6)
    assert torch.equal(x1, x2) and i1["n_iter"] == i2["n_iter"]
    monkeypatch.setenv("DROT_LDU", "0")
    x3, i3, _ = reg_drot.solve_qr(c, p, q, 2.0, 1e-3, 20000, 1e-6)
    assert abs(i1["n_iter"] - i3["n_iter"]) <= 2
    if i1["n_iter"] == i3["n_iter"]:
        _close(x1.cpu().numpy(), x3.cpu().numpy())


@pytest.mark.parametrize("nr,nc,G", [(1500, 1000, 2), (600, 300, 2), (1001, 200, 3)])
def test_ldu_group_lasso_matches_fp64_oracle(cuda, solver_lib, monkeypatch, nr, nc, G):
    # The bar of the default GL kernels: within max(1e-5, 2 x the FP32
    # oracle's own error) of the FP64 oracle on X and the objective.
    import reg_drot
    monkeypatch.setenv("DROT_LDU", "1")
    c, p, q = _problem(nr, nc, nr * 11 + nc + G)
    x, info, _ = reg_drot.solve_gl(c.to(cuda), p.to(cuda), q.to(cuda), G, 2.0, 1e-3, 20000, 1e-4)
    o32 = O.group_lasso_drot(c.numpy(), p.numpy(), q.numpy(), G, 2.0, 1e-3, 20000, 1e-4)
    o64 = O.group_lasso_drot(c.numpy(), p.numpy(), q.numpy(), G, 2.0, 1e-3, 20000, 1e-4,
                             dtype=np.float64)
    assert info["status"] == 0 and info["converged"] == 1
    assert abs(info["n_iter"] - o32["n_iter"]) <= max(1, o32["n_iter"] // 50)
    x64 = o64["x"]
    ref_err = np.linalg.norm(o32["x"] - x64) / np.linalg.norm(x64)
    err = np.linalg.norm(x.cpu().numpy().astype(np.float64) - x64) / np.linalg.norm(x64)
    assert err <= max(RTOL_X, 2.0 * ref_err), (err, ref_err)
