"""GPU: a device wait that runs out ends the launch with a status, and the
device stays usable.

The reference ignores every CUDA error (core/drot_glr.hpp:235 and the other
launch sites); here every grid barrier and mbarrier wait of the solver is
bounded by wall time (DROT_BARRIER_TIMEOUT_MS, 10 s by default): a CTA whose
wait runs out raises the launch's abort flag, every CTA leaves its loop, and
the host gets DROT_ERR_BARRIER_TIMEOUT (3).  No trap, no fault, no endless
wait.

The failure is made with the test hook DROT_TEST_STALL_CTA=k: CTA k does not
arrive at its first grid barrier, so that barrier is a flag nothing sets.
With DROT_BARRIER_TIMEOUT_MS=200 the launch gives up after ~0.2 s.  The next
solve on the same device (hook off) must be correct: it is checked against
the oracle with the parity bars of the other tests.
"""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from oracle import oracle as O  # noqa: E402

BARRIER_TIMEOUT = 3  # DROT_ERR_BARRIER_TIMEOUT


def _problem(nr, nc, seed):
    g = torch.Generator().manual_seed(seed)
    c = torch.rand(nc, nr, generator=g) + 1e-3
    c = c / c.max()
    return c, torch.ones(nr) / nr, torch.ones(nc) / nc


def _close(x, xo):
    x = np.asarray(x, np.float64)
    xo = np.asarray(xo, np.float64)
    assert np.linalg.norm(x - xo) <= 1e-5 * np.linalg.norm(xo)


@pytest.mark.parametrize("kind", ["qr", "gl"])
def test_single_solve_wait_runs_out_then_device_is_usable(cuda, solver_lib, monkeypatch, kind):
    import reg_drot
    c, p, q = _problem(1000, 700, 21)
    cd, pd, qd = c.to(cuda), p.to(cuda), q.to(cuda)
    monkeypatch.setenv("DROT_BARRIER_TIMEOUT_MS", "200")
    monkeypatch.setenv("DROT_TEST_STALL_CTA", "3")
    t0 = time.perf_counter()
    with pytest.raises(reg_drot.DrotError) as err:
        if kind == "qr":
            reg_drot.solve_qr(cd, pd, qd, 2.0, 1e-3, 20000, 1e-4)
        else:
            reg_drot.solve_gl(cd, pd, qd, 2, 2.0, 1e-3, 20000, 1e-4)
    waited = time.perf_counter() - t0
    assert err.value.status == BARRIER_TIMEOUT
    assert waited < 10.0  # the 0.2 s limit, not the 10 s default
    monkeypatch.delenv("DROT_TEST_STALL_CTA")
    monkeypatch.delenv("DROT_BARRIER_TIMEOUT_MS")
    if kind == "qr":
        x, info, _ = reg_drot.solve_qr(cd, pd, qd, 2.0, 1e-3, 20000, 1e-4)
        o = O.quadratic_drot(c.numpy(), p.numpy(), q.numpy(), 2.0, 1e-3, 20000, 1e-4)
    else:
        x, info, _ = reg_drot.solve_gl(cd, pd, qd, 2, 2.0, 1e-3, 20000, 1e-4)
        o = O.group_lasso_drot(c.numpy(), p.numpy(), q.numpy(), 2, 2.0, 1e-3, 20000, 1e-4,
                               dtype=np.float64)
    assert info["status"] == 0 and info["converged"] == 1
    if kind == "qr":
        o = O.quadratic_drot_matching(info["n_iter"], o, c.numpy(), p.numpy(), q.numpy(),
                                      2.0, 1e-3)
        _close(x.cpu().numpy(), o["x"])
    else:
        # the GL bar of the parity tests is relative to the FP32 oracle's
        # own distance from the FP64 solution; 1e-3 covers it on this input
        err64 = np.linalg.norm(x.cpu().numpy().astype(np.float64) - o["x"]) / \
            np.linalg.norm(o["x"])
        assert err64 <= 1e-3, err64


def test_batch_wait_runs_out_then_device_is_usable(cuda, solver_lib, monkeypatch):
    import reg_drot
    from reg_drot.batch import QRBatch
    shapes = [(300, 200), (513, 97), (1000, 700)]
    insts = [_problem(nr, nc, 40 + k) for k, (nr, nc) in enumerate(shapes)]
    B = QRBatch(shapes, 2.0, 1e-3, 1e-4, device=cuda, cols_per_tile=64)
    cb = B.pack_c([ci.to(cuda) for ci, _, _ in insts])
    pb, qb = B.pack_marginals([pi for _, pi, _ in insts], [qi for _, _, qi in insts])
    monkeypatch.setenv("DROT_BARRIER_TIMEOUT_MS", "200")
    monkeypatch.setenv("DROT_TEST_STALL_CTA", "5")
    with pytest.raises(reg_drot.DrotError) as err:
        B.solve(cb, pb, qb, 20000)
    assert err.value.status == BARRIER_TIMEOUT
    monkeypatch.delenv("DROT_TEST_STALL_CTA")
    monkeypatch.delenv("DROT_BARRIER_TIMEOUT_MS")
    x, info = B.solve(cb, pb, qb, 20000)
    for k, (ci, pi, qi) in enumerate(insts):
        o = O.quadratic_drot(ci.numpy(), pi.numpy(), qi.numpy(), 2.0, 1e-3, 20000, 1e-4)
        assert info[k]["converged"] == 1
        assert abs(info[k]["n_iter"] - o["n_iter"]) <= 2
        o = O.quadratic_drot_matching(info[k]["n_iter"], o, ci.numpy(), pi.numpy(), qi.numpy(),
                                      2.0, 1e-3)
        _close(B.view(x, k).cpu().numpy(), o["x"])
