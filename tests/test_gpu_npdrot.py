"""GPU: the numpy-API backend (reg_drot.npdrot) against the reference's own
numpy outputs (tests/golden, generated by importing numpy/npdrot).

Same calls as the reference's solvers (numpy/npdrot/solver.py:191-290):
quaddrot / l1l2drot(init, C, p, q, reg, [groups], max_iters=T-1, eps_abs=-1,
step=s, compute_r_primal=True) with the fixtures' inputs; FP32 device
iterates against numpy's FP64, 1e-5 relative (Frobenius and max entry 1e-4).
The stop test is checked against an FP64 emulation of regdrot's loop
(residual <= eps every iteration) on the oracle.
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from oracle import oracle as O  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden", "npdrot_golden.npz")


def _rel(a, b):
    return (np.linalg.norm(a - b) / np.linalg.norm(b), np.abs(a - b).max() / np.abs(b).max())


def test_numpy_api_matches_reference_numpy_outputs(cuda, solver_lib):
    from reg_drot import npdrot
    z = np.load(GOLD)
    manifest = json.loads(bytes(z["manifest"]).decode())
    cases = [m for m in manifest if m.get("kind") in ("qr", "gl") and m["T"] >= 2]
    assert len(cases) >= 20
    for m in cases:
        inp = m["inputs"]
        C = z[f"{inp}/C"].T  # F-ordered nr x nc, as regdrot asserts
        p, q = z[f"{inp}/p"], z[f"{inp}/q"]
        nr, nc, T, s = m["nr"], m["nc"], m["T"], m["s"]
        init = np.outer(p, q) if m["start"] == "cold" else np.full((nr, nc), s)
        kw = dict(max_iters=T - 1, eps_abs=-1.0, step=s, compute_r_primal=True)
        if m["kind"] == "qr":
            x = npdrot.quaddrot(np.asfortranarray(init), C, p, q, m["r_weight"] * (nr + nc), **kw)
        else:
            b = m["bounds"]
            groups = [(b[g], b[g + 1]) for g in range(len(b) - 1)]
            x = npdrot.l1l2drot(np.asfortranarray(init), C, p, q, m["lam"] / s, groups, **kw)
        ref = z[f"{m['name']}/x"].T
        fro, mx = _rel(x, ref)
        assert fro <= 1e-5 and mx <= 1e-4, (m["name"], fro, mx)


def _numpy_loop_iterations(C, p, q, s, kappa, eps, max_iters):
    """regdrot's loop restated on the FP64 oracle, one iteration per call:
    the number of loop iterations until the primal residual is <= eps."""
    nr, nc = len(p), len(q)
    st = O.initial_state(nr, nc, s, p, q, warm=False, dtype=np.float64)
    for k in range(max_iters):
        o = O.qr_solve(C, p, q, s, kappa, 1, -1.0, state=st, dtype=np.float64)
        st = {key: o[key] for key in ("x", "a", "b", "phi1", "phi2", "alpha")}
        # each one-iteration call is an even step (it reads C and stores the
        # folded X^ - sC): undo the fold before the next call
        st["x"] = np.maximum(st["x"] + s * C, 0.0)
        if o["residual"] <= eps:
            return k + 1
    return max_iters


@pytest.mark.parametrize("nr,nc,seed", [(30, 40, 1), (64, 33, 2)])
def test_numpy_api_stop_rule(cuda, solver_lib, nr, nc, seed):
    from reg_drot import npdrot
    rng = np.random.default_rng(seed)
    C = np.asfortranarray(rng.random((nr, nc)))
    p = rng.dirichlet(np.ones(nr))
    q = rng.dirichlet(np.ones(nc))
    s = 2.0 / (nr + nc)
    reg = 1e-2 * (nr + nc)
    x, log = npdrot.quaddrot(np.asfortranarray(np.outer(p, q)), C, p, q, reg, max_iters=5000,
                             eps_abs=1e-5, compute_r_primal=True, return_log=True)
    k_ref = _numpy_loop_iterations(np.ascontiguousarray(C.T), p, q, s, 1.0 + s * reg, 1e-5, 5000)
    assert abs(log["num_iters"] - k_ref) <= 1, (log["num_iters"], k_ref)
    assert log["primal"][0] <= 1e-5
    # the plan satisfies the marginals to the tolerance
    r = np.sqrt(((x.sum(1) - p) ** 2).sum() + ((x.sum(0) - q) ** 2).sum())
    assert r <= 2e-5
